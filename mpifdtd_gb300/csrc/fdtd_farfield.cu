// fdtd_farfield.cu -- far-field outputs computed from the engine's state.
//
//   spectrum  : ntffTM_TimeOutput / ntffTE_TimeOutput (ntffTM.c:197-275,
//               ntffTE.c:160-238): time-domain far field E_theta (TM) or E_phi
//               (TE) from the U/W accumulators (ntffTM.c:161-194,
//               ntffTE.c:20-55), zero-padded 8192-point FFT per angle with the
//               sign of cfft() (cfft.c:104-179: X[k] = sum x[n] e^{+2 pi i nk/N},
//               no scaling), |E|^2 at 380..700 nm by linear interpolation.
//   frequency : ntffTM_Frequency (ntffTM.c:72-158) / ntffTE_Frequency
//               (ntffTE.c:242-338) on the current fields.
//
// One block per angle.  The FFT runs in shared memory (8192 complex doubles =
// 128 KB): radix-2 decimation in time after a bit-reversal load.
#include <cuda_runtime.h>

#include "fdtd_internal.cuh"

namespace fdtd {

// 360 x 321 spectrum; twiddles w_k = e^{+2 pi i k / 8192}, k < 4096, from the host libm.
__global__ void __launch_bounds__(1024) spectrum_kernel(SpectrumView s)
{
  extern __shared__ double2 buf[];
  const int ang = blockIdx.x;
  const int nlog = 13;
  const double2 *u0 = s.acc[0] + kGuard + (size_t)ang * s.array_size;
  const double2 *u1 = s.acc[1] + kGuard + (size_t)ang * s.array_size;
  const double2 *u2 = s.acc[2] + kGuard + (size_t)ang * s.array_size;
  const double2 d = s.dir[ang];  // (cos phi, sin phi) with the solver's own rounding of phi
  const double px = -d.y, py = d.x, sz = -1.0;  // theta = 0 (ntffTM.c:174-178)
  for (int n = threadIdx.x; n < kNfft; n += blockDim.x) {
    double2 e = make_double2(0.0, 0.0);
    if (n < s.max_time) {
      double2 w;  // the bracket of ETH (TM) or EPH (TE)
      if (s.tm) {  // ETH = coef (-Z0 WTH - UPH), WTH = Wz sz, UPH = Ux px + Uy py
        const double2 ux = u0[n], uy = u1[n], wz = u2[n];
        const double uphr = ux.x * px + uy.x * py, uphi = ux.y * px + uy.y * py;
        w.x = -s.z0 * (wz.x * sz) - uphr;
        w.y = -s.z0 * (wz.y * sz) - uphi;
      } else {     // EPH = coef (-Z0 WPH + UTH), WPH = Wx px + Wy py, UTH = Uz sz
        const double2 wx = u0[n], wy = u1[n], uz = u2[n];
        const double wphr = wx.x * px + wy.x * py, wphi = wx.y * px + wy.y * py;
        w.x = -s.z0 * wphr + uz.x * sz;
        w.y = -s.z0 * wphi + uz.y * sz;
      }
      e.x = s.coef.x * w.x - s.coef.y * w.y;
      e.y = s.coef.x * w.y + s.coef.y * w.x;
    }
    buf[__brev(n) >> (32 - nlog)] = e;
  }
  __syncthreads();
  for (int len = 2, tw = kNfft / 2; len <= kNfft; len <<= 1, tw >>= 1) {
    const int half = len >> 1;
    for (int q = threadIdx.x; q < kNfft / 2; q += blockDim.x) {
      const int grp = q / half, k = q - grp * half;
      const int i0 = grp * len + k, i1 = i0 + half;
      const double2 w = s.twiddle[k * tw];
      const double2 a = buf[i0], b = buf[i1];
      const double2 v = make_double2(b.x * w.x - b.y * w.y, b.x * w.y + b.y * w.x);
      buf[i0] = make_double2(a.x + v.x, a.y + v.y);
      buf[i1] = make_double2(a.x - v.x, a.y - v.y);
    }
    __syncthreads();
  }
  for (int l = threadIdx.x; l <= kLambdaEn - kLambdaSt; l += blockDim.x) {
    const int lam = kLambdaSt + l;
    double p = s.c0 * s.h_u_nm * kNfft / lam;  // ntffTM.c:227
    const int idx = (int)floor(p);
    p = p - idx;
    const double2 a = buf[idx], b = buf[idx + 1];
    const double na = a.x * a.x + a.y * a.y, nb = b.x * b.x + b.y * b.y;
    s.out[(size_t)l * 360 + ang] = ((1 - p) * na + p * nb) / kNfft;
  }
}

// Frequency-domain NTFF of the current fields, one block per angle; global
// cell (x, y) is array cell (x-ox, y-ox).
//   TM (ntffTM.c:72-158): N_z, L_x, L_y over the four sides lt..rt-1 /
//     bm..tp-1, path points on the cell (r2 = (i-cx, j-cy)); bottom/right add,
//     top/left subtract; E = coef (Z0 N_z + L_phi) sqrt(h_u).
//   TE (ntffTE.c:242-338): N_x, N_y, L_z; the bottom side runs lt..rt
//     inclusive, points half a cell along the side (i-cx+0.5 / j-cy+0.5);
//     bottom/right subtract, top/left add; E_phi = coef (Z0 N_phi - L_z) h_u.
//     All four sides use the global index (the shipped function reads three
//     of them through field_subIndex, whose SUB_N_PY is never set: field.c:112).
__device__ __forceinline__ double2 cexp_i(double ph)
{
  double sn, cs;
  sincos(ph, &sn, &cs);
  return make_double2(cs, sn);
}

// complex sample of an FP64 (double2) or FP32 (float2) field, widened to FP64
__device__ __forceinline__ double2 load_c(const void *p, long long k, int f32)
{
  if (f32) {
    const float2 v = ((const float2 *)p)[k];
    return make_double2(v.x, v.y);
  }
  return ((const double2 *)p)[k];
}

__global__ void __launch_bounds__(256) frequency_kernel(FrequencyView f)
{
  __shared__ double red[6][256];
  const int ang = blockIdx.x;
  const double2 d = f.dir[ang];
  const double rx = d.x, ry = d.y;
  // a0: N_z (TM) | L_z (TE) ; a1: L_x | N_x (bottom/top) ; a2: L_y | N_y (right/left)
  double a0r = 0, a0i = 0, a1r = 0, a1i = 0, a2r = 0, a2i = 0;
  const int te = f.tm ? 0 : 1;
  const int nb = f.rt - f.lt, nr = f.tp - f.bm, n0 = nb + te;  // bottom: rt inclusive for TE
  const int ncell = n0 + nb + 2 * nr;
  const double half = te ? 0.5 : 0.0;
  for (int c = threadIdx.x; c < ncell; c += blockDim.x) {
    int x, y, side;
    if (c < n0) { side = 0; x = f.lt + c; y = f.bm; }
    else if (c < n0 + nr) { side = 1; x = f.rt; y = f.bm + (c - n0); }
    else if (c < n0 + nb + nr) { side = 2; x = f.lt + (c - n0 - nr); y = f.tp; }
    else { side = 3; x = f.lt; y = f.bm + (c - n0 - nb - nr); }
    const bool horiz = side == 0 || side == 2;
    const long long k = (long long)(x - f.ox) * f.P + (y - f.ox);
    const long long hoff = horiz ? -1 : -(long long)f.P;
    const void *hp = f.h[horiz ? 0 : 1];
    const double2 ef = load_c(f.e[horiz ? 0 : 1], k, f.f32);
    const double2 ha = load_c(hp, k, f.f32), hb = load_c(hp, k + hoff, f.f32);
    const double hr = 0.5 * (ha.x + hb.x), hi = 0.5 * (ha.y + hb.y);
    const double r2x = horiz ? __dadd_rn((double)x - f.cx, half) : (double)x - f.cx;
    const double r2y = horiz ? (double)y - f.cy : __dadd_rn((double)y - f.cy, half);
    const double inner = __dadd_rn(__dmul_rn(rx, r2x), __dmul_rn(ry, r2y));
    const double2 e = cexp_i(f.k_s * inner);
    double sg = side < 2 ? 1.0 : -1.0;  // TM: bottom/right add, top/left subtract
    if (te) sg = -sg;                   // TE: the other way round
    const double nr_ = sg * (hr * e.x - hi * e.y), ni_ = sg * (hr * e.y + hi * e.x);
    const double er = sg * (ef.x * e.x - ef.y * e.y), ei = sg * (ef.x * e.y + ef.y * e.x);
    if (!te) {
      a0r += nr_; a0i += ni_;
      if (horiz) { a1r += er; a1i += ei; } else { a2r += er; a2i += ei; }
    } else {
      a0r += er; a0i += ei;
      if (horiz) { a1r += nr_; a1i += ni_; } else { a2r += nr_; a2i += ni_; }
    }
  }
  red[0][threadIdx.x] = a0r; red[1][threadIdx.x] = a0i;
  red[2][threadIdx.x] = a1r; red[3][threadIdx.x] = a1i;
  red[4][threadIdx.x] = a2r; red[5][threadIdx.x] = a2i;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int q = 0; q < 6; q++) red[q][threadIdx.x] += red[q][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    // phi component of the bottom/top (x) and right/left (y) sums: -x sin + y cos
    const double pr = -red[2][0] * ry + red[4][0] * rx, pi = -red[3][0] * ry + red[5][0] * rx;
    double br, bi;
    if (!te) { br = f.z0 * red[0][0] + pr; bi = f.z0 * red[1][0] + pi; }   // Z0 N_z + L_phi
    else     { br = f.z0 * pr - red[0][0]; bi = f.z0 * pi - red[1][0]; }    // Z0 N_phi - L_z
    f.out[ang] = make_double2((f.coef.x * br - f.coef.y * bi) * f.scale, (f.coef.x * bi + f.coef.y * br) * f.scale);
  }
}

void launch_spectrum(const SpectrumView &s, cudaStream_t st)
{
  const size_t smem = sizeof(double2) * kNfft;
  static bool configured = false;
  if (!configured) {
    cudaFuncSetAttribute(spectrum_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    configured = true;
  }
  spectrum_kernel<<<360, 1024, smem, st>>>(s);
}

void launch_frequency(const FrequencyView &f, cudaStream_t st) { frequency_kernel<<<360, 256, 0, st>>>(f); }

// A few field samples at given array indices (the elliptic ring's bilinear corners).
__global__ void point_gather_kernel(const void *field, int f32, const long long *idx, int n, double2 *out)
{
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) out[q] = load_c(field, idx[q], f32);
}

void launch_point_gather(const void *field, int f32, const long long *idx, int n, double2 *out, cudaStream_t st)
{
  if (n > 0) point_gather_kernel<<<(n + 255) / 256, 256, 0, st>>>(field, f32, idx, n, out);
}

}  // namespace fdtd
