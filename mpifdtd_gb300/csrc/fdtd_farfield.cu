// fdtd_farfield.cu -- far-field outputs computed from the engine's state.
//
//   spectrum  : ntffTM_TimeOutput / ntffTE_TimeOutput (ntffTM.c:197-275,
//               ntffTE.c:160-238): time-domain far field E_theta (TM) or E_phi
//               (TE) from the U/W accumulators (ntffTM.c:161-194,
//               ntffTE.c:20-55), zero-padded 8192-point FFT per angle with the
//               sign of cfft() (cfft.c:104-179: X[k] = sum x[n] e^{+2 pi i nk/N},
//               no scaling), |E|^2 at 380..700 nm by linear interpolation.
//   frequency : ntffTM_Frequency (ntffTM.c:72-158) on the current fields.
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
        w.x = -kZ0 * (wz.x * sz) - uphr;
        w.y = -kZ0 * (wz.y * sz) - uphi;
      } else {     // EPH = coef (-Z0 WPH + UTH), WPH = Wx px + Wy py, UTH = Uz sz
        const double2 wx = u0[n], wy = u1[n], uz = u2[n];
        const double wphr = wx.x * px + wy.x * py, wphi = wx.y * px + wy.y * py;
        w.x = -kZ0 * wphr + uz.x * sz;
        w.y = -kZ0 * wphi + uz.y * sz;
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
    double p = kC * s.h_u_nm * kNfft / lam;  // ntffTM.c:227
    const int idx = (int)floor(p);
    p = p - idx;
    const double2 a = buf[idx], b = buf[idx + 1];
    const double na = a.x * a.x + a.y * a.y, nb = b.x * b.x + b.y * b.y;
    s.out[(size_t)l * 360 + ang] = ((1 - p) * na + p * nb) / kNfft;
  }
}

// ntffTM_Frequency: N_z, L_x, L_y integrals over the NTFF path of the current
// fields, one block per angle; global-frame cell (x, y) is array cell (x-ox, y-ox).
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
  double nz_r = 0, nz_i = 0, lx_r = 0, lx_i = 0, ly_r = 0, ly_i = 0;
  const int nb = f.rt - f.lt, nr = f.tp - f.bm;
  const int ncell = 2 * nb + 2 * nr;
  for (int c = threadIdx.x; c < ncell; c += blockDim.x) {
    int x, y, side;
    if (c < nb) { side = 0; x = f.lt + c; y = f.bm; }
    else if (c < nb + nr) { side = 1; x = f.rt; y = f.bm + (c - nb); }
    else if (c < 2 * nb + nr) { side = 2; x = f.lt + (c - nb - nr); y = f.tp; }
    else { side = 3; x = f.lt; y = f.bm + (c - 2 * nb - nr); }
    const long long k = (long long)(x - f.ox) * f.P + (y - f.ox);
    const long long hoff = (side == 0 || side == 2) ? -1 : -(long long)f.P;
    const void *hp = f.h[side == 0 || side == 2 ? 0 : 1];
    const double2 ez = load_c(f.e, k, f.f32);
    const double2 ha = load_c(hp, k, f.f32), hb = load_c(hp, k + hoff, f.f32);
    const double hr = 0.5 * (ha.x + hb.x), hi = 0.5 * (ha.y + hb.y);
    const double inner = __dadd_rn(__dmul_rn(rx, (double)x - f.cx), __dmul_rn(ry, (double)y - f.cy));
    const double2 e = cexp_i(f.k_s * inner);
    const double sg = side < 2 ? 1.0 : -1.0;       // bottom/right add, top/left subtract
    nz_r += sg * (hr * e.x - hi * e.y);
    nz_i += sg * (hr * e.y + hi * e.x);
    const double er = sg * (ez.x * e.x - ez.y * e.y), ei = sg * (ez.x * e.y + ez.y * e.x);
    if (side == 0 || side == 2) { lx_r += er; lx_i += ei; }
    else { ly_r += er; ly_i += ei; }
  }
  red[0][threadIdx.x] = nz_r; red[1][threadIdx.x] = nz_i;
  red[2][threadIdx.x] = lx_r; red[3][threadIdx.x] = lx_i;
  red[4][threadIdx.x] = ly_r; red[5][threadIdx.x] = ly_i;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int q = 0; q < 6; q++) red[q][threadIdx.x] += red[q][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    // Lphi = -Lx sin + Ly cos ; result = coef (Z0 Nz + Lphi) sqrt(h_u)   (ntffTM.c:155-156)
    const double lpr = -red[2][0] * ry + red[4][0] * rx, lpi = -red[3][0] * ry + red[5][0] * rx;
    const double br = kZ0 * red[0][0] + lpr, bi = kZ0 * red[1][0] + lpi;
    f.out[ang] = make_double2((f.coef.x * br - f.coef.y * bi) * f.sqrt_hu, (f.coef.x * bi + f.coef.y * br) * f.sqrt_hu);
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

}  // namespace fdtd
