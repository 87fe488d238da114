// fdtd_dft.cu -- running-DFT NTFF: the far field at chosen frequencies
// accumulated during the run instead of the 360 x arraySize time-domain
// accumulators and their FFT (ntffTM.c:197-275, ntffTE.c:160-238).
//
// The time-domain NTFF deposits path value v_c(t) of step t at t + sh(a, c)
// with the three taps (b, a - b, -a) around m0 = floor(t + sh + 1/2)
// (mpiTM_UPML.c:840-847, ntffTM.c:279-288).  For integer t, m0 = t + M and
// a = sh + 1/2 - M are the same every step, so the Fourier sum of one angle's
// series at frequency w (radians per step, the FFT's e^{+i w m}) factorises:
//   X_a(w) = sum_c g_a(c) e^{i w M} (b e^{-i w} + (a - b) - a e^{i w}) S_c(w),
//   S_c(w) = sum_t v_c(t) e^{i w t}
// with g_a(c) the weight of the cell's accumulator in E_theta (TM) or E_phi
// (TE) at angle a (ntffTM.c:174-194, ntffTE.c:20-55).  H samples sit at
// t + 1/2: their M and a come from sh + 1/2.  S_c(w) is accumulated from the
// buffered path samples of the time-blocked NTFF (every flush of the ring);
// the far field sums over the path once, at the end.
#include <cuda_runtime.h>

#include "fdtd_internal.cuh"

namespace fdtd {

namespace {

// P[s][k] = e^{i w_k (t0 + s)}
__global__ void dft_phasor_kernel(const double *omega, int nfreq, int nb, double t0, double2 *P)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb * nfreq) return;
  const int s = i / nfreq, k = i % nfreq;
  double sn, cs;
  sincos(omega[k] * (t0 + s), &sn, &cs);
  P[i] = make_double2(cs, sn);
}

// S[f][c][k] += sum_s vals[s][f][c] P[s][k]; grid (ncell, ceil(nfreq/256), 2)
__global__ void dft_accumulate_kernel(NtffView n, const double2 *P, double2 *S, int nfreq, int nb)
{
  const int c = blockIdx.x, f = blockIdx.z;
  const int k = blockIdx.y * blockDim.x + threadIdx.x;
  if (k >= nfreq) return;
  double2 acc = S[((size_t)f * n.ncell + c) * nfreq + k];
  for (int s = 0; s < nb; s++) {
    const double2 v = n.vals[(size_t)s * 2 * n.ncell + (size_t)f * n.ncell + c];
    const double2 p = P[(size_t)s * nfreq + k];
    acc.x = fma(v.x, p.x, fma(-v.y, p.y, acc.x));
    acc.y = fma(v.x, p.y, fma(v.y, p.x, acc.y));
  }
  S[((size_t)f * n.ncell + c) * nfreq + k] = acc;
}

__device__ __forceinline__ double2 cmul(double2 a, double2 b)
{
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// T[m][k] = e^{i w_k (m + mlo)} for the integer bins m + mlo the far field
// needs (the same sincos of w M the far field would take per element)
__global__ void dft_bin_phasor_kernel(const double *omega, int nfreq, int mlo, int nm, double2 *T)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nm * nfreq) return;
  const int m = i / nfreq, k = i - m * nfreq;
  double sm, cm;
  sincos(omega[k] * (double)(m + mlo), &sm, &cm);
  T[i] = make_double2(cm, sm);
}

// X[a][k] = coef sum_{c, f} g e^{i w M} kappa S ; one block per angle, 128
// threads = 4 groups of path cells x 32 frequencies (lane k), the groups'
// sums added in shared memory.  e^{i w M} comes from the bin table T (the
// sincos fallback covers a bin outside it, which the table's range excludes).
__global__ void __launch_bounds__(128) dft_farfield_kernel(NtffView n, const double2 *S, const double *omega,
                                                           int nfreq, int tm, double z0, const double2 *dir,
                                                           double2 coef, const double2 *T, int mlo, int nm,
                                                           double2 *X)
{
  __shared__ double2 part[4][32];
  const int ang = blockIdx.x, lane = threadIdx.x & 31, grp = threadIdx.x >> 5;
  const double2 d = dir[ang];
  const double px = -d.y, py = d.x, sz = -1.0;
  // weight of accumulators 0, 1, 2 in the angle's far-field component (spectrum_kernel's combination)
  double g[3];
  if (tm) { g[0] = -px; g[1] = -py; g[2] = -z0 * sz; }
  else { g[0] = -z0 * px; g[1] = -z0 * py; g[2] = sz; }
  for (int k0 = 0; k0 < nfreq; k0 += 32) {
    const int k = k0 + lane;
    double2 sum = make_double2(0.0, 0.0);
    if (k < nfreq) {
      const double w = omega[k];
      double sw, cw;
      sincos(w, &sw, &cw);
      for (int c = grp; c < n.ncell; c += 4) {
        const double sh = n.shift[(size_t)ang * n.ncell + c];
        const unsigned char uw = (unsigned char)n.cells[c].uid_wid;
        for (int f = 0; f < 2; f++) {
          const double u = (f == 0 ? sh : sh + 0.5) + 0.5;
          const double M = floor(u);
          const double a = u - M, b = 1.0 - a;
          // kappa = b e^{-iw} + (a - b) - a e^{iw}
          const double2 kap = make_double2(b * cw + (a - b) - a * cw, -b * sw - a * sw);
          const long long m = (long long)M - mlo;
          double2 em;
          if (m >= 0 && m < nm) {
            em = T[(size_t)m * nfreq + k];
          } else {
            double sm, cm;
            sincos(w * M, &sm, &cm);
            em = make_double2(cm, sm);
          }
          const double2 t = cmul(cmul(em, kap), S[((size_t)f * n.ncell + c) * nfreq + k]);
          const double gw = g[f == 0 ? (uw & 15) : (uw >> 4)];
          sum.x += gw * t.x;
          sum.y += gw * t.y;
        }
      }
    }
    part[grp][lane] = sum;
    __syncthreads();
    if (grp == 0 && k < nfreq) {
      const double2 a0 = part[0][lane], a1 = part[1][lane], a2 = part[2][lane], a3 = part[3][lane];
      const double2 tot = make_double2(((a0.x + a1.x) + a2.x) + a3.x, ((a0.y + a1.y) + a2.y) + a3.y);
      X[(size_t)ang * nfreq + k] = cmul(coef, tot);
    }
    __syncthreads();
  }
}

// ---- far fields of many maps that share one path (the broadband batch)
//
// Instances created with the same configuration have the same path, shifts
// and bins, so the weight W = g e^{i w M} kappa of a term (angle, cell,
// field, frequency) is the same for all of them: one block computes it once
// and applies it to a group of up to kFarGroup maps,
//   X_j[a][k] = coef sum_{c, f} W S_j[f][c][k],
// with W and every product rounded by explicit _rn operations, so a map's
// result does not depend on the group it is evaluated in.

constexpr int kFarGroup = 16;

__device__ __forceinline__ double2 ff_weight(double sh, int f, double gw, double w, double cw, double sw, int k,
                                             int nfreq, const double2 *T, int mlo, int nm)
{
  const double u = __dadd_rn(f == 0 ? sh : __dadd_rn(sh, 0.5), 0.5);
  const double M = floor(u);
  const double a = __dsub_rn(u, M), b = __dsub_rn(1.0, a);
  // kappa = b e^{-iw} + (a - b) - a e^{iw} = (b - a)(cos w - 1) - i sin w, scaled by g
  const double kr = __dmul_rn(__dsub_rn(b, a), __dsub_rn(cw, 1.0)), ki = -sw;
  const long long m = (long long)M - mlo;
  double2 em;
  if (m >= 0 && m < nm) {
    em = T[(size_t)m * nfreq + k];
  } else {
    double sm, cm;
    sincos(__dmul_rn(w, M), &sm, &cm);
    em = make_double2(cm, sm);
  }
  const double wr = __fma_rn(em.x, kr, -__dmul_rn(em.y, ki));
  const double wi = __fma_rn(em.x, ki, __dmul_rn(em.y, kr));
  return make_double2(__dmul_rn(gw, wr), __dmul_rn(gw, wi));
}

// grid (360, map groups), 128 threads = 4 groups of path cells x 32
// frequencies (lane k); map j of group g is instance idx[g kFarGroup + j]
__global__ void __launch_bounds__(128) dft_farfield_group_kernel(NtffView n, const double2 *const *S,
                                                                 const int *idx, int nmaps, const double *omega,
                                                                 int nfreq, int tm, double z0, const double2 *dir,
                                                                 double2 coef, const double2 *T, int mlo, int nm,
                                                                 double2 *X, size_t x_stride)
{
  __shared__ double2 part[kFarGroup][4][32];
  const int ang = blockIdx.x, lane = threadIdx.x & 31, grp = threadIdx.x >> 5;
  const int j0 = blockIdx.y * kFarGroup, cnt = min(kFarGroup, nmaps - j0);
  const double2 d = dir[ang];
  const double px = -d.y, py = d.x, sz = -1.0;
  double g[3];
  if (tm) { g[0] = -px; g[1] = -py; g[2] = -z0 * sz; }
  else { g[0] = -z0 * px; g[1] = -z0 * py; g[2] = sz; }
  const double2 *Sj[kFarGroup];
#pragma unroll
  for (int j = 0; j < kFarGroup; j++) Sj[j] = j < cnt ? S[idx[j0 + j]] : nullptr;
  for (int k0 = 0; k0 < nfreq; k0 += 32) {
    const int k = k0 + lane;
    double2 acc[kFarGroup];
#pragma unroll
    for (int j = 0; j < kFarGroup; j++) acc[j] = make_double2(0.0, 0.0);
    if (k < nfreq) {
      const double w = omega[k];
      double sw, cw;
      sincos(w, &sw, &cw);
      for (int c = grp; c < n.ncell; c += 4) {
        const double sh = n.shift[(size_t)ang * n.ncell + c];
        const unsigned char uw = (unsigned char)n.cells[c].uid_wid;
        for (int f = 0; f < 2; f++) {
          const double2 W = ff_weight(sh, f, g[f == 0 ? (uw & 15) : (uw >> 4)], w, cw, sw, k, nfreq, T, mlo, nm);
          const size_t at = ((size_t)f * n.ncell + c) * nfreq + k;
#pragma unroll
          for (int j = 0; j < kFarGroup; j++) {
            if (j < cnt) {
              const double2 v = Sj[j][at];
              acc[j].x = __fma_rn(W.x, v.x, __fma_rn(-W.y, v.y, acc[j].x));
              acc[j].y = __fma_rn(W.x, v.y, __fma_rn(W.y, v.x, acc[j].y));
            }
          }
        }
      }
    }
#pragma unroll
    for (int j = 0; j < kFarGroup; j++) part[j][grp][lane] = acc[j];
    __syncthreads();
    for (int q = threadIdx.x; q < cnt * 32; q += blockDim.x) {
      const int j = q >> 5, l = q & 31, kk = k0 + l;
      if (kk < nfreq) {
        const double2 a0 = part[j][0][l], a1 = part[j][1][l], a2 = part[j][2][l], a3 = part[j][3][l];
        const double2 tot = make_double2(__dadd_rn(__dadd_rn(__dadd_rn(a0.x, a1.x), a2.x), a3.x),
                                         __dadd_rn(__dadd_rn(__dadd_rn(a0.y, a1.y), a2.y), a3.y));
        X[(size_t)idx[j0 + j] * x_stride + (size_t)ang * nfreq + kk] =
            make_double2(__fma_rn(coef.x, tot.x, -__dmul_rn(coef.y, tot.y)),
                         __fma_rn(coef.x, tot.y, __dmul_rn(coef.y, tot.x)));
      }
    }
    __syncthreads();
  }
}

}  // namespace

void launch_dft_accumulate(const NtffView &n, const DftView &d, int nb, double t0, cudaStream_t st)
{
  if (nb <= 0 || d.nfreq <= 0) return;
  dft_phasor_kernel<<<(nb * d.nfreq + 255) / 256, 256, 0, st>>>(d.omega, d.nfreq, nb, t0, d.phasor);
  dft_accumulate_kernel<<<dim3((unsigned)n.ncell, (unsigned)((d.nfreq + 255) / 256), 2), 256, 0, st>>>(
      n, d.phasor, d.S, d.nfreq, nb);
}

void launch_dft_farfield(const NtffView &n, const DftView &d, int tm, double z0, const double2 *dir, double2 coef,
                         const DftBins &bins, double2 *X, cudaStream_t st)
{
  if (bins.nm > 0)
    dft_bin_phasor_kernel<<<(bins.nm * d.nfreq + 255) / 256, 256, 0, st>>>(d.omega, d.nfreq, bins.mlo, bins.nm,
                                                                           bins.T);
  dft_farfield_kernel<<<360, 128, 0, st>>>(n, d.S, d.omega, d.nfreq, tm, z0, dir, coef, bins.T, bins.mlo, bins.nm,
                                          X);
}

void launch_dft_farfield_group(const NtffView &n, const double2 *const *S, const int *idx, int nmaps,
                               const double *omega, int nfreq, int tm, double z0, const double2 *dir, double2 coef,
                               const DftBins &bins, double2 *X, size_t x_stride, cudaStream_t st)
{
  if (nmaps <= 0) return;
  if (bins.nm > 0)
    dft_bin_phasor_kernel<<<(bins.nm * nfreq + 255) / 256, 256, 0, st>>>(omega, nfreq, bins.mlo, bins.nm, bins.T);
  const dim3 grid(360, (unsigned)((nmaps + kFarGroup - 1) / kFarGroup));
  dft_farfield_group_kernel<<<grid, 128, 0, st>>>(n, S, idx, nmaps, omega, nfreq, tm, z0, dir, coef, bins.T, bins.mlo,
                                                  bins.nm, X, x_stride);
}

}  // namespace fdtd
