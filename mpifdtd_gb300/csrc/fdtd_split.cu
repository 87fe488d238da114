// fdtd_split.cu -- the serial solvers without UPML auxiliaries: split-field
// PML (fdtdTM.c, fdtdTE.c) and non-standard FDTD (nsFdtdTM.c, nsFdtdTE.c).
//
// Fields on the N_PX x N_PY global frame (array cell (x, y) at x*P + y),
// updated on 1 <= x <= N_PX-2, 1 <= y <= N_PY-2 as the reference's loops are
// (the outer ring stays zero).  Every coefficient is per cell, as in the
// reference (it depends on both sigma and the local permittivity), and is
// computed once on the host from the permittivity (fdtd_api.cu
// split_coefficients): the device only steps.
//
// Slots: TM 0 Ez 1 Ezx 2 Ezy 3 Hx 4 Hy ; TE 0 Ex 1 Ey 2 Hz 3 Hzx 4 Hzy.
// Coefficients (SplitView::c):
//   TM (split, NS): 0 C_EZX 1 C_EZXLX 2 C_EZY 3 C_EZYLY 4 C_HX 5 C_HXLY 6 C_HY 7 C_HYLX
//   TE (split, NS): 0 C_EX 1 C_EXLY 2 C_EY 3 C_EYLX 4 C_HZX 5 C_HZXLX 6 C_HZY 7 C_HZYLY
//   8 (9): the per-cell source amplitude of the driven component(s):
//     split: EPSILON_0_S/eps - 1 (field_scatteredWaveNotUPML, field.c:179-196)
//     NS   : 1/(n_ u n) - 1      (field_nsScatteredWaveNotUPML, field.c:155-177)
//
// This file is compiled without FMA contraction so that every expression
// rounds as the reference's C does (one rounding per operation).
#include <cuda_runtime.h>

#include "fdtd_internal.cuh"

namespace fdtd {

namespace {

__device__ __forceinline__ double2 cadd2(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub2(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 rmul(double r, double2 a) { return make_double2(r * a.x, r * a.y); }

// a * (cexp(i (kr - w t_hi)) - cexp(i (kr - w t_lo)))
__device__ __forceinline__ double2 wave_step(double a, double kr, double w, double t_hi, double t_lo)
{
  double s1, c1, s0, c0;
  sincos(kr - w * t_hi, &s1, &c1);
  sincos(kr - w * t_lo, &s0, &c0);
  return make_double2(a * (c1 - c0), a * (s1 - s0));
}

__device__ __forceinline__ double kr_at(const SplitView &v, int i, int j, double gx, double gy)
{
  return (i + gx) * v.ks_cos + (j + gy) * v.ks_sin;
}

// ((a1 - a0) + b1) - b0: the reference's EZX(.+1) - EZX(.) + EZY(.+1) - EZY(.)
__device__ __forceinline__ double2 pair_diff(double2 a1, double2 a0, double2 b1, double2 b0)
{
  return csub2(cadd2(csub2(a1, a0), b1), b0);
}

// (a + b) - 2 c
__device__ __forceinline__ double2 second(double2 a, double2 b, double2 c) { return csub2(cadd2(a, b), rmul(2, c)); }

#define SPLIT_CELL                                              \
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;     \
  const int i = blockIdx.y * blockDim.y + threadIdx.y + 1;     \
  if (i > v.n_px - 2 || j > v.n_py - 2) return;                \
  const long long P = v.P;                                      \
  const long long k = (long long)i * P + j;

// ---- split-field TM (fdtdTM.c:290-327): calcH, then calcE, then the source on Ezx

__global__ void split_tm_h(SplitView v)
{
  SPLIT_CELL
  const double2 *Ezx = v.f[1], *Ezy = v.f[2];
  double2 *Hx = v.f[3], *Hy = v.f[4];
  const double2 dx = pair_diff(Ezx[k + 1], Ezx[k], Ezy[k + 1], Ezy[k]);
  const double2 dy = pair_diff(Ezx[k + P], Ezx[k], Ezy[k + P], Ezy[k]);
  Hx[k] = csub2(rmul(v.c[4][k], Hx[k]), rmul(v.c[5][k], dx));
  Hy[k] = cadd2(rmul(v.c[6][k], Hy[k]), rmul(v.c[7][k], dy));
}

__global__ void split_tm_e(SplitView v)
{
  SPLIT_CELL
  double2 *Ez = v.f[0], *Ezx = v.f[1], *Ezy = v.f[2];
  const double2 *Hx = v.f[3], *Hy = v.f[4];
  const double2 ezx = cadd2(rmul(v.c[0][k], Ezx[k]), rmul(v.c[1][k], csub2(Hy[k], Hy[k - P])));
  const double2 ezy = csub2(rmul(v.c[2][k], Ezy[k]), rmul(v.c[3][k], csub2(Hx[k], Hx[k - 1])));
  Ez[k] = cadd2(ezx, ezy);
  // field_scatteredWaveNotUPML(Ezx, EPS_EZ, 0, 0) after Ez = Ezx + Ezy
  Ezx[k] = cadd2(ezx, wave_step(v.ray * v.c[8][k], kr_at(v, i, j, 0.0, 0.0), v.w_s, v.t + 0.5, v.t - 0.5));
  Ezy[k] = ezy;
}

// ---- split-field TE (fdtdTE.c:283-321): calcE, the source on Ey, then calcH

__global__ void split_te_e(SplitView v)
{
  SPLIT_CELL
  double2 *Ex = v.f[0], *Ey = v.f[1];
  const double2 *Hzx = v.f[3], *Hzy = v.f[4];
  const double2 dy = pair_diff(Hzx[k], Hzx[k - 1], Hzy[k], Hzy[k - 1]);
  const double2 dx = pair_diff(Hzx[k], Hzx[k - P], Hzy[k], Hzy[k - P]);
  Ex[k] = cadd2(rmul(v.c[0][k], Ex[k]), rmul(v.c[1][k], dy));
  const double2 ey = csub2(rmul(v.c[2][k], Ey[k]), rmul(v.c[3][k], dx));
  // field_scatteredWaveNotUPML(Ey, EPS_EY, 0.0, 0.5)
  Ey[k] = cadd2(ey, wave_step(v.ray * v.c[8][k], kr_at(v, i, j, 0.0, 0.5), v.w_s, v.t + 0.5, v.t - 0.5));
}

__global__ void split_te_h(SplitView v)
{
  SPLIT_CELL
  const double2 *Ex = v.f[0], *Ey = v.f[1];
  double2 *Hz = v.f[2], *Hzx = v.f[3], *Hzy = v.f[4];
  const double2 hzx = csub2(rmul(v.c[4][k], Hzx[k]), rmul(v.c[5][k], csub2(Ey[k + P], Ey[k])));
  const double2 hzy = cadd2(rmul(v.c[6][k], Hzy[k]), rmul(v.c[7][k], csub2(Ex[k + 1], Ex[k])));
  Hzx[k] = hzx;
  Hzy[k] = hzy;
  Hz[k] = cadd2(hzx, hzy);
}

// ---- NS-FDTD TM (nsFdtdTM.c:68-151): calcH from Ez with the NS operator,
// calcE, the source on Ezy, then Ez = Ezx + Ezy

__global__ void ns_tm_h(SplitView v)
{
  SPLIT_CELL
  const double2 *e = v.f[0];
  double2 *Hx = v.f[3], *Hy = v.f[4];
  const double2 nsx = rmul(v.r_2, csub2(second(e[k + 1 + P], e[k + 1 - P], e[k + 1]), second(e[k + P], e[k - P], e[k])));
  Hx[k] = csub2(rmul(v.c[4][k], Hx[k]), rmul(v.c[5][k], cadd2(csub2(e[k + 1], e[k]), nsx)));
  const double2 nsy = rmul(v.r_2, csub2(second(e[k + P + 1], e[k + P - 1], e[k + P]), second(e[k + 1], e[k - 1], e[k])));
  Hy[k] = cadd2(rmul(v.c[6][k], Hy[k]), rmul(v.c[7][k], cadd2(csub2(e[k + P], e[k]), nsy)));
}

__global__ void ns_tm_e(SplitView v)
{
  SPLIT_CELL
  double2 *Ez = v.f[0], *Ezx = v.f[1], *Ezy = v.f[2];
  const double2 *Hx = v.f[3], *Hy = v.f[4];
  const double2 ezx = cadd2(rmul(v.c[0][k], Ezx[k]), rmul(v.c[1][k], csub2(Hy[k], Hy[k - P])));
  double2 ezy = csub2(rmul(v.c[2][k], Ezy[k]), rmul(v.c[3][k], csub2(Hx[k], Hx[k - 1])));
  // field_nsScatteredWaveNotUPML(Ezy, EPS_EZ, 0, 0, 1.0), then Ez = Ezx + Ezy
  ezy = cadd2(ezy, wave_step(v.ray * v.c[8][k], kr_at(v, i, j, 0.0, 0.0), v.w_s, v.t + 1.0, v.t));
  Ezx[k] = ezx;
  Ezy[k] = ezy;
  Ez[k] = cadd2(ezx, ezy);
}

// ---- NS-FDTD TE (nsFdtdTE.c:233-308): calcH, Hz = Hzx + Hzy, calcE with the
// NS operator, then the sources on Ex (cos) and Ey (sin) of angle + 90 deg

__global__ void ns_te_h(SplitView v)
{
  SPLIT_CELL
  const double2 *Ex = v.f[0], *Ey = v.f[1];
  double2 *Hz = v.f[2], *Hzx = v.f[3], *Hzy = v.f[4];
  const double2 hzx = csub2(rmul(v.c[4][k], Hzx[k]), rmul(v.c[5][k], csub2(Ey[k + P], Ey[k])));
  const double2 hzy = cadd2(rmul(v.c[6][k], Hzy[k]), rmul(v.c[7][k], csub2(Ex[k + 1], Ex[k])));
  Hzx[k] = hzx;
  Hzy[k] = hzy;
  Hz[k] = cadd2(hzx, hzy);
}

__global__ void ns_te_e(SplitView v)
{
  SPLIT_CELL
  double2 *Ex = v.f[0], *Ey = v.f[1];
  const double2 *h = v.f[2];
  const double2 nsx = rmul(v.r_2, csub2(second(h[k + P], h[k - P], h[k]), second(h[k - 1 + P], h[k - 1 - P], h[k - 1])));
  double2 ex = cadd2(rmul(v.c[0][k], Ex[k]), rmul(v.c[1][k], cadd2(csub2(h[k], h[k - 1]), nsx)));
  const double2 nsy = rmul(v.r_2, csub2(second(h[k + 1], h[k - 1], h[k]), second(h[k - P + 1], h[k - P - 1], h[k - P])));
  double2 ey = csub2(rmul(v.c[2][k], Ey[k]), rmul(v.c[3][k], cadd2(csub2(h[k], h[k - P]), nsy)));
  const double kr = kr_at(v, i, j, 0.0, 0.5);
  if (v.co != 0.0) ex = cadd2(ex, wave_step((v.ray * v.co) * v.c[8][k], kr, v.w_s, v.t + 1.0, v.t));
  if (v.si != 0.0) ey = cadd2(ey, wave_step((v.ray * v.si) * v.c[9][k], kr, v.w_s, v.t + 1.0, v.t));
  Ex[k] = ex;
  Ey[k] = ey;
}

}  // namespace

void launch_split_step(const SplitView &v, int solver, cudaStream_t st)
{
  const dim3 b(32, 8);
  const dim3 g((unsigned)((v.n_py - 2 + 31) / 32), (unsigned)((v.n_px - 2 + 7) / 8));
  switch (solver) {
  case 0:  // TM_2D: update() = calcH(); calcE(); source (fdtdTM.c:290-297)
    split_tm_h<<<g, b, 0, st>>>(v);
    split_tm_e<<<g, b, 0, st>>>(v);
    break;
  case 1:  // TE_2D: calcE(); source; calcH() (fdtdTE.c:283-288)
    split_te_e<<<g, b, 0, st>>>(v);
    split_te_h<<<g, b, 0, st>>>(v);
    break;
  case 6:  // NS_TM_2D (nsFdtdTM.c:68-80)
    ns_tm_h<<<g, b, 0, st>>>(v);
    ns_tm_e<<<g, b, 0, st>>>(v);
    break;
  default:  // NS_TE_2D (nsFdtdTE.c:233-252)
    ns_te_h<<<g, b, 0, st>>>(v);
    ns_te_e<<<g, b, 0, st>>>(v);
    break;
  }
}

}  // namespace fdtd
