// stencil_ops.cuh -- per-cell helpers shared by the one-step stencil kernels
// (fdtd_kernels.cu) and the temporally blocked kernels (fdtd_tblock.cu).
#pragma once
#include <cuda_runtime.h>

#include "fdtd_internal.cuh"

namespace fdtd {

template <typename T> __device__ __forceinline__ T cadd(T a, T b) { a.x += b.x; a.y += b.y; return a; }
template <typename T> __device__ __forceinline__ T csub(T a, T b) { a.x -= b.x; a.y -= b.y; return a; }
template <typename T, typename R> __device__ __forceinline__ T cscale(T a, R s) { a.x *= s; a.y *= s; return a; }
template <typename T> __device__ __forceinline__ T ldro(const T *p) { return __ldg(p); }
template <typename T> __device__ __forceinline__ T czero() { T z; z.x = 0; z.y = 0; return z; }

__device__ __forceinline__ bool is_one(double v) { return __double_as_longlong(v) == 0x3FF0000000000000LL; }
__device__ __forceinline__ bool is_one(float v) { return __float_as_int(v) == 0x3F800000; }

// CW scattered-wave increment at array cell (i, j): ray_coef (1/eps - 1) e^{i(kr - w t)}
// (mpiTM_UPML.c:369-370).  kr is split as x*kcos + y*ksin, so e^{ikr} is the
// product of two 1-D tables; (s_re, s_im) = ray_coef e^{-i w t} comes from the
// host per step.  Evaluated in the field precision R: FP64 for the parity
// engine; FP32 for FP32 fields (an FP64 evaluation there costs more than the
// whole FP32 stencil on dielectric cells, GB300's FP64 rate being ~1/56 of FP32).
template <typename R>
__device__ __forceinline__ void cw_add(const StencilView<R> &v, double s_re, double s_im, int i, int j, R ie,
                                       typename Cplx<R>::T &e)
{
  const typename Cplx<R>::T ex = v.ex[i], ey = v.ey[j];
  const R sr = (R)s_re, si = (R)s_im;
  const R pr = ex.x * ey.x - ex.y * ey.y;
  const R pi = ex.x * ey.y + ex.y * ey.x;
  const R amp = ie - (R)1;
  const R qr = (pr * sr - pi * si) * amp;
  const R qi = (pr * si + pi * sr) * amp;
  e.x = e.x + qr;
  e.y = e.y + qi;
}

// The same increment in a blocked launch, at level lvl: the row table of that
// level (v.src_lstride = 0 for the CW source: one table for every level).
template <typename R>
__device__ __forceinline__ void cw_add_level(const StencilView<R> &v, double s_re, double s_im, int lvl, int i,
                                             int j, R ie, typename Cplx<R>::T &e)
{
  const typename Cplx<R>::T ex = v.ex[(size_t)lvl * v.src_lstride + i], ey = v.ey[j];
  const R sr = (R)s_re, si = (R)s_im;
  const R pr = ex.x * ey.x - ex.y * ey.y;
  const R pi = ex.x * ey.y + ex.y * ey.x;
  const R amp = ie - (R)1;
  const R qr = (pr * sr - pi * si) * amp;
  const R qi = (pr * si + pi * sr) * amp;
  e.x = e.x + qr;
  e.y = e.y + qi;
}

template <typename R>
__device__ __forceinline__ void cw_source(const StencilView<R> &v, const SourceStep &s, int i, int j, R ie,
                                          typename Cplx<R>::T &e)
{
  cw_add<R>(v, s.s_re, s.s_im, i, j, ie, e);
}

// Gaussian-pulse scattered field (field.c:224-256) at array cell (i, j), at
// s.time + dt (dt: the level of a blocked launch; integer times add exactly).
template <typename R>
__device__ __forceinline__ void pulse_source(const SourceStep &s, int i, int j, R ie, typename Cplx<R>::T &e,
                                             double dt = 0.0)
{
  const double pos = __dadd_rn(__dmul_rn((double)i + s.gap_x, s.cos_per_c),
                               __dmul_rn((double)j + s.gap_y, s.sin_per_c));
  const double r = __dsub_rn(pos, (s.time + dt) - s.t0);
  const double q = __ddiv_rn(r, 50.0);
  const double g = exp(-(q * q));
  const double amp = s.dot * g * ((double)ie - 1.0);
  double sn, cs;
  sincos(r * s.w, &sn, &cs);
  e.x = (R)((double)e.x + amp * cs);
  e.y = (R)((double)e.y + amp * sn);
}

// The same from a row table entry (pulse at 0 degrees): the operations after
// the pulse's own value are pulse_source's, in its order.
template <typename R>
__device__ __forceinline__ void pulse_row(const PulseRow &p, R ie, typename Cplx<R>::T &e)
{
  const double amp = p.a * ((double)ie - 1.0);
  e.x = (R)((double)e.x + amp * p.c);
  e.y = (R)((double)e.y + amp * p.s);
}

template <typename R>
__device__ __forceinline__ void apply_source(const StencilView<R> &v, const SourceStep &s, int i, int j, R ie,
                                             typename Cplx<R>::T &e)
{
  if (s.kind == 1) cw_source<R>(v, s, i, j, ie, e);
  else if (s.kind == 2) pulse_source<R>(s, i, j, ie, e);
}

template <typename R>
__device__ __forceinline__ bool interior(const StencilView<R> &v, int i, int j)
{
  const int x = i + v.ox, y = j + v.ox;
  return x >= v.in_x0 && x < v.in_x1 && y >= v.in_y0 && y < v.in_y1;
}

// ---- Gedney UPML updates of one PML cell (coefficients from the 1-D tables).
// The interior update (all C_* = 1) is written inline by the callers.

// TM calcJD (mpiTM_UPML.c:431-446): jz old -> new, dz old -> new
template <typename R, typename T>
__device__ __forceinline__ void tm_e_pml(const StencilView<R> &v, int i, int j, const T &curl, T &dz, T &jz)
{
  const Coef4<R> cx = v.tx_i[i], cy = v.ty_i[j];
  T jn;
  jn.x = cx.a * jz.x + cx.b * curl.x;                 // C_JZ Jz + C_JZHXHY curl
  jn.y = cx.a * jz.y + cx.b * curl.y;
  dz.x = (cy.a * dz.x + cy.b * jn.x) - cy.b * jz.x;   // C_DZ Dz + C_DZJZ1 Jz' - C_DZJZ0 Jz
  dz.y = (cy.a * dz.y + cy.b * jn.y) - cy.b * jz.y;
  jz = jn;
}

// TM calcMB + calcH (mpiTM_UPML.c:491-530) with dEx = Ez[j+1] - Ez, dEy = Ez - Ez[i+1]
template <typename R, typename T>
__device__ __forceinline__ void tm_h_pml(const StencilView<R> &v, int i, int j, const T &dEx, const T &dEy, T &hx,
                                         T &hy, T &mx, T &my)
{
  const Coef4<R> cxi = v.tx_i[i], cxh = v.tx_h[i], cyi = v.ty_i[j], cyh = v.ty_h[j];
  T mxn, myn;
  mxn.x = cyh.a * mx.x - cyh.b * dEx.x;          // C_MX Mx - C_MXEZ/mu0 dE
  mxn.y = cyh.a * mx.y - cyh.b * dEx.y;
  hx.x = (hx.x + cxi.c * mxn.x) - cxi.d * mx.x;  // C_BX(=1) H + C_BXMX1 Mx' - C_BXMX0 Mx
  hx.y = (hx.y + cxi.c * mxn.y) - cxi.d * mx.y;
  myn.x = my.x - v.inv_mu * dEy.x;               // C_MY(=1) My - C_MYEZ(=1)/mu0 dE
  myn.y = my.y - v.inv_mu * dEy.y;
  const R c1 = cyi.c * cxh.b, c0 = cyi.d * cxh.b;  // C_BYMY1, C_BYMY0
  hy.x = (cxh.a * hy.x + c1 * myn.x) - c0 * my.x;
  hy.y = (cxh.a * hy.y + c1 * myn.y) - c0 * my.y;
  mx = mxn;
  my = myn;
}

// TE calcJD (mpiTE_UPML.c:337-375) with cxv = Hz - Hz[j-1], cyv = -Hz + Hz[i-1]
template <typename R, typename T>
__device__ __forceinline__ void te_e_pml(const StencilView<R> &v, int i, int j, const T &cxv, const T &cyv, T &dx,
                                         T &dy, T &jx, T &jy)
{
  const Coef4<R> cxh = v.tx_h[i], cxi = v.tx_i[i], cyi = v.ty_i[j], cyh = v.ty_h[j];
  T jxn, jyn;
  jxn.x = cyi.a * jx.x + cyi.b * cxv.x;          // C_JX Jx + C_JXHZ curl
  jxn.y = cyi.a * jx.y + cyi.b * cxv.y;
  dx.x = (dx.x + cxh.a * jxn.x) - cxh.b * jx.x;  // C_DX(=1) Dx + C_DXJX1 Jx' - C_DXJX0 Jx
  dx.y = (dx.y + cxh.a * jxn.y) - cxh.b * jx.y;
  jyn = cadd(jy, cyv);                           // C_JY(=1) Jy + C_JYHZ(=1) curl
  const R c1 = cyh.c * cxi.b, c0 = cyh.d * cxi.b;  // C_DYJY1, C_DYJY0
  dy.x = (cxi.a * dy.x + c1 * jyn.x) - c0 * jy.x;
  dy.y = (cxi.a * dy.y + c1 * jyn.y) - c0 * jy.y;
  jx = jxn;
  jy = jyn;
}

// TE calcMB + calcH (mpiTE_UPML.c:377-399) with ce = Ey[i+1] - Ey - Ex[j+1] + Ex
template <typename R, typename T>
__device__ __forceinline__ void te_h_pml(const StencilView<R> &v, int i, int j, const T &ce, T &hz, T &mz)
{
  const Coef4<R> cxh = v.tx_h[i], cyh = v.ty_h[j];
  T mzn;
  mzn.x = cxh.c * mz.x - cxh.d * ce.x;                   // C_MZ Mz - C_MZEXEY/mu0 curl
  mzn.y = cxh.c * mz.y - cxh.d * ce.y;
  hz.x = (cyh.a * hz.x + cyh.b * mzn.x) - cyh.b * mz.x;  // C_BZ H + C_BZMZ1 Mz' - C_BZMZ0 Mz
  hz.y = (cyh.a * hz.y + cyh.b * mzn.y) - cyh.b * mz.y;
  mz = mzn;
}

}  // namespace fdtd
