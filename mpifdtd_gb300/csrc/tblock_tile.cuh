// tblock_tile.cuh -- one warp tile of the temporally blocked stencil of the
// MPI solvers (fdtd_tblock.cu: one simulation; fdtd_batch.cu: many): K time
// steps (E half then H half, mpiTM_UPML.c:196-217, mpiTE_UPML.c:290-304) per
// pass over the fields in HBM.
//
// A warp owns one tile: a strip of W = 32 CPL - 2K columns and a row segment
// [r0, r1).  Each lane holds CPL adjacent columns (CPL = 1, or 2 for FP32:
// 16-byte loads of a column pair); the 32 lanes cover the strip plus K columns
// on each side.  The warp walks the rows i from r0 - K to r1 + K - 1 and keeps
// K time levels in registers, level l one row behind level l-1.  At front row
// r it loads the level-0 state (D of row r+1, H of row r, two rows ahead of
// use) and, for l = 1..K,
//   E^l at row e = r-l+1 from D^{l-1}(e), H^{l-1}(e) and H^{l-1}(e-1),
//   H^l at row h = r-l   from H^{l-1}(h), E^l(h) and E^l(h+1);
// the column neighbours (H[j-1] for E, E[j+1] for H) are the lane's own other
// column or, at the pair's edge, a warp shuffle.  Every level loses one valid
// column on each side and one valid row at the start, so after K levels the
// centre W columns of rows [r0, r1) are exact and only those are stored.  The
// launch reads one field set and writes the other (ping-pong), so overlapping
// tiles never read each other's results.
//
// HBM traffic per cell and launch: read D, H (+1/eps), write D, E, H: for TM
// FP32 (8+16+4) + (8+8+16) = 60 B per K steps instead of 100 B per step.
//
// Interior tiles (the whole cone has sigma = 0 and lies inside the active
// cells) run a kernel that carries no J/M auxiliaries and skips the
// active-cell tests; the other tiles run the general kernel from a
// packed work-list, with the PML update from the 1-D coefficient tables and
// the zero halo (PEC) ring frozen.
#pragma once
#include <cuda_runtime.h>

#include "fdtd_internal.cuh"
#include "stencil_ops.cuh"

namespace fdtd {
namespace tile {

// first owned column of strip 0: with two columns per lane the lane's first
// column must be even (16-byte aligned pairs: the pitch is a multiple of 8)
template <int K, int CPL> __host__ __device__ constexpr int origin() { return CPL == 1 ? 1 : (K & 1); }
template <int K, int CPL> __host__ __device__ constexpr int width() { return 32 * CPL - 2 * K; }

template <typename T> __device__ __forceinline__ T shup(T v)
{
  T r;
  r.x = __shfl_up_sync(0xffffffffu, v.x, 1);
  r.y = __shfl_up_sync(0xffffffffu, v.y, 1);
  return r;
}
template <typename T> __device__ __forceinline__ T shdn(T v)
{
  T r;
  r.x = __shfl_down_sync(0xffffffffu, v.x, 1);
  r.y = __shfl_down_sync(0xffffffffu, v.y, 1);
  return r;
}

template <typename R> __device__ __forceinline__ bool x_in(const StencilView<R> &v, int i)
{
  const int x = i + v.ox;
  return x >= v.in_x0 && x < v.in_x1;
}
template <typename R> __device__ __forceinline__ bool y_in(const StencilView<R> &v, int j)
{
  const int y = j + v.ox;
  return y >= v.in_y0 && y < v.in_y1;
}

// CPL complex values of a row from column j0 (zero where not active)
template <int CPL, typename T>
__device__ __forceinline__ void ld_cols(const T *p, const bool *act, T *out)
{
  if (CPL == 2 && act[0] && act[1]) {  // FP32 pair: one 16-byte load
    const float4 w = __ldg((const float4 *)p);
    out[0].x = w.x; out[0].y = w.y;
    out[CPL - 1].x = w.z; out[CPL - 1].y = w.w;
    return;
  }
#pragma unroll
  for (int q = 0; q < CPL; q++) out[q] = act[q] ? ldro(p + q) : czero<T>();
}
template <int CPL, typename R>
__device__ __forceinline__ void ld_real(const R *p, const bool *act, R *out)
{
  if (CPL == 2 && act[0] && act[1]) {
    const float2 w = __ldg((const float2 *)p);
    out[0] = w.x;
    out[CPL - 1] = w.y;
    return;
  }
#pragma unroll
  for (int q = 0; q < CPL; q++) out[q] = act[q] ? ldro(p + q) : (R)1;
}
template <int CPL, typename T>
__device__ __forceinline__ void st_cols(T *p, const bool *own, const T *val)
{
  if (CPL == 2 && own[0] && own[1]) {
    *(float4 *)p = make_float4(val[0].x, val[0].y, val[CPL - 1].x, val[CPL - 1].y);
    return;
  }
#pragma unroll
  for (int q = 0; q < CPL; q++)
    if (own[q]) p[q] = val[q];
}

// L2 prefetch of the row holding p[0] .. p[32 CPL - 1] of a warp (elements of
// `bytes` each): the lanes at 128-byte strides and the last lane issue it, so
// every line the warp's row touches is requested once.  The prefetched rows
// are rows the tile loads two row-steps later; a prefetch takes no register.
template <int CPL>
__device__ __forceinline__ void prefetch_row(const void *p, int bytes)
{
  const int lane = threadIdx.x & 31, per_line = 128 / (bytes * CPL);
  if (per_line <= 1 || lane % per_line == 0 || lane == 31)
    asm volatile("prefetch.L2 [%0];" ::"l"(p));
}

// One lane's view of its tile.
template <int CPL>
struct Lane {
  int j;             // array column of the lane's first column
  int r0, r1;        // owned rows [r0, r1)
  bool jact[CPL];    // the column is active (1..nj)
  bool own[CPL];     // the column is one of the tile's W owned columns
  bool yin[CPL];     // the column is PML-free
  int colq[CPL];     // index of the NTFF column line through the column, or -1
  bool lines;        // the lane stores NTFF line samples in this tile
};

template <int K, int CPL, typename R>
__device__ __forceinline__ Lane<CPL> lane_of(const StencilView<R> &v, const TBlockView<R> &tb, int strip, int r0,
                                             int r1)
{
  constexpr int W = width<K, CPL>();
  const int lane = threadIdx.x & 31;
  Lane<CPL> t;
  t.j = origin<K, CPL>() + strip * W - K + lane * CPL;
  t.r0 = r0;
  t.r1 = r1;
  t.lines = false;
  bool any_row = false;
  if (tb.col)
    for (int q = 0; q < 4; q++)
      if (tb.ri[q] >= r0 && tb.ri[q] < r1) any_row = true;
#pragma unroll
  for (int q = 0; q < CPL; q++) {
    const int j = t.j + q, lc = lane * CPL + q;
    t.jact[q] = j >= 1 && j <= v.nj;
    t.own[q] = t.jact[q] && lc >= K && lc < 32 * CPL - K;
    t.yin[q] = y_in(v, j);
    t.colq[q] = -1;
    if (tb.col && t.own[q]) {
      for (int c = 0; c < 4; c++)
        if (j == tb.cj[c]) t.colq[q] = c;
      if (t.colq[q] >= 0 || any_row) t.lines = true;
    }
  }
  return t;
}

// NTFF line sample: field f of level lev at owned cell (i, t.j + q)
template <int CPL, typename R, typename T>
__device__ __forceinline__ void line_put(const StencilView<R> &v, const TBlockView<R> &tb, const Lane<CPL> &t, int q,
                                         int lev, int i, int f, const T &val)
{
  if (t.colq[q] >= 0) tb.col[((size_t)(lev * 4 + t.colq[q]) * 3 + f) * v.nxa + i] = val;
#pragma unroll
  for (int c = 0; c < 4; c++)
    if (i == tb.ri[c]) tb.row[((size_t)(lev * 4 + c) * 3 + f) * v.P + t.j + q] = val;
}

// ------------------------------------------------------------------ TM
// slots 0 Ez 1 Dz 2 Jz 3 Hx 4 Hy 5 Mx 6 My
template <typename R, int K, bool AUX, int CPL = 1>
__device__ __forceinline__ void tm_tile(const StencilView<R> &v, const TBlockView<R> &tb, int strip, int r0,
                                        int r1, int nlev)
{
  static_assert(CPL == 1 || sizeof(R) == 4, "two columns per lane: FP32 only");
  using T = typename Cplx<R>::T;
  struct ES { T d, e, j; R ie; };
  struct HS { T x, y, mx, my; };
  const Lane<CPL> t = lane_of<K, CPL>(v, tb, strip, r0, r1);
  const int j = t.j;
  const size_t P = (size_t)v.P;
  const T *Dz = v.f[1], *Jz = v.f[2], *Hx = v.f[3], *Hy = v.f[4], *Mx = v.f[5], *My = v.f[6];
  const R *IE = v.inv_eps[0];
  ES E[K + 1][CPL];
  HS H[K + 1][CPL];
#pragma unroll
  for (int l = 0; l <= K; l++)
#pragma unroll
    for (int q = 0; q < CPL; q++) {
      E[l][q].d = E[l][q].e = E[l][q].j = czero<T>();
      E[l][q].ie = (R)1;
      H[l][q].x = H[l][q].y = H[l][q].mx = H[l][q].my = czero<T>();
    }
  // level-0 state of front row r: D (J, 1/eps) of row r+1 and H (M) of row r,
  // zero outside the active rows/columns
  auto load0 = [&](int r, ES *n, HS *m) {
    const int a = r + 1;
#pragma unroll
    for (int q = 0; q < CPL; q++) {
      n[q].d = n[q].e = n[q].j = czero<T>();
      n[q].ie = (R)1;
      m[q].x = m[q].y = m[q].mx = m[q].my = czero<T>();
    }
    if (a >= 1 && a <= v.ni) {  // a branch (not straight-line loads) measured 1.3x faster
      const size_t k = (size_t)a * P + j;
      T d[CPL];
      R ie[CPL];
      ld_cols<CPL>(Dz + k, t.jact, d);
      ld_real<CPL>(IE + k, t.jact, ie);
#pragma unroll
      for (int q = 0; q < CPL; q++) {
        n[q].d = d[q];
        n[q].ie = ie[q];
        if (AUX && t.jact[q] && !(t.yin[q] && x_in(v, a))) n[q].j = ldro(Jz + k + q);
      }
    }
    if (r >= 1 && r <= v.ni) {
      const size_t k = (size_t)r * P + j;
      T hx[CPL], hy[CPL];
      ld_cols<CPL>(Hx + k, t.jact, hx);
      ld_cols<CPL>(Hy + k, t.jact, hy);
#pragma unroll
      for (int q = 0; q < CPL; q++) {
        m[q].x = hx[q];
        m[q].y = hy[q];
        if (AUX && t.jact[q] && !(t.yin[q] && x_in(v, r))) {
          m[q].mx = ldro(Mx + k + q);
          m[q].my = ldro(My + k + q);
        }
      }
    }
  };
  ES pe0[CPL], pe1[CPL];
  HS ph0[CPL], ph1[CPL];
  load0(t.r0 - K, pe0, ph0);
  load0(t.r0 - K + 1, pe1, ph1);
#pragma unroll 1
  for (int r = t.r0 - K; r < t.r1 + K; r++) {
    ES eo[CPL];
    HS ho[CPL];
#pragma unroll
    for (int q = 0; q < CPL; q++) {
      eo[q] = E[0][q];
      ho[q] = H[0][q];
      E[0][q] = pe0[q];
      H[0][q] = ph0[q];
      pe0[q] = pe1[q];
      ph0[q] = ph1[q];
    }
    load0(r + 2, pe1, ph1);
    {  // rows the tile loads two row-steps later
      const int rp = r + 4, ap = rp + 1;
      if (ap >= 1 && ap <= v.ni) {
        prefetch_row<CPL>(Dz + (size_t)ap * P + j, sizeof(T));
        prefetch_row<CPL>(IE + (size_t)ap * P + j, sizeof(R));
      }
      if (rp >= 1 && rp <= v.ni) {
        prefetch_row<CPL>(Hx + (size_t)rp * P + j, sizeof(T));
        prefetch_row<CPL>(Hy + (size_t)rp * P + j, sizeof(T));
      }
    }
#pragma unroll
    for (int l = 1; l <= K; l++) {
      const int e = r - l + 1, h = r - l;
      const bool erow = e >= 1 && e <= v.ni, hrow = h >= 1 && h <= v.ni;
      // E half (calcJD + calcE + scatteredWave) at row e
      T hxb[CPL];  // Hx^{l-1}(e, j-1)
      hxb[0] = shup(H[l - 1][CPL - 1].x);
#pragma unroll
      for (int q = 1; q < CPL; q++) hxb[q] = H[l - 1][q - 1].x;
      ES en[CPL];
#pragma unroll
      for (int q = 0; q < CPL; q++) {
        en[q].ie = eo[q].ie;
        en[q].d = en[q].e = en[q].j = czero<T>();
        if (l > nlev) {  // frozen level (the instance stops inside this launch): E^l = E^{l-1}
          en[q] = eo[q];
        } else if (!AUX || (t.jact[q] && erow)) {
          T curl;
          curl.x = ((H[l - 1][q].y.x - ho[q].y.x) - H[l - 1][q].x.x) + hxb[q].x;
          curl.y = ((H[l - 1][q].y.y - ho[q].y.y) - H[l - 1][q].x.y) + hxb[q].y;
          T dz = eo[q].d;
          if (!AUX || (t.yin[q] && x_in(v, e))) {
            dz = cadd(dz, curl);
          } else {
            T jz = eo[q].j;
            tm_e_pml(v, e, j + q, curl, dz, jz);
            en[q].j = jz;
          }
          en[q].d = dz;
          T ez = dz;
          if (!is_one(en[q].ie)) {
            ez = cscale(dz, en[q].ie);
            cw_add_level<R>(v, tb.sc[l - 1].x, tb.sc[l - 1].y, l - 1, e, j + q, en[q].ie, ez);
          }
          en[q].e = ez;
        }
      }
      ES eold[CPL];  // E^l of row h = e-1
#pragma unroll
      for (int q = 0; q < CPL; q++) {
        eold[q] = E[l][q];
        E[l][q] = en[q];
      }
      // H half (calcMB + calcH) at row h
      T ezr[CPL];  // Ez^l(h, j+1)
      ezr[CPL - 1] = shdn(eold[0].e);
#pragma unroll
      for (int q = 0; q + 1 < CPL; q++) ezr[q] = eold[q + 1].e;
      HS hn[CPL];
#pragma unroll
      for (int q = 0; q < CPL; q++) {
        hn[q].x = hn[q].y = hn[q].mx = hn[q].my = czero<T>();
        if (l > nlev) {
          hn[q] = ho[q];
        } else if (!AUX || (t.jact[q] && hrow)) {
          const T dEx = csub(ezr[q], eold[q].e);
          const T dEy = csub(eold[q].e, en[q].e);
          T hx = ho[q].x, hy = ho[q].y;
          if (!AUX || (t.yin[q] && x_in(v, h))) {
            hx.x -= v.inv_mu * dEx.x; hx.y -= v.inv_mu * dEx.y;
            hy.x -= v.inv_mu * dEy.x; hy.y -= v.inv_mu * dEy.y;
          } else {
            T mx = ho[q].mx, my = ho[q].my;
            tm_h_pml(v, h, j + q, dEx, dEy, hx, hy, mx, my);
            hn[q].mx = mx;
            hn[q].my = my;
          }
          hn[q].x = hx;
          hn[q].y = hy;
        }
      }
#pragma unroll
      for (int q = 0; q < CPL; q++) {
        const HS hold = H[l][q];
        H[l][q] = hn[q];
        if (t.lines && t.own[q]) {
          if (e >= t.r0 && e < t.r1) line_put(v, tb, t, q, l - 1, e, 0, en[q].e);
          if (h >= t.r0 && h < t.r1) {
            line_put(v, tb, t, q, l - 1, h, 1, hn[q].x);
            line_put(v, tb, t, q, l - 1, h, 2, hn[q].y);
          }
        }
        eo[q] = eold[q];
        ho[q] = hold;
      }
    }
    {  // level K is final: E of row r-K+1, H of row r-K
      const int e = r - K + 1, h = r - K;
      if (e >= t.r0 && e < t.r1) {
        const size_t k = (size_t)e * P + j;
        T d[CPL], ez[CPL];
#pragma unroll
        for (int q = 0; q < CPL; q++) {
          d[q] = E[K][q].d;
          ez[q] = E[K][q].e;
          if (AUX && t.own[q] && !(t.yin[q] && x_in(v, e))) tb.out[2][k + q] = E[K][q].j;
        }
        st_cols<CPL>(tb.out[1] + k, t.own, d);
        st_cols<CPL>(tb.out[0] + k, t.own, ez);
      }
      if (h >= t.r0 && h < t.r1) {
        const size_t k = (size_t)h * P + j;
        T hx[CPL], hy[CPL];
#pragma unroll
        for (int q = 0; q < CPL; q++) {
          hx[q] = H[K][q].x;
          hy[q] = H[K][q].y;
          if (AUX && t.own[q] && !(t.yin[q] && x_in(v, h))) {
            tb.out[5][k + q] = H[K][q].mx;
            tb.out[6][k + q] = H[K][q].my;
          }
        }
        st_cols<CPL>(tb.out[3] + k, t.own, hx);
        st_cols<CPL>(tb.out[4] + k, t.own, hy);
      }
    }
  }
}

// ------------------------------------------------------------------ TE
// slots 0 Ex 1 Ey 2 Dx 3 Dy 4 Jx 5 Jy 6 Hz 7 Mz; the CW source drives Ey only
// (the MPI TE solver's scatteredWave, mpiTE_UPML.c:250-281).
template <typename R, int K, bool AUX, int CPL = 1>
__device__ __forceinline__ void te_tile(const StencilView<R> &v, const TBlockView<R> &tb, int strip, int r0,
                                        int r1, int nlev)
{
  static_assert(CPL == 1 || sizeof(R) == 4, "two columns per lane: FP32 only");
  using T = typename Cplx<R>::T;
  struct ES { T dx, dy, ex, ey, jx, jy; R iex, iey; };
  struct HS { T z, mz; };
  const Lane<CPL> t = lane_of<K, CPL>(v, tb, strip, r0, r1);
  const int j = t.j;
  const size_t P = (size_t)v.P;
  const T *Dx = v.f[2], *Dy = v.f[3], *Jx = v.f[4], *Jy = v.f[5], *Hz = v.f[6], *Mz = v.f[7];
  const R *IEX = v.inv_eps[0], *IEY = v.inv_eps[1];
  ES E[K + 1][CPL];
  HS H[K + 1][CPL];
#pragma unroll
  for (int l = 0; l <= K; l++)
#pragma unroll
    for (int q = 0; q < CPL; q++) {
      E[l][q].dx = E[l][q].dy = E[l][q].ex = E[l][q].ey = E[l][q].jx = E[l][q].jy = czero<T>();
      E[l][q].iex = E[l][q].iey = (R)1;
      H[l][q].z = H[l][q].mz = czero<T>();
    }
  auto load0 = [&](int r, ES *n, HS *m) {  // D (J, 1/eps) of row r+1, H (M) of row r
    const int a = r + 1;
#pragma unroll
    for (int q = 0; q < CPL; q++) {
      n[q].dx = n[q].dy = n[q].ex = n[q].ey = n[q].jx = n[q].jy = czero<T>();
      n[q].iex = n[q].iey = (R)1;
      m[q].z = m[q].mz = czero<T>();
    }
    if (a >= 1 && a <= v.ni) {  // a branch (not straight-line loads) measured 1.3x faster
      const size_t k = (size_t)a * P + j;
      T dx[CPL], dy[CPL];
      R iex[CPL], iey[CPL];
      ld_cols<CPL>(Dx + k, t.jact, dx);
      ld_cols<CPL>(Dy + k, t.jact, dy);
      ld_real<CPL>(IEX + k, t.jact, iex);
      ld_real<CPL>(IEY + k, t.jact, iey);
#pragma unroll
      for (int q = 0; q < CPL; q++) {
        n[q].dx = dx[q];
        n[q].dy = dy[q];
        n[q].iex = iex[q];
        n[q].iey = iey[q];
        if (AUX && t.jact[q] && !(t.yin[q] && x_in(v, a))) {
          n[q].jx = ldro(Jx + k + q);
          n[q].jy = ldro(Jy + k + q);
        }
      }
    }
    if (r >= 1 && r <= v.ni) {
      const size_t k = (size_t)r * P + j;
      T hz[CPL];
      ld_cols<CPL>(Hz + k, t.jact, hz);
#pragma unroll
      for (int q = 0; q < CPL; q++) {
        m[q].z = hz[q];
        if (AUX && t.jact[q] && !(t.yin[q] && x_in(v, r))) m[q].mz = ldro(Mz + k + q);
      }
    }
  };
  ES pe0[CPL], pe1[CPL];
  HS ph0[CPL], ph1[CPL];
  load0(t.r0 - K, pe0, ph0);
  load0(t.r0 - K + 1, pe1, ph1);
#pragma unroll 1
  for (int r = t.r0 - K; r < t.r1 + K; r++) {
    ES eo[CPL];
    HS ho[CPL];
#pragma unroll
    for (int q = 0; q < CPL; q++) {
      eo[q] = E[0][q];
      ho[q] = H[0][q];
      E[0][q] = pe0[q];
      H[0][q] = ph0[q];
      pe0[q] = pe1[q];
      ph0[q] = ph1[q];
    }
    load0(r + 2, pe1, ph1);
    {  // rows the tile loads two row-steps later
      const int rp = r + 4, ap = rp + 1;
      if (ap >= 1 && ap <= v.ni) {
        prefetch_row<CPL>(Dx + (size_t)ap * P + j, sizeof(T));
        prefetch_row<CPL>(Dy + (size_t)ap * P + j, sizeof(T));
        prefetch_row<CPL>(IEX + (size_t)ap * P + j, sizeof(R));
        prefetch_row<CPL>(IEY + (size_t)ap * P + j, sizeof(R));
      }
      if (rp >= 1 && rp <= v.ni) prefetch_row<CPL>(Hz + (size_t)rp * P + j, sizeof(T));
    }
#pragma unroll
    for (int l = 1; l <= K; l++) {
      const int e = r - l + 1, h = r - l;
      const bool erow = e >= 1 && e <= v.ni, hrow = h >= 1 && h <= v.ni;
      T hzb[CPL];  // Hz^{l-1}(e, j-1)
      hzb[0] = shup(H[l - 1][CPL - 1].z);
#pragma unroll
      for (int q = 1; q < CPL; q++) hzb[q] = H[l - 1][q - 1].z;
      ES en[CPL];
#pragma unroll
      for (int q = 0; q < CPL; q++) {
        en[q].iex = eo[q].iex;
        en[q].iey = eo[q].iey;
        en[q].dx = en[q].dy = en[q].ex = en[q].ey = en[q].jx = en[q].jy = czero<T>();
        if (l > nlev) {  // frozen level (the instance stops inside this launch): E^l = E^{l-1}
          en[q] = eo[q];
        } else if (!AUX || (t.jact[q] && erow)) {
          const T hzk = H[l - 1][q].z;
          const T cxv = csub(hzk, hzb[q]);  // Hz - Hz[j-1]
          T cyv;                            // -Hz + Hz[i-1]
          cyv.x = -hzk.x + ho[q].z.x;
          cyv.y = -hzk.y + ho[q].z.y;
          T dx = eo[q].dx, dy = eo[q].dy;
          if (!AUX || (t.yin[q] && x_in(v, e))) {
            dx = cadd(dx, cxv);
            dy = cadd(dy, cyv);
          } else {
            T jx = eo[q].jx, jy = eo[q].jy;
            te_e_pml(v, e, j + q, cxv, cyv, dx, dy, jx, jy);
            en[q].jx = jx;
            en[q].jy = jy;
          }
          en[q].dx = dx;
          en[q].dy = dy;
          T ex = dx, ey = dy;
          if (!is_one(en[q].iex)) ex = cscale(dx, en[q].iex);
          if (!is_one(en[q].iey)) {
            ey = cscale(dy, en[q].iey);
            cw_add_level<R>(v, tb.sc[l - 1].x, tb.sc[l - 1].y, l - 1, e, j + q, en[q].iey, ey);
          }
          en[q].ex = ex;
          en[q].ey = ey;
        }
      }
      ES eold[CPL];
#pragma unroll
      for (int q = 0; q < CPL; q++) {
        eold[q] = E[l][q];
        E[l][q] = en[q];
      }
      T ext[CPL];  // Ex^l(h, j+1)
      ext[CPL - 1] = shdn(eold[0].ex);
#pragma unroll
      for (int q = 0; q + 1 < CPL; q++) ext[q] = eold[q + 1].ex;
      HS hn[CPL];
#pragma unroll
      for (int q = 0; q < CPL; q++) {
        hn[q].z = hn[q].mz = czero<T>();
        if (l > nlev) {
          hn[q] = ho[q];
        } else if (!AUX || (t.jact[q] && hrow)) {
          T ce;  // Ey[i+1] - Ey - Ex[j+1] + Ex
          ce.x = ((en[q].ey.x - eold[q].ey.x) - ext[q].x) + eold[q].ex.x;
          ce.y = ((en[q].ey.y - eold[q].ey.y) - ext[q].y) + eold[q].ex.y;
          T hz = ho[q].z;
          if (!AUX || (t.yin[q] && x_in(v, h))) {
            hz.x -= v.inv_mu * ce.x;
            hz.y -= v.inv_mu * ce.y;
          } else {
            T mz = ho[q].mz;
            te_h_pml(v, h, j + q, ce, hz, mz);
            hn[q].mz = mz;
          }
          hn[q].z = hz;
        }
      }
#pragma unroll
      for (int q = 0; q < CPL; q++) {
        const HS hold = H[l][q];
        H[l][q] = hn[q];
        if (t.lines && t.own[q]) {
          if (e >= t.r0 && e < t.r1) {
            line_put(v, tb, t, q, l - 1, e, 0, en[q].ex);
            line_put(v, tb, t, q, l - 1, e, 1, en[q].ey);
          }
          if (h >= t.r0 && h < t.r1) line_put(v, tb, t, q, l - 1, h, 2, hn[q].z);
        }
        eo[q] = eold[q];
        ho[q] = hold;
      }
    }
    {
      const int e = r - K + 1, h = r - K;
      if (e >= t.r0 && e < t.r1) {
        const size_t k = (size_t)e * P + j;
        T dx[CPL], dy[CPL], ex[CPL], ey[CPL];
#pragma unroll
        for (int q = 0; q < CPL; q++) {
          dx[q] = E[K][q].dx;
          dy[q] = E[K][q].dy;
          ex[q] = E[K][q].ex;
          ey[q] = E[K][q].ey;
          if (AUX && t.own[q] && !(t.yin[q] && x_in(v, e))) {
            tb.out[4][k + q] = E[K][q].jx;
            tb.out[5][k + q] = E[K][q].jy;
          }
        }
        st_cols<CPL>(tb.out[2] + k, t.own, dx);
        st_cols<CPL>(tb.out[3] + k, t.own, dy);
        st_cols<CPL>(tb.out[0] + k, t.own, ex);
        st_cols<CPL>(tb.out[1] + k, t.own, ey);
      }
      if (h >= t.r0 && h < t.r1) {
        const size_t k = (size_t)h * P + j;
        T hz[CPL];
#pragma unroll
        for (int q = 0; q < CPL; q++) {
          hz[q] = H[K][q].z;
          if (AUX && t.own[q] && !(t.yin[q] && x_in(v, h))) tb.out[7][k + q] = H[K][q].mz;
        }
        st_cols<CPL>(tb.out[6] + k, t.own, hz);
      }
    }
  }
}

// ------------------------------------------------------------------ serial solvers
//
// The serial solvers step H before E (fdtdTM_upml.c:54-66, fdtdTE_upml.c:
// 168-192) and drive E with the Gaussian pulse (field.c:224-256, tb.pulse:
// the block's first step; level l adds l - 1 to its time).  Level l at front
// row r computes H^l and then E^l, both at row h = r - l:
//   H^l(h) from H^{l-1}(h), E^{l-1}(h) and E^{l-1}(h+1),
//   E^l(h) from D^{l-1}(h), H^l(h) and H^l(h-1);
// the level-0 state of front row r is E (D, J, 1/eps) and H (M) of row r.  With
// the first front row r0 - K, E^l is exact from row r0 - K + l and H^l from
// r0 - K + l - 1; each level loses one column on each side (H^l reads E^{l-1}
// of column j+1, E^l reads H^l of column j-1).  The cell updates are those of
// the one-step kernels (tm_h/tm_e, te_h/te_e).

template <typename R, int K, bool AUX, int CPL = 1>
__device__ __forceinline__ void tm_tile_hf(const StencilView<R> &v, const TBlockView<R> &tb, int strip, int r0,
                                           int r1)
{
  static_assert(CPL == 1 || sizeof(R) == 4, "two columns per lane: FP32 only");
  using T = typename Cplx<R>::T;
  struct ES { T d, e, j; R ie; };
  struct HS { T x, y, mx, my; };
  const Lane<CPL> t = lane_of<K, CPL>(v, tb, strip, r0, r1);
  const int j = t.j;
  const size_t P = (size_t)v.P;
  const T *Ez = v.f[0], *Dz = v.f[1], *Jz = v.f[2], *Hx = v.f[3], *Hy = v.f[4], *Mx = v.f[5], *My = v.f[6];
  const R *IE = v.inv_eps[0];
  ES E[K + 1][CPL];
  HS H[K + 1][CPL];
#pragma unroll
  for (int l = 0; l <= K; l++)
#pragma unroll
    for (int q = 0; q < CPL; q++) {
      E[l][q].d = E[l][q].e = E[l][q].j = czero<T>();
      E[l][q].ie = (R)1;
      H[l][q].x = H[l][q].y = H[l][q].mx = H[l][q].my = czero<T>();
    }
  auto load0 = [&](int r, ES *n, HS *m) {  // E (D, J, 1/eps) and H (M) of row r
#pragma unroll
    for (int q = 0; q < CPL; q++) {
      n[q].d = n[q].e = n[q].j = czero<T>();
      n[q].ie = (R)1;
      m[q].x = m[q].y = m[q].mx = m[q].my = czero<T>();
    }
    if (r >= 1 && r <= v.ni) {
      const size_t k = (size_t)r * P + j;
      T ez[CPL], d[CPL], hx[CPL], hy[CPL];
      R ie[CPL];
      ld_cols<CPL>(Ez + k, t.jact, ez);
      ld_cols<CPL>(Dz + k, t.jact, d);
      ld_real<CPL>(IE + k, t.jact, ie);
      ld_cols<CPL>(Hx + k, t.jact, hx);
      ld_cols<CPL>(Hy + k, t.jact, hy);
#pragma unroll
      for (int q = 0; q < CPL; q++) {
        n[q].e = ez[q];
        n[q].d = d[q];
        n[q].ie = ie[q];
        m[q].x = hx[q];
        m[q].y = hy[q];
        if (AUX && t.jact[q] && !(t.yin[q] && x_in(v, r))) {
          n[q].j = ldro(Jz + k + q);
          m[q].mx = ldro(Mx + k + q);
          m[q].my = ldro(My + k + q);
        }
      }
    }
  };
  ES pe0[CPL], pe1[CPL];
  HS ph0[CPL], ph1[CPL];
  load0(t.r0 - K, pe0, ph0);
  load0(t.r0 - K + 1, pe1, ph1);
#pragma unroll 1
  for (int r = t.r0 - K; r < t.r1 + K; r++) {
    ES eo[CPL];  // E^{l-1} of row r - l (the previous front row's), entering level l
    HS ho[CPL];  // H^{l-1} of row r - l
#pragma unroll
    for (int q = 0; q < CPL; q++) {
      eo[q] = E[0][q];
      ho[q] = H[0][q];
      E[0][q] = pe0[q];
      H[0][q] = ph0[q];
      pe0[q] = pe1[q];
      ph0[q] = ph1[q];
    }
    load0(r + 2, pe1, ph1);
    {  // rows the tile loads two row-steps later
      const int rp = r + 4;
      if (rp >= 1 && rp <= v.ni) {
        prefetch_row<CPL>(Ez + (size_t)rp * P + j, sizeof(T));
        prefetch_row<CPL>(Dz + (size_t)rp * P + j, sizeof(T));
        prefetch_row<CPL>(IE + (size_t)rp * P + j, sizeof(R));
        prefetch_row<CPL>(Hx + (size_t)rp * P + j, sizeof(T));
        prefetch_row<CPL>(Hy + (size_t)rp * P + j, sizeof(T));
      }
    }
#pragma unroll
    for (int l = 1; l <= K; l++) {
      const int h = r - l;
      const bool hrow = h >= 1 && h <= v.ni;
      // H half (calcMB + calcH) at row h from E^{l-1} of rows h (eo) and h + 1 (E[l-1])
      T ezr[CPL];  // Ez^{l-1}(h, j+1)
      ezr[CPL - 1] = shdn(eo[0].e);
#pragma unroll
      for (int q = 0; q + 1 < CPL; q++) ezr[q] = eo[q + 1].e;
      HS hn[CPL];
#pragma unroll
      for (int q = 0; q < CPL; q++) {
        hn[q].x = hn[q].y = hn[q].mx = hn[q].my = czero<T>();
        if (!AUX || (t.jact[q] && hrow)) {
          const T dEx = csub(ezr[q], eo[q].e);
          const T dEy = csub(eo[q].e, E[l - 1][q].e);
          T hx = ho[q].x, hy = ho[q].y;
          if (!AUX || (t.yin[q] && x_in(v, h))) {
            hx.x -= v.inv_mu * dEx.x; hx.y -= v.inv_mu * dEx.y;
            hy.x -= v.inv_mu * dEy.x; hy.y -= v.inv_mu * dEy.y;
          } else {
            T mx = ho[q].mx, my = ho[q].my;
            tm_h_pml(v, h, j + q, dEx, dEy, hx, hy, mx, my);
            hn[q].mx = mx;
            hn[q].my = my;
          }
          hn[q].x = hx;
          hn[q].y = hy;
        }
      }
      HS hold[CPL];  // H^l of row h - 1
#pragma unroll
      for (int q = 0; q < CPL; q++) {
        hold[q] = H[l][q];
        H[l][q] = hn[q];
      }
      // E half (calcJD + calcE + pulse) at row h from H^l of rows h (hn) and h - 1 (hold)
      T hxb[CPL];  // Hx^l(h, j-1)
      hxb[0] = shup(hn[CPL - 1].x);
#pragma unroll
      for (int q = 1; q < CPL; q++) hxb[q] = hn[q - 1].x;
      ES en[CPL];
#pragma unroll
      for (int q = 0; q < CPL; q++) {
        en[q].ie = eo[q].ie;
        en[q].d = en[q].e = en[q].j = czero<T>();
        if (!AUX || (t.jact[q] && hrow)) {
          T curl;
          curl.x = ((hn[q].y.x - hold[q].y.x) - hn[q].x.x) + hxb[q].x;
          curl.y = ((hn[q].y.y - hold[q].y.y) - hn[q].x.y) + hxb[q].y;
          T dz = eo[q].d;
          if (!AUX || (t.yin[q] && x_in(v, h))) {
            dz = cadd(dz, curl);
          } else {
            T jz = eo[q].j;
            tm_e_pml(v, h, j + q, curl, dz, jz);
            en[q].j = jz;
          }
          en[q].d = dz;
          T ez = dz;
          if (!is_one(en[q].ie)) {
            ez = cscale(dz, en[q].ie);
            if (tb.pulse[0].kind) {
              if (tb.ptab[0]) pulse_row<R>(tb.ptab[0][(size_t)(l - 1) * v.nxa + h], en[q].ie, ez);
              else pulse_source<R>(tb.pulse[0], h, j + q, en[q].ie, ez, (double)(l - 1));
            }
          }
          en[q].e = ez;
        }
      }
#pragma unroll
      for (int q = 0; q < CPL; q++) {
        const ES eold = E[l][q];  // E^l of row h - 1
        E[l][q] = en[q];
        if (t.lines && t.own[q] && h >= t.r0 && h < t.r1) {
          line_put(v, tb, t, q, l - 1, h, 0, en[q].e);
          line_put(v, tb, t, q, l - 1, h, 1, hn[q].x);
          line_put(v, tb, t, q, l - 1, h, 2, hn[q].y);
        }
        eo[q] = eold;
        ho[q] = hold[q];
      }
    }
    {  // level K is final: E and H of row r - K
      const int h = r - K;
      if (h >= t.r0 && h < t.r1) {
        const size_t k = (size_t)h * P + j;
        T d[CPL], ez[CPL], hx[CPL], hy[CPL];
#pragma unroll
        for (int q = 0; q < CPL; q++) {
          d[q] = E[K][q].d;
          ez[q] = E[K][q].e;
          hx[q] = H[K][q].x;
          hy[q] = H[K][q].y;
          if (AUX && t.own[q] && !(t.yin[q] && x_in(v, h))) {
            tb.out[2][k + q] = E[K][q].j;
            tb.out[5][k + q] = H[K][q].mx;
            tb.out[6][k + q] = H[K][q].my;
          }
        }
        st_cols<CPL>(tb.out[1] + k, t.own, d);
        st_cols<CPL>(tb.out[0] + k, t.own, ez);
        st_cols<CPL>(tb.out[3] + k, t.own, hx);
        st_cols<CPL>(tb.out[4] + k, t.own, hy);
      }
    }
  }
}

template <typename R, int K, bool AUX, int CPL = 1>
__device__ __forceinline__ void te_tile_hf(const StencilView<R> &v, const TBlockView<R> &tb, int strip, int r0,
                                           int r1)
{
  static_assert(CPL == 1 || sizeof(R) == 4, "two columns per lane: FP32 only");
  using T = typename Cplx<R>::T;
  struct ES { T dx, dy, ex, ey, jx, jy; R iex, iey; };
  struct HS { T z, mz; };
  const Lane<CPL> t = lane_of<K, CPL>(v, tb, strip, r0, r1);
  const int j = t.j;
  const size_t P = (size_t)v.P;
  const T *Ex = v.f[0], *Ey = v.f[1], *Dx = v.f[2], *Dy = v.f[3], *Jx = v.f[4], *Jy = v.f[5], *Hz = v.f[6],
          *Mz = v.f[7];
  const R *IEX = v.inv_eps[0], *IEY = v.inv_eps[1];
  ES E[K + 1][CPL];
  HS H[K + 1][CPL];
#pragma unroll
  for (int l = 0; l <= K; l++)
#pragma unroll
    for (int q = 0; q < CPL; q++) {
      E[l][q].dx = E[l][q].dy = E[l][q].ex = E[l][q].ey = E[l][q].jx = E[l][q].jy = czero<T>();
      E[l][q].iex = E[l][q].iey = (R)1;
      H[l][q].z = H[l][q].mz = czero<T>();
    }
  auto load0 = [&](int r, ES *n, HS *m) {  // E (D, J, 1/eps) and H (M) of row r
#pragma unroll
    for (int q = 0; q < CPL; q++) {
      n[q].dx = n[q].dy = n[q].ex = n[q].ey = n[q].jx = n[q].jy = czero<T>();
      n[q].iex = n[q].iey = (R)1;
      m[q].z = m[q].mz = czero<T>();
    }
    if (r >= 1 && r <= v.ni) {
      const size_t k = (size_t)r * P + j;
      T ex[CPL], ey[CPL], dx[CPL], dy[CPL], hz[CPL];
      R iex[CPL], iey[CPL];
      ld_cols<CPL>(Ex + k, t.jact, ex);
      ld_cols<CPL>(Ey + k, t.jact, ey);
      ld_cols<CPL>(Dx + k, t.jact, dx);
      ld_cols<CPL>(Dy + k, t.jact, dy);
      ld_real<CPL>(IEX + k, t.jact, iex);
      ld_real<CPL>(IEY + k, t.jact, iey);
      ld_cols<CPL>(Hz + k, t.jact, hz);
#pragma unroll
      for (int q = 0; q < CPL; q++) {
        n[q].ex = ex[q];
        n[q].ey = ey[q];
        n[q].dx = dx[q];
        n[q].dy = dy[q];
        n[q].iex = iex[q];
        n[q].iey = iey[q];
        m[q].z = hz[q];
        if (AUX && t.jact[q] && !(t.yin[q] && x_in(v, r))) {
          n[q].jx = ldro(Jx + k + q);
          n[q].jy = ldro(Jy + k + q);
          m[q].mz = ldro(Mz + k + q);
        }
      }
    }
  };
  ES pe0[CPL], pe1[CPL];
  HS ph0[CPL], ph1[CPL];
  load0(t.r0 - K, pe0, ph0);
  load0(t.r0 - K + 1, pe1, ph1);
#pragma unroll 1
  for (int r = t.r0 - K; r < t.r1 + K; r++) {
    ES eo[CPL];
    HS ho[CPL];
#pragma unroll
    for (int q = 0; q < CPL; q++) {
      eo[q] = E[0][q];
      ho[q] = H[0][q];
      E[0][q] = pe0[q];
      H[0][q] = ph0[q];
      pe0[q] = pe1[q];
      ph0[q] = ph1[q];
    }
    load0(r + 2, pe1, ph1);
    {  // rows the tile loads two row-steps later
      const int rp = r + 4;
      if (rp >= 1 && rp <= v.ni) {
        prefetch_row<CPL>(Ex + (size_t)rp * P + j, sizeof(T));
        prefetch_row<CPL>(Ey + (size_t)rp * P + j, sizeof(T));
        prefetch_row<CPL>(Dx + (size_t)rp * P + j, sizeof(T));
        prefetch_row<CPL>(Dy + (size_t)rp * P + j, sizeof(T));
        prefetch_row<CPL>(IEX + (size_t)rp * P + j, sizeof(R));
        prefetch_row<CPL>(IEY + (size_t)rp * P + j, sizeof(R));
        prefetch_row<CPL>(Hz + (size_t)rp * P + j, sizeof(T));
      }
    }
#pragma unroll
    for (int l = 1; l <= K; l++) {
      const int h = r - l;
      const bool hrow = h >= 1 && h <= v.ni;
      // H half (calcMB + calcH) at row h from E^{l-1} of rows h (eo) and h + 1 (E[l-1])
      T ext[CPL];  // Ex^{l-1}(h, j+1)
      ext[CPL - 1] = shdn(eo[0].ex);
#pragma unroll
      for (int q = 0; q + 1 < CPL; q++) ext[q] = eo[q + 1].ex;
      HS hn[CPL];
#pragma unroll
      for (int q = 0; q < CPL; q++) {
        hn[q].z = hn[q].mz = czero<T>();
        if (!AUX || (t.jact[q] && hrow)) {
          T ce;  // Ey[i+1] - Ey - Ex[j+1] + Ex
          ce.x = ((E[l - 1][q].ey.x - eo[q].ey.x) - ext[q].x) + eo[q].ex.x;
          ce.y = ((E[l - 1][q].ey.y - eo[q].ey.y) - ext[q].y) + eo[q].ex.y;
          T hz = ho[q].z;
          if (!AUX || (t.yin[q] && x_in(v, h))) {
            hz.x -= v.inv_mu * ce.x;
            hz.y -= v.inv_mu * ce.y;
          } else {
            T mz = ho[q].mz;
            te_h_pml(v, h, j + q, ce, hz, mz);
            hn[q].mz = mz;
          }
          hn[q].z = hz;
        }
      }
      HS hold[CPL];  // H^l of row h - 1
#pragma unroll
      for (int q = 0; q < CPL; q++) {
        hold[q] = H[l][q];
        H[l][q] = hn[q];
      }
      // E half (calcJD + calcE + pulse) at row h from H^l of rows h (hn) and h - 1 (hold)
      T hzb[CPL];  // Hz^l(h, j-1)
      hzb[0] = shup(hn[CPL - 1].z);
#pragma unroll
      for (int q = 1; q < CPL; q++) hzb[q] = hn[q - 1].z;
      ES en[CPL];
#pragma unroll
      for (int q = 0; q < CPL; q++) {
        en[q].iex = eo[q].iex;
        en[q].iey = eo[q].iey;
        en[q].dx = en[q].dy = en[q].ex = en[q].ey = en[q].jx = en[q].jy = czero<T>();
        if (!AUX || (t.jact[q] && hrow)) {
          const T hzk = hn[q].z;
          const T cxv = csub(hzk, hzb[q]);  // Hz - Hz[j-1]
          T cyv;                            // -Hz + Hz[i-1]
          cyv.x = -hzk.x + hold[q].z.x;
          cyv.y = -hzk.y + hold[q].z.y;
          T dx = eo[q].dx, dy = eo[q].dy;
          if (!AUX || (t.yin[q] && x_in(v, h))) {
            dx = cadd(dx, cxv);
            dy = cadd(dy, cyv);
          } else {
            T jx = eo[q].jx, jy = eo[q].jy;
            te_e_pml(v, h, j + q, cxv, cyv, dx, dy, jx, jy);
            en[q].jx = jx;
            en[q].jy = jy;
          }
          en[q].dx = dx;
          en[q].dy = dy;
          T ex = dx, ey = dy;
          if (!is_one(en[q].iex)) {
            ex = cscale(dx, en[q].iex);
            if (tb.pulse[0].kind) {
              if (tb.ptab[0]) pulse_row<R>(tb.ptab[0][(size_t)(l - 1) * v.nxa + h], en[q].iex, ex);
              else pulse_source<R>(tb.pulse[0], h, j + q, en[q].iex, ex, (double)(l - 1));
            }
          }
          if (!is_one(en[q].iey)) {
            ey = cscale(dy, en[q].iey);
            if (tb.pulse[1].kind) {
              if (tb.ptab[1]) pulse_row<R>(tb.ptab[1][(size_t)(l - 1) * v.nxa + h], en[q].iey, ey);
              else pulse_source<R>(tb.pulse[1], h, j + q, en[q].iey, ey, (double)(l - 1));
            }
          }
          en[q].ex = ex;
          en[q].ey = ey;
        }
      }
#pragma unroll
      for (int q = 0; q < CPL; q++) {
        const ES eold = E[l][q];  // E^l of row h - 1
        E[l][q] = en[q];
        if (t.lines && t.own[q] && h >= t.r0 && h < t.r1) {
          line_put(v, tb, t, q, l - 1, h, 0, en[q].ex);
          line_put(v, tb, t, q, l - 1, h, 1, en[q].ey);
          line_put(v, tb, t, q, l - 1, h, 2, hn[q].z);
        }
        eo[q] = eold;
        ho[q] = hold[q];
      }
    }
    {  // level K is final: E and H of row r - K
      const int h = r - K;
      if (h >= t.r0 && h < t.r1) {
        const size_t k = (size_t)h * P + j;
        T dx[CPL], dy[CPL], ex[CPL], ey[CPL], hz[CPL];
#pragma unroll
        for (int q = 0; q < CPL; q++) {
          dx[q] = E[K][q].dx;
          dy[q] = E[K][q].dy;
          ex[q] = E[K][q].ex;
          ey[q] = E[K][q].ey;
          hz[q] = H[K][q].z;
          if (AUX && t.own[q] && !(t.yin[q] && x_in(v, h))) {
            tb.out[4][k + q] = E[K][q].jx;
            tb.out[5][k + q] = E[K][q].jy;
            tb.out[7][k + q] = H[K][q].mz;
          }
        }
        st_cols<CPL>(tb.out[2] + k, t.own, dx);
        st_cols<CPL>(tb.out[3] + k, t.own, dy);
        st_cols<CPL>(tb.out[0] + k, t.own, ex);
        st_cols<CPL>(tb.out[1] + k, t.own, ey);
        st_cols<CPL>(tb.out[6] + k, t.own, hz);
      }
    }
  }
}

// NTFF surface samples of level lev from the line buffers (zero on the halo ring)
template <typename R>
__device__ __forceinline__ bool line_get(const StencilView<R> &v, const TBlockView<R> &tb, int lev, int f, int i,
                                         int j, typename Cplx<R>::T &out)
{
  if (i < 1 || i > v.ni || j < 1 || j > v.nj) {
    out = czero<typename Cplx<R>::T>();
    return true;
  }
  for (int q = 0; q < 4; q++)
    if (j == tb.cj[q]) {
      out = tb.col[((size_t)(lev * 4 + q) * 3 + f) * v.nxa + i];
      return true;
    }
  for (int q = 0; q < 4; q++)
    if (i == tb.ri[q]) {
      out = tb.row[((size_t)(lev * 4 + q) * 3 + f) * v.P + j];
      return true;
    }
  return false;
}

}  // namespace tile
}  // namespace fdtd
