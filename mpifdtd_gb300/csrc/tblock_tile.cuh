// tblock_tile.cuh -- one warp tile of the temporally blocked stencil of the
// MPI solvers (fdtd_tblock.cu: one simulation; fdtd_batch.cu: many): K time
// steps (E half then H half, mpiTM_UPML.c:196-217, mpiTE_UPML.c:290-304) per
// pass over the fields in HBM.
//
// A warp owns one tile: a strip of W = 32 - 2K columns and a row segment
// [r0, r1).  Lane = column j: the 32 lanes cover the strip plus K columns on
// each side.  The warp walks the rows i from r0 - K to r1 + K - 1 and keeps K time levels
// in registers, level l one row behind level l-1.  At front row r it loads
// the level-0 state (D of row r+1, H of row r) and, for l = 1..K,
//   E^l at row e = r-l+1 from D^{l-1}(e), H^{l-1}(e) and H^{l-1}(e-1),
//   H^l at row h = r-l   from H^{l-1}(h), E^l(h) and E^l(h+1);
// the column neighbours (H[j-1] for E, E[j+1] for H) come from warp shuffles.
// Every level loses one valid column on each side and one valid row at the
// start, so after K levels the centre W columns of rows [r0, r1) are exact and
// only those are stored.  The launch reads one field set and writes the other
// (ping-pong), so overlapping tiles never read each other's results.
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

// One lane's view of its tile.
struct Lane {
  int j;        // array column
  int r0, r1;   // owned rows [r0, r1)
  bool jact;    // j is an active column (1..nj)
  bool own;     // j is one of the tile's W owned columns
  int colq;     // index of the NTFF column line through j, or -1
  bool lines;   // the lane stores NTFF line samples in this tile (own column on a column line,
                // or a row line inside [r0, r1))
};

template <int K, typename R>
__device__ __forceinline__ Lane lane_of(const StencilView<R> &v, const TBlockView<R> &tb, int strip, int r0, int r1)
{
  constexpr int W = 32 - 2 * K;
  const int lane = threadIdx.x & 31;
  Lane t;
  t.j = 1 + strip * W - K + lane;
  t.jact = t.j >= 1 && t.j <= v.nj;
  t.own = t.jact && lane >= K && lane < 32 - K;
  t.r0 = r0;
  t.r1 = r1;
  t.colq = -1;
  t.lines = false;
  if (tb.col && t.own) {
    for (int q = 0; q < 4; q++) {
      if (t.j == tb.cj[q]) t.colq = q;
      if (tb.ri[q] >= t.r0 && tb.ri[q] < t.r1) t.lines = true;
    }
    if (t.colq >= 0) t.lines = true;
  }
  return t;
}

// NTFF line sample: field f of level lev at owned cell (i, t.j)
template <typename R, typename T>
__device__ __forceinline__ void line_put(const StencilView<R> &v, const TBlockView<R> &tb, const Lane &t, int lev,
                                         int i, int f, const T &val)
{
  if (t.colq >= 0) tb.col[((size_t)(lev * 4 + t.colq) * 3 + f) * v.nxa + i] = val;
#pragma unroll
  for (int q = 0; q < 4; q++)
    if (i == tb.ri[q]) tb.row[((size_t)(lev * 4 + q) * 3 + f) * v.P + t.j] = val;
}

// ------------------------------------------------------------------ TM
// slots 0 Ez 1 Dz 2 Jz 3 Hx 4 Hy 5 Mx 6 My
template <typename R, int K, bool AUX>
__device__ __forceinline__ void tm_tile(const StencilView<R> &v, const TBlockView<R> &tb, int strip, int r0,
                                        int r1, int nlev)
{
  using T = typename Cplx<R>::T;
  struct ES { T d, e, j; R ie; };
  struct HS { T x, y, mx, my; };
  const Lane t = lane_of<K>(v, tb, strip, r0, r1);
  const int j = t.j;
  const size_t P = (size_t)v.P;
  const T *Dz = v.f[1], *Jz = v.f[2], *Hx = v.f[3], *Hy = v.f[4], *Mx = v.f[5], *My = v.f[6];
  const R *IE = v.inv_eps[0];
  const bool yin = y_in(v, j);
  ES E[K + 1];
  HS H[K + 1];
#pragma unroll
  for (int l = 0; l <= K; l++) {
    E[l].d = E[l].e = E[l].j = czero<T>();
    E[l].ie = (R)1;
    H[l].x = H[l].y = H[l].mx = H[l].my = czero<T>();
  }
  // level-0 state of front row r: D (J, 1/eps) of row r+1 and H (M) of row r,
  // zero outside the active rows/columns; loaded two rows ahead of use
  auto load0 = [&](int r, ES &n, HS &m) {
    const int a = r + 1;
    n.d = n.e = n.j = czero<T>();
    n.ie = (R)1;
    if (t.jact && a >= 1 && a <= v.ni) {  // a branch (not straight-line loads) measured 1.3x faster
      const size_t k = (size_t)a * P + j;
      n.d = ldro(Dz + k);
      n.ie = ldro(IE + k);
      if (AUX && !(yin && x_in(v, a))) n.j = ldro(Jz + k);
    }
    m.x = m.y = m.mx = m.my = czero<T>();
    if (t.jact && r >= 1 && r <= v.ni) {
      const size_t k = (size_t)r * P + j;
      m.x = ldro(Hx + k);
      m.y = ldro(Hy + k);
      if (AUX && !(yin && x_in(v, r))) {
        m.mx = ldro(Mx + k);
        m.my = ldro(My + k);
      }
    }
  };
  ES pe0, pe1;
  HS ph0, ph1;
  load0(t.r0 - K, pe0, ph0);
  load0(t.r0 - K + 1, pe1, ph1);
#pragma unroll 1
  for (int r = t.r0 - K; r < t.r1 + K; r++) {
    ES eo = E[0];
    HS ho = H[0];
    E[0] = pe0;
    H[0] = ph0;
    pe0 = pe1;
    ph0 = ph1;
    load0(r + 2, pe1, ph1);
#pragma unroll
    for (int l = 1; l <= K; l++) {
      const int e = r - l + 1, h = r - l;
      // E half (calcJD + calcE + scatteredWave) at row e
      const T hxb = shup(H[l - 1].x);  // Hx^{l-1}(e, j-1)
      ES en;
      en.ie = eo.ie;
      en.d = en.e = en.j = czero<T>();
      if (l > nlev) {  // frozen level (the instance stops inside this launch): E^l = E^{l-1}
        en = eo;
      } else if (!AUX || (t.jact && e >= 1 && e <= v.ni)) {
        T curl;
        curl.x = ((H[l - 1].y.x - ho.y.x) - H[l - 1].x.x) + hxb.x;
        curl.y = ((H[l - 1].y.y - ho.y.y) - H[l - 1].x.y) + hxb.y;
        T dz = eo.d;
        if (!AUX || (yin && x_in(v, e))) {
          dz = cadd(dz, curl);
        } else {
          T jz = eo.j;
          tm_e_pml(v, e, j, curl, dz, jz);
          en.j = jz;
        }
        en.d = dz;
        T ez = dz;
        if (!is_one(en.ie)) {
          ez = cscale(dz, en.ie);
          cw_add<R>(v, tb.sc[l - 1].x, tb.sc[l - 1].y, e, j, en.ie, ez);
        }
        en.e = ez;
      }
      const ES eold = E[l];  // E^l of row h = e-1
      E[l] = en;
      // H half (calcMB + calcH) at row h
      const T ezr = shdn(eold.e);  // Ez^l(h, j+1)
      HS hn;
      hn.x = hn.y = hn.mx = hn.my = czero<T>();
      if (l > nlev) {
        hn = ho;
      } else if (!AUX || (t.jact && h >= 1 && h <= v.ni)) {
        const T dEx = csub(ezr, eold.e);
        const T dEy = csub(eold.e, en.e);
        T hx = ho.x, hy = ho.y;
        if (!AUX || (yin && x_in(v, h))) {
          hx.x -= v.inv_mu * dEx.x; hx.y -= v.inv_mu * dEx.y;
          hy.x -= v.inv_mu * dEy.x; hy.y -= v.inv_mu * dEy.y;
        } else {
          T mx = ho.mx, my = ho.my;
          tm_h_pml(v, h, j, dEx, dEy, hx, hy, mx, my);
          hn.mx = mx;
          hn.my = my;
        }
        hn.x = hx;
        hn.y = hy;
      }
      const HS hold = H[l];
      H[l] = hn;
      if (t.lines) {
        if (e >= t.r0 && e < t.r1) line_put(v, tb, t, l - 1, e, 0, en.e);
        if (h >= t.r0 && h < t.r1) {
          line_put(v, tb, t, l - 1, h, 1, hn.x);
          line_put(v, tb, t, l - 1, h, 2, hn.y);
        }
      }
      eo = eold;
      ho = hold;
    }
    if (t.own) {  // level K is final: E of row r-K+1, H of row r-K
      const int e = r - K + 1, h = r - K;
      if (e >= t.r0 && e < t.r1) {
        const size_t k = (size_t)e * P + j;
        tb.out[1][k] = E[K].d;
        tb.out[0][k] = E[K].e;
        if (AUX && !(yin && x_in(v, e))) tb.out[2][k] = E[K].j;
      }
      if (h >= t.r0 && h < t.r1) {
        const size_t k = (size_t)h * P + j;
        tb.out[3][k] = H[K].x;
        tb.out[4][k] = H[K].y;
        if (AUX && !(yin && x_in(v, h))) {
          tb.out[5][k] = H[K].mx;
          tb.out[6][k] = H[K].my;
        }
      }
    }
  }
}

// ------------------------------------------------------------------ TE
// slots 0 Ex 1 Ey 2 Dx 3 Dy 4 Jx 5 Jy 6 Hz 7 Mz; the CW source drives Ey only
// (the MPI TE solver's scatteredWave, mpiTE_UPML.c:250-281).
template <typename R, int K, bool AUX>
__device__ __forceinline__ void te_tile(const StencilView<R> &v, const TBlockView<R> &tb, int strip, int r0,
                                        int r1, int nlev)
{
  using T = typename Cplx<R>::T;
  struct ES { T dx, dy, ex, ey, jx, jy; R iex, iey; };
  struct HS { T z, mz; };
  const Lane t = lane_of<K>(v, tb, strip, r0, r1);
  const int j = t.j;
  const size_t P = (size_t)v.P;
  const T *Dx = v.f[2], *Dy = v.f[3], *Jx = v.f[4], *Jy = v.f[5], *Hz = v.f[6], *Mz = v.f[7];
  const R *IEX = v.inv_eps[0], *IEY = v.inv_eps[1];
  const bool yin = y_in(v, j);
  ES E[K + 1];
  HS H[K + 1];
#pragma unroll
  for (int l = 0; l <= K; l++) {
    E[l].dx = E[l].dy = E[l].ex = E[l].ey = E[l].jx = E[l].jy = czero<T>();
    E[l].iex = E[l].iey = (R)1;
    H[l].z = H[l].mz = czero<T>();
  }
  auto load0 = [&](int r, ES &n, HS &m) {  // D (J, 1/eps) of row r+1, H (M) of row r
    const int a = r + 1;
    n.dx = n.dy = n.ex = n.ey = n.jx = n.jy = czero<T>();
    n.iex = n.iey = (R)1;
    if (t.jact && a >= 1 && a <= v.ni) {  // a branch (not straight-line loads) measured 1.3x faster
      const size_t k = (size_t)a * P + j;
      n.dx = ldro(Dx + k);
      n.dy = ldro(Dy + k);
      n.iex = ldro(IEX + k);
      n.iey = ldro(IEY + k);
      if (AUX && !(yin && x_in(v, a))) {
        n.jx = ldro(Jx + k);
        n.jy = ldro(Jy + k);
      }
    }
    m.z = m.mz = czero<T>();
    if (t.jact && r >= 1 && r <= v.ni) {
      const size_t k = (size_t)r * P + j;
      m.z = ldro(Hz + k);
      if (AUX && !(yin && x_in(v, r))) m.mz = ldro(Mz + k);
    }
  };
  ES pe0, pe1;
  HS ph0, ph1;
  load0(t.r0 - K, pe0, ph0);
  load0(t.r0 - K + 1, pe1, ph1);
#pragma unroll 1
  for (int r = t.r0 - K; r < t.r1 + K; r++) {
    ES eo = E[0];
    HS ho = H[0];
    E[0] = pe0;
    H[0] = ph0;
    pe0 = pe1;
    ph0 = ph1;
    load0(r + 2, pe1, ph1);
#pragma unroll
    for (int l = 1; l <= K; l++) {
      const int e = r - l + 1, h = r - l;
      const T hzk = H[l - 1].z;
      const T hzb = shup(hzk);  // Hz^{l-1}(e, j-1)
      ES en;
      en.iex = eo.iex;
      en.iey = eo.iey;
      en.dx = en.dy = en.ex = en.ey = en.jx = en.jy = czero<T>();
      if (l > nlev) {  // frozen level (the instance stops inside this launch): E^l = E^{l-1}
        en = eo;
      } else if (!AUX || (t.jact && e >= 1 && e <= v.ni)) {
        const T cxv = csub(hzk, hzb);  // Hz - Hz[j-1]
        T cyv;                         // -Hz + Hz[i-1]
        cyv.x = -hzk.x + ho.z.x;
        cyv.y = -hzk.y + ho.z.y;
        T dx = eo.dx, dy = eo.dy;
        if (!AUX || (yin && x_in(v, e))) {
          dx = cadd(dx, cxv);
          dy = cadd(dy, cyv);
        } else {
          T jx = eo.jx, jy = eo.jy;
          te_e_pml(v, e, j, cxv, cyv, dx, dy, jx, jy);
          en.jx = jx;
          en.jy = jy;
        }
        en.dx = dx;
        en.dy = dy;
        T ex = dx, ey = dy;
        if (!is_one(en.iex)) ex = cscale(dx, en.iex);
        if (!is_one(en.iey)) {
          ey = cscale(dy, en.iey);
          cw_add<R>(v, tb.sc[l - 1].x, tb.sc[l - 1].y, e, j, en.iey, ey);
        }
        en.ex = ex;
        en.ey = ey;
      }
      const ES eold = E[l];
      E[l] = en;
      const T ext = shdn(eold.ex);  // Ex^l(h, j+1)
      HS hn;
      hn.z = hn.mz = czero<T>();
      if (l > nlev) {
        hn = ho;
      } else if (!AUX || (t.jact && h >= 1 && h <= v.ni)) {
        T ce;  // Ey[i+1] - Ey - Ex[j+1] + Ex
        ce.x = ((en.ey.x - eold.ey.x) - ext.x) + eold.ex.x;
        ce.y = ((en.ey.y - eold.ey.y) - ext.y) + eold.ex.y;
        T hz = ho.z;
        if (!AUX || (yin && x_in(v, h))) {
          hz.x -= v.inv_mu * ce.x;
          hz.y -= v.inv_mu * ce.y;
        } else {
          T mz = ho.mz;
          te_h_pml(v, h, j, ce, hz, mz);
          hn.mz = mz;
        }
        hn.z = hz;
      }
      const HS hold = H[l];
      H[l] = hn;
      if (t.lines) {
        if (e >= t.r0 && e < t.r1) {
          line_put(v, tb, t, l - 1, e, 0, en.ex);
          line_put(v, tb, t, l - 1, e, 1, en.ey);
        }
        if (h >= t.r0 && h < t.r1) line_put(v, tb, t, l - 1, h, 2, hn.z);
      }
      eo = eold;
      ho = hold;
    }
    if (t.own) {
      const int e = r - K + 1, h = r - K;
      if (e >= t.r0 && e < t.r1) {
        const size_t k = (size_t)e * P + j;
        tb.out[2][k] = E[K].dx;
        tb.out[3][k] = E[K].dy;
        tb.out[0][k] = E[K].ex;
        tb.out[1][k] = E[K].ey;
        if (AUX && !(yin && x_in(v, e))) {
          tb.out[4][k] = E[K].jx;
          tb.out[5][k] = E[K].jy;
        }
      }
      if (h >= t.r0 && h < t.r1) {
        const size_t k = (size_t)h * P + j;
        tb.out[6][k] = H[K].z;
        if (AUX && !(yin && x_in(v, h))) tb.out[7][k] = H[K].mz;
      }
    }
  }
}

}  // namespace tile
}  // namespace fdtd
