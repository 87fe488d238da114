// fdtd_tblock.cu -- the temporally blocked stencil of one simulation: the
// interior-tile and work-list kernels around tile::tm_tile / tile::te_tile
// (tblock_tile.cuh), and the gather of the NTFF line samples into the
// time-blocked NTFF buffer.
#include <cuda_runtime.h>

#include "fdtd_internal.cuh"
#include "stencil_ops.cuh"
#include "tblock_tile.cuh"

namespace fdtd {

namespace {

using tile::tm_tile;
using tile::te_tile;

constexpr int kWarps = 4;  // warps (tiles) per block

// Register cap through the resident-block count (blocks of 4 warps per SM):
// measured on the 16416^2 FP32 grid, TM at K = 4 is fastest at 4 blocks (128
// registers; 5 spills), TE at K = 4 at 5 blocks (102 registers, fewer live
// values), K <= 2 at 6 blocks; FP64 and K = 8 keep 3-4 (their levels need
// more registers); two columns per lane double the level state (3-4 blocks).
template <typename R, int K, bool TM, int CPL> constexpr int interior_min_blocks()
{
  return CPL == 2 ? (K > 2 ? 3 : 4)
                  : sizeof(R) == 8 ? (K > 2 ? 3 : 4) : (K >= 8 ? 3 : K == 4 ? (TM ? 4 : 5) : 6);
}

// interior tiles: strips [s0, s1) x segments of rows [ra, rb), no auxiliaries
template <typename R, int K, bool TM, int CPL>
__global__ void __launch_bounds__(32 * kWarps, (interior_min_blocks<R, K, TM, CPL>()))
    tblock_interior_kernel(StencilView<R> v, TBlockView<R> tb)
{
  const int strip = tb.s0 + (int)blockIdx.x * kWarps + (int)(threadIdx.x >> 5);
  if (strip >= tb.s1) return;  // whole warp
  const int r0 = tb.ra + (int)blockIdx.y * tb.L;
  const int r1 = min(r0 + tb.L, tb.rb);
  if (TM) tm_tile<R, K, false, CPL>(v, tb, strip, r0, r1, K);
  else te_tile<R, K, false, CPL>(v, tb, strip, r0, r1, K);
}

// every other tile, from the work-list (3 resident blocks: 14 % faster on the
// sweep of small instances, where these tiles are a fifth of the cells, than 2)
template <typename R, int K, bool TM, int CPL>
__global__ void __launch_bounds__(32 * kWarps, 3) tblock_general_kernel(StencilView<R> v, TBlockView<R> tb)
{
  const int w = (int)blockIdx.x * kWarps + (int)(threadIdx.x >> 5);
  if (w >= tb.ntiles) return;  // whole warp
  const int4 t4 = tb.tiles[w];
  if (TM) tm_tile<R, K, true, CPL>(v, tb, t4.x, t4.y, t4.z, K);
  else te_tile<R, K, true, CPL>(v, tb, t4.x, t4.y, t4.z, K);
}

// Same values as ntff_gather_kernel, for the K steps of one blocked launch.
template <typename R>
__global__ void line_gather_kernel(StencilView<R> v, TBlockView<R> tb, NtffView n, double coef, int slot0, int tm)
{
  using T = typename Cplx<R>::T;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int lev = blockIdx.y;
  if (c >= n.ncell) return;
  const SurfCell sc = n.cells[c];
  const int i = (int)(sc.k / v.P), j = (int)(sc.k % v.P);
  const int fe = tm ? 0 : sc.e_slot;                    // TE: 0 Ex (bottom/top), 1 Ey (right/left)
  const int fh = tm ? (sc.h_slot == 3 ? 1 : 2) : 2;     // TM: Hx / Hy ; TE: Hz
  const int i1 = sc.hoff == -1 ? i : i - 1, j1 = sc.hoff == -1 ? j - 1 : j;
  T e, h0, h1;
  if (!tile::line_get(v, tb, lev, fe, i, j, e) || !tile::line_get(v, tb, lev, fh, i, j, h0) ||
      !tile::line_get(v, tb, lev, fh, i1, j1, h1)) {
    atomicOr(n.status, kStatusNtffRange);
    return;
  }
  const double sg = sc.sign;
  double2 ev, hv;
  ev.x = sg * (double)e.x * coef;
  ev.y = sg * (double)e.y * coef;
  hv.x = (sg * 0.5) * ((double)h0.x + (double)h1.x) * coef;
  hv.y = (sg * 0.5) * ((double)h0.y + (double)h1.y) * coef;
  double2 *vals = n.vals + (size_t)(slot0 + lev) * 2 * n.ncell;
  vals[c] = ev;
  vals[n.ncell + c] = hv;
}

template <typename R, int K, int CPL>
void launch_depth(const StencilView<R> &v, const TBlockView<R> &tb, bool tm, cudaStream_t st)
{
  const dim3 blk(32 * kWarps);
  if (tb.s1 > tb.s0 && tb.nseg > 0) {
    const dim3 g((unsigned)((tb.s1 - tb.s0 + kWarps - 1) / kWarps), (unsigned)tb.nseg);
    if (tm) tblock_interior_kernel<R, K, true, CPL><<<g, blk, 0, st>>>(v, tb);
    else tblock_interior_kernel<R, K, false, CPL><<<g, blk, 0, st>>>(v, tb);
  }
  if (tb.ntiles > 0) {
    const dim3 g((unsigned)((tb.ntiles + kWarps - 1) / kWarps));
    if (tm) tblock_general_kernel<R, K, true, CPL><<<g, blk, 0, st>>>(v, tb);
    else tblock_general_kernel<R, K, false, CPL><<<g, blk, 0, st>>>(v, tb);
  }
}

}  // namespace

template <typename R>
void launch_tblock(const StencilView<R> &v, const TBlockView<R> &tb, int K, bool tm, cudaStream_t st)
{
  constexpr bool f32 = sizeof(R) == 4;
  if (f32 && tb.cpl == 2) {  // two columns per lane: K = 2 or 4 (the host checks)
    if (K == 2) launch_depth<R, 2, f32 ? 2 : 1>(v, tb, tm, st);
    else if (K == 4) launch_depth<R, 4, f32 ? 2 : 1>(v, tb, tm, st);
    return;
  }
  switch (K) {
  case 1: launch_depth<R, 1, 1>(v, tb, tm, st); break;
  case 2: launch_depth<R, 2, 1>(v, tb, tm, st); break;
  case 4: launch_depth<R, 4, 1>(v, tb, tm, st); break;
  case 8:  // FP32 only: eight FP64 levels do not fit the register file
    if (f32) launch_depth<R, f32 ? 8 : 4, 1>(v, tb, tm, st);
    break;
  default: break;  // the host accepts 1, 2, 4 and (FP32) 8 only
  }
}

template <typename R>
void launch_line_gather(const StencilView<R> &v, const TBlockView<R> &tb, const NtffView &n, double coef, int K,
                        int slot0, bool tm, cudaStream_t st)
{
  const dim3 g((unsigned)((n.ncell + 255) / 256), (unsigned)K);
  line_gather_kernel<R><<<g, 256, 0, st>>>(v, tb, n, coef, slot0, tm ? 1 : 0);
}

template void launch_tblock<double>(const StencilView<double> &, const TBlockView<double> &, int, bool, cudaStream_t);
template void launch_tblock<float>(const StencilView<float> &, const TBlockView<float> &, int, bool, cudaStream_t);
template void launch_line_gather<double>(const StencilView<double> &, const TBlockView<double> &, const NtffView &,
                                         double, int, int, bool, cudaStream_t);
template void launch_line_gather<float>(const StencilView<float> &, const TBlockView<float> &, const NtffView &,
                                        double, int, int, bool, cudaStream_t);

}  // namespace fdtd
