// fdtd_tblock_serial.cu -- the temporally blocked stencil of the serial UPML
// solvers (TM_UPML, TE_UPML: H half-step first, Gaussian pulse): the interior
// and work-list kernels around tile::tm_tile_hf / tile::te_tile_hf
// (tblock_tile.cuh), on the tiles and NTFF line buffers of the MPI solvers'
// blocking (fdtd_tblock.cu).
#include <cuda_runtime.h>

#include "fdtd_internal.cuh"
#include "stencil_ops.cuh"
#include "tblock_tile.cuh"

namespace fdtd {

namespace {

using tile::te_tile_hf;
using tile::tm_tile_hf;

constexpr int kWarps = 4;  // warps (tiles) per block

// resident blocks per SM of the interior kernel: the E-first tile's choice for
// TM; TE keeps E, D and 1/eps of two components per level and loads E as well
// as D, so it gets the registers of one block fewer
template <typename R, int K, bool TM, int CPL> constexpr int hf_min_blocks()
{
  return CPL == 2 ? (K > 2 ? 3 : 4)
                  : sizeof(R) == 8 ? (K > 1 ? 3 : 4) : (K == 4 ? 4 : K == 2 ? (TM ? 6 : 5) : 6);
}

template <typename R, int K, bool TM, int CPL>
__global__ void __launch_bounds__(32 * kWarps, (hf_min_blocks<R, K, TM, CPL>()))
    tblock_hf_interior_kernel(StencilView<R> v, TBlockView<R> tb)
{
  const int strip = tb.s0 + (int)blockIdx.x * kWarps + (int)(threadIdx.x >> 5);
  if (strip >= tb.s1) return;  // whole warp
  const int r0 = tb.ra + (int)blockIdx.y * tb.L;
  const int r1 = min(r0 + tb.L, tb.rb);
  if (TM) tm_tile_hf<R, K, false, CPL>(v, tb, strip, r0, r1);
  else te_tile_hf<R, K, false, CPL>(v, tb, strip, r0, r1);
}

template <typename R, int K, bool TM, int CPL>
__global__ void __launch_bounds__(32 * kWarps, 3) tblock_hf_general_kernel(StencilView<R> v, TBlockView<R> tb)
{
  const int w = (int)blockIdx.x * kWarps + (int)(threadIdx.x >> 5);
  if (w >= tb.ntiles) return;  // whole warp
  const int4 t4 = tb.tiles[w];
  if (TM) tm_tile_hf<R, K, true, CPL>(v, tb, t4.x, t4.y, t4.z);
  else te_tile_hf<R, K, true, CPL>(v, tb, t4.x, t4.y, t4.z);
}

template <typename R, int K, int CPL>
void launch_depth_hf(const StencilView<R> &v, const TBlockView<R> &tb, bool tm, cudaStream_t st)
{
  const dim3 blk(32 * kWarps);
  if (tb.s1 > tb.s0 && tb.nseg > 0) {
    const dim3 g((unsigned)((tb.s1 - tb.s0 + kWarps - 1) / kWarps), (unsigned)tb.nseg);
    if (tm) tblock_hf_interior_kernel<R, K, true, CPL><<<g, blk, 0, st>>>(v, tb);
    else tblock_hf_interior_kernel<R, K, false, CPL><<<g, blk, 0, st>>>(v, tb);
  }
  if (tb.ntiles > 0) {
    const dim3 g((unsigned)((tb.ntiles + kWarps - 1) / kWarps));
    if (tm) tblock_hf_general_kernel<R, K, true, CPL><<<g, blk, 0, st>>>(v, tb);
    else tblock_hf_general_kernel<R, K, false, CPL><<<g, blk, 0, st>>>(v, tb);
  }
}

// tab[l][i]: pulse_source's values for row i at step s.time + l, its
// operations in its order (the column term is 0 x (j + gap) = +0 at 0 degrees)
__global__ void pulse_row_kernel(SourceStep s, int K, int nrow, PulseRow *tab)
{
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= K * nrow) return;
  const int l = q / nrow, i = q - l * nrow;
  const double pos = __dadd_rn(__dmul_rn((double)i + s.gap_x, s.cos_per_c), 0.0);
  const double r = __dsub_rn(pos, (s.time + (double)l) - s.t0);
  const double qq = __ddiv_rn(r, 50.0);
  const double g = exp(-(qq * qq));
  double sn, cs;
  sincos(r * s.w, &sn, &cs);
  PulseRow p;
  p.a = s.dot * g;
  p.c = cs;
  p.s = sn;
  p.pad = 0.0;
  tab[q] = p;
}

}  // namespace

void launch_pulse_rows(const SourceStep &s, int K, int nrow, PulseRow *tab, cudaStream_t st)
{
  pulse_row_kernel<<<(K * nrow + 255) / 256, 256, 0, st>>>(s, K, nrow, tab);
}

template <typename R>
void launch_tblock_serial(const StencilView<R> &v, const TBlockView<R> &tb, int K, bool tm, cudaStream_t st)
{
  constexpr bool f32 = sizeof(R) == 4;
  if (f32 && tb.cpl == 2) {  // two columns per lane: K = 2 or 4 (the host checks)
    if (K == 2) launch_depth_hf<R, 2, f32 ? 2 : 1>(v, tb, tm, st);
    else if (K == 4) launch_depth_hf<R, 4, f32 ? 2 : 1>(v, tb, tm, st);
    return;
  }
  switch (K) {
  case 1: launch_depth_hf<R, 1, 1>(v, tb, tm, st); break;
  case 2: launch_depth_hf<R, 2, 1>(v, tb, tm, st); break;
  case 4: launch_depth_hf<R, 4, 1>(v, tb, tm, st); break;
  default: break;  // the host accepts 1, 2 and 4 only
  }
}

template void launch_tblock_serial<double>(const StencilView<double> &, const TBlockView<double> &, int, bool,
                                           cudaStream_t);
template void launch_tblock_serial<float>(const StencilView<float> &, const TBlockView<float> &, int, bool,
                                          cudaStream_t);

}  // namespace fdtd
