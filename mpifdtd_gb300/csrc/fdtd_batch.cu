// fdtd_batch.cu -- many independent simulations advanced together: a sweep of
// scatterer / wavelength instances of one MPI solver with uneven grids and
// step counts (the task parallelism the reference gets from one process per
// structure, main.c:114-138, on one GPU).
//
// Every instance is an ordinary fdtd_sim (own fields, tables and
// permittivity; the caller fills and reads it through the fdtd_* calls).  The
// batch adds each instance's spare field set, a device clock, and two packed
// work-lists of (instance, strip, segment) tiles over all instances -- the
// PML-free interior tiles and the others -- for the temporally blocked tile
// code (tblock_tile.cuh), each sorted by tile height (largest first).  One
// K-step block is four launches:
//   source  : ray_coef e^{-i w t} of every instance at the block's K times
//   interior: persistent kernel whose warps claim interior tiles one by one
//             (an atomic counter in the clock record)
//   general : the same over the other tiles (on a second stream forked and
//             joined inside the graph: runs beside interior)
//   clock   : t += K, set parity flips, tile counters reset
// captured once in a CUDA graph and replayed until the instance with the
// largest step_num has finished.  An instance whose step_num ends inside a
// block freezes its remaining levels; a finished one is skipped, so its
// fields stay in the set of its last block.  The batch does no time-domain
// NTFF: the far field of a CW instance is fdtd_frequency (ntffTM_Frequency)
// of its final fields.
//
// Broadband mode (fdtd_batch_broadband, TM at 0 degrees): the source is the
// reference's Gaussian pulse (field.c:224-256) instead of the CW wave, and the
// far field at many wavelengths comes from one run.  Two more launches per
// block: before the tiles, a pulse kernel writes each instance's per-level
// row table of the pulse (at 0 degrees it depends on x and t only; the tile
// code reads it through the CW path's row table, one table per level) and the
// phasors e^{i w t} of the block's sample time; after the tiles, a DFT kernel
// reads the NTFF path samples the tiles left in their line buffers and adds
// v e^{i w t} of the block's last level, every FDTD_OPT_DFT_STRIDE steps
// (16 by default, a whole number of blocks), into per-instance sums
// S[2][path][nfreq] (FP64), from which the time-domain NTFF's far field at
// each frequency follows (fdtd_dft.cu).  Sparse samples suffice: the pulse's
// spectrum (a Gaussian of width 1/50 rad per step about its carrier, 0.03-0.06
// rad per step for 400-700 nm on 5 nm cells) is negligible long before the
// Nyquist frequency pi/stride of the sampled series (its nearest alias of a
// wavelength of interest lies ~0.7 rad per step away at stride 8, where the
// Gaussian is below e^-100), so the Fourier sums at the wavelengths of
// interest are those of every step divided by the stride; the incident
// pulse's sum (the normalisation) is taken over the same times.  The sums
// hold the samples' sign and H average but not their 1/(4 pi C R), which the
// far field applies.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "fdtd_internal.cuh"
#include "fdtd_sim.h"
#include "stencil_ops.cuh"
#include "tblock_tile.cuh"

namespace fdtd {

namespace {

struct BatchClock {
  double t;     // engine time of the block's first step
  int q;        // blocks run so far (field-set parity)
  int next[2];  // next unclaimed tile of the interior [0] / general [1] list (reset by the clock kernel)
};

// Per instance and per field-set parity p (blocks q with q % 2 == p): the
// view reading set p and the blocked view writing the other set; the source
// kernel stores the block's per-level source values into tb[p].sc.
template <typename R>
struct BatchInst {
  StencilView<R> v[2];
  TBlockView<R> tb[2];
  int n_steps;
  // broadband mode (src null: CW)
  typename Cplx<R>::T *src;  // [K][nxa] pulse rows of the current block (v[p].ex, level stride nxa)
  double2 *S;                // [2][ncell][nfreq] sum_t v e^{i w t} of the E / H path samples
  const SurfCell *cells;
  int ncell;
  double t0, w, inv_c;       // field.c:224-256: t0 = 500 - centre peak, carrier w_s, cos(0)/C
  double coef;               // NTFF sample scale 1/(4 pi C R), mpiTM_UPML.c:852-854 (applied by the far field)
};

constexpr int kBWarps = 4;

template <typename R>
__global__ void batch_source_kernel(BatchInst<R> *inst, const double *omega, int n, int K, const BatchClock *clk)
{
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= n * K) return;
  const int i = id / K, l = id - i * K;
  const double t = clk->t + l;
  const double rc = 1.0 - exp(-pow(0.01 * t, 2.0));  // field.c:312-315
  double sn, cs;
  sincos(omega[i] * t, &sn, &cs);
  // a pulse instance carries its whole source in the row table (the pulse has no ramp)
  inst[i].tb[clk->q & 1].sc[l] = inst[i].src ? make_double2(1.0, 0.0) : make_double2(rc * cs, -rc * sn);
}

// Broadband: the Gaussian pulse of field.c:224-256 at 0 degrees (cos_per_c =
// 1/C, sin_per_c = 0, no gap) as per-level row tables: value at array row i
// (global x = i + ox) and level l (time t + l) = g(r) e^{i r w}, g = exp(-(r/50)^2),
// r = x/C - (t + l - t0); grid (chunks, instances).  Block (0, 0) also writes
// the block's DFT phasors P[k] = e^{i w_k (t + K - 2)}: the E sample time of
// the last level, the one the DFT takes (the far field adds the H samples'
// half step).
template <typename R>
__global__ void batch_pulse_kernel(BatchInst<R> *inst, int K, const BatchClock *clk, const double *freq, int nfreq,
                                   double2 *P)
{
  using T = typename Cplx<R>::T;
  const BatchInst<R> &I = inst[blockIdx.y];
  const double t = clk->t;
  if (blockIdx.x == 0 && blockIdx.y == 0)
    for (int k = threadIdx.x; k < nfreq; k += blockDim.x) {
      double sn, cs;
      sincos(freq[k] * (t + K - 2.0), &sn, &cs);
      P[k] = make_double2(cs, sn);
    }
  if (!I.src) return;
  const int nxa = I.v[0].nxa, ox = I.v[0].ox;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < K * nxa; q += gridDim.x * blockDim.x) {
    const int l = q / nxa, i = q - l * nxa;
    const double r = (double)(i + ox) * I.inv_c - ((t + l) - I.t0);
    const double g = exp(-(r / 50.0) * (r / 50.0));
    double sn, cs;
    sincos(r * I.w, &sn, &cs);
    T v;
    v.x = (R)(g * cs);
    v.y = (R)(g * sn);
    I.src[q] = v;
  }
}

// Broadband: one warp per (instance, path cell), one lane per frequency.  The
// E and H samples of the block's last level come from the tiles' line buffers
// as line_gather_kernel forms them (sign, H average), in the fields' own
// precision (GB300 issues one FP64 warp-instruction per 16 clocks per SM:
// only the conversions and the accumulation run in FP64); each lane adds
// v P[k] to the cell's sums.  Runs after both tile kernels of the block and
// before the clock advances (the parity is the block's), in every `every`-th
// block.  An instance whose step_num ends inside the block takes no sample.
template <typename R, int K>
__global__ void __launch_bounds__(128) batch_dft_kernel(const BatchInst<R> *inst, const BatchClock *clk,
                                                         const double2 *P, int nfreq, int every)
{
  using T = typename Cplx<R>::T;
  if ((clk->q + 1) % every != 0) return;
  const BatchInst<R> &I = inst[blockIdx.y];
  if (!I.src) return;
  const int c = blockIdx.x * 4 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (c >= I.ncell) return;  // whole warp
  if (I.n_steps - (int)clk->t < K) return;
  const int p = clk->q & 1;
  const StencilView<R> &v = I.v[p];
  const TBlockView<R> &tb = I.tb[p];
  const SurfCell sc = I.cells[c];
  const int i = (int)(sc.k / v.P), j = (int)(sc.k % v.P);
  const int fh = sc.h_slot == 3 ? 1 : 2;  // TM: Hx (bottom/top), Hy (right/left)
  const int i1 = sc.hoff == -1 ? i : i - 1, j1 = sc.hoff == -1 ? j - 1 : j;
  T e = czero<T>(), h0 = czero<T>(), h1 = czero<T>();  // path cells always lie on a sampled line
  tile::line_get(v, tb, K - 1, 0, i, j, e);
  tile::line_get(v, tb, K - 1, fh, i, j, h0);
  tile::line_get(v, tb, K - 1, fh, i1, j1, h1);
  const R sg = (R)sc.sign, hs = sg * (R)0.5;  // exact: +-1, +-1/2
  const double2 ev = make_double2((double)(sg * e.x), (double)(sg * e.y));
  const double2 hv = make_double2((double)(hs * (h0.x + h1.x)), (double)(hs * (h0.y + h1.y)));
  for (int k = lane; k < nfreq; k += 32) {
    double2 *se = I.S + (size_t)c * nfreq + k, *sh = I.S + ((size_t)I.ncell + c) * nfreq + k;
    double2 ae = *se, ah = *sh;
    const double2 ph = P[k];
    ae.x = fma(ev.x, ph.x, fma(-ev.y, ph.y, ae.x));
    ae.y = fma(ev.x, ph.y, fma(ev.y, ph.x, ae.y));
    ah.x = fma(hv.x, ph.x, fma(-hv.y, ph.y, ah.x));
    ah.y = fma(hv.x, ph.y, fma(hv.y, ph.x, ah.y));
    *se = ae;
    *sh = ah;
  }
}

__global__ void batch_clock_kernel(BatchClock *clk, int K)
{
  clk->t += K;
  clk->q += 1;
  clk->next[0] = clk->next[1] = 0;  // both tile kernels of the block have finished (after the join)
}

// resident blocks per SM of the interior tile kernel (see interior_min_blocks in fdtd_tblock.cu)
template <typename R, int K, bool TM, int CPL> constexpr int batch_min_blocks()
{
  return CPL == 2 ? (K > 2 ? 3 : 4)
                  : sizeof(R) == 8 ? (K > 2 ? 3 : 4) : (K >= 8 ? 3 : K == 4 ? (TM ? 4 : 5) : 6);
}

// The PML / edge work-list kernel runs 3 resident blocks per SM (162
// registers for FP32 TM at K = 4), or 4 (WIDE: 128 registers, a few bytes of
// spill) where the tile fits them (TM, FP32, one column per lane, K <= 4) and
// the list has at least one tile per warp of 4 blocks per SM: each tile then
// runs slower, but more run at once.  Sweeps of 256 / 64 / 32 cylinders: 287 /
// 208 / 102 structures/s at 4 blocks, 272 / 196 / 128 at 3 (32 cylinders:
// 1576 tiles for 2432 warps); 256 at 5 blocks (96 registers, 344 bytes of
// spill): 241.
template <typename R, int K, bool TM, int CPL> constexpr bool batch_aux_wide_ok()
{
  return TM && sizeof(R) == 4 && CPL == 1 && K <= 4;
}

// Persistent: each warp claims the next tile of the list (sorted by cost,
// largest first) until the list is exhausted, so the tail is one tile long
// whatever the mix of tile heights and finished instances.
template <typename R, int K, bool AUX, bool TM, int CPL, bool WIDE = false>
__global__ void __launch_bounds__(32 * kBWarps, (AUX ? (WIDE ? 4 : 3) : batch_min_blocks<R, K, TM, CPL>()))
    batch_tile_kernel(const BatchInst<R> *__restrict__ inst, const int4 *__restrict__ tiles, int ntiles,
                      BatchClock *clk)
{
  const double t = clk->t;
  const int p = clk->q & 1;
  int *next = &clk->next[AUX ? 1 : 0];
  for (;;) {
    int w = 0;
    if ((threadIdx.x & 31) == 0) w = atomicAdd(next, 1);
    w = __shfl_sync(0xffffffffu, w, 0);
    if (w >= ntiles) break;  // whole warp
    const int4 tl = tiles[w];
    const BatchInst<R> &I = inst[tl.x];
    const int left = I.n_steps - (int)t;
    if (left <= 0) continue;  // finished instance (whole warp)
    const int nlev = left < K ? left : K;
    if (TM) tile::tm_tile<R, K, AUX, CPL>(I.v[p], I.tb[p], tl.y, tl.z, tl.w, nlev);
    else tile::te_tile<R, K, AUX, CPL>(I.v[p], I.tb[p], tl.y, tl.z, tl.w, nlev);
  }
}

template <typename R, int K, bool AUX, bool TM, int CPL, bool WIDE = false>
int persistent_grid(int ntiles)
{
  int dev = 0, nsm = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, batch_tile_kernel<R, K, AUX, TM, CPL, WIDE>, 32 * kBWarps, 0);
  cudaGetLastError();
  const int want = (ntiles + kBWarps - 1) / kBWarps;
  return std::max(1, std::min(want, std::max(1, nsm) * std::max(1, per)));
}

}  // namespace

}  // namespace fdtd

using namespace fdtd;

struct fdtd_batch {
  int solver = 0;
  bool tm = false, f32 = false;
  int K = 4, L = 0, cols = 1;
  std::vector<fdtd_sim *> sims;
  cudaStream_t stream = nullptr, stream2 = nullptr;  // stream2: the work-list kernel, forked in the graph
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  void *d_inst = nullptr, *d_tint = nullptr, *d_tgen = nullptr, *d_clock = nullptr, *d_omega = nullptr;
  int n_int = 0, n_gen = 0, grid_int = 0, grid_gen = 0;
  bool aux_wide = false;        // the work-list kernel at 4 blocks per SM (batch_aux_wide_ok, long list)
  int dft_stride = 16, dft_every = 4;  // FDTD_OPT_DFT_STRIDE; blocks between DFT samples (stride / K)
  int planned_k = 0, planned_l = -1, planned_c = 0;
  std::vector<int> rows;  // tile rows of each instance
  cudaGraphExec_t graph = nullptr;
  int graph_blocks = 0;
  long long launches = 0;
  // broadband mode (fdtd_batch_broadband)
  std::vector<int> bb_lam;      // wavelengths (nm); empty: CW
  void *d_bb_freq = nullptr;    // [nfreq] radians per step
  void *d_bb_phase = nullptr;   // [nfreq] phasors of the current block's sample time
  std::vector<void *> bb_src;   // per instance: [kMaxTBlock][nxa] pulse rows (field precision)
  std::vector<void *> bb_S;     // per instance: [2][ncell][nfreq] DFT sums
  void *d_bb_X = nullptr;       // [n][360][nfreq] far fields of every instance
  void *d_bb_Sptr = nullptr;    // [n] device copy of bb_S (the far field of a group of instances)
  void *d_bb_idx = nullptr;     // [n] instances ordered by configuration group
  int max_nxa = 0, max_ncell = 0;
  std::vector<double> bb_freq;  // host copy of d_bb_freq
  // |A(w)|^2 of the incident pulse per (t0, carrier, step_num): the instances of a sweep share it
  std::vector<std::pair<std::array<double, 4>, std::vector<double>>> bb_a2;
};

static void batch_free(fdtd_batch *b)
{
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (fdtd_sim *s : b->sims) fdtd_destroy(s);
  cudaFree(b->d_inst);
  cudaFree(b->d_tint);
  cudaFree(b->d_tgen);
  cudaFree(b->d_clock);
  cudaFree(b->d_omega);
  cudaFree(b->d_bb_freq);
  cudaFree(b->d_bb_phase);
  cudaFree(b->d_bb_X);
  cudaFree(b->d_bb_Sptr);
  cudaFree(b->d_bb_idx);
  for (void *p : b->bb_src) cudaFree(p);
  for (void *p : b->bb_S) cudaFree(p);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  if (b->ev_fork) cudaEventDestroy(b->ev_fork);
  if (b->ev_join) cudaEventDestroy(b->ev_join);
  if (b->stream2) cudaStreamDestroy(b->stream2);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

#define BCK(x)                                                                                     \
  do {                                                                                             \
    cudaError_t e_ = (x);                                                                          \
    if (e_ != cudaSuccess) {                                                                       \
      cudaGetLastError();                                                                          \
      return set_error(FDTD_E_CUDA, "%s: %s", #x, cudaGetErrorString(e_));                        \
    }                                                                                              \
  } while (0)

extern "C" int fdtd_batch_create(int solver, const fdtd_config *cfgs, int n, fdtd_batch **out)
{
  if (!cfgs || !out || n <= 0) return set_error(FDTD_E_ARG, "bad batch arguments");
  *out = nullptr;
  if (solver != FDTD_MPI_TM_UPML && solver != FDTD_MPI_TE_UPML)
    return set_error(FDTD_E_UNSUPPORTED, "a batch runs an MPI solver (E then H half-step)");
  for (int i = 1; i < n; i++)
    if (cfgs[i].precision != cfgs[0].precision) return set_error(FDTD_E_ARG, "instances differ in precision");
  fdtd_batch *b = new (std::nothrow) fdtd_batch();
  if (!b) return set_error(FDTD_E_NOMEM, "host allocation failed");
  b->solver = solver;
  b->tm = solver == FDTD_MPI_TM_UPML;
  b->f32 = cfgs[0].precision == FDTD_F32;
  for (int i = 0; i < n; i++) {
    fdtd_sim *s = nullptr;
    if (int rc = fdtd_create(solver, &cfgs[i], &s)) {
      batch_free(b);
      return rc;
    }
    b->sims.push_back(s);
  }
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->stream2, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    batch_free(b);
    return set_error(FDTD_E_CUDA, "stream / event creation failed");
  }
  *out = b;
  return FDTD_OK;
}

extern "C" int fdtd_batch_destroy(fdtd_batch *b)
{
  batch_free(b);
  return FDTD_OK;
}

extern "C" int fdtd_batch_size(const fdtd_batch *b) { return b ? (int)b->sims.size() : 0; }

extern "C" int fdtd_batch_instance(fdtd_batch *b, int index, fdtd_sim **sim)
{
  if (!b || !sim || index < 0 || index >= (int)b->sims.size()) return set_error(FDTD_E_ARG, "bad instance index");
  *sim = b->sims[index];
  return FDTD_OK;
}

extern "C" int fdtd_batch_set_option(fdtd_batch *b, int key, int value)
{
  if (!b) return set_error(FDTD_E_ARG, "null batch");
  switch (key) {
  case FDTD_OPT_TBLOCK:
    if (value != 1 && value != 2 && value != 4 && value != 8)
      return set_error(FDTD_E_ARG, "batch blocking depth must be 1, 2, 4 or 8");
    if (value == 8 && !b->f32) return set_error(FDTD_E_ARG, "blocking depth 8 needs FP32 fields");
    b->K = value;
    return FDTD_OK;
  case FDTD_OPT_TBLOCK_ROWS:
    if (value < 0 || value > (1 << 20)) return set_error(FDTD_E_ARG, "tile rows must be in [0, 2^20]");
    b->L = value;
    return FDTD_OK;
  case FDTD_OPT_DFT_STRIDE:
    if (value < 1 || value > 64) return set_error(FDTD_E_ARG, "DFT stride must be 1..64 steps");
    b->dft_stride = value;
    b->planned_k = 0;  // the graph bakes the stride in
    return FDTD_OK;
  case FDTD_OPT_TBLOCK_COLS:
    if (value != 1 && value != 2) return set_error(FDTD_E_ARG, "columns per lane must be 1 or 2");
    if (value == 2 && !b->f32) return set_error(FDTD_E_ARG, "two columns per lane need FP32 fields");
    b->cols = value;
    return FDTD_OK;
  }
  return set_error(FDTD_E_ARG, "unknown batch option %d", key);
}

extern "C" long long fdtd_batch_launch_count(const fdtd_batch *b) { return b ? b->launches : 0; }

// columns per lane: two (FP32, K = 2 or 4) when asked for
static int batch_cols(const fdtd_batch *b) { return b->cols == 2 && b->f32 && (b->K == 2 || b->K == 4) ? 2 : 1; }

// rows per interior tile segment of one instance (the work-list over all
// instances provides the parallelism; the PML bands get their own thin tiles)
static int batch_rows(const fdtd_batch *b, const fdtd_sim *s)
{
  if (b->L > 0) return b->L;
  // 96: fastest on the 256-cylinder sweep (236^2..643^2) once the tiles prefetch
  // their rows (32: 242, 48: 259, 64: 266, 96: 271 structures/s)
  return std::max(16, std::min(96, s->ni));
}

// Instance descriptors from the current field sets (fdtd_batch_run swaps an
// instance's sets after a run, so they are rebuilt before every run).
template <typename R>
static int batch_descriptors(fdtd_batch *b)
{
  const int n = (int)b->sims.size();
  std::vector<BatchInst<R>> inst(n);
  for (int i = 0; i < n; i++) {
    fdtd_sim *s = b->sims[i];
    BatchInst<R> &I = inst[i];
    I = BatchInst<R>{};
    I.v[0] = fdtd_view_of<R>(s);  // reads set A (the current d_f): blocks of even parity
    I.v[1] = I.v[0];
    for (int a = 0; a < kMaxSlots; a++) {
      I.v[1].f[a] = (typename Cplx<R>::T *)s->d_f2[a];
      I.tb[0].out[a] = I.v[1].f[a];
      I.tb[1].out[a] = I.v[0].f[a];
    }
    for (int p = 0; p < 2; p++) I.tb[p].L = b->rows[i];  // CW: no NTFF lines (col/row null)
    I.n_steps = s->cfg.step_num;
    if (!b->bb_lam.empty()) {  // broadband: pulse rows as the source table, path samples into the line buffers
      using T = typename Cplx<R>::T;
      const fdtd_geometry &g = s->geo;
      const int cj[4] = {g.ntff_bottom - 1, g.ntff_bottom, g.ntff_top - 1, g.ntff_top};
      const int ri[4] = {g.ntff_left - 1, g.ntff_left, g.ntff_right - 1, g.ntff_right};
      I.src = (T *)b->bb_src[i];
      I.S = (double2 *)b->bb_S[i];
      I.cells = (const SurfCell *)s->d_cells;
      I.ncell = s->ncell;
      const double C0 = s->c0;
      const double cos_per_c = cos(0.0) / C0;  // field.c:230 at 0 degrees
      I.inv_c = cos_per_c;
      I.t0 = -((g.n_px / 2.0) * cos_per_c) + 500;  // field.c:231-232
      I.w = g.omega_s;
      I.coef = 1.0 / (4 * M_PI * C0 * 1.0e6);
      for (int p = 0; p < 2; p++) {
        I.v[p].ex = I.src;
        I.v[p].src_lstride = s->nxa;
        I.tb[p].col = (T *)s->d_tbcol;
        I.tb[p].row = (T *)s->d_tbrow;
        for (int q = 0; q < 4; q++) {
          I.tb[p].cj[q] = cj[q];
          I.tb[p].ri[q] = ri[q];
        }
      }
    }
  }
  BCK(cudaMemcpyAsync(b->d_inst, inst.data(), sizeof(BatchInst<R>) * n, cudaMemcpyHostToDevice, b->stream));
  BCK(cudaStreamSynchronize(b->stream));  // inst is a host temporary
  return FDTD_OK;
}

// Spare field sets, tile work-lists and device buffers for depth K.
template <typename R>
static int batch_plan(fdtd_batch *b)
{
  const int K = b->K, n = (int)b->sims.size();
  std::vector<int4> tint, tgen;
  std::vector<double> omega(n);
  b->rows.assign(n, 0);
  for (int i = 0; i < n; i++) {
    fdtd_sim *s = b->sims[i];
    const size_t bytes = (size_t)s->nxa * s->pitch * s->esize;
    if (!s->d_f2[0])
      for (int a = 0; a < s->nslots; a++) {
        BCK(cudaMalloc(&s->d_f2[a], bytes));
        BCK(cudaMemsetAsync(s->d_f2[a], 0, bytes, s->stream));
      }
    const int L = batch_rows(b, s);
    TilePlan plan;
    if (int rc = fdtd_plan_tiles(s, K, L, batch_cols(b), &plan)) return rc;
    for (int g = 0; g < plan.nseg; g++) {
      const int r0 = plan.ra + g * L, r1 = std::min(r0 + L, plan.rb);
      for (int st = plan.s0; st < plan.s1; st++) tint.push_back(make_int4(i, st, r0, r1));
    }
    for (const int4 &t : plan.general) tgen.push_back(make_int4(i, t.x, t.y, t.z));
    b->rows[i] = L;
    omega[i] = s->geo.omega_s;
    if (!b->bb_lam.empty()) {  // broadband buffers: pulse rows, DFT sums, NTFF line buffers
      const int nfreq = (int)b->bb_lam.size();
      if (!b->bb_src[i]) BCK(cudaMalloc(&b->bb_src[i], (size_t)kMaxTBlock * s->nxa * s->esize));
      if (!b->bb_S[i]) BCK(cudaMalloc(&b->bb_S[i], sizeof(double2) * 2 * (size_t)s->ncell * nfreq));
      if (!s->d_tbcol) {
        BCK(cudaMalloc(&s->d_tbcol, (size_t)kMaxTBlock * 12 * s->nxa * s->esize));
        BCK(cudaMalloc(&s->d_tbrow, (size_t)kMaxTBlock * 12 * s->pitch * s->esize));
      }
      b->max_nxa = std::max(b->max_nxa, s->nxa);
      b->max_ncell = std::max(b->max_ncell, s->ncell);
    }
  }
  // largest tiles first (rows walked = height + 2K), so the warps that take the
  // last tiles of a launch finish together
  auto taller = [](const int4 &a, const int4 &c) { return a.w - a.z > c.w - c.z; };
  std::stable_sort(tint.begin(), tint.end(), taller);
  std::stable_sort(tgen.begin(), tgen.end(), taller);
  for (fdtd_sim *s : b->sims) BCK(cudaStreamSynchronize(s->stream));
  cudaFree(b->d_inst);
  cudaFree(b->d_tint);
  cudaFree(b->d_tgen);
  cudaFree(b->d_omega);
  b->d_inst = b->d_tint = b->d_tgen = b->d_omega = nullptr;
  BCK(cudaMalloc(&b->d_inst, sizeof(BatchInst<R>) * n));
  BCK(cudaMalloc(&b->d_tint, sizeof(int4) * std::max<size_t>(1, tint.size())));
  BCK(cudaMalloc(&b->d_tgen, sizeof(int4) * std::max<size_t>(1, tgen.size())));
  if (!tint.empty()) BCK(cudaMemcpy(b->d_tint, tint.data(), sizeof(int4) * tint.size(), cudaMemcpyHostToDevice));
  if (!tgen.empty()) BCK(cudaMemcpy(b->d_tgen, tgen.data(), sizeof(int4) * tgen.size(), cudaMemcpyHostToDevice));
  BCK(cudaMalloc(&b->d_omega, sizeof(double) * n));
  BCK(cudaMemcpy(b->d_omega, omega.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
  if (!b->d_clock) BCK(cudaMalloc(&b->d_clock, sizeof(BatchClock)));
  b->n_int = (int)tint.size();
  b->n_gen = (int)tgen.size();
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  b->planned_k = K;
  b->dft_every = std::max(1, (b->dft_stride + K - 1) / K);
  b->planned_l = b->L;
  b->planned_c = batch_cols(b);
  return FDTD_OK;
}

template <typename R, int K, bool TM, int CPL>
static void batch_block(fdtd_batch *b)
{
  cudaStream_t st = b->stream;
  const int n = (int)b->sims.size();
  auto *inst = (BatchInst<R> *)b->d_inst;
  auto *clk = (BatchClock *)b->d_clock;
  batch_source_kernel<R><<<(n * K + 127) / 128, 128, 0, st>>>(inst, (const double *)b->d_omega, n, K, clk);
  const int nfreq = (int)b->bb_lam.size();
  if (nfreq > 0)
    batch_pulse_kernel<R><<<dim3((unsigned)((K * b->max_nxa + 255) / 256), (unsigned)n), 256, 0, st>>>(
        inst, K, clk, (const double *)b->d_bb_freq, nfreq, (double2 *)b->d_bb_phase);
  // the two tile kernels run side by side (fork onto the second stream, join)
  cudaEventRecord(b->ev_fork, st);
  cudaStreamWaitEvent(b->stream2, b->ev_fork, 0);
  constexpr bool wide_ok = batch_aux_wide_ok<R, K, TM, CPL>();
  if (b->n_gen > 0 && wide_ok && b->aux_wide)
    batch_tile_kernel<R, K, true, TM, CPL, wide_ok><<<b->grid_gen, 32 * kBWarps, 0, b->stream2>>>(
        inst, (const int4 *)b->d_tgen, b->n_gen, clk);
  else if (b->n_gen > 0)
    batch_tile_kernel<R, K, true, TM, CPL><<<b->grid_gen, 32 * kBWarps, 0, b->stream2>>>(
        inst, (const int4 *)b->d_tgen, b->n_gen, clk);
  cudaEventRecord(b->ev_join, b->stream2);
  if (b->n_int > 0)
    batch_tile_kernel<R, K, false, TM, CPL><<<b->grid_int, 32 * kBWarps, 0, st>>>(inst, (const int4 *)b->d_tint,
                                                                             b->n_int, clk);
  cudaStreamWaitEvent(st, b->ev_join, 0);
  if (nfreq > 0)
    batch_dft_kernel<R, K><<<dim3((unsigned)((b->max_ncell + 3) / 4), (unsigned)n), 128, 0, st>>>(
        inst, clk, (const double2 *)b->d_bb_phase, nfreq, b->dft_every);
  batch_clock_kernel<<<1, 1, 0, st>>>((BatchClock *)b->d_clock, K);
}

// persistent grid sizes (resident blocks on every SM, at most one warp per tile)
template <typename R, int K, bool TM, int CPL>
static void batch_grids(fdtd_batch *b)
{
  b->grid_int = persistent_grid<R, K, false, TM, CPL>(b->n_int);
  // the wide work-list kernel once the list gives every warp of 4 blocks per SM a tile
  constexpr bool wide_ok = batch_aux_wide_ok<R, K, TM, CPL>();
  int dev = 0, nsm = 152;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev))
    cudaGetLastError();
  b->aux_wide = wide_ok && b->n_gen >= 4 * kBWarps * nsm;
  b->grid_gen = b->aux_wide ? persistent_grid<R, K, true, TM, CPL, wide_ok>(b->n_gen)
                            : persistent_grid<R, K, true, TM, CPL>(b->n_gen);
}

// dispatch on (K, columns per lane, TM) of the batch
template <typename R, bool GRIDS>
static void batch_dispatch(fdtd_batch *b)
{
  constexpr bool f32 = sizeof(R) == 4;
  const bool tm = b->tm;
  if (f32 && batch_cols(b) == 2) {
    if (b->K == 2) {
      if (GRIDS) tm ? batch_grids<R, 2, true, f32 ? 2 : 1>(b) : batch_grids<R, 2, false, f32 ? 2 : 1>(b);
      else tm ? batch_block<R, 2, true, f32 ? 2 : 1>(b) : batch_block<R, 2, false, f32 ? 2 : 1>(b);
    } else {
      if (GRIDS) tm ? batch_grids<R, 4, true, f32 ? 2 : 1>(b) : batch_grids<R, 4, false, f32 ? 2 : 1>(b);
      else tm ? batch_block<R, 4, true, f32 ? 2 : 1>(b) : batch_block<R, 4, false, f32 ? 2 : 1>(b);
    }
    return;
  }
  switch (b->K) {
  case 1:
    if (GRIDS) tm ? batch_grids<R, 1, true, 1>(b) : batch_grids<R, 1, false, 1>(b);
    else tm ? batch_block<R, 1, true, 1>(b) : batch_block<R, 1, false, 1>(b);
    break;
  case 2:
    if (GRIDS) tm ? batch_grids<R, 2, true, 1>(b) : batch_grids<R, 2, false, 1>(b);
    else tm ? batch_block<R, 2, true, 1>(b) : batch_block<R, 2, false, 1>(b);
    break;
  case 4:
    if (GRIDS) tm ? batch_grids<R, 4, true, 1>(b) : batch_grids<R, 4, false, 1>(b);
    else tm ? batch_block<R, 4, true, 1>(b) : batch_block<R, 4, false, 1>(b);
    break;
  default:  // 8: FP32 only (checked by fdtd_batch_set_option)
    if (f32) {
      if (GRIDS) tm ? batch_grids<R, f32 ? 8 : 4, true, 1>(b) : batch_grids<R, f32 ? 8 : 4, false, 1>(b);
      else tm ? batch_block<R, f32 ? 8 : 4, true, 1>(b) : batch_block<R, f32 ? 8 : 4, false, 1>(b);
    }
    break;
  }
}

// blocks per graph replay
static const int kGraphBlocks = 4;

extern "C" int fdtd_batch_run(fdtd_batch *b)
{
  if (!b) return set_error(FDTD_E_ARG, "null batch");
  int max_n = 0;
  for (fdtd_sim *s : b->sims) {
    if (s->time != 0) return set_error(FDTD_E_STATE, "batch_run starts every instance at time 0 (fdtd_reset)");
    max_n = std::max(max_n, s->cfg.step_num);
  }
  if (b->planned_k != b->K || b->planned_l != b->L || b->planned_c != batch_cols(b)) {
    if (int rc = b->f32 ? batch_plan<float>(b) : batch_plan<double>(b)) return rc;
    if (b->f32) batch_dispatch<float, true>(b);
    else batch_dispatch<double, true>(b);
  }
  for (fdtd_sim *s : b->sims) BCK(cudaStreamSynchronize(s->stream));
  if (int rc = b->f32 ? batch_descriptors<float>(b) : batch_descriptors<double>(b)) return rc;
  BatchClock c0{0.0, 0, {0, 0}};
  BCK(cudaMemcpyAsync(b->d_clock, &c0, sizeof c0, cudaMemcpyHostToDevice, b->stream));
  for (size_t i = 0; i < b->bb_S.size(); i++)  // broadband: the DFT sums start at zero every run
    BCK(cudaMemsetAsync(b->bb_S[i], 0, sizeof(double2) * 2 * (size_t)b->sims[i]->ncell * b->bb_lam.size(),
                        b->stream));
  if (!b->graph) {
    cudaGraph_t g = nullptr;
    BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    for (int q = 0; q < kGraphBlocks; q++) {
      if (b->f32) batch_dispatch<float, false>(b);
      else batch_dispatch<double, false>(b);
    }
    const cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
    if (ce != cudaSuccess) {
      cudaGetLastError();
      return set_error(FDTD_E_CUDA, "graph capture failed: %s", cudaGetErrorString(ce));
    }
    const cudaError_t ie = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
      cudaGetLastError();
      b->graph = nullptr;
      return set_error(FDTD_E_CUDA, "graph instantiate failed: %s", cudaGetErrorString(ie));
    }
    b->graph_blocks = kGraphBlocks;
  }
  const int nblocks = (max_n + b->K - 1) / b->K;
  const int reps = (nblocks + b->graph_blocks - 1) / b->graph_blocks;
  const int per_block = 2 + (b->n_int > 0) + (b->n_gen > 0) + (b->bb_lam.empty() ? 0 : 2);
  for (int r = 0; r < reps; r++) BCK(cudaGraphLaunch(b->graph, b->stream));
  b->launches += (long long)reps * b->graph_blocks * per_block;
  BCK(cudaStreamSynchronize(b->stream));
  for (fdtd_sim *s : b->sims) {  // the fields of instance i are in the set its last block wrote
    const int blocks = (s->cfg.step_num + b->K - 1) / b->K;
    if (blocks & 1)
      for (int a = 0; a < kMaxSlots; a++) std::swap(s->d_f[a], s->d_f2[a]);
    s->time = s->cfg.step_num;
    s->ray_coef = 1.0 - exp(-pow(0.01 * s->time, 2));
  }
  return FDTD_OK;
}

extern "C" int fdtd_batch_reset(fdtd_batch *b)
{
  if (!b) return set_error(FDTD_E_ARG, "null batch");
  for (fdtd_sim *s : b->sims)
    if (int rc = fdtd_reset(s)) return rc;
  return FDTD_OK;
}

extern "C" int fdtd_batch_broadband(fdtd_batch *b, int nlam, const int *lambda_nm)
{
  if (!b || !lambda_nm || nlam < 1 || nlam > 64) return set_error(FDTD_E_ARG, "1..64 wavelengths");
  if (!b->tm) return set_error(FDTD_E_UNSUPPORTED, "the broadband batch runs MPI_TM_UPML");
  const fdtd_sim *s0 = b->sims[0];
  for (const fdtd_sim *s : b->sims) {
    if (s->cfg.angle_deg != 0) return set_error(FDTD_E_UNSUPPORTED, "the broadband pulse runs at 0 degrees");
    if (!s->d_cells || s->ncell <= 0)
      return set_error(FDTD_E_STATE, "broadband instances need the NTFF path (no FDTD_CFG_NO_TIME_NTFF)");
    if (s->cfg.h_u_nm != s0->cfg.h_u_nm || s->c0 != s0->c0)
      return set_error(FDTD_E_ARG, "broadband instances share one cell size and Courant number");
  }
  std::vector<double> freq(nlam);
  for (int k = 0; k < nlam; k++) {
    if (lambda_nm[k] <= 0) return set_error(FDTD_E_ARG, "wavelength %d nm", lambda_nm[k]);
    const double lambda_s = (double)lambda_nm[k] / s0->cfg.h_u_nm;  // field.c:105-109: w = C k, k = 2 pi / lambda_s
    freq[k] = s0->c0 * (2 * M_PI / lambda_s);
  }
  BCK(cudaStreamSynchronize(b->stream));
  cudaFree(b->d_bb_freq);
  cudaFree(b->d_bb_phase);
  cudaFree(b->d_bb_X);
  cudaFree(b->d_bb_Sptr);
  cudaFree(b->d_bb_idx);
  for (void *p : b->bb_src) cudaFree(p);
  for (void *p : b->bb_S) cudaFree(p);
  b->d_bb_freq = b->d_bb_phase = b->d_bb_X = b->d_bb_Sptr = b->d_bb_idx = nullptr;
  b->bb_src.assign(b->sims.size(), nullptr);
  b->bb_S.assign(b->sims.size(), nullptr);
  b->bb_lam.assign(lambda_nm, lambda_nm + nlam);
  b->bb_freq = freq;
  b->bb_a2.clear();
  BCK(cudaMalloc(&b->d_bb_freq, sizeof(double) * nlam));
  BCK(cudaMemcpy(b->d_bb_freq, freq.data(), sizeof(double) * nlam, cudaMemcpyHostToDevice));
  BCK(cudaMalloc(&b->d_bb_phase, sizeof(double2) * (size_t)nlam));
  BCK(cudaMalloc(&b->d_bb_X, sizeof(double2) * 360 * (size_t)nlam * b->sims.size()));
  BCK(cudaMalloc(&b->d_bb_Sptr, sizeof(void *) * b->sims.size()));
  BCK(cudaMalloc(&b->d_bb_idx, sizeof(int) * b->sims.size()));
  b->planned_k = 0;  // buffers and graph are made again by the next run
  return FDTD_OK;
}

// |A(w_k)|^2 of instance s: the incident pulse at x = 0 (field.c:224-256)
// transformed with the samples' e^{i w t} at the times the DFT sampled (the
// last level of every `dft_every`-th full K-step block: clock t = D-1,
// 2D-1, ... with D = dft_every K); dividing by it leaves the response to a
// unit incident wave, the CW run's steady state.  Cached by (t0, carrier,
// step_num, D): the instances of a sweep share it.
static const std::vector<double> &pulse_spectrum2(fdtd_batch *b, const fdtd_sim *s)
{
  const int nfreq = (int)b->bb_lam.size(), D = b->planned_k * b->dft_every;
  const double t0 = -((s->geo.n_px / 2.0) * (cos(0.0) / s->c0)) + 500, w = s->geo.omega_s;
  const std::array<double, 4> key{t0, w, (double)s->cfg.step_num, (double)D};
  for (const auto &e : b->bb_a2)
    if (e.first == key) return e.second;
  std::vector<double> a2(nfreq);
  for (int k = 0; k < nfreq; k++) {
    double ar = 0, ai = 0;
    for (int t = D - 1; t < s->cfg.step_num; t += D) {
      const double r = -(t - t0), g = exp(-(r / 50.0) * (r / 50.0));
      const double ph = r * w + b->bb_freq[k] * (t - 1.0);
      ar += g * cos(ph);
      ai += g * sin(ph);
    }
    a2[k] = ar * ar + ai * ai;
  }
  b->bb_a2.emplace_back(key, std::move(a2));
  return b->bb_a2.back().second;
}

// Far fields of instances [i0, i1) into out[(i - i0)][nlam][360].  Instances
// created with the same configuration share one path: each such group is one
// launch over all its maps (fdtd_far_field_of_sums_group), then one copy back.
static int broadband_spectra(fdtd_batch *b, int i0, int i1, double *out)
{
  if (b->bb_lam.empty()) return set_error(FDTD_E_STATE, "no broadband run (fdtd_batch_broadband)");
  const int nfreq = (int)b->bb_lam.size();
  const size_t per = 360 * (size_t)nfreq;
  std::vector<std::vector<int>> groups;
  for (int i = i0; i < i1; i++) {
    fdtd_sim *s = b->sims[i];
    if (!b->bb_S[i]) return set_error(FDTD_E_STATE, "no broadband run (fdtd_batch_broadband)");
    if (s->time != s->cfg.step_num) return set_error(FDTD_E_STATE, "instance %d has not run to its step_num", i);
    bool placed = false;
    for (auto &g : groups)
      if (std::memcmp(&b->sims[g[0]]->cfg, &s->cfg, sizeof(fdtd_config)) == 0) {
        g.push_back(i);
        placed = true;
        break;
      }
    if (!placed) groups.push_back({i});
  }
  std::vector<int> order;
  for (const auto &g : groups) order.insert(order.end(), g.begin(), g.end());
  BCK(cudaMemcpyAsync(b->d_bb_Sptr, b->bb_S.data(), sizeof(void *) * b->bb_S.size(), cudaMemcpyHostToDevice,
                      b->stream));
  BCK(cudaMemcpyAsync(b->d_bb_idx, order.data(), sizeof(int) * order.size(), cudaMemcpyHostToDevice, b->stream));
  size_t off = 0;
  for (const auto &g : groups) {
    fdtd_sim *s = b->sims[g[0]];
    if (int rc = fdtd_far_field_of_sums_group(s, (const double *)b->d_bb_freq, nfreq, (const double2 *const *)b->d_bb_Sptr,
                                              (const int *)b->d_bb_idx + off, (int)g.size(), (double2 *)b->d_bb_X,
                                              per, 1.0 / (4 * M_PI * s->c0 * 1.0e6), b->stream))
      return rc;
    off += g.size();
  }
  std::vector<double2> X(per * (size_t)(i1 - i0));
  BCK(cudaMemcpyAsync(X.data(), (double2 *)b->d_bb_X + (size_t)i0 * per, sizeof(double2) * X.size(),
                      cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaStreamSynchronize(b->stream));  // also keeps `order` alive until its copy is done
  for (int i = i0; i < i1; i++) {
    const std::vector<double> &a2 = pulse_spectrum2(b, b->sims[i]);
    const double2 *x = X.data() + (size_t)(i - i0) * per;
    double *o = out + (size_t)(i - i0) * per;
    for (int k = 0; k < nfreq; k++)
      for (int ang = 0; ang < 360; ang++) {
        const double2 v = x[(size_t)ang * nfreq + k];
        o[(size_t)k * 360 + ang] = (v.x * v.x + v.y * v.y) / a2[k];
      }
  }
  return FDTD_OK;
}

extern "C" int fdtd_batch_broadband_spectrum(fdtd_batch *b, int index, double *out)
{
  if (!b || !out || index < 0 || index >= (int)b->sims.size()) return set_error(FDTD_E_ARG, "bad instance index");
  return broadband_spectra(b, index, index + 1, out);
}

extern "C" int fdtd_batch_broadband_spectra(fdtd_batch *b, double *out)
{
  if (!b || !out) return set_error(FDTD_E_ARG, "null argument");
  return broadband_spectra(b, 0, (int)b->sims.size(), out);
}
