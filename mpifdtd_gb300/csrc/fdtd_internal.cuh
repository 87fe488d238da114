// fdtd_internal.cuh -- device-side data structures of the GB300 FDTD engine.
//
// Layout in HBM (one simulation):
//   every field is a pitched 2-D array of complex values, rows i in [0, nxa),
//   columns j in [0, P), y (j) contiguous as in the reference (field.c:70-74).
//   Active cells are i in [1, ni], j in [1, nj]; the ring around them is a
//   zero halo (PEC): for the MPI solvers it is the one-rank sub-domain halo
//   of mpiTM_UPML.c:737-741 (global x = i-1), for the serial solvers it is
//   the boundary ring the reference never updates (global x = i).
//   P is a multiple of 8 complex values so every row starts on a 128-byte
//   boundary and a warp's 32 consecutive j are one coalesced 512-byte (FP64)
//   or 256-byte (FP32) transaction.
//
// PML coefficients are separable (every C_* of mpiTM_UPML.c:697-713 and
// mpiTE_UPML.c:517-533 depends on sigma_x at one stagger and/or sigma_y at
// one stagger), so they live in four 1-D tables per simulation instead of the
// reference's 15 per-cell arrays.
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>

#include "../../include/mpifdtd_gb300.h"

namespace fdtd {

constexpr double kC = 0.7071;                 // field.h:70 C_0_S
constexpr double kEps0 = 1.0;                 // field.h:73
constexpr double kZ0 = 1.41422712488;         // field.h:75
constexpr int kGuard = 16;                    // NTFF guard cells each side
constexpr int kMaxNtffBlock = 64;             // steps buffered per time-blocked NTFF deposit
constexpr int kNfft = 8192;                   // ntff.h:6 NTFF_NUM
constexpr int kLambdaSt = 380, kLambdaEn = 700;  // ntff.h:4-5

template <typename R> struct Cplx;
template <> struct Cplx<double> { using T = double2; };
template <> struct Cplx<float> { using T = float2; };

// One entry of a 1-D coefficient table (meaning depends on table, see
// fdtd_api.cu build_coefficients()).
template <typename R> struct Coef4 { R a, b, c, d; };

// Field slots.  TM: 0 Ez 1 Dz 2 Jz 3 Hx 4 Hy 5 Mx 6 My (M scaled by 1/mu0)
//               TE: 0 Ex 1 Ey 2 Dx 3 Dy 4 Jx 5 Jy 6 Hz 7 Mz (M scaled by 1/mu0)
constexpr int kMaxSlots = 8;

template <typename R>
struct StencilView {
  typename Cplx<R>::T *f[kMaxSlots];
  const R *inv_eps[2];          // TM: [0] 1/EPS_EZ ; TE: [0] 1/EPS_EX, [1] 1/EPS_EY
  const Coef4<R> *tx_i, *tx_h;  // indexed by row i (sigma_x at x, x+1/2)
  const Coef4<R> *ty_i, *ty_h;  // indexed by column j (sigma_y at y, y+1/2)
  const typename Cplx<R>::T *ex, *ey;  // CW source phase tables e^{i x kcos}, e^{i y ksin} in R
  // Elements between the ex tables of consecutive levels of a blocked launch:
  // 0 (one table for every level, the CW source) or nxa (a batched Gaussian
  // pulse at 0 degrees, whose row table changes with the level's time).
  int src_lstride;
  int P, nxa, ni, nj, ox;
  int in_x0, in_x1, in_y0, in_y1;  // interior (all sigma = 0): x in [in_x0,in_x1)
  int rows;                        // rows per thread of the stencil kernels (1, 2, 4, 8)
  R inv_mu;
};

// Per-step source description.
// Gaussian pulse of one row at one step, for 0 degrees (the pulse then depends
// on the row only): a = dot g, (c, s) = (cos, sin) of its phase (stencil_ops.cuh
// pulse_source computes the same values per cell)
struct PulseRow {
  double a, c, s, pad;
};

struct SourceStep {
  int kind;          // 0 none, 1 CW scattered wave (MPI solvers), 2 Gaussian pulse (serial)
  double s_re, s_im; // CW: ray_coef * e^{-i w t}
  // pulse (field.c:224-256), applied to field slot `slot` with permittivity table `eps_slot`
  double time, t0, w, cos_per_c, sin_per_c, gap_x, gap_y, dot;
};

// Surface cell of the NTFF integration path.
struct SurfCell {
  long long k;       // array index of the E sample
  int hoff;          // offset of the second H sample (-1 bottom/top, -P right/left)
  signed char sign;  // +1 / -1 (normal orientation, mpiTM_UPML.c:877-1035)
  signed char e_slot, h_slot, uid_wid;   // uid_wid = uid | (wid << 4)
};

struct NtffView {
  double2 *acc[3];        // base pointers incl. guard (flat [360][AS] + 2*guard)
  const double *shift;    // [360][ncell] retarded-time shift per (angle, cell)
  const SurfCell *cells;
  double2 *vals;          // [slot][2][ncell] surface values (E then H) of buffered steps
  double4 *dg;            // [j][2][ncell] (d_j, e_j): differences of the buffered values (block deposit)
  int ncell, array_size;
  long long len;          // elements of each accumulator incl. guards
  unsigned int *status;   // device status word (kStatus* bits)
};

// Shared-memory window variant of the NTFF deposit.  The path is cut into
// chunks (consecutive cells of one side); along a side the retarded-time
// shift is linear in the cell index, so the bins one chunk touches in one step
// form a short contiguous range [base, base+W) with base = floor(timeE) + lo.
struct NtffWindow {
  const int2 *chunk;      // [nchunk] (first cell, cell count)
  const int2 *lo;         // [360][nchunk] (lo_e, lo_h) bin offsets
  int nchunk, width;      // width W of both windows (bins)
};

// Device status bits (fdtd_get_status).
constexpr unsigned int kStatusNtffRange = 1u;   // a deposit fell outside the accumulator
constexpr unsigned int kStatusBadEps = 2u;      // a permittivity value was not finite and > 0
constexpr unsigned int kStatusNonFinite = 4u;   // fdtd_check_finite found a non-finite field value

// Launchers (fdtd_kernels.cu).  All take the stream they run on.
template <typename R>
void launch_tm_e(const StencilView<R> &v, const SourceStep &s, cudaStream_t st);
template <typename R>
void launch_tm_h(const StencilView<R> &v, cudaStream_t st);
template <typename R>
void launch_te_e(const StencilView<R> &v, const SourceStep &sx, const SourceStep &sy, cudaStream_t st);
template <typename R>
void launch_te_h(const StencilView<R> &v, cudaStream_t st);
template <typename R>
void launch_ntff_gather(const StencilView<R> &v, const NtffView &n, double coef, int slot, cudaStream_t st);
void launch_ntff_accumulate(const NtffView &n, double timeE, double timeH, cudaStream_t st);
void launch_ntff_window(const NtffView &n, const NtffWindow &w, double timeE, double timeH, cudaStream_t st);
// Deposit nb buffered steps (slots 0..nb-1) whose first step has timeE = t0.
void launch_ntff_block(const NtffView &n, int nb, double t0, cudaStream_t st);

// ---- temporally blocked stencil (fdtd_tblock.cu)
//
// K steps of an MPI solver per launch.  A warp owns a tile: a strip of
// W = 32 cpl - 2K columns (cpl columns per lane; strip s owns columns
// o + s W .. o + s W + W - 1, o = 1 for cpl 1 and K mod 2 for cpl 2) and a row
// segment [r0, r1).  Interior tiles (cone free of PML and halo) cover strips [s0, s1)
// x rows [ra, rb) in segments of L rows; every other tile is an entry
// (strip, r0, r1) of the work-list.  The launch reads the field set of
// StencilView::f and writes the set `out` (ping-pong), plus the E and H
// samples of the NTFF lines of every level.
constexpr int kMaxTBlock = 8;

template <typename R>
struct TBlockView {
  typename Cplx<R>::T *out[kMaxSlots];  // destination field set
  // NTFF line samples per level (null: none):
  //   col[((level*4 + q)*3 + f)*nxa + i]   q-th sampled column cj[q], rows i
  //   row[((level*4 + q)*3 + f)*P + j]     q-th sampled row ri[q], columns j
  // f: TM 0 Ez, 1 Hx, 2 Hy ; TE 0 Ex, 1 Ey, 2 Hz
  typename Cplx<R>::T *col, *row;
  int cj[4], ri[4];
  const int4 *tiles;   // (strip, r0, r1, -) tiles of the general kernel
  int ntiles;
  int s0, s1;          // interior kernel: strips [s0, s1) x
  int ra, rb, nseg;    //   rows [ra, rb) in nseg segments of L rows
  int L;
  int cpl;             // columns per lane: 1, or 2 (FP32, K = 2 or 4)
  double2 sc[kMaxTBlock];  // CW source per level: ray_coef e^{-i w t}
  SourceStep pulse[2];     // serial solvers: the pulse of the block's first step (TM [0] on Ez; TE [0] Ex, [1] Ey)
  const PulseRow *ptab[2]; // 0 degrees: pulse[p] per level and row, [K][nxa] (null: per cell)
};

// Runs the interior and the general kernel of depth K (1, 2, 4 or 8).
template <typename R>
void launch_tblock(const StencilView<R> &v, const TBlockView<R> &tb, int K, bool tm, cudaStream_t st);
// The same for the serial solvers (H half-step first, pulse source; K = 1, 2 or 4),
// fdtd_tblock_serial.cu.
template <typename R>
void launch_tblock_serial(const StencilView<R> &v, const TBlockView<R> &tb, int K, bool tm, cudaStream_t st);
// tab[l][i] = the pulse s at step s.time + l of array row i (l < K, i < nrow), 0 degrees only
void launch_pulse_rows(const SourceStep &s, int K, int nrow, PulseRow *tab, cudaStream_t st);
// vals slots slot0 .. slot0+K-1 from the NTFF line samples of a blocked launch
// (the samples ntff_gather_kernel takes from the fields after each step).
template <typename R>
void launch_line_gather(const StencilView<R> &v, const TBlockView<R> &tb, const NtffView &n, double coef, int K,
                        int slot0, bool tm, cudaStream_t st);

}  // namespace fdtd

#include "models_eval.h"

namespace fdtd {

// fdtd_farfield.cu
struct SpectrumView {
  const double2 *acc[3];   // NTFF accumulators incl. guard
  int array_size, max_time, tm, h_u_nm;
  double c0, z0;           // Courant number and impedance (field.h:70, :75 by default)
  const double2 *dir;      // [360] (cos phi, sin phi)
  const double2 *twiddle;  // [4096] e^{+2 pi i k / 8192}
  double2 coef;            // 1/(4 pi C) sqrt(2 pi C / (i w))  (ntffTM.c:165)
  double *out;             // [321][360]
};
struct FrequencyView {
  // global cell (x,y) at array (x-ox)*P + (y-ox)
  const void *e[2];        // TM: Ez, Ez ; TE: Ex (bottom/top sides), Ey (right/left)
  const void *h[2];        // TM: Hx (bottom/top), Hy (right/left) ; TE: Hz, Hz
  int tm;                  // ntffTM_Frequency, else ntffTE_Frequency
  int f32;                 // fields are float2 (FP32 mode) instead of double2
  int P, ox, lt, rt, bm, tp;
  double cx, cy, k_s, scale;  // scale: sqrt(h_u_nm) (TM), h_u_nm (TE)
  double z0;               // impedance (field.h:75 by default)
  const double2 *dir;      // [360] (cos, sin)
  double2 coef;            // csqrt(i k/(8 pi R0)) e^{i k R0}  (ntffTM.c:82, ntffTE.c:256)
  double2 *out;            // [360]
};
void launch_spectrum(const SpectrumView &s, cudaStream_t st);

// fdtd_dft.cu: running DFT of the buffered path samples at nfreq frequencies
struct DftView {
  const double *omega;  // [nfreq] radians per step
  int nfreq;
  double2 *phasor;      // [kMaxNtffBlock][nfreq] scratch
  double2 *S;           // [2][ncell][nfreq] sum_t v_c(t) e^{i w t} (E samples, H samples)
};
void launch_dft_accumulate(const NtffView &n, const DftView &d, int nb, double t0, cudaStream_t st);
// Table of e^{i w_k m} for the integer retarded bins m in [mlo, mlo + nm) of
// a path (the caller's device buffer, nm x nfreq; nm = 0: no table).
struct DftBins {
  double2 *T;
  int mlo, nm;
};
void launch_dft_farfield(const NtffView &n, const DftView &d, int tm, double z0, const double2 *dir, double2 coef,
                         const DftBins &bins, double2 *X, cudaStream_t st);
// The same far field for nmaps maps that share the path of n (one
// configuration): map j's sums are S[idx[j]] ([2][ncell][nfreq]) and its far
// field goes to X + idx[j] x_stride ([360][nfreq]); S and idx are device arrays.
void launch_dft_farfield_group(const NtffView &n, const double2 *const *S, const int *idx, int nmaps,
                               const double *omega, int nfreq, int tm, double z0, const double2 *dir, double2 coef,
                               const DftBins &bins, double2 *X, size_t x_stride, cudaStream_t st);
// The settings of a configuration that the reference hard-codes (fdtd_config:
// courant_e4, pml_order, ntff_inset; 0 = the reference's value).
inline double config_courant(const fdtd_config &c) { return c.courant_e4 > 0 ? c.courant_e4 / 1.0e4 : kC; }
// field.h:75 writes sqrt(mu0/eps0) = 1/C as the literal 1.41422712488 for C = 0.7071
inline double config_z0(const fdtd_config &c) { return c.courant_e4 > 0 ? 1.0 / config_courant(c) : kZ0; }
inline int config_pml_order(const fdtd_config &c) { return c.pml_order > 0 ? c.pml_order : 2; }
inline int config_ntff_inset(const fdtd_config &c) { return c.ntff_inset > 0 ? c.ntff_inset : 5; }
void launch_frequency(const FrequencyView &f, cudaStream_t st);
// fdtd_split.cu: split-field PML and NS-FDTD solvers (one step = two launches)
struct SplitView {
  double2 *f[5];         // TM: 0 Ez 1 Ezx 2 Ezy 3 Hx 4 Hy ; TE: 0 Ex 1 Ey 2 Hz 3 Hzx 4 Hzy
  const double *c[10];   // per-cell coefficients (fdtd_split.cu)
  int P, n_px, n_py;
  double ray, t, w_s, ks_cos, ks_sin;  // source: ray_coef, time, omega, k (cos, sin of the wave angle)
  double r_2, co, si;                  // NS operator weight; NS TE source directions
};
void launch_split_step(const SplitView &v, int solver, cudaStream_t st);

// out[q] = field[idx[q]] widened to FP64 (FP32 fields: f32 = 1), q < n
void launch_point_gather(const void *field, int f32, const long long *idx, int n, double2 *out, cudaStream_t st);

// Sets the calling thread's fdtd_last_error() message and returns code (fdtd_api.cu).
int set_error(int code, const char *fmt, ...);

// fdtd_setup.cu
// alt: TM -- the MPI / split-field / NS staggering (HX at D_Y, HY at D_X) instead
// of the serial UPML one (D_XY everywhere); TE -- HZ sampled once at D_XY (NS TE)
// instead of the mean of D_X and D_Y
void launch_eps_model(double *e0, double *e1, double *e2, int P, int nxa, int ncols, int ox, int n_px, int n_py,
                      bool tm, bool alt, const mdl_params &m, cudaStream_t st);
void launch_inv_eps(const double *eps, double *ie64, float *ie32, size_t count, unsigned int *status,
                    cudaStream_t st);
void launch_fill(double *p, double v, size_t count, cudaStream_t st);

}  // namespace fdtd
