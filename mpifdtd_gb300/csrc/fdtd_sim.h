// fdtd_sim.h -- host-side state of one simulation (opaque fdtd_sim of the C ABI).
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "../../include/mpifdtd_gb300.h"
#include "fdtd_internal.cuh"

struct fdtd_sim {
  int solver = 0;
  bool tm = false, mpi = false, f32 = false;
  int family = 0;               // 0 UPML, 1 split-field PML (fdtdTM.c / fdtdTE.c), 2 NS-FDTD (nsFdtd*.c)
  void *d_coef = nullptr;       // family 1, 2: per-cell coefficients (fdtd_split.cu), ncoef x nxa x pitch
  int ncoef = 0;
  bool coef_dirty = true;       // the permittivity changed since the coefficients were made
  fdtd_config cfg{};
  fdtd_geometry geo{};
  double c0 = fdtd::kC, z0 = fdtd::kZ0;  // Courant number, impedance (config_courant, config_z0)
  // array frame (see fdtd_internal.cuh)
  int ox = 0, ni = 0, nj = 0, nxa = 0, ncols = 0, pitch = 0;
  size_t esize = 0;
  int nslots = 0;
  int in_x0 = 0, in_x1 = 0, in_y0 = 0, in_y1 = 0;
  double inv_mu = 0;
  cudaStream_t stream = nullptr;
  void *d_f[fdtd::kMaxSlots] = {};
  void *d_ieps64[2] = {}, *d_ieps32[2] = {};
  void *d_tab64[4] = {}, *d_tab32[4] = {};
  void *d_ex = nullptr, *d_ey = nullptr;      // CW phase tables, FP64
  void *d_ex32 = nullptr, *d_ey32 = nullptr;  // and FP32 copies (FP32 fields)
  // NTFF
  void *d_cells = nullptr, *d_shift = nullptr, *d_vals = nullptr, *d_dg = nullptr;
  void *d_ntff[3] = {};
  unsigned int *d_status = nullptr;
  int ncell = 0;
  size_t ntff_len = 0;
  std::vector<double> h_shift;   // [360][ncell], kept to rebuild the window tables
  std::vector<int> h_side;       // side of each path cell (0 bottom, 1 right, 2 top, 3 left)
  // NTFF deposit: 0 direct, 1 shared window, 2 time-blocked (default)
  int ntff_mode = 2, ntff_chunk = 1024, ntff_block = 32;
  int rows = 1;                 // stencil rows per thread (FDTD_OPT_ROWS)
  // temporal blocking (MPI solvers): K steps per launch, ping-pong field sets
  int tblock = 0;               // depth K (FDTD_OPT_TBLOCK), 0 = one launch pair per step
  int tb_rows = 0;              // rows per tile segment (FDTD_OPT_TBLOCK_ROWS), 0 = automatic
  void *d_f2[fdtd::kMaxSlots] = {};  // the other field set
  void *d_tbcol = nullptr, *d_tbrow = nullptr;  // NTFF line samples of kMaxTBlock levels
  void *d_ptab = nullptr;       // serial solvers at 0 degrees: pulse row tables [2][kMaxTBlock][nxa] (PulseRow)
  void *d_tiles = nullptr;      // int4 (strip, r0, r1, -) work-list of the general kernel
  int ntiles = 0, tiles_cap = 0;
  int tb_s0 = 0, tb_s1 = 0, tb_ra = 1, tb_rb = 1, tb_nseg = 0, tb_L = 0;
  int tb_cols = 1;               // columns per lane (FDTD_OPT_TBLOCK_COLS)
  int tb_built_k = 0, tb_built_l = 0, tb_built_c = 0;
  std::vector<double> tune_table;  // last fdtd_autotune: (K, rows, columns per lane, ms per step) per candidate
  int nb_pending = 0;           // buffered steps not yet deposited (mode 2)
  double pending_t0 = 0;        // timeE of the first buffered step
  void *d_chunk = nullptr, *d_lo = nullptr;
  int nchunk = 0, win_width = 0;
  bool window_dirty = true;
  void *d_eps[3] = {};            // permittivity as given, padded array frame (fdtd_get_eps)
  // engine clock (field.c:21-22 time, ray_coef)
  double time = 0, ray_coef = 0;
  long long launches = 0;
  // running-DFT NTFF (fdtd_dft_enable): two FFT bins per wavelength
  std::vector<int> dft_lam;
  std::vector<double> dft_frac;  // interpolation weight of the upper bin per wavelength
  void *d_dft_omega = nullptr, *d_dft_P = nullptr, *d_dft_S = nullptr, *d_dft_X = nullptr;
  void *d_dft_T = nullptr;        // far-field bin table e^{i w m} (fdtd_dft.cu DftBins), d_dft_T_bytes long
  size_t d_dft_T_bytes = 0;
  int bin_mlo = 0, bin_nm = -1;   // retarded bins of the path's shifts (-1: not yet derived)
  // far-field outputs (allocated on first use)
  void *d_spec = nullptr, *d_dirs = nullptr, *d_twiddle = nullptr, *d_freq = nullptr;
  // per-kernel event timing (fdtd_profile_*): 5 events per step
  bool profiling = false;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  long long prof_steps = 0;
};

// Temporal-blocking tiles of a simulation (fdtd_api.cu), cpl columns per lane: interior strips
// [s0, s1) x rows [ra, rb) in nseg segments of L rows, and the list of the
// other tiles (strip, r0, r1, 0).
struct TilePlan {
  int s0 = 0, s1 = 0, ra = 1, rb = 1, L = 0, nseg = 0;
  std::vector<int4> general;
};
int fdtd_plan_tiles(const fdtd_sim *s, int K, int L, int cpl, TilePlan *plan);

// The stencil view of a simulation's current field set (fdtd_api.cu).
template <typename R>
fdtd::StencilView<R> fdtd_view_of(fdtd_sim *s);

// Far field X[360][nfreq] (device) of the running-DFT sums S[2][ncell][nfreq]
// (device, E then H path samples, phasors of the E sample times) at the
// frequencies omega[nfreq] (device, radians per step), with the simulation's
// own path, shifts and spectrum coefficient (fdtd_api.cu; the broadband batch
// keeps its sums outside the simulation), times `scale` (the batch's sums
// leave out the samples' 1/(4 pi C R)).
int fdtd_far_field_of_sums(fdtd_sim *s, const double *d_omega, int nfreq, const double2 *d_S, double2 *d_X,
                           double scale);
// The same for nmaps instances that share s's configuration (hence its path):
// instance idx[j]'s sums are d_S[idx[j]] and its far field goes to
// d_X + idx[j] x_stride (d_S, d_idx: device arrays), launched on st.
int fdtd_far_field_of_sums_group(fdtd_sim *s, const double *d_omega, int nfreq, const double2 *const *d_S,
                                 const int *d_idx, int nmaps, double2 *d_X, size_t x_stride, double scale,
                                 cudaStream_t st);

// 1/eps of the E components (or, for the split-field / NS solvers, a rebuild of
// the per-cell coefficients before the next step) from the permittivity on the
// device (fdtd_api.cu); FDTD_E_ARG if a value is not finite and > 0.
int fdtd_derive_inv_eps(fdtd_sim *s);
