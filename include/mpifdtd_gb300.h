/*
 * mpifdtd_gb300.h -- C ABI of the GB300 (sm_103a) 2-D UPML FDTD engine.
 *
 * The engine time-steps the reference's TM_UPML / TE_UPML solvers
 * (rennone/mpiFDTD) on one GPU: the fused Yee + UPML auxiliary updates of
 * mpiTM_UPML.c / mpiTE_UPML.c (and of the serial fdtdTM_upml.c /
 * fdtdTE_upml.c), the scattered-field sources of field.c, and the
 * time-domain near-to-far-field (NTFF) accumulation into the flat
 * [360][arraySize] U/W arrays; besides those, the split-field PML and
 * non-standard FDTD solvers (fdtdTM.c, fdtdTE.c, nsFdtdTM.c, nsFdtdTE.c),
 * batched sweeps, the running-DFT NTFF and the reference's file outputs.
 * Plain C types only: no CUDA or torch types.
 *
 * The reference's own entry points (mpi_fdtdTM_upml_getUpdate() ... ) are
 * provided on top of this ABI by libmpifdtd_upml.so, see mpifdtd_upml.h.
 *
 * Every call returns FDTD_OK (0) or an error code; fdtd_last_error() gives a
 * message for the calling thread.  Nothing here falls back to the CPU: if no
 * usable GPU is present fdtd_create() fails with FDTD_E_CUDA.
 */
#ifndef MPIFDTD_GB300_H
#define MPIFDTD_GB300_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define FDTD_OK 0
#define FDTD_E_ARG 1           /* invalid argument or configuration            */
#define FDTD_E_CUDA 2          /* CUDA runtime error (no device, launch error)  */
#define FDTD_E_NOMEM 3         /* device or host allocation failed              */
#define FDTD_E_STATE 4         /* call not valid in the simulation's state      */
#define FDTD_E_UNSUPPORTED 5   /* valid request the engine does not implement   */

/* Solver ids: the values of enum SOLVER in simulator.h:8-18. */
#define FDTD_TM_2D 0           /* serial TM split-field PML (fdtdTM.c), FP64 only   */
#define FDTD_TE_2D 1           /* serial TE split-field PML (fdtdTE.c), FP64 only   */
#define FDTD_TM_UPML 2         /* serial TM UPML  (fdtdTM_upml.c)  */
#define FDTD_TE_UPML 3         /* serial TE UPML  (fdtdTE_upml.c)  */
#define FDTD_MPI_TM_UPML 4     /* MPI TM UPML     (mpiTM_UPML.c), one-rank semantics */
#define FDTD_MPI_TE_UPML 5     /* MPI TE UPML     (mpiTE_UPML.c), one-rank semantics */
#define FDTD_NS_TM_2D 6        /* serial TM non-standard FDTD (nsFdtdTM.c), FP64 only */
#define FDTD_NS_TE_2D 7        /* serial TE non-standard FDTD (nsFdtdTE.c), FP64 only */
/* The split-field and NS solvers have no NTFF (the reference's have none):
 * they run, give fields, permittivity and the elliptic ring; the NTFF,
 * spectrum, frequency and blocking calls return FDTD_E_STATE / UNSUPPORTED. */

/* Field precision of the stencil.  The NTFF accumulation is FP64 in both. */
#define FDTD_F64 0
#define FDTD_F32 1

/* Built-in permittivity models evaluated on the GPU (models.c:139-164 ids). */
#define FDTD_MODEL_NONE 0      /* noModel.c                                     */
#define FDTD_MODEL_CIRCLE 1    /* circleModel.c: {radius_nm, eps}                */
#define FDTD_MODEL_MORPHO 3    /* morphoScaleModel.c: {width_nm, thick0_nm, thick1_nm,
                                  layers, branch_nm, edge_rate, eps, per_lamella(0/1),
                                  width_0_nm, width_1_nm, ...}                   */
#define FDTD_MODEL_ZIGZAG 5    /* zigzagModel.c: {width_nm, thickness_nm, layers,
                                  degree, n (<=0: 1.56)}                          */

/* Which array: fields (TM: 0 Ez, 1 Hx, 2 Hy; TE: 0 Ex, 1 Ey, 2 Hz; the
 * split-field and NS solvers add 3, 4: TM Ezx, Ezy; TE Hzx, Hzy),
 * NTFF accumulators (TM: 0 Ux, 1 Uy, 2 Wz; TE: 0 Wx, 1 Wy, 2 Uz). */

/* Layout of copied-out fields / permittivity:
 *   FDTD_LAYOUT_GLOBAL : N_PX x N_PY cells, y contiguous (global frame)
 *   FDTD_LAYOUT_SOLVER : the reference solver's own array: (N_PX+2) x (N_PY+2)
 *                        with a zero halo for the MPI solvers
 *                        (mpiTM_UPML.c:737-741), N_PX x N_PY for the serial ones */
#define FDTD_LAYOUT_GLOBAL 0
#define FDTD_LAYOUT_SOLVER 1

typedef struct fdtd_config {
  /* field.h:20-28 FieldInfo, physical sizes in nm */
  int width_nm, height_nm, h_u_nm, pml, lambda_nm, angle_deg, step_num;
  int precision;       /* FDTD_F64 or FDTD_F32                                 */
  int flags;           /* FDTD_CFG_* bits                                      */
  /* Settings the reference hard-codes; 0 keeps the reference's value.  The
   * UPML solvers (2-5) take any; the split-field / NS solvers only 0. */
  int courant_e4;      /* Courant number x 10^4, 1..7071 (2-D Yee stability
                          needs <= 1/sqrt 2); 0: C_0_S = 0.7071 (field.h:70).
                          It sets mu0 = 1/C^2 (the H update), omega = C k, the
                          PML's sig_max, the NTFF time shifts and coefficients,
                          the pulse source and the spectrum bins             */
  int pml_order;       /* exponent M of the sigma grading, 1..8; 0: 2
                          (field.c:259-283; sig_max uses M + 1 as there)      */
  int ntff_inset;      /* cells between the PML and the NTFF path, >= 1;
                          0: 5 (field.c:136-139)                              */
  int reserved[4];     /* must be zero                                         */
} fdtd_config;

/* No time-domain NTFF state (accumulators, path tables): for CW runs whose
 * far field is fdtd_frequency of the final fields, e.g. batch sweeps with
 * thousands of instances.  NTFF mode is then 3 and fdtd_get_ntff /
 * fdtd_spectrum return FDTD_E_STATE. */
#define FDTD_CFG_NO_TIME_NTFF 1

/* Grid and NTFF geometry derived exactly as field_init() does (field.c:89-143). */
typedef struct fdtd_geometry {
  int n_px, n_py, n_pml, n_x, n_y;
  int ntff_top, ntff_bottom, ntff_left, ntff_right, ntff_cx, ntff_cy;
  double rf_per_c;
  int array_size;      /* NTFFInfo.arraySize = stepNum + 2*RFperC              */
  double lambda_s, k_s, omega_s;
} fdtd_geometry;

typedef struct fdtd_sim fdtd_sim;

/* Computes the geometry without touching the GPU. */
int fdtd_geometry_of(const fdtd_config *cfg, fdtd_geometry *out);

/* Allocates the device state (all fields zero, time 0, ray_coef 0).
 * Replaces: the solver init() bodies mpiTM_UPML.c:187-193 / mpiTE_UPML.c:283-288
 * (allocation and coefficients; permittivity comes from fdtd_set_eps or
 * fdtd_fill_eps_model). */
int fdtd_create(int solver, const fdtd_config *cfg, fdtd_sim **out);
int fdtd_destroy(fdtd_sim *sim);
int fdtd_get_geometry(const fdtd_sim *sim, fdtd_geometry *out);

/* Permittivity in the global frame, N_PX*N_PY doubles each, host pointers.
 * TM: e0 = EPS_EZ(x,y,D_XY), e1 = EPS_HX(x,y+.5,D_Y), e2 = EPS_HY(x+.5,y,D_X)
 * TE: e0 = EPS_EX(x+.5,y,D_Y), e1 = EPS_EY(x,y+.5,D_X), e2 = EPS_HZ
 * (mpiTM_UPML.c:680-682, mpiTE_UPML.c:503-505; the serial solvers use the
 * modes of fdtdTM_upml.c:237-239).  e1/e2 may be NULL for TM and e2 for TE:
 * the updates read only the E-component permittivity. */
int fdtd_set_eps(fdtd_sim *sim, const double *e0, const double *e1, const double *e2);
/* Evaluates a built-in model on the GPU at the same staggered points and
 * sub-cell modes as the solver's setCoefficient(). */
int fdtd_fill_eps_model(fdtd_sim *sim, int model, const double *params, int n_params);

/* One update() at the caller's clock (drop-in path: the caller owns time and
 * ray_coef, as simulator_calc() + field_nextStep() do, simulator.c:247-251).
 * time must lie in [0, step_num-1]: the reference's driver stops at maxTime
 * (field.c:317-319) and the flat NTFF index is only allocated up to there. */
int fdtd_update(fdtd_sim *sim, double time, double ray_coef);
/* n steps of update() followed by the engine's own field_nextStep()
 * (field.c:312-315); starts from the engine clock (fdtd_get_time). */
int fdtd_run(fdtd_sim *sim, int n_steps);
int fdtd_get_time(const fdtd_sim *sim, double *time);
int fdtd_set_time(fdtd_sim *sim, double time);
int fdtd_synchronize(fdtd_sim *sim);
/* Enqueues the deposit of every buffered NTFF step (NTFF mode 2) on the
 * engine's stream and returns without waiting: after it, work recorded on
 * that stream (a CUDA event, a copy) follows the complete time-domain NTFF of
 * every step taken so far.  The reference deposits inside each update()
 * (mpiTM_UPML.c:196-217); the engine buffers up to FDTD_OPT_NTFF_BLOCK steps
 * and deposits them together, so a timer that stops between steps calls this
 * first.  A no-op when nothing is buffered. */
int fdtd_flush(fdtd_sim *sim);

/* Copy-out.  Sizes in complex elements: GLOBAL n_px*n_py, SOLVER
 * (n_px+2)*(n_py+2) for MPI solvers, n_px*n_py for serial ones. */
int fdtd_get_field(fdtd_sim *sim, int which, int layout, double *out_complex);
int fdtd_get_eps(fdtd_sim *sim, int which, int layout, double *out);
/* NTFF accumulator: 360*array_size complex, the reference's flat indexing. */
int fdtd_get_ntff(fdtd_sim *sim, int which, double *out_complex);
/* Values the flat indexing wrote outside the 360*array_size block (each side
 * has `guard` cells; the reference writes past its allocation there). */
int fdtd_get_ntff_guard(fdtd_sim *sim, int which, double *out_complex, int *guard);

/* Far-field spectrum of ntffTM_TimeOutput / ntffTE_TimeOutput
 * (ntffTM.c:197-275, ntffTE.c:160-238): E_theta (TM) or E_phi (TE) from the
 * NTFF accumulators, zero-padded 8192-point FFT per angle, |E|^2 at every nm
 * from 380 to 700.  out: double[321][360], the layout ntff_outputEnormBin
 * writes (ntff.c:20-33).  step_num > 8192 returns FDTD_E_UNSUPPORTED (the
 * reference's FFT buffer overflows there, ntffTM.c:214-221). */
int fdtd_spectrum(fdtd_sim *sim, double *out);
/* Frequency-domain NTFF of the current fields, ntffTM_Frequency
 * (ntffTM.c:72-158: E_z far field) or ntffTE_Frequency (ntffTE.c:242-338:
 * E_phi), R0 = 1e6 * 500 nm in cells; out: 360 complex.  For TE all four
 * sides of the path use the global index (the shipped function reads three of
 * them through field_subIndex, whose sub-domain record field_init no longer
 * fills, field.c:112).  Angle a is the direction a + 180 degrees of the
 * e^{-i w t} convention (the transform's kernel is e^{+i k r.r'}). */
int fdtd_frequency(fdtd_sim *sim, double *out_complex);
/* field_outputElliptic (field.c:322-343): |field|^2, bilinear as cbilinear
 * (myComplex.c:40-52), on the circle of radius 1.2 lambda_s about the grid
 * centre at ang = 180 .. 0 degrees; out[q] (181 doubles) is printed line
 * q = 180 - ang.  which: fdtd_get_field numbering (the reference calls it on
 * Ez for TM, Ey for TE).  A ring that leaves the grid is FDTD_E_ARG. */
int fdtd_elliptic(fdtd_sim *sim, int which, double *out181);
/* The same ring written as field_outputElliptic's text file ("%d %lf \n"). */
int fdtd_write_elliptic(fdtd_sim *sim, int which, const char *path);
/* drawer_outputImage (drawer.c:253-298): 24-bit BMP of permittivity `which`
 * in the global frame (the reference draws getEps(): EPS_EZ for TM, EPS_EY
 * for TE), (N_PX rounded down to a multiple of 4) x N_PY pixels, colour
 * modelColorTransform (drawer.c:230-251), header as putBmpHeader. */
int fdtd_write_model_image(fdtd_sim *sim, int which, const char *path);

/* Running-DFT NTFF (no counterpart in the reference): accumulates, from the
 * time-blocked NTFF ring (mode 2), sum_t v(t) e^{i w t} of every path sample at
 * the two 8192-point FFT bins around each wavelength, and at the end forms
 * the far field of ntff*_TimeOutput at those bins without the 360 x arraySize
 * accumulators or the FFT.  Call before the first step.  The time-domain
 * spectrum transforms only the first step_num bins of each angle's series
 * (ntffTM.c:214-221); the DFT sums every deposit, so the two agree once the
 * pulse has left the NTFF box.
 * fdtd_dft_far_field: out[360][2*nlam] complex (lower, upper bin per wavelength).
 * fdtd_dft_spectrum: out[nlam][360], |E|^2 interpolated as the spectrum is. */
int fdtd_dft_enable(fdtd_sim *sim, int nlam, const int *lambda_nm);
int fdtd_dft_far_field(fdtd_sim *sim, double *out_complex);
int fdtd_dft_spectrum(fdtd_sim *sim, double *out);

/* reset() of the solvers (mpiTM_UPML.c:219-232): zero every field; the
 * serial solvers also zero the NTFF arrays (fdtdTM_upml.c:110-113). The
 * engine clock returns to 0. */
int fdtd_reset(fdtd_sim *sim);

/* The CUDA stream (cudaStream_t) every launch of this simulation is issued on. */
int fdtd_get_stream(fdtd_sim *sim, void **stream);

/* Device pointers of the state for zero-copy consumers (pitch in elements). */
int fdtd_device_field(fdtd_sim *sim, int which, void **dptr, int *pitch, int *rows);

/* Device status word: bit 0 = an NTFF deposit fell outside the accumulator
 * and was dropped (cannot happen within [0, step_num) on valid geometry);
 * bit 2 = fdtd_check_finite found a non-finite field value. */
#define FDTD_STATUS_NTFF_RANGE 1u
#define FDTD_STATUS_NONFINITE 4u
int fdtd_get_status(fdtd_sim *sim, unsigned int *flags);

/* Failure detection (the reference has none; a blown-up run only shows as
 * NaN in its output files): counts the field values (every slot of the
 * solver, PML auxiliaries included) with a non-finite real or imaginary part,
 * on the device, and sets FDTD_STATUS_NONFINITE when there are any.  Nothing
 * traps: the simulation stays usable. */
int fdtd_check_finite(fdtd_sim *sim, long long *count);

/* Checkpoint / resume (the reference has none: its reset only zeroes the
 * fields, mpiTM_UPML.c:219-232).  An image holds the whole time-stepping
 * state: the permittivity as given, every field slot, the time-domain NTFF
 * accumulators, the running-DFT sums, the clock and the tuning options; the
 * buffered NTFF steps are deposited first.  It loads into a simulation created
 * with the same solver and fdtd_config (FDTD_E_ARG otherwise; a simulation
 * without a running DFT takes the image's wavelengths), after which runs
 * continue as the saved simulation's would have: the fields and the DFT sums
 * bit for bit, the NTFF accumulators to rounding (their deposit adds with
 * FP64 atomics in no fixed order, as in any two runs).
 *   fdtd_checkpoint_size   bytes of the image
 *   fdtd_checkpoint_save   image into a host buffer of exactly that size
 *   fdtd_checkpoint_load   image from a host buffer
 *   fdtd_checkpoint_write  image into a file (64 MiB pinned staging chunks)
 *   fdtd_checkpoint_read   image from a file */
int fdtd_checkpoint_size(fdtd_sim *sim, size_t *bytes);
int fdtd_checkpoint_save(fdtd_sim *sim, void *buf, size_t bytes);
int fdtd_checkpoint_load(fdtd_sim *sim, const void *buf, size_t bytes);
int fdtd_checkpoint_write(fdtd_sim *sim, const char *path);
int fdtd_checkpoint_read(fdtd_sim *sim, const char *path);

/* Tuning knobs (results are the same up to summation order).
 * NTFF deposit modes: 0 direct (three atomic adds per tap set every step),
 * 1 shared-memory window per side chunk, 2 time-blocked (default): the path
 * samples of FDTD_OPT_NTFF_BLOCK consecutive steps are buffered and each
 * (angle, cell) pair deposits them in one pass.  Buffered steps are deposited
 * before any NTFF read-out, fdtd_synchronize, fdtd_reset or option change.
 * Mode 3 skips the time-domain NTFF (the accumulators stay as they are): for
 * CW runs whose far field comes from fdtd_frequency at the end. */
#define FDTD_OPT_NTFF_MODE 1     /* 0, 1, 2 or 3 (default 2)                           */
#define FDTD_OPT_NTFF_CHUNK 2    /* mode 1: cells of a side per block (64..4096, 1024)  */
#define FDTD_OPT_NTFF_BLOCK 3    /* mode 2: steps per deposit (1..64, default 32)       */
#define FDTD_OPT_ROWS 4          /* stencil rows per thread: 1 (default), 2, 4 or 8     */
/* Temporal blocking (UPML solvers, NTFF mode 2 or 3): fdtd_run advances K
 * steps per pass over the fields in HBM (K = 1, 2, 4, and 8 in FP32 for the
 * MPI solvers; 0 = off, the default) in tiles of 32-2K columns x
 * FDTD_OPT_TBLOCK_ROWS rows (0 = automatic).  The serial solvers (TM_UPML,
 * TE_UPML) block their own order, H half-step then E with the pulse
 * (fdtdTM_upml.c:54-66, fdtdTE_upml.c:168-192).  It
 * holds a second set of fields on the device, and the fields move between the
 * two sets, so a pointer from fdtd_device_field is valid until the next
 * fdtd_run or fdtd_update.  fdtd_update (one step per call) never blocks. */
#define FDTD_OPT_TBLOCK 5
#define FDTD_OPT_TBLOCK_ROWS 6
#define FDTD_OPT_TBLOCK_COLS 7   /* columns per lane of a tile: 1 (default), 2 (FP32, K = 2 or 4) */
/* Broadband batch: steps between the running DFT's samples (rounded up to a
 * multiple of the blocking depth K; default 16).  The pulse's spectrum lies
 * far below the Nyquist frequency pi / stride of the sampled series for
 * strides up to a few tens of steps on 5 nm cells, so the far field does not
 * depend on it beyond rounding; fewer samples cost less FP64 work. */
#define FDTD_OPT_DFT_STRIDE 8
int fdtd_set_option(fdtd_sim *sim, int key, int value);
int fdtd_get_option(fdtd_sim *sim, int key, int *value);

/* Autotuner of the temporal blocking (UPML solvers): times the one-step kernels and the
 * blocked kernel at each depth K and tile height on this simulation's own
 * grid and fields (into the spare field set: the state does not change),
 * sets FDTD_OPT_TBLOCK / _ROWS / _COLS to the fastest, returns K and rows
 * with its stencil time per step in ms (*k_out = 0: one-step kernels won). */
int fdtd_autotune(fdtd_sim *sim, int *k_out, int *rows_out, double *ms_per_step_out);
/* The candidates the last fdtd_autotune timed: up to cap quadruples
 * (K, rows, columns per lane, ms per step) into out, K = 0 being the one-step
 * kernels; returns the number of candidates (negative status on error). */
int fdtd_autotune_report(const fdtd_sim *sim, double *out, int cap);

/* Per-kernel timing with CUDA events recorded on the engine's own stream
 * around every launch class while enabled.  ms_out[4] receives the summed
 * milliseconds of: 0 E half-step, 1 H half-step, 2 NTFF gather, 3 NTFF deposit;
 * *steps the number of steps timed.  Reading synchronizes and clears. */
int fdtd_profile_enable(fdtd_sim *sim, int on);
int fdtd_profile_read(fdtd_sim *sim, double *ms_out, long long *steps);

/* ---- Batched sweeps (no counterpart in the reference; it runs one process
 * per structure, main.c:114-138) ---------------------------------------------
 * n independent instances of one MPI solver, each with its own fdtd_config
 * (grid, wavelength, step_num; one precision for all), advanced together on
 * one GPU: a packed work-list of the temporally blocked tiles of every
 * instance, stepped by persistent kernels captured in one CUDA graph per
 * K-step block.  Each instance is an fdtd_sim handle owned by the batch
 * (fdtd_batch_instance): fill its permittivity and read its fields and
 * fdtd_frequency far field with the single-simulation calls.
 * fdtd_batch_run advances every instance from time 0 to its own step_num;
 * the batch does no time-domain NTFF (the instances' accumulators stay zero).
 * Options: FDTD_OPT_TBLOCK (K = 1, 2, 4 (default), 8 for FP32) and
 * FDTD_OPT_TBLOCK_ROWS (0 = per-instance automatic). */
typedef struct fdtd_batch fdtd_batch;
int fdtd_batch_create(int solver, const fdtd_config *cfgs, int n, fdtd_batch **out);
int fdtd_batch_destroy(fdtd_batch *batch);
int fdtd_batch_size(const fdtd_batch *batch);
int fdtd_batch_instance(fdtd_batch *batch, int index, fdtd_sim **sim);
int fdtd_batch_set_option(fdtd_batch *batch, int key, int value);
int fdtd_batch_run(fdtd_batch *batch);
int fdtd_batch_reset(fdtd_batch *batch);
long long fdtd_batch_launch_count(const fdtd_batch *batch);

/* Broadband batch: the far field of every instance at many wavelengths from
 * one run.  The reference's broadband run is a serial solver driven by
 * field_scatteredPulse (field.c:224-256) whose ntffTM_TimeOutput spectrum
 * (ntffTM.c:197-275) covers 380..700 nm; here every instance of an
 * MPI_TM_UPML batch at 0 degrees gets that Gaussian pulse (carrier: its own
 * lambda_nm) instead of the CW wave, and the NTFF path samples of every step
 * feed a running DFT at the nlam given wavelengths (exact frequencies
 * w = C 2 pi h_u / lambda).  The instances must be created with the
 * time-domain NTFF state (no FDTD_CFG_NO_TIME_NTFF), one cell size and
 * Courant number for all; call before fdtd_batch_run.
 * fdtd_batch_broadband_spectrum: out[nlam][360] = |X(w)|^2 / |A(w)|^2 of
 * instance `index` after its run, X the far-field component the spectrum
 * transforms (E_theta, ntffTM.c:161-194) at w from the DFT sums, A the DFT of
 * the incident pulse at x = 0 over the same steps: the far-field intensity of
 * the structure's response to a unit incident plane wave at each wavelength,
 * which the CW run approaches at its steady state.  step_num must let the
 * pulse and the structure's ringing leave the grid. */
int fdtd_batch_broadband(fdtd_batch *batch, int nlam, const int *lambda_nm);
int fdtd_batch_broadband_spectrum(fdtd_batch *batch, int index, double *out);
/* The same for every instance: out[n][nlam][360]. */
int fdtd_batch_broadband_spectra(fdtd_batch *batch, double *out);

/* Number of kernel launches the engine issued since creation. */
long long fdtd_launch_count(const fdtd_sim *sim);

/* ---- Allocation-free NTFF step (no counterpart in the reference) ---------
 * For callers that may not allocate device memory, directly or through this
 * library: a host application whose memory manager owns every device buffer
 * of the process, or a loop that must not pay the device-wide
 * synchronisation cudaMalloc/cudaFree imply.  Such a caller keeps the fields
 * and the NTFF accumulators in its own device buffers and calls this once per
 * update(): it adds that step's 360-angle time-domain NTFF contribution of an
 * MPI UPML solver (mpiTM_UPML.c:849-1037, mpiTE_UPML.c:611-794), the same
 * arithmetic as the engine's own NTFF kernels.
 *
 * No cudaMalloc, cudaFree or allocating library call is made.  The path
 * samples are staged in one file-scope __device__ array sized for
 * FDTD_NOALLOC_MAX_PATH path cells (2 MB, held by every GPU that loads the
 * library until the process exits); a larger path is rejected with
 * FDTD_E_ARG.  The first call on a device looks the array up and uploads the
 * 360 direction cosines, so make that first call before any stream capture.
 * The set-up belongs to the device's CUDA context: after a cudaDeviceReset
 * the next call finds a new context and sets up again (it asks the driver
 * for the context's id, cuCtxGetId; a driver without it keeps the first
 * set-up, and calls after a reset then fail or use stale tables).
 * Every call reuses the same array (each call writes the 2 x path entries it
 * reads before reading them), so calls that overlap on the GPU -- on
 * different streams, or from several host threads -- race; order them on
 * one stream.  A tap whose flat index falls outside the block and its guard
 * cells is skipped without an error: with time in [0, step_num-1] and
 * accumulators sized as below none does, so a skip means the accumulators
 * do not match cfg.
 *
 * args->e0/e1/h0/h1: device FP64 complex fields in the one-rank layout of the
 *   MPI solvers: row i, column j at (i*pitch + j), i in [0, N_PX+2), global
 *   x = i-1 (TM: e0 Ez, h0 Hx, h1 Hy; TE: e0 Ex, e1 Ey, h0 Hz).
 * args->acc[3]: device accumulators (TM Ux, Uy, Wz; TE Wx, Wy, Uz), each
 *   pointing at element 0 of its flat 360*array_size complex block and owning
 *   FDTD_NTFF_GUARD complex elements before and after it (the flat index of
 *   the reference reaches past the block at corner angles).
 * args->time: the clock of the update() these fields come from, in
 *   [0, step_num-1].  stream: cudaStream_t to launch on (NULL: default). */
#define FDTD_NOALLOC_MAX_PATH 65536
#define FDTD_NTFF_GUARD 16
typedef struct fdtd_ntff_step_args {
  int solver;                /* FDTD_MPI_TM_UPML or FDTD_MPI_TE_UPML           */
  fdtd_config cfg;           /* the grid, as for fdtd_create                    */
  const void *e0, *e1, *h0, *h1;
  int pitch;                 /* complex elements per row, >= N_PY + 2           */
  double time;
  void *acc[3];
} fdtd_ntff_step_args;
int fdtd_ntff_step_noalloc(const fdtd_ntff_step_args *args, void *stream);

const char *fdtd_last_error(void);
const char *fdtd_version(void);

#ifdef __cplusplus
}
#endif
#endif
