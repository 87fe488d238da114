/*
 * mpifdtd_upml.h -- the reference's UPML solver entry points, served by the
 * GB300 engine (libmpifdtd_upml.so on top of libmpifdtd_gb300.so).
 *
 * Drop-in for the eight solver translation units of rennone/mpiFDTD that
 * simulator.c binds (simulator.c:32-205): link libmpifdtd_upml.so instead of
 * mpiTM_UPML.c, mpiTE_UPML.c, fdtdTM_upml.c, fdtdTE_upml.c, fdtdTM.c,
 * fdtdTE.c, nsFdtdTM.c and nsFdtdTE.c; simulator.c,
 * field.c, models.c and the models stay as they are.  The library calls back
 * into the host program's field_getFieldInfo(), field_getTime(),
 * field_getRayCoef(), field_getWaveAngle() and models_eps() exactly where the
 * reference solvers read them, so the host keeps owning time (field_nextStep
 * after update(), simulator.c:247-251) and the permittivity callback.
 *
 * Semantics per entry point:
 *   init()   allocates the device state, fills the permittivity through
 *            models_eps() at the solver's staggered points and modes
 *   update() one time step on the GPU at field_getTime()/field_getRayCoef()
 *   reset()  zeroes the fields (serial UPML solvers first write the far-field
 *            spectrum files, as ntffTM_TimeOutput does; split-field / NS ones
 *            the field_outputElliptic ring file)
 *   finish() releases everything (serial solvers write the spectrum first)
 *   get*()   borrowed host pointers in the reference solver's own layout,
 *            refreshed from the device on each call after an update()
 * Differences from the reference: finish() of the MPI solvers does not run
 * ntff*_FrequencySplit or MPI_Finalize (fdtd_frequency gives the frequency
 * far field); update() at a time outside [0, stepNum-1] is refused, since the
 * reference's flat NTFF index leaves its allocation there; errors print and
 * exit(2) as the reference does, or, after mpifdtd_upml_set_error_mode(1),
 * are stored for mpifdtd_upml_last_status() instead.
 * This header is C only (double complex), like the reference's headers.
 */
#ifndef MPIFDTD_UPML_H
#define MPIFDTD_UPML_H
#include <complex.h>

/* mpiTM_UPML.h:5-18 */
extern void (*mpi_fdtdTM_upml_getUpdate(void))(void);
extern void (*mpi_fdtdTM_upml_getFinish(void))(void);
extern void (*mpi_fdtdTM_upml_getReset(void))(void);
extern void (*mpi_fdtdTM_upml_getInit(void))(void);
extern double complex *mpi_fdtdTM_upml_getHx(void);
extern double complex *mpi_fdtdTM_upml_getHy(void);
extern double complex *mpi_fdtdTM_upml_getEz(void);
extern double *mpi_fdtdTM_upml_getEps(void);
extern int mpi_fdtdTM_upml_getSubNx(void);
extern int mpi_fdtdTM_upml_getSubNy(void);
extern int mpi_fdtdTM_upml_getSubNpx(void);
extern int mpi_fdtdTM_upml_getSubNpy(void);
extern int mpi_fdtdTM_upml_getSubNcell(void);

/* mpiTE_UPML.h:5-19 */
extern void (*mpi_fdtdTE_upml_getUpdate(void))(void);
extern void (*mpi_fdtdTE_upml_getFinish(void))(void);
extern void (*mpi_fdtdTE_upml_getReset(void))(void);
extern void (*mpi_fdtdTE_upml_getInit(void))(void);
extern double complex *mpi_fdtdTE_upml_getEx(void);
extern double complex *mpi_fdtdTE_upml_getEy(void);
extern double complex *mpi_fdtdTE_upml_getHz(void);
extern int mpi_fdtdTE_upml_getSubNx(void);
extern int mpi_fdtdTE_upml_getSubNy(void);
extern int mpi_fdtdTE_upml_getSubNpx(void);
extern int mpi_fdtdTE_upml_getSubNpy(void);
extern int mpi_fdtdTE_upml_getSubNcell(void);
extern double *mpi_fdtdTE_upml_getEps(void);

/* fdtdTM_upml.h:5-14 */
extern void (*fdtdTM_upml_getUpdate(void))(void);
extern void (*fdtdTM_upml_getFinish(void))(void);
extern void (*fdtdTM_upml_getReset(void))(void);
extern void (*fdtdTM_upml_getInit(void))(void);
extern double complex *fdtdTM_upml_getHx(void);
extern double complex *fdtdTM_upml_getHy(void);
extern double complex *fdtdTM_upml_getEz(void);
extern double *fdtdTM_upml_getEps(void);

/* fdtdTE_upml.h:5-14 */
extern void (*fdtdTE_upml_getUpdate(void))(void);
extern void (*fdtdTE_upml_getFinish(void))(void);
extern void (*fdtdTE_upml_getInit(void))(void);
extern void (*fdtdTE_upml_getReset(void))(void);
extern double complex *fdtdTE_upml_getEx(void);
extern double complex *fdtdTE_upml_getEy(void);
extern double complex *fdtdTE_upml_getHz(void);
extern double *fdtdTE_upml_getEps(void);

/* fdtdTM.h (split-field PML TM) */
extern void (*fdtdTM_getUpdate(void))(void);
extern void (*fdtdTM_getFinish(void))(void);
extern void (*fdtdTM_getReset(void))(void);
extern void (*fdtdTM_getInit(void))(void);
extern double complex *fdtdTM_getEzx(void);
extern double complex *fdtdTM_getEzy(void);
extern double complex *fdtdTM_getEz(void);
extern double complex *fdtdTM_getHy(void);
extern double complex *fdtdTM_getHx(void);
extern double *fdtdTM_getEps(void);

/* fdtdTE.h (split-field PML TE) */
extern void (*fdtdTE_getUpdate(void))(void);
extern void (*fdtdTE_getFinish(void))(void);
extern void (*fdtdTE_getReset(void))(void);
extern void (*fdtdTE_getInit(void))(void);
extern double complex *fdtdTE_getEx(void);
extern double complex *fdtdTE_getEy(void);
extern double complex *fdtdTE_getHzx(void);
extern double complex *fdtdTE_getHzy(void);
extern double complex *fdtdTE_getHz(void);
extern double *fdtdTE_getEps(void);

/* nsFdtdTM.h (non-standard FDTD TM); getEpsX/Y/Z are public in nsFdtdTM.c:33-35.
 * nsFdtdTM_getSolver (a Solver record whose fields the reference leaves unset)
 * is not provided. */
extern void (*nsFdtdTM_getUpdate(void))(void);
extern void (*nsFdtdTM_getFinish(void))(void);
extern void (*nsFdtdTM_getReset(void))(void);
extern void (*nsFdtdTM_getInit(void))(void);
extern double complex *nsFdtdTM_getEzx(void);
extern double complex *nsFdtdTM_getEzy(void);
extern double complex *nsFdtdTM_getEz(void);
extern double complex *nsFdtdTM_getHy(void);
extern double complex *nsFdtdTM_getHx(void);
extern double *nsFdtdTM_getEps(void);
extern double *nsFdtdTM_getEpsX(void);
extern double *nsFdtdTM_getEpsY(void);
extern double *nsFdtdTM_getEpsZ(void);

/* nsFdtdTE.h (non-standard FDTD TE); getEpsX/Y/Z are public in nsFdtdTE.c:33-35.
 * nsFdtdTE_getSolver is not provided (as for TM). */
extern void (*nsFdtdTE_getUpdate(void))(void);
extern void (*nsFdtdTE_getFinish(void))(void);
extern void (*nsFdtdTE_getReset(void))(void);
extern void (*nsFdtdTE_getInit(void))(void);
extern double complex *nsFdtdTE_getHzx(void);
extern double complex *nsFdtdTE_getHzy(void);
extern double complex *nsFdtdTE_getHz(void);
extern double complex *nsFdtdTE_getEy(void);
extern double complex *nsFdtdTE_getEx(void);
extern double *nsFdtdTE_getEps(void);
extern double *nsFdtdTE_getEpsX(void);
extern double *nsFdtdTE_getEpsY(void);
extern double *nsFdtdTE_getEpsZ(void);

/* Extensions (no counterpart in the reference).
 * The reference reports errors with printf + exit(2) (function.c:27-32,
 * simulator.c:234-237); the drop-in does the same by default.  Mode 1 makes
 * the void entry points return instead and keeps the status for
 * mpifdtd_upml_last_status() (FDTD_OK or an FDTD_E_* code). */
extern void mpifdtd_upml_set_error_mode(int return_instead_of_exit);
extern int mpifdtd_upml_last_status(void);
/* The engine simulation behind a solver (enum SOLVER value 0..7), or
 * NULL before init(): lets a host use the extended C ABI of mpifdtd_gb300.h. */
struct fdtd_sim;
extern struct fdtd_sim *mpifdtd_upml_engine(int solver);

#endif
