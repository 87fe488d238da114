/*
 * fdtd_oracle.h -- CPU restatement of rennone/mpiFDTD's UPML time-stepping
 * path.  TEST INFRASTRUCTURE: only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py may load it, and only as the reference the
 * results are compared with or as the timed CPU baseline.  The product (mpifdtd_gb300) never links or calls it.
 *
 * Parity pin: the restatement is checked against golden vectors produced by
 * the reference's own C sources compiled unmodified (oracle/ref.mk ->
 * oracle/_ref/libfdtdref.so, vectors in tests/golden/).
 */
#ifndef FDTD_ORACLE_H
#define FDTD_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* Solver selection, numbered like enum SOLVER in simulator.h:8-18 (0, 1, 6, 7:
 * the split-field PML and NS-FDTD solvers, no NTFF). */
enum { OF_TM_2D = 0, OF_TE_2D = 1, OF_TM_UPML = 2, OF_TE_UPML = 3, OF_MPI_TM_UPML = 4, OF_MPI_TE_UPML = 5,
       OF_NS_TM_2D = 6, OF_NS_TE_2D = 7 };

/* Models: the reference's noModel.c / circleModel.c / morphoScaleModel.c /
 * zigzagModel.c, plus
 * a seeded "discs" map used to make golden vectors with permittivity inside the
 * PML and several materials (it goes through the reference's models_eps
 * callback path, models.c:132-150, via the harness). */
enum { OF_MODEL_NONE = 0, OF_MODEL_CIRCLE = 1, OF_MODEL_MORPHO = 2, OF_MODEL_DISCS = 3, OF_MODEL_ZIGZAG = 4 };

typedef struct of_field_info {      /* field.h:20-28 FieldInfo */
  int width_nm, height_nm, h_u_nm, pml, lambda_nm, angle_deg, step_num;
  /* Settings the reference hard-codes, 0 = the reference's value (UPML
   * solvers only; the split-field / NS solvers refuse others):
   * courant: C_0_S = 0.7071 (field.h:70), which also sets MU_0_S = 1/C^2 and
   * Z_0_S = 1/C (field.h:74-75); pml_order: the sigma grading exponent M = 2
   * (field.c:259-283); ntff_inset: NTFF path 5 cells inside the PML
   * (field.c:136-139). */
  double courant;
  int pml_order, ntff_inset;
} of_field_info;

/* circle: p = {radius_nm, eps (<=0: N=1.6 default)}
 * morpho: p = {width_nm, thick0_nm, thick1_nm, layers, branch_nm, edge_rate, eps (<=0: 1.56^2)}
 * discs : p = {n, cx0, cy0, r0, eps0, cx1, ...} in cell units, n <= 8
 * zigzag: p = {width_nm, thickness_nm, layers, degree, n (<=0: N_0 = 1.56)}     */
typedef struct of_model { int kind; double p[40]; } of_model;

typedef struct of_sim of_sim;

of_sim *of_create(int solver, const of_field_info *fi, const of_model *m);
void    of_destroy(of_sim *s);
void    of_step(of_sim *s, int n);                 /* update() + field_nextStep(), n times */
double  of_time(const of_sim *s);
/* array layout: MPI solvers (N_PX+2) x (N_PY+2) with one halo cell per side,
 * serial solvers N_PX x N_PY; index i*ny + j (y contiguous). */
void    of_dims(const of_sim *s, int *nx, int *ny, int *n_px, int *n_py);
double *of_field(of_sim *s, int which);            /* complex interleaved; TM: 0 Ez 1 Hx 2 Hy, TE: 0 Ex 1 Ey 2 Hz */
double *of_eps(of_sim *s, int which);              /* TM: 0 EZ 1 HX 2 HY; TE: 0 EX 1 EY 2 HZ */
int     of_ntff_info(const of_sim *s, int *top, int *bottom, int *left, int *right, int *cx, int *cy, double *rf);
int     of_array_size(const of_sim *s);            /* NTFFInfo.arraySize */
int     of_ntff_guard(void);                       /* guard cells before/after the flat 360*arraySize block */
/* flat NTFF accumulator incl. guards: length 360*arraySize + 2*guard complex.
 * TM: 0 Ux 1 Uy 2 Wz ; TE: 0 Wx 1 Wy 2 Uz */
double *of_ntff(of_sim *s, int which);
/* Spectrum of ntffTM/TE_TimeOutput: out[321*360] = |E|^2 per nm 380..700 x angle.
 * Returns -1 if step_num > 8192 (the reference overflows its FFT buffer there). */
int     of_time_output(of_sim *s, double *out);
/* Frequency-domain NTFF (ntffTM_Frequency) of the current fields: out[360] complex */
int     of_frequency(of_sim *s, double *out);
/* Times n_threads independent simulations of `steps` steps each (task
 * parallel, as main.c:114-138 uses ranks); returns wall seconds of the
 * stepping phase only (setup excluded). */
double  of_bench(int solver, const of_field_info *fi, const of_model *m, int steps, int n_threads);
double  of_bench_opts(int solver, const of_field_info *fi, const of_model *m, int steps, int n_threads,
                      int flags);

#ifdef __cplusplus
}
#endif
#endif
