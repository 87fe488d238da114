/*
 * compat_upml.c -- the reference's UPML solver entry points (include/mpifdtd_upml.h)
 * on top of the GB300 engine (include/mpifdtd_gb300.h).
 *
 * Each of the eight solvers of the reference (mpiTM_UPML.c, mpiTE_UPML.c,
 * fdtdTM_upml.c, fdtdTE_upml.c, and the split-field / NS ones fdtdTM.c,
 * fdtdTE.c, nsFdtdTM.c, nsFdtdTE.c) keeps its state in file statics and is
 * driven through function pointers by simulator.c; here each is one slot
 * holding an engine simulation plus host mirrors of what the getters return.
 *
 * Calls back into the host program (symbols of field.c / models.c):
 *   field_getFieldInfo()  grid of init()            (field.h:138)
 *   field_getTime(), field_getRayCoef()  clock of update()  (field.c:46,50)
 *   field_getWaveAngle()  file names of the spectrum  (ntffTM.c:240-245)
 *   models_eps()          permittivity of init()   (models.c:166-184)
 */
#define _GNU_SOURCE
#include <complex.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "mpifdtd_gb300.h"
#include "mpifdtd_upml.h"

/* field.h:20-28 (same layout) and the host-program functions used here */
typedef struct FieldInfo {
  int width_nm, height_nm, h_u_nm, pml, lambda_nm, angle_deg, stepNum;
} FieldInfo;
extern FieldInfo field_getFieldInfo(void);
extern double field_getTime(void);
extern double field_getRayCoef(void);
extern double field_getWaveAngle(void);
extern double models_eps(double x, double y, int mode);  /* enum MODE: D_X 0, D_Y 1, D_XY 2 (models.h:16-21) */

enum { MODE_DX = 0, MODE_DY = 1, MODE_DXY = 2 };
enum { SLOT_SER_TM = 0, SLOT_SER_TE = 1, SLOT_MPI_TM = 2, SLOT_MPI_TE = 3,
       SLOT_SPLIT_TM = 4, SLOT_SPLIT_TE = 5, SLOT_NS_TM = 6, SLOT_NS_TE = 7, NSLOT = 8 };

typedef struct slot {
  int solver;
  fdtd_sim *sim;
  int n_px, n_py, nx, ny;        /* nx x ny: the reference solver's array (MPI: +2 halo) */
  double complex *field[5];      /* getter mirrors in the solver layout (3, 4: split parts) */
  double *eps;                   /* getEps mirror in the solver layout */
  double *eps_all[3];            /* nsFdtd*_getEpsX/Y/Z mirrors (NS solvers) */
  int fresh[5];
} slot;

static slot g_slot[NSLOT] = {{FDTD_TM_UPML}, {FDTD_TE_UPML}, {FDTD_MPI_TM_UPML}, {FDTD_MPI_TE_UPML},
                             {FDTD_TM_2D}, {FDTD_TE_2D}, {FDTD_NS_TM_2D}, {FDTD_NS_TE_2D}};

static int is_split(int solver)
{
  return solver == FDTD_TM_2D || solver == FDTD_TE_2D || solver == FDTD_NS_TM_2D || solver == FDTD_NS_TE_2D;
}
static int g_return_mode = 0;
static int g_status = FDTD_OK;

void mpifdtd_upml_set_error_mode(int m) { g_return_mode = m != 0; }
int mpifdtd_upml_last_status(void) { return g_status; }

struct fdtd_sim *mpifdtd_upml_engine(int solver)
{
  for (int q = 0; q < NSLOT; q++)
    if (g_slot[q].solver == solver) return g_slot[q].sim;
  return NULL;
}

/* the reference prints and exits on errors (function.c:27-32) */
static int check(int rc, const char *where)
{
  g_status = rc;
  if (rc == FDTD_OK) return 0;
  printf("mpifdtd_gb300: %s: %s\n", where, fdtd_last_error());
  if (!g_return_mode) exit(2);
  return 1;
}

static void release(slot *s)
{
  if (s->sim) fdtd_destroy(s->sim);
  s->sim = NULL;
  for (int q = 0; q < 5; q++) { free(s->field[q]); s->field[q] = NULL; }
  free(s->eps);
  s->eps = NULL;
  for (int q = 0; q < 3; q++) { free(s->eps_all[q]); s->eps_all[q] = NULL; }
}

/* setCoefficient()'s permittivity: mpiTM_UPML.c:680-682, mpiTE_UPML.c:503-505,
 * fdtdTM_upml.c:237-239, fdtdTE_upml.c:374-376, fdtdTM.c:209-211,
 * fdtdTE.c:210-212, nsFdtdTM.c:244-246, nsFdtdTE.c:119-121 (inner cells only),
 * on the global frame. */
static void fill_eps(const slot *s, double *e0, double *e1, double *e2)
{
  const int tm = s->solver == FDTD_TM_UPML || s->solver == FDTD_MPI_TM_UPML || s->solver == FDTD_TM_2D ||
                 s->solver == FDTD_NS_TM_2D;
  const int alt = s->solver != FDTD_TM_UPML;  /* TM: HX at D_Y, HY at D_X */
  const int ns_te = s->solver == FDTD_NS_TE_2D;
  for (int x = 0; x < s->n_px; x++)
    for (int y = 0; y < s->n_py; y++) {
      const size_t k = (size_t)x * s->n_py + y;
      if (tm) {
        e0[k] = models_eps(x, y, MODE_DXY);
        e1[k] = models_eps(x, y + 0.5, alt ? MODE_DY : MODE_DXY);
        e2[k] = models_eps(x + 0.5, y, alt ? MODE_DX : MODE_DXY);
      } else if (ns_te) {
        const int inner = x > 0 && y > 0 && x < s->n_px - 1 && y < s->n_py - 1;
        e0[k] = inner ? models_eps(x + 0.5, y, MODE_DY) : 0.0;
        e1[k] = inner ? models_eps(x, y + 0.5, MODE_DX) : 0.0;
        e2[k] = inner ? models_eps(x + 0.5, y + 0.5, MODE_DXY) : 0.0;
      } else {
        e0[k] = models_eps(x + 0.5, y, MODE_DY);
        e1[k] = models_eps(x, y + 0.5, MODE_DX);
        e2[k] = 0.5 * (models_eps(x + 0.5, y + 0.5, MODE_DX) + models_eps(x + 0.5, y + 0.5, MODE_DY));
      }
    }
}

static void slot_init(slot *s)
{
  release(s);
  const FieldInfo fi = field_getFieldInfo();
  fdtd_config cfg;
  memset(&cfg, 0, sizeof cfg);
  cfg.width_nm = fi.width_nm;
  cfg.height_nm = fi.height_nm;
  cfg.h_u_nm = fi.h_u_nm;
  cfg.pml = fi.pml;
  cfg.lambda_nm = fi.lambda_nm;
  cfg.angle_deg = fi.angle_deg;
  cfg.step_num = fi.stepNum;
  const char *prec = getenv("MPIFDTD_PRECISION");
  cfg.precision = (prec && !strcmp(prec, "f32")) ? FDTD_F32 : FDTD_F64;
  if (check(fdtd_create(s->solver, &cfg, &s->sim), "init")) return;
  fdtd_geometry g;
  fdtd_get_geometry(s->sim, &g);
  s->n_px = g.n_px;
  s->n_py = g.n_py;
  const int mpi = s->solver == FDTD_MPI_TM_UPML || s->solver == FDTD_MPI_TE_UPML;
  s->nx = mpi ? g.n_px + 2 : g.n_px;
  s->ny = mpi ? g.n_py + 2 : g.n_py;
  const size_t n = (size_t)g.n_px * g.n_py;
  double *e[3];
  for (int q = 0; q < 3; q++) e[q] = (double *)malloc(sizeof(double) * n);
  fill_eps(s, e[0], e[1], e[2]);
  int rc = fdtd_set_eps(s->sim, e[0], e[1], e[2]);
  for (int q = 0; q < 3; q++) free(e[q]);
  if (check(rc, "init (permittivity)")) return;
  const size_t na = (size_t)s->nx * s->ny;
  const int nf = is_split(s->solver) ? 5 : 3;
  for (int q = 0; q < nf; q++) s->field[q] = (double complex *)calloc(na, sizeof(double complex));
  s->eps = (double *)calloc(na, sizeof(double));
  /* getEps: EPS_EZ (TM), EPS_EY (MPI TE mpiTE_UPML.c:104-106, split TE fdtdTE.c:71-74,
   * NS TE nsFdtdTE.c:36), EPS_EX (serial UPML TE, fdtdTE_upml.c:93-96) */
  const int te_ey = s->solver == FDTD_MPI_TE_UPML || s->solver == FDTD_TE_2D || s->solver == FDTD_NS_TE_2D;
  check(fdtd_get_eps(s->sim, te_ey ? 1 : 0, FDTD_LAYOUT_SOLVER, s->eps), "init (getEps)");
  if (s->solver == FDTD_NS_TM_2D || s->solver == FDTD_NS_TE_2D)
    for (int q = 0; q < 3; q++) {
      s->eps_all[q] = (double *)calloc(na, sizeof(double));
      check(fdtd_get_eps(s->sim, q, FDTD_LAYOUT_SOLVER, s->eps_all[q]), "init (getEps)");
    }
  for (int q = 0; q < 5; q++) s->fresh[q] = 0;
}

static void slot_update(slot *s)
{
  if (!s->sim) { check(FDTD_E_STATE, "update before init"); return; }
  check(fdtd_update(s->sim, field_getTime(), field_getRayCoef()), "update");
  for (int q = 0; q < 5; q++) s->fresh[q] = 0;
}

static double complex *slot_field(slot *s, int which)
{
  if (!s->sim) return NULL;
  if (!s->fresh[which]) {
    if (check(fdtd_get_field(s->sim, which, FDTD_LAYOUT_SOLVER, (double *)s->field[which]), "get field")) return NULL;
    s->fresh[which] = 1;
  }
  return s->field[which];
}

/* ntff_outputEnormTxt / ntff_outputEnormBin (ntff.c:6-33), names of ntffTM.c:240-247 */
static void write_spectrum(const double *spec)
{
  char name[256], cwd[512];
  if (!getcwd(cwd, sizeof cwd)) cwd[0] = 0;
  const int ang = (int)field_getWaveAngle();
  snprintf(name, sizeof name, "%d[deg].txt", ang);
  FILE *fp = fopen(name, "w");
  if (!fp) { printf("cannot open file %s \n", name); if (!g_return_mode) exit(2); return; }
  for (int lam = 380; lam <= 700; lam++) {
    fprintf(fp, "%d ", lam);
    for (int a = 0; a < 360; a++) fprintf(fp, "%lf.20 ", spec[(lam - 380) * 360 + a]);
    fprintf(fp, "\n");
  }
  fclose(fp);
  printf("saved %s/%s\n", cwd, name);
  snprintf(name, sizeof name, "%d[deg]_%dnm_%dnm_b.dat", ang, 380, 700);
  fp = fopen(name, "wb");
  if (!fp) { printf("cannot open file %s \n", name); if (!g_return_mode) exit(2); return; }
  if (fwrite(spec, sizeof(double), 321 * 360, fp) < 321 * 360) {
    printf("error in write binary %s\n", name);
    if (!g_return_mode) exit(2);
  }
  fclose(fp);
  printf("saved %s/%s\n", cwd, name);
}

/* field_outputElliptic of the E field the split-field / NS reset() writes:
 * fdtdTM.c:158-159 "tm_%dnm.txt" (Ez), fdtdTE.c:273-274 "te_%dnm.txt" (Ey),
 * nsFdtdTM.c:163-164 "ns_tm_%dnm.txt", nsFdtdTE.c:222-223 "ns_te_%dnm.txt" */
static void write_elliptic(slot *s)
{
  static const char *fmt[4] = {"tm_%dnm.txt", "te_%dnm.txt", "ns_tm_%dnm.txt", "ns_te_%dnm.txt"};
  const int q = s->solver == FDTD_TM_2D ? 0 : s->solver == FDTD_TE_2D ? 1 : s->solver == FDTD_NS_TM_2D ? 2 : 3;
  char name[128];
  snprintf(name, sizeof name, fmt[q], field_getFieldInfo().h_u_nm);
  printf("output start\n");
  if (!check(fdtd_write_elliptic(s->sim, (q & 1) ? 1 : 0, name), "reset (elliptic)"))
    printf("output to %s end\n", name);
}

static void slot_reset(slot *s)
{
  if (!s->sim) return;
  if (is_split(s->solver)) write_elliptic(s);
  const int serial = s->solver == FDTD_TM_UPML || s->solver == FDTD_TE_UPML;
  if (serial) {  /* fdtdTM_upml.c:85-87: the spectrum of the finished run first */
    double *spec = (double *)malloc(sizeof(double) * 321 * 360);
    if (!check(fdtd_spectrum(s->sim, spec), "reset (spectrum)")) write_spectrum(spec);
    free(spec);
  }
  check(fdtd_reset(s->sim), "reset");
  for (int q = 0; q < 5; q++) s->fresh[q] = 0;
}

static void slot_finish(slot *s)
{
  if (!s->sim) return;
  const int serial = s->solver == FDTD_TM_UPML || s->solver == FDTD_TE_UPML || is_split(s->solver);
  if (serial) slot_reset(s);   /* fdtdTM_upml.c:78-82 */
  release(s);
}

/* ---------------------------------------------------------------- MPI TM */
static void mtm_init(void) { slot_init(&g_slot[SLOT_MPI_TM]); }
static void mtm_update(void) { slot_update(&g_slot[SLOT_MPI_TM]); }
static void mtm_reset(void) { slot_reset(&g_slot[SLOT_MPI_TM]); }
static void mtm_finish(void) { slot_finish(&g_slot[SLOT_MPI_TM]); }
void (*mpi_fdtdTM_upml_getUpdate(void))(void) { return mtm_update; }
void (*mpi_fdtdTM_upml_getFinish(void))(void) { return mtm_finish; }
void (*mpi_fdtdTM_upml_getReset(void))(void) { return mtm_reset; }
void (*mpi_fdtdTM_upml_getInit(void))(void) { return mtm_init; }
double complex *mpi_fdtdTM_upml_getEz(void) { return slot_field(&g_slot[SLOT_MPI_TM], 0); }
double complex *mpi_fdtdTM_upml_getHx(void) { return slot_field(&g_slot[SLOT_MPI_TM], 1); }
double complex *mpi_fdtdTM_upml_getHy(void) { return slot_field(&g_slot[SLOT_MPI_TM], 2); }
double *mpi_fdtdTM_upml_getEps(void) { return g_slot[SLOT_MPI_TM].eps; }
/* one rank: SUB_N_X = N_PX, SUB_N_PX = N_PX + 2 (mpiTM_UPML.c:737-741) */
int mpi_fdtdTM_upml_getSubNx(void) { return g_slot[SLOT_MPI_TM].n_px; }
int mpi_fdtdTM_upml_getSubNy(void) { return g_slot[SLOT_MPI_TM].n_py; }
int mpi_fdtdTM_upml_getSubNpx(void) { return g_slot[SLOT_MPI_TM].nx; }
int mpi_fdtdTM_upml_getSubNpy(void) { return g_slot[SLOT_MPI_TM].ny; }
int mpi_fdtdTM_upml_getSubNcell(void) { return g_slot[SLOT_MPI_TM].nx * g_slot[SLOT_MPI_TM].ny; }

/* ---------------------------------------------------------------- MPI TE */
static void mte_init(void) { slot_init(&g_slot[SLOT_MPI_TE]); }
static void mte_update(void) { slot_update(&g_slot[SLOT_MPI_TE]); }
static void mte_reset(void) { slot_reset(&g_slot[SLOT_MPI_TE]); }
static void mte_finish(void) { slot_finish(&g_slot[SLOT_MPI_TE]); }
void (*mpi_fdtdTE_upml_getUpdate(void))(void) { return mte_update; }
void (*mpi_fdtdTE_upml_getFinish(void))(void) { return mte_finish; }
void (*mpi_fdtdTE_upml_getReset(void))(void) { return mte_reset; }
void (*mpi_fdtdTE_upml_getInit(void))(void) { return mte_init; }
double complex *mpi_fdtdTE_upml_getEx(void) { return slot_field(&g_slot[SLOT_MPI_TE], 0); }
double complex *mpi_fdtdTE_upml_getEy(void) { return slot_field(&g_slot[SLOT_MPI_TE], 1); }
double complex *mpi_fdtdTE_upml_getHz(void) { return slot_field(&g_slot[SLOT_MPI_TE], 2); }
double *mpi_fdtdTE_upml_getEps(void) { return g_slot[SLOT_MPI_TE].eps; }
int mpi_fdtdTE_upml_getSubNx(void) { return g_slot[SLOT_MPI_TE].n_px; }
int mpi_fdtdTE_upml_getSubNy(void) { return g_slot[SLOT_MPI_TE].n_py; }
int mpi_fdtdTE_upml_getSubNpx(void) { return g_slot[SLOT_MPI_TE].nx; }
int mpi_fdtdTE_upml_getSubNpy(void) { return g_slot[SLOT_MPI_TE].ny; }
int mpi_fdtdTE_upml_getSubNcell(void) { return g_slot[SLOT_MPI_TE].nx * g_slot[SLOT_MPI_TE].ny; }

/* ---------------------------------------------------------------- serial TM */
static void stm_init(void) { slot_init(&g_slot[SLOT_SER_TM]); }
static void stm_update(void) { slot_update(&g_slot[SLOT_SER_TM]); }
static void stm_reset(void) { slot_reset(&g_slot[SLOT_SER_TM]); }
static void stm_finish(void) { slot_finish(&g_slot[SLOT_SER_TM]); }
void (*fdtdTM_upml_getUpdate(void))(void) { return stm_update; }
void (*fdtdTM_upml_getFinish(void))(void) { return stm_finish; }
void (*fdtdTM_upml_getReset(void))(void) { return stm_reset; }
void (*fdtdTM_upml_getInit(void))(void) { return stm_init; }
double complex *fdtdTM_upml_getEz(void) { return slot_field(&g_slot[SLOT_SER_TM], 0); }
double complex *fdtdTM_upml_getHx(void) { return slot_field(&g_slot[SLOT_SER_TM], 1); }
double complex *fdtdTM_upml_getHy(void) { return slot_field(&g_slot[SLOT_SER_TM], 2); }
double *fdtdTM_upml_getEps(void) { return g_slot[SLOT_SER_TM].eps; }

/* ---------------------------------------------------------------- serial TE */
static void ste_init(void) { slot_init(&g_slot[SLOT_SER_TE]); }
static void ste_update(void) { slot_update(&g_slot[SLOT_SER_TE]); }
static void ste_reset(void) { slot_reset(&g_slot[SLOT_SER_TE]); }
static void ste_finish(void) { slot_finish(&g_slot[SLOT_SER_TE]); }
void (*fdtdTE_upml_getUpdate(void))(void) { return ste_update; }
void (*fdtdTE_upml_getFinish(void))(void) { return ste_finish; }
void (*fdtdTE_upml_getReset(void))(void) { return ste_reset; }
void (*fdtdTE_upml_getInit(void))(void) { return ste_init; }
double complex *fdtdTE_upml_getEx(void) { return slot_field(&g_slot[SLOT_SER_TE], 0); }
double complex *fdtdTE_upml_getEy(void) { return slot_field(&g_slot[SLOT_SER_TE], 1); }
double complex *fdtdTE_upml_getHz(void) { return slot_field(&g_slot[SLOT_SER_TE], 2); }
double *fdtdTE_upml_getEps(void) { return g_slot[SLOT_SER_TE].eps; }

/* ------------------------------------------- split-field PML TM (fdtdTM.h) */
static void ftm_init(void) { slot_init(&g_slot[SLOT_SPLIT_TM]); }
static void ftm_update(void) { slot_update(&g_slot[SLOT_SPLIT_TM]); }
static void ftm_reset(void) { slot_reset(&g_slot[SLOT_SPLIT_TM]); }
static void ftm_finish(void) { slot_finish(&g_slot[SLOT_SPLIT_TM]); }
void (*fdtdTM_getUpdate(void))(void) { return ftm_update; }
void (*fdtdTM_getFinish(void))(void) { return ftm_finish; }
void (*fdtdTM_getReset(void))(void) { return ftm_reset; }
void (*fdtdTM_getInit(void))(void) { return ftm_init; }
double complex *fdtdTM_getEz(void) { return slot_field(&g_slot[SLOT_SPLIT_TM], 0); }
double complex *fdtdTM_getHx(void) { return slot_field(&g_slot[SLOT_SPLIT_TM], 1); }
double complex *fdtdTM_getHy(void) { return slot_field(&g_slot[SLOT_SPLIT_TM], 2); }
double complex *fdtdTM_getEzx(void) { return slot_field(&g_slot[SLOT_SPLIT_TM], 3); }
double complex *fdtdTM_getEzy(void) { return slot_field(&g_slot[SLOT_SPLIT_TM], 4); }
double *fdtdTM_getEps(void) { return g_slot[SLOT_SPLIT_TM].eps; }

/* ------------------------------------------- split-field PML TE (fdtdTE.h) */
static void fte_init(void) { slot_init(&g_slot[SLOT_SPLIT_TE]); }
static void fte_update(void) { slot_update(&g_slot[SLOT_SPLIT_TE]); }
static void fte_reset(void) { slot_reset(&g_slot[SLOT_SPLIT_TE]); }
static void fte_finish(void) { slot_finish(&g_slot[SLOT_SPLIT_TE]); }
void (*fdtdTE_getUpdate(void))(void) { return fte_update; }
void (*fdtdTE_getFinish(void))(void) { return fte_finish; }
void (*fdtdTE_getReset(void))(void) { return fte_reset; }
void (*fdtdTE_getInit(void))(void) { return fte_init; }
double complex *fdtdTE_getEx(void) { return slot_field(&g_slot[SLOT_SPLIT_TE], 0); }
double complex *fdtdTE_getEy(void) { return slot_field(&g_slot[SLOT_SPLIT_TE], 1); }
double complex *fdtdTE_getHz(void) { return slot_field(&g_slot[SLOT_SPLIT_TE], 2); }
double complex *fdtdTE_getHzx(void) { return slot_field(&g_slot[SLOT_SPLIT_TE], 3); }
double complex *fdtdTE_getHzy(void) { return slot_field(&g_slot[SLOT_SPLIT_TE], 4); }
double *fdtdTE_getEps(void) { return g_slot[SLOT_SPLIT_TE].eps; }

/* ------------------------------------------- NS-FDTD TM (nsFdtdTM.h) */
static void ntm_init(void) { slot_init(&g_slot[SLOT_NS_TM]); }
static void ntm_update(void) { slot_update(&g_slot[SLOT_NS_TM]); }
static void ntm_reset(void) { slot_reset(&g_slot[SLOT_NS_TM]); }
static void ntm_finish(void) { slot_finish(&g_slot[SLOT_NS_TM]); }
void (*nsFdtdTM_getUpdate(void))(void) { return ntm_update; }
void (*nsFdtdTM_getFinish(void))(void) { return ntm_finish; }
void (*nsFdtdTM_getReset(void))(void) { return ntm_reset; }
void (*nsFdtdTM_getInit(void))(void) { return ntm_init; }
double complex *nsFdtdTM_getEz(void) { return slot_field(&g_slot[SLOT_NS_TM], 0); }
double complex *nsFdtdTM_getHx(void) { return slot_field(&g_slot[SLOT_NS_TM], 1); }
double complex *nsFdtdTM_getHy(void) { return slot_field(&g_slot[SLOT_NS_TM], 2); }
double complex *nsFdtdTM_getEzx(void) { return slot_field(&g_slot[SLOT_NS_TM], 3); }
double complex *nsFdtdTM_getEzy(void) { return slot_field(&g_slot[SLOT_NS_TM], 4); }
double *nsFdtdTM_getEps(void) { return g_slot[SLOT_NS_TM].eps; }
double *nsFdtdTM_getEpsX(void) { return g_slot[SLOT_NS_TM].eps_all[1]; }  /* EPS_HX (nsFdtdTM.c:33-35) */
double *nsFdtdTM_getEpsY(void) { return g_slot[SLOT_NS_TM].eps_all[2]; }  /* EPS_HY */
double *nsFdtdTM_getEpsZ(void) { return g_slot[SLOT_NS_TM].eps_all[0]; }  /* EPS_EZ */

/* ------------------------------------------- NS-FDTD TE (nsFdtdTE.h) */
static void nte_init(void) { slot_init(&g_slot[SLOT_NS_TE]); }
static void nte_update(void) { slot_update(&g_slot[SLOT_NS_TE]); }
static void nte_reset(void) { slot_reset(&g_slot[SLOT_NS_TE]); }
static void nte_finish(void) { slot_finish(&g_slot[SLOT_NS_TE]); }
void (*nsFdtdTE_getUpdate(void))(void) { return nte_update; }
void (*nsFdtdTE_getFinish(void))(void) { return nte_finish; }
void (*nsFdtdTE_getReset(void))(void) { return nte_reset; }
void (*nsFdtdTE_getInit(void))(void) { return nte_init; }
double complex *nsFdtdTE_getEx(void) { return slot_field(&g_slot[SLOT_NS_TE], 0); }
double complex *nsFdtdTE_getEy(void) { return slot_field(&g_slot[SLOT_NS_TE], 1); }
double complex *nsFdtdTE_getHz(void) { return slot_field(&g_slot[SLOT_NS_TE], 2); }
double complex *nsFdtdTE_getHzx(void) { return slot_field(&g_slot[SLOT_NS_TE], 3); }
double complex *nsFdtdTE_getHzy(void) { return slot_field(&g_slot[SLOT_NS_TE], 4); }
double *nsFdtdTE_getEps(void) { return g_slot[SLOT_NS_TE].eps; }
double *nsFdtdTE_getEpsX(void) { return g_slot[SLOT_NS_TE].eps_all[0]; }  /* EPS_EX (nsFdtdTE.c:33-35) */
double *nsFdtdTE_getEpsY(void) { return g_slot[SLOT_NS_TE].eps_all[1]; }  /* EPS_EY */
double *nsFdtdTE_getEpsZ(void) { return g_slot[SLOT_NS_TE].eps_all[2]; }  /* EPS_HZ */
