/* Oracle build only: drives the reference exactly as simulator.c does
 * (simulator.c:258-266 init, simulator.c:247-251 calc), with hooks between
 * models_initModel() and the solver init so that a test can override the
 * models' compile-time parameters (circleModel.c:6-10, morphoScaleModel.c:14-64)
 * without editing the reference. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "simulator.h"
#include "field.h"
#include "models.h"
#include <complex.h>

extern void refh_mpitm_init(void);
extern void refh_mpite_init(void);
extern void refh_sertm_init(void);
extern void refh_serte_init(void);
extern void refh_splittm_init(void);
extern void refh_splitte_init(void);
extern void refh_nstm_init(void);
extern void refh_nste_init(void);
extern void refh_models_set_callback(double (*fn)(double, double, int, int));
extern void refh_circle_set_radius_nm(int r);
extern void refh_circle_set_eps(double e);
extern void refh_morpho_set(int width, int thick0, int thick1, int layers, int branch, double edge_rate);
extern void refh_morpho_set_eps(double e);
extern void refh_zigzag_set(int width, int thick, int layers, int deg);

enum { RM_NONE = 0, RM_CIRCLE = 1, RM_MORPHO = 2, RM_CALLBACK = 3, RM_ZIGZAG = 4 };

/* model params: circle {radius_nm, eps (<=0: reference default)};
 * morpho {width, thick0, thick1, layers, branch, edge_rate, eps (<=0: default)};
 * zigzag {width, thickness, layers, degree} (index N_0 = 1.56 is a #define) */
int refh_setup(int solver, int width_nm, int height_nm, int h_u_nm, int pml,
               int lambda_nm, int angle_deg, int step_num,
               int model, const double *mp, double (*cb)(double, double, int, int))
{
  simulator_setSolver((enum SOLVER)solver);
  switch (model) {
  case RM_NONE: models_setModel(NO_MODEL); break;
  case RM_CIRCLE: models_setModel(MIE_CYLINDER); refh_circle_set_radius_nm((int)mp[0]); break;
  case RM_MORPHO:
    models_setModel(MORPHO_SCALE);
    refh_morpho_set((int)mp[0], (int)mp[1], (int)mp[2], (int)mp[3], (int)mp[4], mp[5]);
    break;
  case RM_CALLBACK: refh_models_set_callback(cb); break;
  case RM_ZIGZAG:
    models_setModel(ZIGZAG);
    refh_zigzag_set((int)mp[0], (int)mp[1], (int)mp[2], (int)mp[3]);
    break;
  default: return -1;
  }
  FieldInfo fi;
  fi.width_nm = width_nm; fi.height_nm = height_nm; fi.h_u_nm = h_u_nm; fi.pml = pml;
  fi.lambda_nm = lambda_nm; fi.angle_deg = angle_deg; fi.stepNum = step_num;
  field_init(fi);
  models_initModel();
  if (model == RM_CIRCLE && mp[1] > 0) refh_circle_set_eps(mp[1]);
  if (model == RM_MORPHO && mp[6] > 0) refh_morpho_set_eps(mp[6]);
  switch (solver) {
  case MPI_TM_UPML_2D: refh_mpitm_init(); break;
  case MPI_TE_UPML_2D: refh_mpite_init(); break;
  case TM_UPML_2D: refh_sertm_init(); break;
  case TE_UPML_2D: refh_serte_init(); break;
  case TM_2D: refh_splittm_init(); break;
  case TE_2D: refh_splitte_init(); break;
  case NS_TM_2D: refh_nstm_init(); break;
  case NS_TE_2D: refh_nste_init(); break;
  default: return -2;
  }
  return 0;
}

void refh_step(int n)
{
  for (int s = 0; s < n; s++) simulator_calc();
}

/* Seeded test map installed through the reference's models_eps callback
 * path: the last disc containing the point wins (point sample). */
static int discs_n;
static double discs_p[32];
static double discs_eps(double x, double y, int col, int row)
{
  (void)col; (void)row;
  double e = EPSILON_0_S;
  for (int d = 0; d < discs_n; d++) {
    double dx = x - discs_p[4 * d], dy = y - discs_p[4 * d + 1], r = discs_p[4 * d + 2];
    if (dx * dx + dy * dy <= r * r) e = discs_p[4 * d + 3];
  }
  return e;
}
void *refh_discs_callback(int n, const double *p)
{
  discs_n = n > 8 ? 8 : n;
  for (int q = 0; q < 4 * discs_n; q++) discs_p[q] = p[q];
  return (void *)discs_eps;
}

/* ntffTM_init() sets R0 (ntffTM.c:27-64); the MPI solvers never call it
 * (mpiTM_UPML.c:187-193), so a harness must before ntffTM_Frequency. */
extern void ntffTM_init(void);
extern void ntffTM_Frequency(double complex *Hx, double complex *Hy, double complex *Ez, double complex res[360]);
void refh_tm_frequency(double complex *Hx, double complex *Hy, double complex *Ez, double complex *res)
{
  ntffTM_init();
  ntffTM_Frequency(Hx, Hy, Ez, res);
}
