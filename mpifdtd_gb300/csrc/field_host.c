/*
 * field_host.c -- the host API of the reference's field.h and models.h
 * (libmpifdtd_field.so), for programs that use the drop-in solver library
 * without the reference's own field.c / models.c.
 *
 * field.c keeps the run's parameters and clock in globals; so does this file:
 *   field_init      field.c:89-143 (grid and NTFF box from fdtd_geometry_of)
 *   field_nextStep  field.c:312-315, field_isFinish field.c:317-319
 *   field_sigmaX/Y  field.c:259-283, field_pmlCoef* field.c:288-295
 *   models_*        models.c:139-194 with the built-in noModel / circleModel /
 *                   morphoScaleModel evaluators of models_eval.h; the model
 *                   parameters the reference fixes at compile time
 *                   (circleModel.c:6-10, morphoScaleModel.c:14-64) are set with
 *                   mpifdtd_models_set_params().
 */
#include <math.h>
#include <stdio.h>
#include <string.h>

#include "mpifdtd_gb300.h"
#include "models_eval.h"

#define C_0_S 0.7071

/* field.h:20-68 (same layouts) */
typedef struct FieldInfo { int width_nm, height_nm, h_u_nm, pml, lambda_nm, angle_deg, stepNum; } FieldInfo;
typedef struct FieldInfo_S { int N_X, N_Y, N_PX, N_PY, N_CELL, N_PML, DX, DY; } FieldInfo_S;
typedef struct SubFieldInfo_S {
  int OFFSET_X, OFFSET_Y, SUB_N_X, SUB_N_Y, SUB_N_PX, SUB_N_PY, SUB_N_CELL, Rank, RtRank, LtRank, TpRank, BmRank;
} SubFieldInfo_S;
typedef struct WaveInfo_S { double Lambda_s, T_s, Omega_s, K_s, K_0_s, Angle_deg; } WaveInfo_S;
typedef struct NTFFInfo { int top, bottom, left, right, cx, cy; double RFperC; int arraySize; } NTFFInfo;

int N_X, N_Y, N_CELL, N_PML, N_PX, N_PY;          /* field.h:77-82 */

static FieldInfo g_fi;
static FieldInfo_S g_fs;
static SubFieldInfo_S g_sub;
static WaveInfo_S g_wave;
static NTFFInfo g_ntff;
static double g_time, g_ray, g_max_time, g_lambda_s, g_k_s, g_w_s, g_T_s;

static int g_model = 0;                          /* models.h enum MODEL */
static double g_params[64];
static int g_nparams = 0;
static mdl_params g_mdl;

/* ------------------------------------------------------------ field.h */

void field_init(FieldInfo fi)
{
  g_fi = fi;
  fdtd_config cfg;
  memset(&cfg, 0, sizeof cfg);
  cfg.width_nm = fi.width_nm; cfg.height_nm = fi.height_nm; cfg.h_u_nm = fi.h_u_nm; cfg.pml = fi.pml;
  cfg.lambda_nm = fi.lambda_nm; cfg.angle_deg = fi.angle_deg; cfg.step_num = fi.stepNum;
  fdtd_geometry g;
  if (fdtd_geometry_of(&cfg, &g) != FDTD_OK) {
    printf("field_init: %s\n", fdtd_last_error());
    return;
  }
  g_fs.N_PX = g.n_px; g_fs.N_PY = g.n_py; g_fs.N_PML = g.n_pml;
  g_fs.N_X = g.n_x; g_fs.N_Y = g.n_y; g_fs.N_CELL = g.n_px * g.n_py; g_fs.DX = g.n_py; g_fs.DY = 1;
  N_PX = g.n_px; N_PY = g.n_py; N_PML = g.n_pml; N_X = g.n_x; N_Y = g.n_y; N_CELL = g.n_px * g.n_py;
  g_wave.Lambda_s = g.lambda_s;
  g_wave.T_s = g.lambda_s / C_0_S;
  g_wave.K_s = g.k_s;
  g_wave.K_0_s = g.k_s;
  g_wave.Omega_s = g.omega_s;
  g_wave.Angle_deg = fi.angle_deg;
  g_lambda_s = g.lambda_s; g_k_s = g.k_s; g_w_s = g.omega_s; g_T_s = 2 * M_PI / g_w_s;
  g_time = 0;
  g_ray = 0;
  g_max_time = fi.stepNum;
  g_ntff.cx = g.ntff_cx; g_ntff.cy = g.ntff_cy; g_ntff.top = g.ntff_top; g_ntff.bottom = g.ntff_bottom;
  g_ntff.left = g.ntff_left; g_ntff.right = g.ntff_right; g_ntff.RFperC = g.rf_per_c;
  g_ntff.arraySize = g.array_size;
  memset(&g_sub, 0, sizeof g_sub);               /* field.c:112: mpiSplit() is not called either */
}

void field_reset(void) { g_time = 0; g_ray = 0; }
void field_nextStep(void)
{
  g_time += 1.0;
  g_ray = 1.0 - exp(-pow(0.01 * g_time, 2));
}
int field_isFinish(void) { return g_time >= g_max_time; }
void field_setWaveAngle(int deg) { g_fi.angle_deg = deg; g_wave.Angle_deg = deg; }

double field_getT(void) { return g_wave.T_s; }
double field_getK(void) { return g_wave.K_s; }
double field_getRayCoef(void) { return g_ray; }
double field_getOmega(void) { return g_wave.Omega_s; }
double field_getLambda(void) { return g_lambda_s; }
double field_getWaveAngle(void) { return g_wave.Angle_deg; }
double field_getTime(void) { return g_time; }
double field_getMaxTime(void) { return g_max_time; }
NTFFInfo field_getNTFFInfo(void) { return g_ntff; }
WaveInfo_S field_getWaveInfo_S(void) { return g_wave; }
SubFieldInfo_S field_getSubFieldInfo_S(void) { return g_sub; }
FieldInfo_S field_getFieldInfo_S(void) { return g_fs; }
FieldInfo field_getFieldInfo(void) { return g_fi; }

int field_getOffsetX(void) { return g_sub.OFFSET_X; }
int field_getOffsetY(void) { return g_sub.OFFSET_Y; }
int field_getSubNx(void) { return g_sub.SUB_N_X; }
int field_getSubNy(void) { return g_sub.SUB_N_Y; }
int field_getSubNpx(void) { return g_sub.SUB_N_PX; }
int field_getSubNpy(void) { return g_sub.SUB_N_PY; }
int field_getSubNcell(void) { return g_sub.SUB_N_CELL; }
int field_subIndex(int i, int j) { return i * g_sub.SUB_N_PY + j; }
int field_index(int i, int j) { return i * g_fs.N_PY + j; }
int ind(const int i, const int j) { return i * N_PY + j; }
double field_toCellUnit(const double p) { return p / g_fi.h_u_nm; }
double field_toPhisycalUnit(const double c) { return c * g_fi.h_u_nm; }

double field_sigmaX(const double x, const double y)
{
  (void)y;
  const int M = 2;
  if (x < N_PML) return pow(1.0 * (N_PML - x) / N_PML, M);
  if (N_PML <= x && x < (N_X + N_PML)) return 0;
  return pow(1.0 * (x - (N_PX - N_PML - 1)) / N_PML, M);
}
double field_sigmaY(const double x, double y)
{
  (void)x;
  const int M = 2;
  if (y < N_PML) return pow(1.0 * (N_PML - y) / N_PML, M);
  if (y >= N_PML && y < (N_Y + N_PML)) return 0.0;
  return pow(1.0 * (y - (N_PY - N_PML - 1)) / N_PML, M);
}
double field_pmlCoef(double ep_mu, double sig) { return (1.0 - sig / ep_mu) / (1.0 + sig / ep_mu); }
double field_pmlCoef_LXY(double ep_mu, double sig) { return 1.0 / (ep_mu + sig); }

/* ------------------------------------------------------------ models.h */

/* Parameters of the built-in models (cell-independent, in nm):
 *   MIE_CYLINDER (1): {radius_nm, eps}        default {500, 1.6^2}   circleModel.c:6-10
 *   MORPHO_SCALE (3): {width, thick0, thick1, layers, branch, edge_rate, eps,
 *                      per_lamella, widths...} default {300, 90, 90, 6, 0, 0, 1.56^2, 0}
 *   ZIGZAG (5):       {width, thickness, layers, degree, n} default {300, 80, 5, 10, 1.56}
 *                                                          zigzagModel.c:9-31
 * Returns 0, -1 on an unknown model. */
int mpifdtd_models_set_params(int model, const double *p, int n)
{
  if (model != 0 && model != 1 && model != 3 && model != 5) return -1;
  g_model = model;
  g_nparams = n > 64 ? 64 : n;
  if (g_nparams > 0) memcpy(g_params, p, sizeof(double) * g_nparams);
  return 0;
}

void models_setModel(int model)
{
  static const double circle[2] = {500, 0};
  static const double morpho[8] = {300, 90, 90, 6, 0, 0.0, 0, 0};
  static const double zigzag[5] = {300, 80, 5, 10, 0};
  if (model == 1 && g_model != 1) mpifdtd_models_set_params(1, circle, 2);
  else if (model == 3 && g_model != 3) mpifdtd_models_set_params(3, morpho, 8);
  else if (model == 5 && g_model != 5) mpifdtd_models_set_params(5, zigzag, 5);
  else if (model == 0) mpifdtd_models_set_params(0, NULL, 0);
  else if (model != 1 && model != 3 && model != 5) {
    printf("mpifdtd_gb300: model %d is not built in (NO_MODEL, MIE_CYLINDER, MORPHO_SCALE, ZIGZAG)\n", model);
    g_model = 0;
  }
}

void models_initModel(void)
{
  if (mdl_init(&g_mdl, g_model, g_params, g_nparams, N_PX, N_PY, N_PML, g_fi.h_u_nm) != 0) {
    printf("mpifdtd_gb300: bad parameters for model %d\n", g_model);
    mdl_init(&g_mdl, 0, NULL, 0, N_PX, N_PY, N_PML, g_fi.h_u_nm);
  }
}

double models_eps(double x, double y, int mode)
{
  switch (mode) {
  case 0: return mdl_eps(&g_mdl, x, y, 1, 0);   /* D_X  */
  case 1: return mdl_eps(&g_mdl, x, y, 0, 1);   /* D_Y  */
  default: return mdl_eps(&g_mdl, x, y, 1, 1);  /* D_XY */
  }
}

int models_isFinish(void) { return 1; }
void models_moveDirectory(void) {}
void models_needSize(int *x_nm, int *y_nm)
{
  *x_nm = 1000;
  *y_nm = 1000;
}
