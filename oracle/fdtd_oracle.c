/*
 * fdtd_oracle.c -- CPU restatement of the reference's 2-D UPML FDTD path.
 *
 * TEST INFRASTRUCTURE (the oracle).  It exists to check the GPU product and to
 * serve as the timed CPU baseline; the product never links or calls it.
 *
 * What it restates (reference file:line, paths within rennone/mpiFDTD):
 *   field parameters      field.c:89-143 (field_init), field.c:312-319 (nextStep)
 *   PML sigma profiles    field.c:259-283
 *   models                noModel.c:5-8, circleModel.c:27-58,74-81,
 *                         morphoScaleModel.c:101-253,379-422, zigzagModel.c:41-79,
 *                         146-161, models.c:166-184
 *   MPI TM UPML (np=1)    mpiTM_UPML.c:196-217 update, :431-530 kernels,
 *                         :337-374 source, :663-716 coefficients, :840-1037 ntff
 *   MPI TE UPML (np=1)    mpiTE_UPML.c:290-304 update, :337-399 kernels,
 *                         :250-281 source, :489-536 coefficients, :602-794 ntff
 *   serial TM UPML        fdtdTM_upml.c:54-66, :155-274; ntffTM.c:279-371
 *   serial TE UPML        fdtdTE_upml.c:168-192, :252-412; ntffTE.c:57-157
 *   pulse source          field.c:224-256
 *   spectrum output       ntffTM.c:161-275, ntffTE.c:20-55,160-238, cfft.c:104-179
 *   split-field PML       fdtdTM.c:167-242, :290-327; fdtdTE.c:170-238, :283-321
 *   NS-FDTD               nsFdtdTM.c:68-151, :221-307; nsFdtdTE.c:90-181, :233-308;
 *                         sources field.c:155-196
 *   frequency NTFF        ntffTM.c:72-158, ntffTE.c:242-338 (TE: global index
 *                         on all four sides, see of_frequency)
 *
 * The MPI solvers are restated for one rank: the sub-domain is the whole grid
 * with a one-cell halo that stays zero (mpiTM_UPML.c:718-748 with
 * MPI_PROC_NULL neighbours), so array index i holds global x = i-1.
 *
 * Parity pin: tests/test_oracle_golden.py checks this file against golden
 * vectors made by the reference's own sources compiled unmodified
 * (oracle/ref.mk, tests/golden/make_golden.py).
 */
#define _GNU_SOURCE
#include <complex.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include "fdtd_oracle.h"

#ifndef M_PI
#define M_PI 3.1415926535897932384626433832795
#endif

#define OF_C 0.7071                      /* field.h:70 C_0_S */
#define OF_EPS0 1.0                      /* field.h:73 */
#define OF_MU0 (1.0 / OF_C / OF_C)       /* field.h:74 */
#define OF_Z0 1.41422712488              /* field.h:75 */
#define OF_GUARD 16
#define OF_NFFT 8192                     /* ntff.h:6 NTFF_NUM */
#define OF_LAMBDA_ST 380                 /* ntff.h:4 */
#define OF_LAMBDA_EN 700                 /* ntff.h:5 */

typedef double complex cplx;

struct of_sim {
  int solver, tm, mpi;
  int family;                            /* 0 UPML, 1 split-field PML, 2 NS-FDTD */
  of_field_info fi;
  /* field.c:89-143 */
  int n_px, n_py, n_pml, n_x, n_y;
  double lambda_s, k_s, w_s;
  double time, ray_coef, max_time;
  int top, bottom, left, right, cx, cy, array_size;
  double rf;
  /* model state (kept per simulation so several can run in threads) */
  of_model model;
  double c_radius, c_eps, c_posx, c_posy;
  double m_width[16], m_width_max, m_thick[2], m_branch, m_height, m_ox, m_oy, m_ep, m_edge;
  int m_layers;
  double m_a[16], m_b1[16], m_b2[16];
  int z_layers;
  double z_rad, z_width, z_thick, z_height, z_exw, z_exh, z_ox, z_oy, z_ep;
  /* arrays */
  int nx, ny, ncell, ox;                 /* array dims; global x = i + ox */
  cplx *f[9];
  double *c[15];
  double *eps[3];
  cplx *nt_base[3], *nt[3];
  int skip_ntff;                         /* of_bench_opts: leave the time-domain NTFF out (timing only) */
  double c0, mu0, z0;                    /* Courant number, 1/C^2, impedance (field.h:70-75 by default) */
  int pml_m, inset;                      /* sigma grading exponent, NTFF inset (field.c:259-283, :136-139) */
};

/* ---------------------------------------------------------------- models */

/* circleModel.c:27-58 */
static double eps_circle(const of_sim *s, double x, double y, int col, int row)
{
  if (x < s->n_pml || y < s->n_pml || x > s->n_x + s->n_pml || y > s->n_y + s->n_pml)
    return OF_EPS0;
  double dx = x - s->c_posx, dy = y - s->c_posy;
  double len = dx * dx + dy * dy;
  double r = s->c_radius;
  if (len >= (r + 1) * (r + 1)) return OF_EPS0;
  if (len <= (r - 1) * (r - 1)) return s->c_eps;
  const double split = 10, half = split / 2;
  double sum = 0;
  for (double i = -half + 0.5; i < half; i += 1)
    for (double j = -half + 0.5; j < half; j += 1) {
      double px = dx + col * i / split, py = dy + row * j / split;
      if (px * px + py * py <= r * r) sum += 1;
    }
  sum /= split * split;
  return s->c_eps * sum + OF_EPS0 * (1 - sum);
}

/* morphoScaleModel.c:101-104 inLamela */
static int in_lamella(const of_sim *s, int id, double x, double y)
{
  return s->m_a[id] * x + s->m_b1[id] <= y && y <= s->m_a[id] * x + s->m_b2[id];
}

/* morphoScaleModel.c:107-125 getWidth (no edge randomness: RANDOMNESS 0, CURVE 0) */
static double lamella_width(const of_sim *s, double sx, double sy, int id)
{
  double b = sy - sx * s->m_a[id];
  double p = 1 - b / s->m_height;
  double width_p = p + (1 - p) * s->m_edge;
  double half_width = s->m_width[id] / 2.0;
  return width_p * (half_width * (1 - 0.0));
}

/* morphoScaleModel.c:128-145 calcLamela: first lamella whose band holds a corner */
static int find_lamella(const of_sim *s, double lft, double rht, double btm, double top)
{
  for (int i = 0; i < s->m_layers; i++)
    if (in_lamella(s, i, lft, btm) || in_lamella(s, i, rht, btm) ||
        in_lamella(s, i, lft, top) || in_lamella(s, i, rht, top))
      return i;
  return -1;
}

/* morphoScaleModel.c:147-253 eps (symmetric, no gap, no anisotropy) */
static double eps_morpho(const of_sim *s, double x, double y, int col, int row)
{
  double X = x - s->m_ox, Y = y - s->m_oy;
  if (fabs(X) > 0.5 * sqrt(s->m_width_max * s->m_width_max + s->m_thick[0] * s->m_thick[0]) + 0.5)
    return OF_EPS0;
  int lam_id[2] = {-1, -1};              /* [0] left (x<0), [1] right */
  if (fabs(X) > 0.5) {
    lam_id[X < 0 ? 0 : 1] = find_lamella(s, X - 0.5, X + 0.5, Y - 0.5, Y + 0.5);
  } else {
    lam_id[0] = find_lamella(s, X - 0.5, 0, Y - 0.5, Y + 0.5);
    lam_id[1] = find_lamella(s, 0, X + 0.5, Y - 0.5, Y + 0.5);
  }
  double cnt = 0;
  const double split = 10, half = split / 2;
  for (double i = -half + 0.5; i < half; i += 1)
    for (double j = -half + 0.5; j < half; j += 1) {
      double sx = X + col * i / split, sy = Y + row * j / split;
      if (sy >= 0 && sy <= s->m_height) {          /* trunk */
        double p = 1 - sy / s->m_height;
        double width_p = p + (1 - p) * s->m_edge;
        if (fabs(sx) < s->m_branch / 2.0 * width_p) { cnt += 1; continue; }
      }
      int id = lam_id[sx < 0 ? 0 : 1];
      if (id < 0) continue;
      if (in_lamella(s, id, sx, sy)) {
        double w = lamella_width(s, sx, sy, id);
        if (sx * sx * (1 + s->m_a[id] * s->m_a[id]) < w * w) { cnt += 1; continue; }
      }
      for (int k = -1; k < 2; k += 2) {            /* neighbouring lamellae */
        int nid = id + k;
        if (nid < 0 || nid >= s->m_layers) continue;
        if (in_lamella(s, nid, sx, sy)) {
          double w = lamella_width(s, sx, sy, nid);
          if (sx * sx * (1 + s->m_a[nid] * s->m_a[nid]) < w * w) { cnt += 1; break; }
        }
      }
    }
  cnt /= split * split;
  return OF_EPS0 * (1 - cnt) + s->m_ep * cnt;
}

/* seeded test map: the last disc that contains the point wins (point sample) */
static double eps_discs(const of_sim *s, double x, double y)
{
  const double *p = s->model.p;
  int n = (int)p[0];
  double e = OF_EPS0;
  for (int d = 0; d < n && d < 8; d++) {
    double dx = x - p[1 + 4 * d], dy = y - p[2 + 4 * d], r = p[3 + 4 * d];
    if (dx * dx + dy * dy <= r * r) e = p[4 + 4 * d];
  }
  return e;
}

/* zigzagModel.c:41-79 eps: lamellae as thick lines zig-zagging up a
 * trunkless ridge, 10x10 sub-cell area/line average */
static double eps_zigzag(const of_sim *s, double _x, double _y, int col, int row)
{
  double x = _x - s->z_ox, y = _y - s->z_oy;
  const double rad = s->z_rad, width_s = s->z_width, thickness_s = s->z_thick;
  const double height_s = s->z_height, exw = s->z_exw, exh = s->z_exh;
  if (fabs(x) > width_s / 2.0 + exw + 0.5 || y < -exh - 0.5 || y > height_s + exh + 0.5) return OF_EPS0;
  double cnt = 0;
  const double split = 10, half = split / 2;
  for (double i = -half + 0.5; i < half; i += 1)
    for (double j = -half + 0.5; j < half; j += 1) {
      double sx = x + col * i / split, sy = y + row * j / split;
      if (fabs(sx) > width_s / 2 + exw || sy < -exh || sy > height_s + exh) continue;
      double q = sy / (width_s * sin(rad) + cos(rad) * thickness_s / 2);
      double m = 0 > q ? 0 : q;
      int k = (int)(s->z_layers - 1 < m ? s->z_layers - 1 : m);   /* min(layerNum-1, max(0, q)) */
      double px = -width_s * cos(rad) / 2.0;
      double py = floor((k + 1) / 2) * 2 * (width_s * sin(rad)) + k * cos(rad) * thickness_s / 2;
      double vx = (1 - ((k & 1) << 1)) * cos(rad);
      double vy = sin(rad);
      double sqr = pow(sx - px, 2) + pow(sy - py, 2) - pow((sx - px) * vx + (sy - py) * vy, 2);
      if (sqr <= thickness_s * thickness_s) cnt += 1;
    }
  cnt /= split * split;
  return OF_EPS0 * (1 - cnt) + s->z_ep * cnt;
}

/* models.c:166-184 (D_X -> (1,0), D_Y -> (0,1), D_XY -> (1,1)) */
static double model_eps(const of_sim *s, double x, double y, int col, int row)
{
  switch (s->model.kind) {
  case OF_MODEL_CIRCLE: return eps_circle(s, x, y, col, row);
  case OF_MODEL_MORPHO: return eps_morpho(s, x, y, col, row);
  case OF_MODEL_DISCS: return eps_discs(s, x, y);
  case OF_MODEL_ZIGZAG: return eps_zigzag(s, x, y, col, row);
  default: return OF_EPS0;
  }
}
enum { DX_ = 0, DY_ = 1, DXY_ = 2 };
static double meps(const of_sim *s, double x, double y, int mode)
{
  if (mode == DX_) return model_eps(s, x, y, 1, 0);
  if (mode == DY_) return model_eps(s, x, y, 0, 1);
  return model_eps(s, x, y, 1, 1);
}

/* circleModel.c:74-81, morphoScaleModel.c:379-422, zigzagModel.c:146-161 */
static void model_init(of_sim *s)
{
  const double *p = s->model.p;
  double hu = s->fi.h_u_nm;
  if (s->model.kind == OF_MODEL_ZIGZAG) {
    const int layers = (int)p[2];
    s->z_layers = layers;
    s->z_rad = (int)p[3] * M_PI / 180.0;
    s->z_width = (int)p[0] / hu;
    s->z_thick = (int)p[1] / hu;
    s->z_height = (s->z_width * sin(s->z_rad)) * layers + layers * s->z_thick / 2 * cos(s->z_rad);
    s->z_exw = s->z_thick / 2.0 * sin(s->z_rad);
    s->z_exh = s->z_thick / 2.0 * cos(s->z_rad);
    s->z_ox = s->n_px / 2.0;
    s->z_oy = (s->n_py - s->z_height) / 2.0;
    s->z_ep = p[4] > 0 ? p[4] * p[4] * OF_EPS0 : 1.56 * 1.56 * OF_EPS0;
  } else if (s->model.kind == OF_MODEL_CIRCLE) {
    s->c_radius = p[0] / hu;
    s->c_posx = s->n_px / 2;
    s->c_posy = s->n_py / 2;
    s->c_eps = p[1] > 0 ? p[1] : 1.6 * 1.6 * OF_EPS0;
  } else if (s->model.kind == OF_MODEL_MORPHO) {
    int layers = (int)p[3];
    if (layers > 16) layers = 16;
    s->m_layers = layers;
    s->m_thick[0] = p[1] / hu;
    s->m_thick[1] = p[2] / hu;
    s->m_branch = p[4] / hu;
    s->m_edge = p[5];
    s->m_ep = p[6] > 0 ? p[6] : 1.56 * 1.56 * OF_EPS0;
    s->m_width_max = 0;
    for (int i = 0; i < layers; i++) {
      /* p[7] > 0 selects per-lamella widths p[8..8+layers) (an extension);
       * otherwise every lamella has the reference's single width p[0]. */
      s->m_width[i] = (p[7] > 0 ? p[8 + i] : p[0]) / hu;
      if (s->m_width[i] > s->m_width_max) s->m_width_max = s->m_width[i];
    }
    s->m_height = (s->m_thick[0] + s->m_thick[1]) * layers + (s->m_thick[0] + s->m_thick[1]);
    s->m_oy = s->n_py / 2 - s->m_height / 2;
    s->m_ox = s->n_px / 2;
    double thick = s->m_thick[0] + s->m_thick[1], half = 0.5 * s->m_thick[0];
    for (int i = 0; i < layers; i++) {
      s->m_a[i] = tan(0.0);
      s->m_b1[i] = thick * i + half - half / cos(0.0);
      s->m_b2[i] = thick * i + half + half / cos(0.0);
    }
  }
}

/* ---------------------------------------------------------------- field */

/* field.c:259-283: pow(t, M), M = 2 in the reference (t * t, the same value) */
static double grade(const of_sim *s, double t) { return s->pml_m == 2 ? t * t : pow(t, (double)s->pml_m); }
static double sigma_x(const of_sim *s, double x)
{
  if (x < s->n_pml) return grade(s, 1.0 * (s->n_pml - x) / s->n_pml);
  if (x < s->n_x + s->n_pml) return 0;
  return grade(s, 1.0 * (x - (s->n_px - s->n_pml - 1)) / s->n_pml);
}
static double sigma_y(const of_sim *s, double y)
{
  if (y < s->n_pml) return grade(s, 1.0 * (s->n_pml - y) / s->n_pml);
  if (y < s->n_y + s->n_pml) return 0.0;
  return grade(s, 1.0 * (y - (s->n_py - s->n_pml - 1)) / s->n_pml);
}

static void field_setup(of_sim *s)
{
  const of_field_info *f = &s->fi;
  s->n_px = (int)((double)f->width_nm / f->h_u_nm);
  s->n_py = (int)((double)f->height_nm / f->h_u_nm);
  s->n_pml = f->pml;
  s->n_x = s->n_px - 2 * s->n_pml;
  s->n_y = s->n_py - 2 * s->n_pml;
  s->lambda_s = (double)f->lambda_nm / f->h_u_nm;
  s->k_s = 2 * M_PI / s->lambda_s;
  s->w_s = s->c0 * s->k_s;
  s->time = 0;
  s->ray_coef = 0;
  s->max_time = f->step_num;
  s->cx = s->n_px / 2;
  s->cy = s->n_py / 2;
  s->top = s->n_py - s->n_pml - s->inset;
  s->bottom = s->n_pml + s->inset;
  s->left = s->n_pml + s->inset;
  s->right = s->n_px - s->n_pml - s->inset;
  double len = (s->top - s->bottom) / 2;
  s->rf = len * 2;
  s->array_size = (int)(s->max_time + 2 * s->rf);
}

/* ---------------------------------------------------------- allocation */

/* malloc + memset as the reference's allocateMemories() does
 * (mpiTM_UPML.c:604-661): every page is touched at setup, not in the timed loop */
static void *zalloc(size_t n)
{
  void *p = malloc(n);
  if (p) memset(p, 0, n);
  return p;
}

static void coefficients(of_sim *s)
{
  const double R = 1.0e-8, M = (double)s->pml_m;
  double sig_max;
  if (s->tm) /* mpiTM_UPML.c:672, fdtdTM_upml.c:232 (extra 1/cos(pi/3)) */
    sig_max = -(M + 1.0) * OF_EPS0 * s->c0 / 2.0 / s->n_pml / cos(M_PI / 3) * log(R);
  else       /* mpiTE_UPML.c:497, fdtdTE_upml.c:369 */
    sig_max = -(M + 1.0) * OF_EPS0 * s->c0 / 2.0 / s->n_pml * log(R);
  const double e2 = 2 * OF_EPS0, sz = 0;
  /* MPI: cells 1..n-2 of the padded array (global x=i-1); serial: every cell */
  int i0 = s->mpi ? 1 : 0, i1 = s->mpi ? s->nx - 1 : s->nx;
  int j0 = s->mpi ? 1 : 0, j1 = s->mpi ? s->ny - 1 : s->ny;
  for (int i = i0; i < i1; i++)
    for (int j = j0; j < j1; j++) {
      int k = i * s->ny + j;
      double x = i + s->ox, y = j + s->ox;
      double **c = s->c;
      if (s->tm) {
        if (s->mpi) {   /* mpiTM_UPML.c:680-682 */
          s->eps[0][k] = meps(s, x, y, DXY_);
          s->eps[1][k] = meps(s, x, y + 0.5, DY_);
          s->eps[2][k] = meps(s, x + 0.5, y, DX_);
        } else {        /* fdtdTM_upml.c:237-239 */
          s->eps[0][k] = meps(s, x, y, DXY_);
          s->eps[1][k] = meps(s, x, y + 0.5, DXY_);
          s->eps[2][k] = meps(s, x + 0.5, y, DXY_);
        }
        double sex = sig_max * sigma_x(s, x), sey = sig_max * sigma_y(s, y);
        double shxx = sig_max * sigma_x(s, x), shxy = sig_max * sigma_y(s, y + 0.5);
        double shyx = sig_max * sigma_x(s, x + 0.5), shyy = sig_max * sigma_y(s, y);
        /* mpiTM_UPML.c:697-713 : JZ JZHXHY DZ DZJZ1 DZJZ0 MX MXEZ BX BXMX1 BXMX0 MY MYEZ BY BYMY1 BYMY0 */
        c[0][k] = (e2 - sex) / (e2 + sex);
        c[1][k] = (e2) / (e2 + sex);
        c[2][k] = (e2 - sey) / (e2 + sey);
        c[3][k] = (e2 + sz) / (e2 + sey);
        c[4][k] = (e2 - sz) / (e2 + sey);
        c[5][k] = (e2 - shxy) / (e2 + shxy);
        c[6][k] = (e2) / (e2 + shxy);
        c[7][k] = (e2 - sz) / (e2 + sz);
        c[8][k] = (e2 + shxx) / (e2 + sz);
        c[9][k] = (e2 - shxx) / (e2 + sz);
        c[10][k] = (e2 - sz) / (e2 + sz);
        c[11][k] = (e2) / (e2 + sz);
        c[12][k] = (e2 - shyx) / (e2 + shyx);
        c[13][k] = (e2 + shyy) / (e2 + shyx);
        c[14][k] = (e2 - shyy) / (e2 + shyx);
      } else {
        /* mpiTE_UPML.c:503-505, fdtdTE_upml.c:374-376 */
        s->eps[0][k] = meps(s, x + 0.5, y, DY_);
        s->eps[1][k] = meps(s, x, y + 0.5, DX_);
        s->eps[2][k] = 0.5 * (meps(s, x + 0.5, y + 0.5, DX_) + meps(s, x + 0.5, y + 0.5, DY_));
        double sexx = sig_max * sigma_x(s, x + 0.5), sexy = sig_max * sigma_y(s, y);
        double seyx = sig_max * sigma_x(s, x), seyy = sig_max * sigma_y(s, y + 0.5);
        double shzx = sig_max * sigma_x(s, x + 0.5), shzy = sig_max * sigma_y(s, y + 0.5);
        /* mpiTE_UPML.c:517-533 : JX JXHZ DX DXJX1 DXJX0 JY JYHZ DY DYJY1 DYJY0 MZ MZEXEY BZ BZMZ1 BZMZ0 */
        c[0][k] = (e2 - sexy) / (e2 + sexy);
        c[1][k] = (e2) / (e2 + sexy);
        c[2][k] = (e2 - sz) / (e2 + sz);
        c[3][k] = (e2 + sexx) / (e2 + sz);
        c[4][k] = (e2 - sexx) / (e2 + sz);
        c[5][k] = (e2 - sz) / (e2 + sz);
        c[6][k] = (e2) / (e2 + sz);
        c[7][k] = (e2 - seyx) / (e2 + seyx);
        c[8][k] = (e2 + seyy) / (e2 + seyx);
        c[9][k] = (e2 - seyy) / (e2 + seyx);
        c[10][k] = (e2 - shzx) / (e2 + shzx);
        c[11][k] = (e2) / (e2 + shzx);
        c[12][k] = (e2 - shzy) / (e2 + shzy);
        c[13][k] = (e2 + sz) / (e2 + shzy);
        c[14][k] = (e2 - sz) / (e2 + shzy);
      }
    }
}

static void coefficients_split(of_sim *s);

of_sim *of_create(int solver, const of_field_info *fi, const of_model *m)
{
  if (solver != OF_TM_UPML && solver != OF_TE_UPML && solver != OF_MPI_TM_UPML && solver != OF_MPI_TE_UPML &&
      solver != OF_TM_2D && solver != OF_TE_2D && solver != OF_NS_TM_2D && solver != OF_NS_TE_2D)
    return NULL;
  of_sim *s = (of_sim *)zalloc(sizeof(of_sim));
  s->solver = solver;
  s->tm = (solver == OF_TM_UPML || solver == OF_MPI_TM_UPML || solver == OF_TM_2D || solver == OF_NS_TM_2D);
  s->mpi = (solver == OF_MPI_TM_UPML || solver == OF_MPI_TE_UPML);
  s->family = (solver == OF_TM_2D || solver == OF_TE_2D) ? 1 : (solver == OF_NS_TM_2D || solver == OF_NS_TE_2D) ? 2 : 0;
  s->fi = *fi;
  if (m) s->model = *m;
  if ((s->family && (fi->courant != 0 || fi->pml_order || fi->ntff_inset)) || fi->courant < 0 ||
      fi->courant > 0.7071 || fi->pml_order < 0 || fi->ntff_inset < 0) { free(s); return NULL; }
  s->c0 = fi->courant > 0 ? fi->courant : OF_C;
  s->mu0 = 1.0 / s->c0 / s->c0;                            /* field.h:74 */
  s->z0 = fi->courant > 0 ? 1.0 / fi->courant : OF_Z0;     /* field.h:75 (the literal for 0.7071) */
  s->pml_m = fi->pml_order > 0 ? fi->pml_order : 2;
  s->inset = fi->ntff_inset > 0 ? fi->ntff_inset : 5;
  field_setup(s);
  if (s->n_pml <= 0 || s->n_px < 2 * (s->n_pml + s->inset + 1) || s->n_py < 2 * (s->n_pml + s->inset + 1)) {
    free(s);
    return NULL;
  }
  model_init(s);
  s->nx = s->mpi ? s->n_px + 2 : s->n_px;
  s->ny = s->mpi ? s->n_py + 2 : s->n_py;
  s->ox = s->mpi ? -1 : 0;
  s->ncell = s->nx * s->ny;
  for (int a = 0; a < 9; a++) s->f[a] = (cplx *)zalloc(sizeof(cplx) * s->ncell);
  for (int a = 0; a < 15; a++) s->c[a] = (double *)zalloc(sizeof(double) * s->ncell);
  for (int a = 0; a < 3; a++) s->eps[a] = (double *)zalloc(sizeof(double) * s->ncell);
  if (s->family) {  /* no NTFF in these solvers */
    coefficients_split(s);
    return s;
  }
  size_t nt = (size_t)360 * s->array_size + 2 * OF_GUARD;
  for (int a = 0; a < 3; a++) { s->nt_base[a] = (cplx *)zalloc(sizeof(cplx) * nt); s->nt[a] = s->nt_base[a] + OF_GUARD; }
  coefficients(s);
  return s;
}

void of_destroy(of_sim *s)
{
  if (!s) return;
  for (int a = 0; a < 9; a++) free(s->f[a]);
  for (int a = 0; a < 15; a++) free(s->c[a]);
  for (int a = 0; a < 3; a++) { free(s->eps[a]); free(s->nt_base[a]); }
  free(s);
}

/* ------------------------------------------------------------- TM update */
/* field slots: TM 0 Ez 1 Jz 2 Dz 3 Hx 4 Mx 5 Bx 6 Hy 7 My 8 By */

static void tm_jd_e(of_sim *s)     /* mpiTM_UPML.c:431-458 / fdtdTM_upml.c:155-178 */
{
  cplx *Ez = s->f[0], *Jz = s->f[1], *Dz = s->f[2], *Hx = s->f[3], *Hy = s->f[6];
  double **c = s->c; int ny = s->ny;
  for (int i = 1; i < s->nx - 1; i++)
    for (int j = 1; j < ny - 1; j++) {
      int k = i * ny + j;
      cplx now = Jz[k];
      Jz[k] = c[0][k] * Jz[k] + c[1][k] * (+Hy[k] - Hy[k - ny] - Hx[k] + Hx[k - 1]);
      Dz[k] = c[2][k] * Dz[k] + c[3][k] * Jz[k] - c[4][k] * now;
    }
  for (int i = 1; i < s->nx - 1; i++)
    for (int j = 1; j < ny - 1; j++) {
      int k = i * ny + j;
      Ez[k] = Dz[k] / s->eps[0][k];
    }
}

static void tm_mb_h(of_sim *s)     /* mpiTM_UPML.c:491-530 / fdtdTM_upml.c:181-219 */
{
  cplx *Ez = s->f[0], *Hx = s->f[3], *Mx = s->f[4], *Bx = s->f[5], *Hy = s->f[6], *My = s->f[7], *By = s->f[8];
  double **c = s->c; int ny = s->ny;
  for (int i = 1; i < s->nx - 1; i++)
    for (int j = 1; j < ny - 1; j++) {
      int k = i * ny + j;
      cplx now = Mx[k];
      Mx[k] = c[5][k] * Mx[k] - c[6][k] * (Ez[k + 1] - Ez[k]);
      Bx[k] = c[7][k] * Bx[k] + c[8][k] * Mx[k] - c[9][k] * now;
    }
  for (int i = 1; i < s->nx - 1; i++)
    for (int j = 1; j < ny - 1; j++) {
      int k = i * ny + j;
      cplx now = My[k];
      My[k] = c[10][k] * My[k] - c[11][k] * (-Ez[k + ny] + Ez[k]);
      By[k] = c[12][k] * By[k] + c[13][k] * My[k] - c[14][k] * now;
    }
  for (int i = 1; i < s->nx - 1; i++)
    for (int j = 1; j < ny - 1; j++) {
      int k = i * ny + j;
      Hx[k] = Bx[k] / s->mu0;
      Hy[k] = By[k] / s->mu0;
    }
}

/* ------------------------------------------------------------- TE update */
/* field slots: TE 0 Ex 1 Ey 2 Hz 3 Jx 4 Dx 5 Jy 6 Dy 7 Mz 8 Bz */

static void te_jd_e(of_sim *s)     /* mpiTE_UPML.c:337-375 / fdtdTE_upml.c:252-291 */
{
  cplx *Ex = s->f[0], *Ey = s->f[1], *Hz = s->f[2], *Jx = s->f[3], *Dx = s->f[4], *Jy = s->f[5], *Dy = s->f[6];
  double **c = s->c; int ny = s->ny;
  for (int i = 1; i < s->nx - 1; i++)
    for (int j = 1; j < ny - 1; j++) {
      int k = i * ny + j;
      cplx now = Jx[k];
      Jx[k] = c[0][k] * Jx[k] + c[1][k] * (Hz[k] - Hz[k - 1]);
      Dx[k] = c[2][k] * Dx[k] + c[3][k] * Jx[k] - c[4][k] * now;
    }
  for (int i = 1; i < s->nx - 1; i++)
    for (int j = 1; j < ny - 1; j++) {
      int k = i * ny + j;
      cplx now = Jy[k];
      Jy[k] = c[5][k] * Jy[k] + c[6][k] * (-Hz[k] + Hz[k - ny]);
      Dy[k] = c[7][k] * Dy[k] + c[8][k] * Jy[k] - c[9][k] * now;
    }
  for (int i = 1; i < s->nx - 1; i++)
    for (int j = 1; j < ny - 1; j++) { int k = i * ny + j; Ex[k] = Dx[k] / s->eps[0][k]; }
  for (int i = 1; i < s->nx - 1; i++)
    for (int j = 1; j < ny - 1; j++) { int k = i * ny + j; Ey[k] = Dy[k] / s->eps[1][k]; }
}

static void te_mb_h(of_sim *s)     /* mpiTE_UPML.c:377-399 / fdtdTE_upml.c:293-314 */
{
  cplx *Ex = s->f[0], *Ey = s->f[1], *Hz = s->f[2], *Mz = s->f[7], *Bz = s->f[8];
  double **c = s->c; int ny = s->ny;
  for (int i = 1; i < s->nx - 1; i++)
    for (int j = 1; j < ny - 1; j++) {
      int k = i * ny + j;
      cplx now = Mz[k];
      Mz[k] = c[10][k] * Mz[k] - c[11][k] * (Ey[k + ny] - Ey[k] - Ex[k + 1] + Ex[k]);
      Bz[k] = c[12][k] * Bz[k] + c[13][k] * Mz[k] - c[14][k] * now;
    }
  for (int i = 1; i < s->nx - 1; i++)
    for (int j = 1; j < ny - 1; j++) { int k = i * ny + j; Hz[k] = Bz[k] / s->mu0; }
}

/* ---------------------------------------------------------------- sources */

/* CW scattered-field source: mpiTM_UPML.c:337-374 (cexp form, TM) and
 * mpiTE_UPML.c:250-281 (cos + i sin form, TE on Ey); x = i-1 for one rank. */
static void cw_source(of_sim *s, cplx *p, const double *eps)
{
  double rad = s->fi.angle_deg * M_PI / 180.0;
  double ks_cos = cos(rad) * s->k_s, ks_sin = sin(rad) * s->k_s;
  double t = s->time, w = s->w_s, rc = s->ray_coef;
  for (int i = 1; i < s->nx - 1; i++)
    for (int j = 1; j < s->ny - 1; j++) {
      int k = i * s->ny + j;
      int x = i + s->ox, y = j + s->ox;
      double kr = x * ks_cos + y * ks_sin;
      if (s->tm)
        p[k] += rc * (OF_EPS0 / eps[k] - 1.0) * cexp(I * (kr - w * t));
      else
        p[k] += rc * (OF_EPS0 / eps[k] - 1) * (cos(kr - w * t) + I * sin(kr - w * t));
    }
}

/* Gaussian-pulse scattered-field source, field.c:224-256 */
static void pulse_source(of_sim *s, cplx *p, const double *eps, double gapX, double gapY, double dot)
{
  double t = s->time, w = s->w_s;
  double rad = s->fi.angle_deg * M_PI / 180.0;
  double cos_per_c = cos(rad) / s->c0, sin_per_c = sin(rad) / s->c0;
  const double beam_width = 50;
  const double center_peak = (s->n_px / 2.0 + gapX) * cos_per_c + (s->n_py / 2 + gapY) * sin_per_c;
  const double t0 = -center_peak + 500;
  for (int i = 1; i < s->n_px - 1; i++)
    for (int j = 1; j < s->n_py - 1; j++) {
      int k = i * s->n_py + j;
      if (OF_EPS0 == eps[k]) continue;
      const double r = (i + gapX) * cos_per_c + (j + gapY) * sin_per_c - (t - t0);
      const double g = exp(-pow(r / beam_width, 2));
      p[k] += dot * g * (OF_EPS0 / eps[k] - 1) * cexp(I * r * w);
    }
}

/* ------------------------------------------------------------------ NTFF */

/* mpiTM_UPML.c:840-847: three-tap retarded-time deposit, flat [360][arraySize] */
static inline void deposit(cplx *U, int stp, double time, double shift, cplx v, double coef, int scale)
{
  double t = time + shift;
  int m = (int)floor(t + 0.5);
  double a = (0.5 + t - m), b = 1.0 - a, ab = a - b;
  if (scale) {
    U[stp + m - 1] += v * b * coef;
    U[stp + m] += v * ab * coef;
    U[stp + m + 1] -= v * a * coef;
  } else {                               /* ntffTM.c:279-288 (no coef) */
    U[stp + m - 1] += v * b;
    U[stp + m] += v * ab;
    U[stp + m + 1] -= v * a;
  }
}

/* MPI NTFF, one rank: mpiTM_UPML.c:849-1037 (TM) and mpiTE_UPML.c:611-794 (TE).
 * The surface indices are used directly as padded-array indices (the
 * reference's sub-domain frame), so the box sits one cell left/below the
 * serial one in global coordinates. */
static void ntff_mpi(of_sim *s)
{
  const double C = s->c0, R = 1.0e6;
  const double coef = 1.0 / (4 * M_PI * C * R);
  const int cx = s->n_px / 2, cy = s->n_py / 2, ny = s->ny;
  const double timeE = s->time - 1, timeH = s->time - 0.5;
  const int tp = s->top, bm = s->bottom, rt = s->right, lt = s->left;
  const int sx0 = lt > 1 ? lt : 1, sx1 = rt < s->nx ? rt : s->nx;
  const int sy0 = bm > 1 ? bm : 1, sy1 = tp < s->ny ? tp : s->ny;
  for (int ang = 0; ang < 360; ang++) {
    double rad = ang * M_PI / 180.0;
    double r1x = cos(rad), r1y = sin(rad);
    const int stp = ang * s->array_size;
    if (s->tm) {
      cplx *Ez = s->f[0], *Hx = s->f[3], *Hy = s->f[6];
      cplx *Ux = s->nt[0], *Uy = s->nt[1], *Wz = s->nt[2];
      for (int i = sx0; i < sx1; i++) {          /* bottom: U=(Ez,0,0) W=(0,0,Hx) */
        double sh = -(r1x * (i - cx) + r1y * (bm - cy)) / C + s->rf;
        int k = i * ny + bm;
        deposit(Ux, stp, timeE, sh, Ez[k], coef, 1);
        deposit(Wz, stp, timeH, sh, 0.5 * (Hx[k] + Hx[k - 1]), coef, 1);
      }
      for (int j = sy0; j < sy1; j++) {          /* right: U=(0,Ez,0) W=(0,0,Hy) */
        double sh = -(r1x * (rt - cx) + r1y * (j - cy)) / C + s->rf;
        int k = rt * ny + j;
        deposit(Uy, stp, timeE, sh, Ez[k], coef, 1);
        deposit(Wz, stp, timeH, sh, 0.5 * (Hy[k] + Hy[k - ny]), coef, 1);
      }
      for (int i = sx0; i < sx1; i++) {          /* top: U=(-Ez,0,0) W=(0,0,-Hx) */
        double sh = -(r1x * (i - cx) + r1y * (tp - cy)) / C + s->rf;
        int k = i * ny + tp;
        deposit(Ux, stp, timeE, sh, -Ez[k], coef, 1);
        deposit(Wz, stp, timeH, sh, -0.5 * (Hx[k] + Hx[k - 1]), coef, 1);
      }
      for (int j = sy0; j < sy1; j++) {          /* left: U=(0,-Ez,0) W=(0,0,-Hy) */
        double sh = -(r1x * (lt - cx) + r1y * (j - cy)) / C + s->rf;
        int k = lt * ny + j;
        deposit(Uy, stp, timeE, sh, -Ez[k], coef, 1);
        deposit(Wz, stp, timeH, sh, -0.5 * (Hy[k] + Hy[k - ny]), coef, 1);
      }
    } else {
      cplx *Ex = s->f[0], *Ey = s->f[1], *Hz = s->f[2];
      cplx *Wx = s->nt[0], *Wy = s->nt[1], *Uz = s->nt[2];
      for (int i = sx0; i < sx1; i++) {          /* bottom: U=(0,0,-Ex) W=(-Hz,0,0) */
        double sh = -(r1x * (i - cx + 0.5) + r1y * (bm - cy)) / C + s->rf;
        int k = i * ny + bm;
        deposit(Uz, stp, timeE, sh, -Ex[k], coef, 1);
        deposit(Wx, stp, timeH, sh, -0.5 * (Hz[k] + Hz[k - 1]), coef, 1);
      }
      for (int j = sy0; j < sy1; j++) {          /* right: U=(0,0,-Ey) W=(0,-Hz,0) */
        double sh = -(r1x * (rt - cx) + r1y * (j - cy + 0.5)) / C + s->rf;
        int k = rt * ny + j;
        deposit(Uz, stp, timeE, sh, -Ey[k], coef, 1);
        deposit(Wy, stp, timeH, sh, -0.5 * (Hz[k] + Hz[k - ny]), coef, 1);
      }
      for (int i = sx0; i < sx1; i++) {          /* top: U=(0,0,Ex) W=(Hz,0,0) */
        double sh = -(r1x * (i - cx + 0.5) + r1y * (tp - cy)) / C + s->rf;
        int k = i * ny + tp;
        deposit(Uz, stp, timeE, sh, Ex[k], coef, 1);
        deposit(Wx, stp, timeH, sh, 0.5 * (Hz[k] + Hz[k - 1]), coef, 1);
      }
      for (int j = sy0; j < sy1; j++) {          /* left: U=(0,0,Ey) W=(0,Hz,0) */
        double sh = -(r1x * (lt - cx) + r1y * (j - cy + 0.5)) / C + s->rf;
        int k = lt * ny + j;
        deposit(Uz, stp, timeE, sh, Ey[k], coef, 1);
        deposit(Wy, stp, timeH, sh, 0.5 * (Hz[k] + Hz[k - ny]), coef, 1);
      }
    }
  }
}

/* Serial NTFF: ntffTM.c:293-371 (TM) and ntffTE.c:68-157 (TE).  The retarded
 * time along a side is advanced incrementally, as the reference does. */
static void ntff_serial(of_sim *s)
{
  const int ny = s->n_py;
  const double timeE = s->time - 1, timeH = s->time - 0.5;
  const double lt_cx = s->left - s->cx, rt_cx = s->right - s->cx;
  const double bm_cy = s->bottom - s->cy, tp_cy = s->top - s->cy;
  const int lb = s->left * ny + s->bottom, ltp = s->left * ny + s->top;
  const int rb = s->right * ny + s->bottom, rtp = s->right * ny + s->top;
  for (int ang = 0; ang < 360; ang++) {
    double rad = ang * (M_PI / 180.0);
    double r1x = cos(rad) / s->c0, r1y = sin(rad) / s->c0;
    const int stp = ang * s->array_size;
    if (s->tm) {
      cplx *Ez = s->f[0], *Hx = s->f[3], *Hy = s->f[6];
      cplx *Ux = s->nt[0], *Uy = s->nt[1], *Wz = s->nt[2];
      double sh = -(r1x * lt_cx + r1y * bm_cy) + s->rf;
      for (int k = lb; k < rb; k += ny) {        /* bottom */
        deposit(Ux, stp, timeE, sh, Ez[k], 0, 0);
        deposit(Wz, stp, timeH, sh, 0.5 * (Hx[k] + Hx[k - 1]), 0, 0);
        sh -= r1x;
      }
      sh = -(r1x * rt_cx + r1y * bm_cy) + s->rf;
      for (int k = rb; k < rtp; k++) {           /* right */
        deposit(Uy, stp, timeE, sh, Ez[k], 0, 0);
        deposit(Wz, stp, timeH, sh, 0.5 * (Hy[k] + Hy[k - ny]), 0, 0);
        sh -= r1y;
      }
      sh = -(r1x * lt_cx + r1y * tp_cy) + s->rf;
      for (int k = ltp; k < rtp; k += ny) {      /* top */
        deposit(Ux, stp, timeE, sh, -Ez[k], 0, 0);
        deposit(Wz, stp, timeH, sh, -0.5 * (Hx[k] + Hx[k - 1]), 0, 0);
        sh -= r1x;
      }
      sh = -(r1x * lt_cx + r1y * bm_cy) + s->rf;
      for (int k = lb; k < ltp; k++) {           /* left */
        deposit(Uy, stp, timeE, sh, -Ez[k], 0, 0);
        deposit(Wz, stp, timeH, sh, -0.5 * (Hy[k] + Hy[k - ny]), 0, 0);
        sh -= r1y;
      }
    } else {
      cplx *Ex = s->f[0], *Ey = s->f[1], *Hz = s->f[2];
      cplx *Wx = s->nt[0], *Wy = s->nt[1], *Uz = s->nt[2];
      double sh = -(r1x * (lt_cx + 0.5) + r1y * bm_cy) + s->rf;
      for (int k = lb; k < rb; k += ny) {        /* bottom */
        deposit(Uz, stp, timeE, sh, -Ex[k], 0, 0);
        deposit(Wx, stp, timeH, sh, -0.5 * (Hz[k] + Hz[k - 1]), 0, 0);
        sh -= r1x;
      }
      sh = -(r1x * rt_cx + r1y * (bm_cy + 0.5)) + s->rf;
      for (int k = rb; k < rtp; k++) {           /* right */
        deposit(Uz, stp, timeE, sh, -Ey[k], 0, 0);
        deposit(Wy, stp, timeH, sh, -0.5 * (Hz[k] + Hz[k - ny]), 0, 0);
        sh -= r1y;
      }
      sh = -(r1x * (lt_cx + 0.5) + r1y * tp_cy) + s->rf;
      for (int k = ltp; k < rtp; k += ny) {      /* top */
        deposit(Uz, stp, timeE, sh, Ex[k], 0, 0);
        deposit(Wx, stp, timeH, sh, 0.5 * (Hz[k] + Hz[k - 1]), 0, 0);
        sh -= r1x;
      }
      sh = -(r1x * lt_cx + r1y * (bm_cy + 0.5)) + s->rf;
      for (int k = lb; k < ltp; k++) {           /* left */
        deposit(Uz, stp, timeE, sh, Ey[k], 0, 0);
        deposit(Wy, stp, timeH, sh, 0.5 * (Hz[k] + Hz[k - ny]), 0, 0);
        sh -= r1y;
      }
    }
  }
}

/* ------------------------------------------- split-field PML and NS-FDTD */
/* fdtdTM.c, fdtdTE.c, nsFdtdTM.c, nsFdtdTE.c on the N_PX x N_PY frame.
 * field slots: TM 0 Ez 1 Ezx 2 Ezy 3 Hx 4 Hy ; TE 0 Ex 1 Ey 2 Hz 3 Hzx 4 Hzy
 * coefficients, as the reference names them:
 *   TM 0 C_EZX 1 C_EZXLX 2 C_EZY 3 C_EZYLY 4 C_HX 5 C_HXLY 6 C_HY 7 C_HYLX
 *   TE 0 C_EX 1 C_EXLY 2 C_EY 3 C_EYLX 4 C_HZX 5 C_HZXLX 6 C_HZY 7 C_HZYLY */

static double pml_coef(double ep_mu, double sig) { return (1.0 - sig / ep_mu) / (1.0 + sig / ep_mu); } /* field.c:288-291 */
static double pml_lxy(double ep_mu, double sig) { return 1.0 / (ep_mu + sig); }                      /* field.c:292-295 */
static double ns_beta(double a) { return tanh(a) / (1 + pow(tanh(a), 2)); }                          /* nsFdtdTM.c:221-224 */
static double ns_coef1(double a, double b) { return (1 - b) / (1 + b); }                              /* nsFdtdTM.c:226-229 */
static double ns_u(const of_sim *s, double e)   /* sin(w/2) / sin(k n / 2), n = sqrt(eps) */
{
  double n = sqrt(e / OF_EPS0);
  double k = s->k_s * n;
  return sin(s->w_s * 0.5) / sin(k * 0.5);
}

static void coefficients_split(of_sim *s)
{
  const double R = 1.0e-8, M = 2.0;
  double **c = s->c, **e = s->eps;
  const int NX = s->n_px, NY = s->n_py;
  if (s->solver == OF_TM_2D) {                        /* fdtdTM.c:167-242 */
    const double sig_max = -(M + 1.0) * OF_EPS0 * OF_C / 2.0 / s->n_pml * log(R);
    for (int i = 0; i < NX; i++)
      for (int j = 0; j < NY; j++) {
        int k = i * NY + j;
        e[0][k] = meps(s, i, j, DXY_);
        e[1][k] = meps(s, i, j + 0.5, DY_);
        e[2][k] = meps(s, i + 0.5, j, DX_);
        double sig_ez_x = sig_max * sigma_x(s, i), sig_ez_y = sig_max * sigma_y(s, j);
        double sig_hx_y = sig_max * sigma_y(s, j + 0.5), sig_hx_yy = OF_MU0 / OF_EPS0 * sig_hx_y;
        double sig_hy_x = sig_max * sigma_x(s, i + 0.5), sig_hy_xx = OF_MU0 / OF_EPS0 * sig_hy_x;
        c[0][k] = pml_coef(e[0][k], sig_ez_x);
        c[1][k] = pml_lxy(e[0][k], sig_ez_x);
        c[2][k] = pml_coef(e[0][k], sig_ez_y);
        c[3][k] = pml_lxy(e[0][k], sig_ez_y);
        c[4][k] = pml_coef(OF_MU0, sig_hx_yy);
        c[5][k] = pml_lxy(OF_MU0, sig_hx_yy);
        c[6][k] = pml_coef(OF_MU0, sig_hy_xx);
        c[7][k] = pml_lxy(OF_MU0, sig_hy_xx);
      }
  } else if (s->solver == OF_TE_2D) {                 /* fdtdTE.c:170-238 */
    const double sig_max = -(M + 1.0) * OF_EPS0 * OF_C / 2.0 / s->n_pml * log(R);
    for (int i = 0; i < NX; i++)
      for (int j = 0; j < NY; j++) {
        int k = i * NY + j;
        e[0][k] = meps(s, i + 0.5, j, DY_);
        e[1][k] = meps(s, i, j + 0.5, DX_);
        e[2][k] = 0.5 * (meps(s, i + 0.5, j + 0.5, DX_) + meps(s, i + 0.5, j + 0.5, DY_));
        double sig_ex_y = sig_max * sigma_y(s, j), sig_ey_x = sig_max * sigma_x(s, i);
        double sig_hz_xx = OF_MU0 / OF_EPS0 * (sig_max * sigma_x(s, i + 0.5));
        double sig_hz_yy = OF_MU0 / OF_EPS0 * (sig_max * sigma_y(s, j + 0.5));
        c[0][k] = pml_coef(e[0][k], sig_ex_y);
        c[1][k] = pml_lxy(e[0][k], sig_ex_y);
        c[2][k] = pml_coef(e[1][k], sig_ey_x);
        c[3][k] = pml_lxy(e[1][k], sig_ey_x);
        c[4][k] = pml_coef(OF_MU0, sig_hz_xx);
        c[5][k] = pml_lxy(OF_MU0, sig_hz_xx);
        c[6][k] = pml_coef(OF_MU0, sig_hz_yy);
        c[7][k] = pml_lxy(OF_MU0, sig_hz_yy);
      }
  } else if (s->solver == OF_NS_TM_2D) {              /* nsFdtdTM.c:231-307 */
    const double sig_max = -(M + 1.0) * OF_EPS0 * OF_C / s->n_pml * log(R);
    for (int i = 0; i < NX; i++)
      for (int j = 0; j < NY; j++) {
        int k = i * NY + j;
        e[0][k] = meps(s, i, j, DXY_);
        e[1][k] = meps(s, i, j + 0.5, DY_);
        e[2][k] = meps(s, i + 0.5, j, DX_);
        double sig_ez_x = sig_max * sigma_x(s, i), sig_ez_y = sig_max * sigma_y(s, j);
        double sig_hx_y = sig_max * sigma_y(s, j + 0.5), sig_hy_x = sig_max * sigma_x(s, i + 0.5);
        double a_hx_y = sig_hx_y / (2 * OF_EPS0), a_hy_x = sig_hy_x / (2 * OF_EPS0);
        double a_ez_x = sig_ez_x / (2 * OF_EPS0), a_ez_y = sig_ez_y / (2 * OF_EPS0);
        double b_hx_y = ns_beta(a_hx_y), b_hy_x = ns_beta(a_hy_x), b_ez_x = ns_beta(a_ez_x), b_ez_y = ns_beta(a_ez_y);
        double z_ez = sqrt(OF_MU0 / e[0][k]), u_ez = ns_u(s, e[0][k]);
        c[0][k] = ns_coef1(a_ez_x, b_ez_x);
        c[1][k] = u_ez * z_ez / (1 + b_ez_x);
        c[2][k] = ns_coef1(a_ez_y, b_ez_y);
        c[3][k] = u_ez * z_ez / (1.0 + b_ez_x);        /* nsFdtdTM.c:287: b_ez_x, as written */
        double z_hx = sqrt(OF_MU0 / e[1][k]), u_hx = ns_u(s, e[1][k]);
        c[4][k] = ns_coef1(a_hx_y, b_hx_y);
        c[5][k] = u_hx / z_hx / (1.0 + b_hx_y);
        double z_hy = sqrt(OF_MU0 / e[2][k]), u_hy = ns_u(s, e[2][k]);
        c[6][k] = ns_coef1(a_hy_x, b_hy_x);
        c[7][k] = u_hy / z_hy / (1.0 + b_hy_x);
      }
  } else {                                            /* nsFdtdTE.c:100-181, inner cells only */
    const double sig_max = -(M + 1.0) * OF_EPS0 * OF_C / s->n_pml * log(R);
    for (int i = 1; i < NX - 1; i++)
      for (int j = 1; j < NY - 1; j++) {
        int k = i * NY + j;
        e[0][k] = meps(s, i + 0.5, j, DY_);
        e[1][k] = meps(s, i, j + 0.5, DX_);
        e[2][k] = meps(s, i + 0.5, j + 0.5, DXY_);
        double sig_ex_y = sig_max * sigma_y(s, j), sig_ey_x = sig_max * sigma_x(s, i);
        double sig_hz_x = sig_max * sigma_x(s, i + 0.5), sig_hz_y = sig_max * sigma_y(s, j + 0.5);
        double a_ex_y = sig_ex_y / (2 * e[0][k]), a_ey_x = sig_ey_x / (2 * e[1][k]);
        double a_hz_x = sig_hz_x / (2 * e[2][k]), a_hz_y = sig_hz_y / (2 * e[2][k]);
        double b_ex_y = ns_beta(a_ex_y), b_ey_x = ns_beta(a_ey_x), b_hz_x = ns_beta(a_hz_x), b_hz_y = ns_beta(a_hz_y);
        double z_hz = sqrt(OF_MU0 / e[2][k]), u_hz = ns_u(s, e[2][k]);
        c[4][k] = ns_coef1(a_hz_x, b_hz_x);
        c[5][k] = u_hz / z_hz / (1.0 + b_hz_x);
        c[6][k] = ns_coef1(a_hz_y, b_hz_y);
        c[7][k] = u_hz / z_hz / (1.0 + b_hz_y);
        double z_ex = sqrt(OF_MU0 / e[0][k]), u_ex = ns_u(s, e[0][k]);
        c[0][k] = ns_coef1(a_ex_y, b_ex_y);
        c[1][k] = u_ex * z_ex / (1.0 + b_ex_y);
        double z_ey = sqrt(OF_MU0 / e[1][k]), u_ey = ns_u(s, e[1][k]);
        c[2][k] = ns_coef1(a_ey_x, b_ey_x);
        c[3][k] = u_ey * z_ey / (1.0 + b_ey_x);
      }
  }
}

/* field_scatteredWaveNotUPML (field.c:179-196) and field_nsScatteredWaveNotUPML
 * (field.c:155-177): the CW source of the split-field / NS solvers on cells
 * 1..N-2 of the global frame */
static void wave_not_upml(of_sim *s, cplx *p, const double *eps, double gx, double gy)
{
  double rad = s->fi.angle_deg * M_PI / 180.0;
  double ks_cos = cos(rad) * s->k_s, ks_sin = sin(rad) * s->k_s;
  for (int i = 1; i < s->n_px - 1; i++)
    for (int j = 1; j < s->n_py - 1; j++) {
      int k = i * s->n_py + j;
      double kr = (i + gx) * ks_cos + (j + gy) * ks_sin;
      p[k] += s->ray_coef * (OF_EPS0 / eps[k] - 1.0) *
              (cexp(I * (kr - s->w_s * (s->time + 0.5))) - cexp(I * (kr - s->w_s * (s->time - 0.5))));
    }
}
static void ns_wave_not_upml(of_sim *s, cplx *p, const double *eps, double gx, double gy, double dot)
{
  double ray_coef = s->ray_coef * dot;
  double rad = s->fi.angle_deg * M_PI / 180.0;
  double ks_cos = cos(rad) * s->k_s, ks_sin = sin(rad) * s->k_s;
  for (int i = 1; i < s->n_px - 1; i++)
    for (int j = 1; j < s->n_py - 1; j++) {
      int k = i * s->n_py + j;
      double kr = (i + gx) * ks_cos + (j + gy) * ks_sin;
      double n = sqrt(eps[k] / OF_EPS0);
      double u0 = sin(s->w_s * 0.5) / sin(s->k_s * 0.5);
      double u1 = sin(s->w_s * 0.5) / sin(n * s->k_s * 0.5);
      double _n = u0 / u1;
      p[k] += ray_coef * (1.0 / (_n * n) - 1.0) *
              (cexp(I * (kr - s->w_s * (s->time + 1.0))) - cexp(I * (kr - s->w_s * (s->time))));
    }
}

#define SPLIT_FOR for (int i = 1; i < s->n_px - 1; i++) for (int j = 1; j < s->n_py - 1; j++)

static void update_split(of_sim *s)
{
  const int NY = s->n_py, dx = NY, dy = 1;
  cplx **f = s->f;
  double **c = s->c;
  if (s->solver == OF_TM_2D) {                       /* fdtdTM.c:290-327 */
    cplx *Ez = f[0], *Ezx = f[1], *Ezy = f[2], *Hx = f[3], *Hy = f[4];
    SPLIT_FOR { int k = i * NY + j; Hx[k] = c[4][k] * Hx[k] - c[5][k] * (Ezx[k + 1] - Ezx[k] + Ezy[k + 1] - Ezy[k]); }
    SPLIT_FOR { int k = i * NY + j; Hy[k] = c[6][k] * Hy[k] + c[7][k] * (Ezx[k + dx] - Ezx[k] + Ezy[k + dx] - Ezy[k]); }
    SPLIT_FOR { int k = i * NY + j; Ezx[k] = c[0][k] * Ezx[k] + c[1][k] * (Hy[k] - Hy[k - dx]); }
    SPLIT_FOR { int k = i * NY + j; Ezy[k] = c[2][k] * Ezy[k] - c[3][k] * (Hx[k] - Hx[k - 1]); }
    SPLIT_FOR { int k = i * NY + j; Ez[k] = Ezx[k] + Ezy[k]; }
    wave_not_upml(s, Ezx, s->eps[0], 0.0, 0.0);
  } else if (s->solver == OF_TE_2D) {                /* fdtdTE.c:283-321 */
    cplx *Ex = f[0], *Ey = f[1], *Hz = f[2], *Hzx = f[3], *Hzy = f[4];
    SPLIT_FOR { int k = i * NY + j; Ex[k] = c[0][k] * Ex[k] + c[1][k] * (Hzx[k] - Hzx[k - 1] + Hzy[k] - Hzy[k - 1]); }
    SPLIT_FOR { int k = i * NY + j; Ey[k] = c[2][k] * Ey[k] - c[3][k] * (Hzx[k] - Hzx[k - dx] + Hzy[k] - Hzy[k - dx]); }
    wave_not_upml(s, Ey, s->eps[1], 0.0, 0.5);
    SPLIT_FOR { int k = i * NY + j; Hzx[k] = c[4][k] * Hzx[k] - c[5][k] * (Ey[k + dx] - Ey[k]); }
    SPLIT_FOR { int k = i * NY + j; Hzy[k] = c[6][k] * Hzy[k] + c[7][k] * (Ex[k + 1] - Ex[k]); }
    SPLIT_FOR { int k = i * NY + j; Hz[k] = Hzx[k] + Hzy[k]; }
  } else if (s->solver == OF_NS_TM_2D) {             /* nsFdtdTM.c:68-151 */
    cplx *Ez = f[0], *Ezx = f[1], *Ezy = f[2], *Hx = f[3], *Hy = f[4];
    double k_s = s->k_s;
    double r = 1.0 / 6.0 + k_s * k_s / 180.0 - pow(k_s, 4) / 23040, r_2 = r / 2.0;
    SPLIT_FOR {
      int k = i * NY + j;
      cplx ns = r_2 * ((Ez[k + dy + dx] + Ez[k + dy - dx] - 2 * Ez[k + dy]) - (Ez[k + dx] + Ez[k - dx] - 2 * Ez[k]));
      Hx[k] = c[4][k] * Hx[k] - c[5][k] * (Ez[k + dy] - Ez[k] + ns);
    }
    SPLIT_FOR {
      int k = i * NY + j;
      cplx ns = r_2 * ((Ez[k + dx + dy] + Ez[k + dx - dy] - 2 * Ez[k + dx]) - (Ez[k + dy] + Ez[k - dy] - 2 * Ez[k]));
      Hy[k] = c[6][k] * Hy[k] + c[7][k] * (Ez[k + dx] - Ez[k] + ns);
    }
    SPLIT_FOR { int k = i * NY + j; Ezx[k] = c[0][k] * Ezx[k] + c[1][k] * (Hy[k] - Hy[k - dx]); }
    SPLIT_FOR { int k = i * NY + j; Ezy[k] = c[2][k] * Ezy[k] - c[3][k] * (Hx[k] - Hx[k - dy]); }
    ns_wave_not_upml(s, Ezy, s->eps[0], 0, 0, 1.0);
    SPLIT_FOR { int k = i * NY + j; Ez[k] = Ezx[k] + Ezy[k]; }
  } else {                                           /* nsFdtdTE.c:233-308 */
    cplx *Ex = f[0], *Ey = f[1], *Hz = f[2], *Hzx = f[3], *Hzy = f[4];
    SPLIT_FOR { int k = i * NY + j; Hzx[k] = c[4][k] * Hzx[k] - c[5][k] * (Ey[k + dx] - Ey[k]); }
    SPLIT_FOR { int k = i * NY + j; Hzy[k] = c[6][k] * Hzy[k] + c[7][k] * (Ex[k + dy] - Ex[k]); }
    SPLIT_FOR { int k = i * NY + j; Hz[k] = Hzx[k] + Hzy[k]; }
    double k_s = s->k_s;
    double r = 1.0 / 6.0 + k_s * k_s / 180.0 - pow(k_s, 4) / 23040, r_2 = r / 2.0;
    SPLIT_FOR {
      int k = i * NY + j;
      cplx ns = r_2 * ((Hz[k + dx] + Hz[k - dx] - 2 * Hz[k]) - (Hz[k - dy + dx] + Hz[k - dy - dx] - 2 * Hz[k - dy]));
      Ex[k] = c[0][k] * Ex[k] + c[1][k] * (Hz[k] - Hz[k - dy] + ns);
    }
    SPLIT_FOR {
      int k = i * NY + j;
      cplx ns = r_2 * ((Hz[k + dy] + Hz[k - dy] - 2 * Hz[k]) - (Hz[k - dx + dy] + Hz[k - dx - dy] - 2 * Hz[k - dx]));
      Ey[k] = c[2][k] * Ey[k] - c[3][k] * (Hz[k] - Hz[k - dx] + ns);
    }
    double co = cos((s->fi.angle_deg + 90) * M_PI / 180.0);
    double si = sin((s->fi.angle_deg + 90) * M_PI / 180.0);
    if (co != 0.0) ns_wave_not_upml(s, Ex, s->eps[0], 0, 0.5, co);
    if (si != 0.0) ns_wave_not_upml(s, Ey, s->eps[1], 0, 0.5, si);
  }
}
#undef SPLIT_FOR

/* ------------------------------------------------------------------ step */

static void update(of_sim *s)
{
  if (s->family) {
    update_split(s);
    return;
  }
  if (s->mpi) {
    /* mpiTM_UPML.c:196-217 / mpiTE_UPML.c:290-304 (halo exchange is a no-op
     * for one rank; the halos stay zero) */
    if (s->tm) { tm_jd_e(s); cw_source(s, s->f[0], s->eps[0]); tm_mb_h(s); }
    else       { te_jd_e(s); cw_source(s, s->f[1], s->eps[1]); te_mb_h(s); }
    if (!s->skip_ntff) ntff_mpi(s);
  } else if (s->tm) {      /* fdtdTM_upml.c:54-66 */
    tm_mb_h(s); tm_jd_e(s);
    pulse_source(s, s->f[0], s->eps[0], 0, 0, 1.0);
    ntff_serial(s);
  } else {                 /* fdtdTE_upml.c:168-192 */
    te_mb_h(s); te_jd_e(s);
    double co = cos((s->fi.angle_deg + 90) * M_PI / 180.0);
    double si = sin((s->fi.angle_deg + 90) * M_PI / 180.0);
    if (co != 0.0) pulse_source(s, s->f[0], s->eps[0], 0.5, 0.0, co);
    if (si != 0.0) pulse_source(s, s->f[1], s->eps[1], 0.0, 0.5, si);
    ntff_serial(s);
  }
}

void of_step(of_sim *s, int n)
{
  for (int q = 0; q < n; q++) {
    update(s);
    s->time += 1.0;                                        /* field.c:312-315 */
    s->ray_coef = 1.0 - exp(-pow(0.01 * s->time, 2));
  }
}

double of_time(const of_sim *s) { return s->time; }
void of_dims(const of_sim *s, int *nx, int *ny, int *n_px, int *n_py)
{ *nx = s->nx; *ny = s->ny; *n_px = s->n_px; *n_py = s->n_py; }
double *of_field(of_sim *s, int which)
{
  static const int tm_slot[3] = {0, 3, 6}, te_slot[3] = {0, 1, 2}, split_tm_slot[3] = {0, 3, 4};
  if (which < 0 || which > 2) return NULL;
  if (s->family) return (double *)s->f[s->tm ? split_tm_slot[which] : te_slot[which]];
  return (double *)s->f[s->tm ? tm_slot[which] : te_slot[which]];
}
double *of_eps(of_sim *s, int which) { return (which >= 0 && which < 3) ? s->eps[which] : NULL; }
int of_ntff_info(const of_sim *s, int *top, int *bottom, int *left, int *right, int *cx, int *cy, double *rf)
{
  *top = s->top; *bottom = s->bottom; *left = s->left; *right = s->right; *cx = s->cx; *cy = s->cy; *rf = s->rf;
  return s->array_size;
}
int of_array_size(const of_sim *s) { return s->array_size; }
int of_ntff_guard(void) { return OF_GUARD; }
double *of_ntff(of_sim *s, int which) { return (which >= 0 && which < 3 && !s->family) ? (double *)s->nt_base[which] : NULL; }

/* ------------------------------------------------------- spectrum output */

/* Radix-2 FFT with the sign of the reference's cfft() (cfft.c:104-179,
 * flag 0): X[k] = sum_n x[n] exp(+2 pi i n k / N), no scaling. */
static void fft_pos(cplx *a, int n)
{
  for (int i = 1, j = 0; i < n; i++) {                 /* bit reversal */
    int bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) { cplx t = a[i]; a[i] = a[j]; a[j] = t; }
  }
  for (int len = 2; len <= n; len <<= 1) {             /* decimation in time */
    int half = len >> 1;
    for (int k = 0; k < half; k++) {
      cplx w = cexp(I * (M_PI * k / half));
      for (int st = 0; st < n; st += len) {
        cplx u = a[st + k], v = a[st + k + half] * w;
        a[st + k] = u + v;
        a[st + k + half] = u - v;
      }
    }
  }
}

/* ntffTM.c:161-275 / ntffTE.c:20-55,160-238.  TM transforms E_theta, TE E_phi. */
int of_time_output(of_sim *s, double *out)
{
  if (s->family) return -1;  /* no NTFF */
  const int maxTime = (int)s->max_time;
  if (maxTime > OF_NFFT) return -1;
  const double complex coef = 1.0 / (4 * M_PI * s->c0) * csqrt(2 * M_PI * s->c0 / (I * s->w_s));
  cplx *buf = (cplx *)malloc(sizeof(cplx) * OF_NFFT);
  for (int ang = 0; ang < 360; ang++) {
    double phi = ang * (M_PI / 180.0), theta = 0;
    double sx = cos(theta) * cos(phi), sy = cos(theta) * sin(phi), sz = -cos(theta);
    double px = -sin(phi), py = cos(phi);
    int k = ang * s->array_size;
    memset(buf, 0, sizeof(cplx) * OF_NFFT);
    for (int i = 0; i < maxTime; i++) {
      if (s->tm) {
        cplx Ux = s->nt[0][k + i], Uy = s->nt[1][k + i], Wz = s->nt[2][k + i];
        cplx WTH = Wz * sz, UPH = Ux * px + Uy * py;
        buf[i] = coef * (-s->z0 * WTH - UPH);                 /* E_theta */
      } else {
        cplx Wx = s->nt[0][k + i], Wy = s->nt[1][k + i], Uz = s->nt[2][k + i];
        cplx WPH = Wx * px + Wy * py, UTH = Uz * sz;
        buf[i] = coef * (-s->z0 * WPH + UTH);                 /* E_phi */
        (void)sx; (void)sy;
      }
    }
    fft_pos(buf, OF_NFFT);
    for (int lam = OF_LAMBDA_ST; lam <= OF_LAMBDA_EN; lam++) {
      double p = s->c0 * s->fi.h_u_nm * OF_NFFT / lam;
      int idx = (int)floor(p);
      p = p - idx;
      double n0 = creal(buf[idx]) * creal(buf[idx]) + cimag(buf[idx]) * cimag(buf[idx]);
      double n1 = creal(buf[idx + 1]) * creal(buf[idx + 1]) + cimag(buf[idx + 1]) * cimag(buf[idx + 1]);
      out[(lam - OF_LAMBDA_ST) * 360 + ang] = ((1 - p) * n0 + p * n1) / OF_NFFT;
    }
  }
  free(buf);
  return 0;
}

/* ntffTE.c:242-338 (E_phi of the H-polarised far field) on global-frame Ex,
 * Ey, Hz.  The shipped function reads the bottom side through field_index and
 * the other three through field_subIndex, whose SUB_N_PY stays 0 because
 * field_init no longer calls mpiSplit (field.c:112); here all four sides use
 * the global index, as ntffTM_Frequency does.  Everything else follows the
 * shipped loops: the bottom side runs lt..rt inclusive, the others stop before
 * rt / tp, path points sit half a cell along the side (r2 = i-cx+0.5 or
 * j-cy+0.5), and the result scales by h_u_nm (not its square root). */
static void frequency_te(const of_sim *s, const cplx *Ex, const cplx *Ey, const cplx *Hz, int NY, double *out)
{
  const double cx = s->cx, cy = s->cy, k_s = s->k_s;
  const double R0 = 1.0e6 * (500.0 / s->fi.h_u_nm);
  const double complex coef = csqrt(I * k_s / (8 * M_PI * R0)) * cexp(I * k_s * R0);
  const int tp = s->top, bm = s->bottom, rt = s->right, lt = s->left;
  for (int ang = 0; ang < 360; ang++) {
    double rad = ang * M_PI / 180.0, rx = cos(rad), ry = sin(rad);
    cplx Nx = 0, Ny = 0, Lz = 0;
    for (int i = lt; i <= rt; i++) {                       /* n = (0,-1) */
      int k = i * NY + bm;
      cplx e = cexp(I * k_s * (rx * (i - cx + 0.5) + ry * (bm - cy)));
      Nx -= 0.5 * (Hz[k] + Hz[k - 1]) * e; Lz -= Ex[k] * e;
    }
    for (int j = bm; j < tp; j++) {                        /* n = (1,0) */
      int k = rt * NY + j;
      cplx e = cexp(I * k_s * (rx * (rt - cx) + ry * (j - cy + 0.5)));
      Ny -= 0.5 * (Hz[k] + Hz[k - NY]) * e; Lz -= Ey[k] * e;
    }
    for (int i = lt; i < rt; i++) {                        /* n = (0,1) */
      int k = i * NY + tp;
      cplx e = cexp(I * k_s * (rx * (i - cx + 0.5) + ry * (tp - cy)));
      Nx += 0.5 * (Hz[k] + Hz[k - 1]) * e; Lz += Ex[k] * e;
    }
    for (int j = bm; j < tp; j++) {                        /* n = (-1,0) */
      int k = lt * NY + j;
      cplx e = cexp(I * k_s * (rx * (lt - cx) + ry * (j - cy + 0.5)));
      Ny += 0.5 * (Hz[k] + Hz[k - NY]) * e; Lz += Ey[k] * e;
    }
    cplx Nphi = -Nx * sin(rad) + Ny * cos(rad);
    cplx r = coef * (s->z0 * Nphi - Lz) * s->fi.h_u_nm;
    out[2 * ang] = creal(r); out[2 * ang + 1] = cimag(r);
  }
}

/* ntffTM.c:72-158 (TM) or ntffTE.c:242-338 (TE, frequency_te) on
 * global-frame fields (for the MPI solvers the one-rank sub-domain is
 * gathered to global x = i-1 first). */
int of_frequency(of_sim *s, double *out)
{
  if (s->family) return -1;  /* no NTFF */
  const int NX = s->n_px, NY = s->n_py;
  cplx *g[3];
  for (int q = 0; q < 3; q++) {
    g[q] = (cplx *)malloc(sizeof(cplx) * NX * NY);
    const cplx *src = (const cplx *)of_field(s, q);
    for (int x = 0; x < NX; x++)
      for (int y = 0; y < NY; y++)
        g[q][x * NY + y] = s->mpi ? src[(x + 1) * s->ny + (y + 1)] : src[x * NY + y];
  }
  if (!s->tm) {
    frequency_te(s, g[0], g[1], g[2], NY, out);
    for (int q = 0; q < 3; q++) free(g[q]);
    return 0;
  }
  cplx *Ez = g[0], *Hx = g[1], *Hy = g[2];
  const double cx = s->cx, cy = s->cy, k_s = s->k_s;
  const double R0 = 1.0e6 * (500.0 / s->fi.h_u_nm);
  const double complex coef = csqrt(I * k_s / (8 * M_PI * R0)) * cexp(I * k_s * R0);
  const int tp = s->top, bm = s->bottom, rt = s->right, lt = s->left;
  for (int ang = 0; ang < 360; ang++) {
    double rad = ang * M_PI / 180.0, rx = cos(rad), ry = sin(rad);
    cplx Nz = 0, Lx = 0, Ly = 0;
    for (int i = lt; i < rt; i++) {
      int k = i * NY + bm;
      cplx e = cexp(I * k_s * (rx * (i - cx) + ry * (bm - cy)));
      Nz += 0.5 * (Hx[k] + Hx[k - 1]) * e; Lx += Ez[k] * e;
    }
    for (int j = bm; j < tp; j++) {
      int k = rt * NY + j;
      cplx e = cexp(I * k_s * (rx * (rt - cx) + ry * (j - cy)));
      Nz += 0.5 * (Hy[k] + Hy[k - NY]) * e; Ly += Ez[k] * e;
    }
    for (int i = lt; i < rt; i++) {
      int k = i * NY + tp;
      cplx e = cexp(I * k_s * (rx * (i - cx) + ry * (tp - cy)));
      Nz -= 0.5 * (Hx[k] + Hx[k - 1]) * e; Lx -= Ez[k] * e;
    }
    for (int j = bm; j < tp; j++) {
      int k = lt * NY + j;
      cplx e = cexp(I * k_s * (rx * (lt - cx) + ry * (j - cy)));
      Nz -= 0.5 * (Hy[k] + Hy[k - NY]) * e; Ly -= Ez[k] * e;
    }
    cplx Lphi = -Lx * sin(rad) + Ly * cos(rad);
    cplx r = coef * (s->z0 * Nz + Lphi) * sqrt((double)s->fi.h_u_nm);
    out[2 * ang] = creal(r); out[2 * ang + 1] = cimag(r);
  }
  for (int q = 0; q < 3; q++) free(g[q]);
  return 0;
}

/* ------------------------------------------------------------ CPU bench */

typedef struct {
  int solver, steps, skip_ntff; of_field_info fi; of_model m;
  pthread_barrier_t *bar; of_sim *sim;
} bench_arg;

static void *bench_worker(void *p)
{
  bench_arg *a = (bench_arg *)p;
  a->sim = of_create(a->solver, &a->fi, &a->m);
  if (a->sim) a->sim->skip_ntff = a->skip_ntff;
  pthread_barrier_wait(a->bar);         /* setup done everywhere */
  if (a->sim) of_step(a->sim, a->steps);
  pthread_barrier_wait(a->bar);         /* stepping done everywhere */
  return NULL;
}

static double now_s(void)
{
  struct timespec ts; clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

double of_bench(int solver, const of_field_info *fi, const of_model *m, int steps, int n_threads)
{
  return of_bench_opts(solver, fi, m, steps, n_threads, 0);
}

/* flags bit 0: the MPI solvers skip their time-domain NTFF, so that the
 * stencil's and the NTFF's shares of a step can be told apart. */
double of_bench_opts(int solver, const of_field_info *fi, const of_model *m, int steps, int n_threads, int flags)
{
  if (n_threads < 1) n_threads = 1;
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * n_threads);
  bench_arg *args = (bench_arg *)calloc(n_threads, sizeof(bench_arg));
  pthread_barrier_t bar;
  pthread_barrier_init(&bar, NULL, n_threads + 1);
  for (int t = 0; t < n_threads; t++) {
    args[t].solver = solver; args[t].steps = steps; args[t].fi = *fi; args[t].skip_ntff = flags & 1;
    if (m) args[t].m = *m;
    args[t].bar = &bar;
    pthread_create(&th[t], NULL, bench_worker, &args[t]);
  }
  pthread_barrier_wait(&bar);
  double t0 = now_s();
  pthread_barrier_wait(&bar);
  double dt = now_s() - t0;
  int ok = 1;
  for (int t = 0; t < n_threads; t++) {
    pthread_join(th[t], NULL);
    if (!args[t].sim) ok = 0;
    of_destroy(args[t].sim);
  }
  pthread_barrier_destroy(&bar);
  free(th); free(args);
  return ok ? dt : -1.0;
}
