/*
 * models_eval.h -- permittivity of the reference's built-in models at one
 * staggered point, usable from host C/C++ and from CUDA device code.
 *
 *   circleModel.c:27-58   Mie cylinder, 10x10 sub-cell area/line average
 *   morphoScaleModel.c:101-253, :379-422   lamella ridge + trunk
 *   zigzagModel.c:41-79, :146-161          zig-zag lamellae (thick lines)
 *   noModel.c:5-8
 * dispatched like models_eps (models.c:166-184): D_X -> (col,row) = (1,0),
 * D_Y -> (0,1), D_XY -> (1,1).
 *
 * Only the reference's default morpho options are modelled (no edge
 * randomness, CURVE 0, no gap, no anisotropy; morphoScaleModel.c:14-64), plus
 * one extension: a width per lamella.  One shortcut is added that does not
 * change any result: a cell that no lamella band reaches and that lies wholly
 * above or below the trunk returns 1 before the sub-cell loop (every sub-sample
 * would fail both tests, so the reference also returns exactly 1 there).
 */
#ifndef MPIFDTD_MODELS_EVAL_H
#define MPIFDTD_MODELS_EVAL_H
#include <math.h>

#ifdef __CUDACC__
#define MDL_FN __host__ __device__ static inline
#else
#define MDL_FN static inline
#endif

#define MDL_MAX_LAYERS 32

typedef struct mdl_params {
  int kind;                       /* 0 none, 1 circle, 3 morpho (models.h enum MODEL) */
  int n_pml, n_x, n_y;            /* field geometry the circle tests against */
  /* circle (cell units) */
  double radius, eps_c, posx, posy;
  /* morpho (cell units) */
  int layers;
  double width[MDL_MAX_LAYERS], width_max, thick0, thick1, branch, height, ox, oy, ep, edge;
  double a[MDL_MAX_LAYERS], b1[MDL_MAX_LAYERS], b2[MDL_MAX_LAYERS];
  /* zigzag (cell units); sin/cos of the angle taken once on the host, so the
   * device evaluates with the host libm's values */
  int zz_layers;
  double zz_sin, zz_cos, zz_width, zz_thick, zz_height, zz_exw, zz_exh, zz_ox, zz_oy, zz_ep;
} mdl_params;

/* circleModel.c:27-58 */
MDL_FN double mdl_circle(const mdl_params *m, double x, double y, int col, int row)
{
  if (x < m->n_pml || y < m->n_pml || x > m->n_x + m->n_pml || y > m->n_y + m->n_pml) return 1.0;
  const double dx = x - m->posx, dy = y - m->posy;
  const double len = dx * dx + dy * dy, r = m->radius;
  if (len >= (r + 1) * (r + 1)) return 1.0;
  if (len <= (r - 1) * (r - 1)) return m->eps_c;
  const double split = 10, half = split / 2;
  double sum = 0;
  for (double i = -half + 0.5; i < half; i += 1)
    for (double j = -half + 0.5; j < half; j += 1) {
      const double px = dx + col * i / split, py = dy + row * j / split;
      if (px * px + py * py <= r * r) sum += 1;
    }
  sum /= split * split;
  return m->eps_c * sum + 1.0 * (1 - sum);
}

MDL_FN int mdl_in_lamella(const mdl_params *m, int id, double x, double y)
{
  return m->a[id] * x + m->b1[id] <= y && y <= m->a[id] * x + m->b2[id];
}

/* morphoScaleModel.c:107-125 (no randomness, CURVE 0) */
MDL_FN double mdl_lamella_width(const mdl_params *m, double sx, double sy, int id)
{
  const double b = sy - sx * m->a[id];
  const double p = 1 - b / m->height;
  const double width_p = p + (1 - p) * m->edge;
  const double half_width = m->width[id] / 2.0;
  return width_p * (half_width * (1 - 0.0));
}

/* morphoScaleModel.c:128-145 */
MDL_FN int mdl_find_lamella(const mdl_params *m, double lft, double rht, double btm, double top)
{
  for (int i = 0; i < m->layers; i++)
    if (mdl_in_lamella(m, i, lft, btm) || mdl_in_lamella(m, i, rht, btm) || mdl_in_lamella(m, i, lft, top) ||
        mdl_in_lamella(m, i, rht, top))
      return i;
  return -1;
}

/* morphoScaleModel.c:147-253 */
MDL_FN double mdl_morpho(const mdl_params *m, double x, double y, int col, int row)
{
  const double X = x - m->ox, Y = y - m->oy;
  if (fabs(X) > 0.5 * sqrt(m->width_max * m->width_max + m->thick0 * m->thick0) + 0.5) return 1.0;
  int idl = -1, idr = -1;
  if (fabs(X) > 0.5) {
    const int id = mdl_find_lamella(m, X - 0.5, X + 0.5, Y - 0.5, Y + 0.5);
    if (X < 0) idl = id; else idr = id;
  } else {
    idl = mdl_find_lamella(m, X - 0.5, 0, Y - 0.5, Y + 0.5);
    idr = mdl_find_lamella(m, 0, X + 0.5, Y - 0.5, Y + 0.5);
  }
  if (idl < 0 && idr < 0 && (Y + 0.5 < 0 || Y - 0.5 > m->height)) return 1.0;  /* see header */
  double cnt = 0;
  const double split = 10, half = split / 2;
  for (double i = -half + 0.5; i < half; i += 1)
    for (double j = -half + 0.5; j < half; j += 1) {
      const double sx = X + col * i / split, sy = Y + row * j / split;
      if (sy >= 0 && sy <= m->height) {
        const double p = 1 - sy / m->height;
        const double width_p = p + (1 - p) * m->edge;
        if (fabs(sx) < m->branch / 2.0 * width_p) { cnt += 1; continue; }
      }
      const int id = sx < 0 ? idl : idr;
      if (id < 0) continue;
      if (mdl_in_lamella(m, id, sx, sy)) {
        const double w = mdl_lamella_width(m, sx, sy, id);
        if (sx * sx * (1 + m->a[id] * m->a[id]) < w * w) { cnt += 1; continue; }
      }
      for (int k = -1; k < 2; k += 2) {
        const int nid = id + k;
        if (nid < 0 || nid >= m->layers) continue;
        if (mdl_in_lamella(m, nid, sx, sy)) {
          const double w = mdl_lamella_width(m, sx, sy, nid);
          if (sx * sx * (1 + m->a[nid] * m->a[nid]) < w * w) { cnt += 1; break; }
        }
      }
    }
  cnt /= split * split;
  return 1.0 * (1 - cnt) + m->ep * cnt;
}

/* zigzagModel.c:41-79: sub-sample (sx, sy) is inside when its distance to
 * the centre line of lamella k is at most the thickness; k from the height,
 * clamped to [0, layers-1] as min(layerNum-1, max(0, .)) does.  pow(v, 2) of
 * the reference is v * v (one rounding either way). */
MDL_FN double mdl_zigzag(const mdl_params *m, double _x, double _y, int col, int row)
{
  const double x = _x - m->zz_ox, y = _y - m->zz_oy;
  const double sn = m->zz_sin, cs = m->zz_cos, w = m->zz_width, t = m->zz_thick;
  const double h = m->zz_height, exw = m->zz_exw, exh = m->zz_exh;
  if (fabs(x) > w / 2.0 + exw + 0.5 || y < -exh - 0.5 || y > h + exh + 0.5) return 1.0;
  const double rise = w * sn + cs * t / 2;  /* one lamella's step up */
  const double px = -w * cs / 2.0;
  double cnt = 0;
  const double split = 10, half = split / 2;
  for (double i = -half + 0.5; i < half; i += 1)
    for (double j = -half + 0.5; j < half; j += 1) {
      const double sx = x + col * i / split, sy = y + row * j / split;
      if (fabs(sx) > w / 2 + exw || sy < -exh || sy > h + exh) continue;
      const double q = sy / rise;
      const double qm = 0 > q ? 0 : q;
      const int k = (int)(m->zz_layers - 1 < qm ? m->zz_layers - 1 : qm);
      const double py = floor((double)((k + 1) / 2)) * 2 * (w * sn) + k * cs * t / 2;
      const double vx = (1 - ((k & 1) << 1)) * cs, vy = sn;
      const double ax = sx - px, ay = sy - py, proj = ax * vx + ay * vy;
      const double d2 = ax * ax + ay * ay - proj * proj;
      if (d2 <= t * t) cnt += 1;
    }
  cnt /= split * split;
  return 1.0 * (1 - cnt) + m->zz_ep * cnt;
}

MDL_FN double mdl_eps(const mdl_params *m, double x, double y, int col, int row)
{
  if (m->kind == 1) return mdl_circle(m, x, y, col, row);
  if (m->kind == 3) return mdl_morpho(m, x, y, col, row);
  if (m->kind == 5) return mdl_zigzag(m, x, y, col, row);
  return 1.0;
}

/* circleModel.c:74-81, morphoScaleModel.c:379-422 (cell units from nm).
 * circle p = {radius_nm, eps (<=0: 1.6^2)}
 * morpho p = {width_nm, thick0_nm, thick1_nm, layers, branch_nm, edge_rate, eps (<=0: 1.56^2),
 *             per_lamella (0/1), width_0_nm, width_1_nm, ...}
 * zigzag p = {width_nm, thickness_nm, layers, degree, n (<=0: N_0 = 1.56)}; the reference's
 *             statics are integers, so width, thickness, layers and degree are truncated
 * Returns 0, or -1 on a bad parameter vector. */
MDL_FN int mdl_init(mdl_params *m, int kind, const double *p, int np, int n_px, int n_py, int n_pml, double h_u)
{
  m->kind = kind;
  m->n_pml = n_pml;
  m->n_x = n_px - 2 * n_pml;
  m->n_y = n_py - 2 * n_pml;
  if (kind == 0) return 0;
  if (kind == 1) {
    if (np < 1) return -1;
    m->radius = p[0] / h_u;
    m->posx = n_px / 2;
    m->posy = n_py / 2;
    m->eps_c = (np > 1 && p[1] > 0) ? p[1] : 1.6 * 1.6 * 1.0;
    return 0;
  }
  if (kind == 5) {
    if (np < 4) return -1;
    const int width = (int)p[0], thick = (int)p[1], layers = (int)p[2], degree = (int)p[3];
    if (layers < 1 || width < 0 || thick < 0) return -1;
    const double rad = degree * M_PI / 180.0;
    m->zz_layers = layers;
    m->zz_sin = sin(rad);
    m->zz_cos = cos(rad);
    m->zz_width = width / h_u;
    m->zz_thick = thick / h_u;
    m->zz_height = (m->zz_width * m->zz_sin) * layers + layers * m->zz_thick / 2 * m->zz_cos;
    m->zz_exw = m->zz_thick / 2.0 * m->zz_sin;
    m->zz_exh = m->zz_thick / 2.0 * m->zz_cos;
    m->zz_ox = n_px / 2.0;
    m->zz_oy = (n_py - m->zz_height) / 2.0;
    m->zz_ep = (np > 4 && p[4] > 0) ? p[4] * p[4] * 1.0 : 1.56 * 1.56 * 1.0;
    return 0;
  }
  if (kind == 3) {
    if (np < 6) return -1;
    const int layers = (int)p[3];
    if (layers < 1 || layers > MDL_MAX_LAYERS) return -1;
    const int per = np > 7 && p[7] > 0;
    if (per && np < 8 + layers) return -1;
    m->layers = layers;
    m->thick0 = p[1] / h_u;
    m->thick1 = p[2] / h_u;
    m->branch = p[4] / h_u;
    m->edge = p[5];
    m->ep = (np > 6 && p[6] > 0) ? p[6] : 1.56 * 1.56 * 1.0;
    m->width_max = 0;
    for (int i = 0; i < layers; i++) {
      m->width[i] = (per ? p[8 + i] : p[0]) / h_u;
      if (m->width[i] > m->width_max) m->width_max = m->width[i];
    }
    m->height = (m->thick0 + m->thick1) * layers + (m->thick0 + m->thick1);
    m->oy = n_py / 2 - m->height / 2;
    m->ox = n_px / 2;
    const double thick = m->thick0 + m->thick1, halfv = 0.5 * m->thick0;
    for (int i = 0; i < layers; i++) {
      m->a[i] = tan(0.0);
      m->b1[i] = thick * i + halfv - halfv / cos(0.0);
      m->b2[i] = thick * i + halfv + halfv / cos(0.0);
    }
    return 0;
  }
  return -1;
}

#endif
