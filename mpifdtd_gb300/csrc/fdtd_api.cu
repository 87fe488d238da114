// fdtd_api.cu -- host side of the C ABI declared in include/mpifdtd_gb300.h.
//
// Host responsibilities: derive the grid exactly as field_init() does
// (field.c:89-143), build the 1-D PML coefficient tables with the
// reference's own formulas (mpiTM_UPML.c:663-716, mpiTE_UPML.c:489-536,
// fdtdTM_upml.c:224-274, fdtdTE_upml.c:361-412), build the NTFF surface and
// retarded-time shift tables (mpiTM_UPML.c:849-1037, ntffTM.c:293-371), and
// sequence the per-step launches.  All arithmetic that the reference does once
// per run (sigma, coefficients, shifts, source phases) is done here in double
// with the same expressions; this file must be compiled with
// -ffp-contract=off so the host compiler does not fuse them.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <type_traits>
#include <vector>

#include "fdtd_internal.cuh"
#include "fdtd_sim.h"

using namespace fdtd;

namespace {

thread_local std::string g_err;

int fail(int code, const char *fmt, ...)
{
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CK(call)                                                                                   \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) return fail(FDTD_E_CUDA, "%s: %s", #call, cudaGetErrorString(e_));      \
  } while (0)

bool is_tm(int solver)
{
  return solver == FDTD_TM_UPML || solver == FDTD_MPI_TM_UPML || solver == FDTD_TM_2D || solver == FDTD_NS_TM_2D;
}
// 0 UPML, 1 split-field PML, 2 NS-FDTD
int family_of(int solver)
{
  if (solver == FDTD_TM_2D || solver == FDTD_TE_2D) return 1;
  if (solver == FDTD_NS_TM_2D || solver == FDTD_NS_TE_2D) return 2;
  return 0;
}
bool is_mpi(int solver) { return solver == FDTD_MPI_TM_UPML || solver == FDTD_MPI_TE_UPML; }

// field.c:259-283 (the reference's M = 2; config pml_order sets M)
double sigma_axis(double x, int n_pml, int n_inner, int n_full, int M = 2)
{
  if (x < n_pml) return std::pow(1.0 * (n_pml - x) / n_pml, M);
  if (x < n_inner + n_pml) return 0;
  return std::pow(1.0 * (x - (n_full - n_pml - 1)) / n_pml, M);
}

}  // namespace

int fdtd::set_error(int code, const char *fmt, ...)
{
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

extern "C" const char *fdtd_last_error(void) { return g_err.c_str(); }
extern "C" const char *fdtd_version(void) { return "mpifdtd_gb300 0.1 (sm_103a)"; }

extern "C" int fdtd_geometry_of(const fdtd_config *cfg, fdtd_geometry *g)
{
  if (!cfg || !g) return fail(FDTD_E_ARG, "null argument");
  if (cfg->h_u_nm <= 0 || cfg->width_nm <= 0 || cfg->height_nm <= 0 || cfg->lambda_nm <= 0)
    return fail(FDTD_E_ARG, "sizes must be positive");
  if (cfg->pml <= 0) return fail(FDTD_E_ARG, "pml must be positive (field.c:259-283 divides by it)");
  if (cfg->step_num < 0) return fail(FDTD_E_ARG, "step_num must be >= 0");
  if (cfg->courant_e4 < 0 || cfg->courant_e4 > 7071)
    return fail(FDTD_E_ARG, "courant_e4 %d outside [0, 7071] (Courant number <= 1/sqrt 2)", cfg->courant_e4);
  if (cfg->pml_order < 0 || cfg->pml_order > 8) return fail(FDTD_E_ARG, "pml_order %d outside [0, 8]", cfg->pml_order);
  if (cfg->ntff_inset < 0) return fail(FDTD_E_ARG, "ntff_inset %d < 0", cfg->ntff_inset);
  for (int r = 0; r < 4; r++)
    if (cfg->reserved[r]) return fail(FDTD_E_ARG, "reserved fields of fdtd_config must be zero");
  const int inset = config_ntff_inset(*cfg);
  // field.c:95-100 (field_toCellUnit divides as double, the int conversion truncates)
  g->n_px = (int)((double)cfg->width_nm / cfg->h_u_nm);
  g->n_py = (int)((double)cfg->height_nm / cfg->h_u_nm);
  g->n_pml = cfg->pml;
  g->n_x = g->n_px - 2 * g->n_pml;
  g->n_y = g->n_py - 2 * g->n_pml;
  // field.c:105-109
  g->lambda_s = (double)cfg->lambda_nm / cfg->h_u_nm;
  g->k_s = 2 * M_PI / g->lambda_s;
  g->omega_s = config_courant(*cfg) * g->k_s;
  // field.c:133-142
  g->ntff_cx = g->n_px / 2;
  g->ntff_cy = g->n_py / 2;
  g->ntff_top = g->n_py - g->n_pml - inset;
  g->ntff_bottom = g->n_pml + inset;
  g->ntff_left = g->n_pml + inset;
  g->ntff_right = g->n_px - g->n_pml - inset;
  double len = (g->ntff_top - g->ntff_bottom) / 2;
  g->rf_per_c = len * 2;
  g->array_size = (int)(cfg->step_num + 2 * g->rf_per_c);
  if (g->ntff_right - g->ntff_left < 2 || g->ntff_top - g->ntff_bottom < 2)
    return fail(FDTD_E_ARG, "grid %dx%d too small for pml %d plus the %d-cell NTFF inset", g->n_px, g->n_py,
                g->n_pml, inset);
  return FDTD_OK;
}

// ---------------------------------------------------------------- create

static int build_tables(fdtd_sim *s)
{
  const fdtd_geometry &g = s->geo;
  const bool tm = s->tm;
  const int order = config_pml_order(s->cfg);
  const double R = 1.0e-8, M = (double)order, C0 = s->c0;
  // mpiTM_UPML.c:672 / fdtdTM_upml.c:232 (TM, with 1/cos(pi/3)); mpiTE_UPML.c:497 (TE)
  const double sig_max = tm ? -(M + 1.0) * kEps0 * C0 / 2.0 / g.n_pml / cos(M_PI / 3) * log(R)
                            : -(M + 1.0) * kEps0 * C0 / 2.0 / g.n_pml * log(R);
  const double e2 = 2 * kEps0, sz = 0;
  const double mu0 = 1.0 / C0 / C0;  // field.h:74
  const double inv_mu = 1.0 / mu0;
  s->inv_mu = inv_mu;
  std::vector<Coef4<double>> txi(s->nxa), txh(s->nxa), tyi(s->ncols), tyh(s->ncols);
  for (int i = 0; i < s->nxa; i++) {
    const double x = i + s->ox;
    const double si = sig_max * sigma_axis(x, g.n_pml, g.n_x, g.n_px, order);
    const double sh = sig_max * sigma_axis(x + 0.5, g.n_pml, g.n_x, g.n_px, order);
    if (tm) {
      txi[i] = {(e2 - si) / (e2 + si), (e2) / (e2 + si), (e2 + si) / (e2 + sz), (e2 - si) / (e2 + sz)};
      txh[i] = {(e2 - sh) / (e2 + sh), 1.0 / (e2 + sh), 0, 0};
    } else {
      txi[i] = {(e2 - si) / (e2 + si), 1.0 / (e2 + si), 0, 0};
      txh[i] = {(e2 + sh) / (e2 + sz), (e2 - sh) / (e2 + sz), (e2 - sh) / (e2 + sh), (e2) / (e2 + sh) * inv_mu};
    }
  }
  for (int j = 0; j < s->ncols; j++) {
    const double y = j + s->ox;
    const double si = sig_max * sigma_axis(y, g.n_pml, g.n_y, g.n_py, order);
    const double sh = sig_max * sigma_axis(y + 0.5, g.n_pml, g.n_y, g.n_py, order);
    if (tm) {
      tyi[j] = {(e2 - si) / (e2 + si), (e2 + sz) / (e2 + si), e2 + si, e2 - si};
      tyh[j] = {(e2 - sh) / (e2 + sh), (e2) / (e2 + sh) * inv_mu, 0, 0};
    } else {
      tyi[j] = {(e2 - si) / (e2 + si), (e2) / (e2 + si), 0, 0};
      tyh[j] = {(e2 - sh) / (e2 + sh), (e2 + sz) / (e2 + sh), e2 + sh, e2 - sh};
    }
  }
  // interior: every sigma zero (field.c:265,278): x in [n_pml, n_px - n_pml)
  s->in_x0 = g.n_pml;
  s->in_x1 = g.n_px - g.n_pml;
  s->in_y0 = g.n_pml;
  s->in_y1 = g.n_py - g.n_pml;
  auto up = [&](std::vector<Coef4<double>> &h, void **d64, void **d32) -> int {
    CK(cudaMalloc(d64, h.size() * sizeof(Coef4<double>)));
    CK(cudaMemcpy(*d64, h.data(), h.size() * sizeof(Coef4<double>), cudaMemcpyHostToDevice));
    std::vector<Coef4<float>> f(h.size());
    for (size_t q = 0; q < h.size(); q++) f[q] = {(float)h[q].a, (float)h[q].b, (float)h[q].c, (float)h[q].d};
    CK(cudaMalloc(d32, f.size() * sizeof(Coef4<float>)));
    CK(cudaMemcpy(*d32, f.data(), f.size() * sizeof(Coef4<float>), cudaMemcpyHostToDevice));
    return FDTD_OK;
  };
  int rc;
  if ((rc = up(txi, &s->d_tab64[0], &s->d_tab32[0]))) return rc;
  if ((rc = up(txh, &s->d_tab64[1], &s->d_tab32[1]))) return rc;
  if ((rc = up(tyi, &s->d_tab64[2], &s->d_tab32[2]))) return rc;
  if ((rc = up(tyh, &s->d_tab64[3], &s->d_tab32[3]))) return rc;

  // CW source phase tables (mpiTM_UPML.c:343-347, :369): kr = x ks_cos + y ks_sin
  const double rad = s->cfg.angle_deg * M_PI / 180;
  const double ks_cos = cos(rad) * g.k_s, ks_sin = sin(rad) * g.k_s;
  std::vector<double2> ex(s->nxa), ey(s->ncols);
  for (int i = 0; i < s->nxa; i++) {
    const int x = i + s->ox;
    const double ph = x * ks_cos;
    ex[i] = make_double2(cos(ph), sin(ph));
  }
  for (int j = 0; j < s->ncols; j++) {
    const int y = j + s->ox;
    const double ph = y * ks_sin;
    ey[j] = make_double2(cos(ph), sin(ph));
  }
  CK(cudaMalloc(&s->d_ex, ex.size() * sizeof(double2)));
  CK(cudaMemcpy(s->d_ex, ex.data(), ex.size() * sizeof(double2), cudaMemcpyHostToDevice));
  CK(cudaMalloc(&s->d_ey, ey.size() * sizeof(double2)));
  CK(cudaMemcpy(s->d_ey, ey.data(), ey.size() * sizeof(double2), cudaMemcpyHostToDevice));
  // FP32 copies for the FP32 stencil, which evaluates the source in FP32
  std::vector<float2> ex32(ex.size()), ey32(ey.size());
  for (size_t q = 0; q < ex.size(); q++) ex32[q] = make_float2((float)ex[q].x, (float)ex[q].y);
  for (size_t q = 0; q < ey.size(); q++) ey32[q] = make_float2((float)ey[q].x, (float)ey[q].y);
  CK(cudaMalloc(&s->d_ex32, ex32.size() * sizeof(float2)));
  CK(cudaMemcpy(s->d_ex32, ex32.data(), ex32.size() * sizeof(float2), cudaMemcpyHostToDevice));
  CK(cudaMalloc(&s->d_ey32, ey32.size() * sizeof(float2)));
  CK(cudaMemcpy(s->d_ey32, ey32.data(), ey32.size() * sizeof(float2), cudaMemcpyHostToDevice));
  return FDTD_OK;
}

// NTFF path cells in the reference's side order and their per-angle shifts.
static int build_ntff(fdtd_sim *s)
{
  if (s->cfg.flags & FDTD_CFG_NO_TIME_NTFF) {  // status word only
    s->ntff_mode = 3;
    CK(cudaMalloc(&s->d_status, sizeof(unsigned int)));
    CK(cudaMemsetAsync(s->d_status, 0, sizeof(unsigned int), s->stream));
    return FDTD_OK;
  }
  const fdtd_geometry &g = s->geo;
  const bool tm = s->tm, mpi = s->mpi;
  const int P = s->pitch;
  const int tp = g.ntff_top, bm = g.ntff_bottom, rt = g.ntff_right, lt = g.ntff_left;
  const int cx = g.ntff_cx, cy = g.ntff_cy;
  std::vector<SurfCell> cells;
  // geometry of each cell for the shift: r2 = (rx, ry) (double), side id
  std::vector<double> r2x, r2y;
  std::vector<int> side;
  auto add = [&](int i, int j, int hoff, int sign, int eslot, int hslot, int uid, int wid, double rx, double ry,
                 int sd) {
    SurfCell c;
    c.k = (long long)i * P + j;
    c.hoff = hoff;
    c.sign = (signed char)sign;
    c.e_slot = (signed char)eslot;
    c.h_slot = (signed char)hslot;
    c.uid_wid = (signed char)(uid | (wid << 4));
    cells.push_back(c);
    r2x.push_back(rx);
    r2y.push_back(ry);
    side.push_back(sd);
  };
  // array row/col range of the path: MPI clips to the sub-domain
  // (mpiTM_UPML.c:886-887,926-927), serial uses [left,right) x [bottom,top)
  const int nrow = s->nxa, ncol = s->ncols;
  const int i0 = mpi ? (lt > 1 ? lt : 1) : lt, i1 = mpi ? (rt < nrow ? rt : nrow) : rt;
  const int j0 = mpi ? (bm > 1 ? bm : 1) : bm, j1 = mpi ? (tp < ncol ? tp : ncol) : tp;
  const double hx = tm ? 0.0 : 0.5;  // TE samples sit half a cell along the side
  // TM: U slots Ux 0 / Uy 1, W Wz 2 ; TE: U Uz 2, W Wx 0 / Wy 1
  if (tm) {
    for (int i = i0; i < i1; i++) add(i, bm, -1, +1, 0, 3, 0, 2, i - cx, bm - cy, 0);        // bottom
    for (int j = j0; j < j1; j++) add(rt, j, -P, +1, 0, 4, 1, 2, rt - cx, j - cy, 1);        // right
    for (int i = i0; i < i1; i++) add(i, tp, -1, -1, 0, 3, 0, 2, i - cx, tp - cy, 2);        // top
    for (int j = j0; j < j1; j++) add(lt, j, -P, -1, 0, 4, 1, 2, lt - cx, j - cy, 3);        // left
  } else {
    for (int i = i0; i < i1; i++) add(i, bm, -1, -1, 0, 6, 2, 0, i - cx + hx, bm - cy, 0);
    for (int j = j0; j < j1; j++) add(rt, j, -P, -1, 1, 6, 2, 1, rt - cx, j - cy + hx, 1);
    for (int i = i0; i < i1; i++) add(i, tp, -1, +1, 0, 6, 2, 0, i - cx + hx, tp - cy, 2);
    for (int j = j0; j < j1; j++) add(lt, j, -P, +1, 1, 6, 2, 1, lt - cx, j - cy + hx, 3);
  }
  const int n = (int)cells.size();
  s->ncell = n;
  std::vector<double> shift((size_t)360 * n);
  for (int ang = 0; ang < 360; ang++) {
    double *row = &shift[(size_t)ang * n];
    if (mpi) {
      // mpiTM_UPML.c:875-876, :894 ; mpiTE_UPML.c:634-635, :654
      const double rad = ang * M_PI / 180.0;
      const double r1x = cos(rad), r1y = sin(rad);
      for (int c = 0; c < n; c++) row[c] = -(r1x * r2x[c] + r1y * r2y[c]) / s->c0 + g.rf_per_c;
    } else {
      // ntffTM.c:318-368 / ntffTE.c:92-155: shift advanced incrementally along each side
      const double rad = ang * (M_PI / 180.0);
      const double r1x = cos(rad) / s->c0, r1y = sin(rad) / s->c0;
      int c = 0;
      for (int sd = 0; sd < 4; sd++) {
        int c0 = c;
        while (c < n && side[c] == sd) c++;
        if (c == c0) continue;
        // start point of the side in the reference's loop (left/bottom corner frame)
        double sx0 = r2x[c0], sy0 = r2y[c0];
        double sh = -(r1x * sx0 + r1y * sy0) + g.rf_per_c;
        const double step = (sd == 0 || sd == 2) ? r1x : r1y;
        for (int q = c0; q < c; q++) {
          row[q] = sh;
          sh -= step;
        }
      }
    }
  }
  CK(cudaMalloc(&s->d_cells, sizeof(SurfCell) * n));
  CK(cudaMemcpy(s->d_cells, cells.data(), sizeof(SurfCell) * n, cudaMemcpyHostToDevice));
  CK(cudaMalloc(&s->d_shift, sizeof(double) * shift.size()));
  CK(cudaMemcpy(s->d_shift, shift.data(), sizeof(double) * shift.size(), cudaMemcpyHostToDevice));
  s->h_shift.swap(shift);
  s->h_side.swap(side);
  s->window_dirty = true;
  CK(cudaMalloc(&s->d_vals, sizeof(double2) * 2 * (size_t)n * kMaxNtffBlock));
  CK(cudaMalloc(&s->d_dg, sizeof(double4) * 2 * (size_t)n * (kMaxNtffBlock + 2)));
  s->ntff_len = (size_t)360 * g.array_size + 2 * kGuard;
  for (int a = 0; a < 3; a++) {
    CK(cudaMalloc(&s->d_ntff[a], sizeof(double2) * s->ntff_len));
    CK(cudaMemsetAsync(s->d_ntff[a], 0, sizeof(double2) * s->ntff_len, s->stream));
  }
  CK(cudaMalloc(&s->d_status, sizeof(unsigned int)));
  CK(cudaMemsetAsync(s->d_status, 0, sizeof(unsigned int), s->stream));
  return FDTD_OK;
}

static void free_sim(fdtd_sim *s)
{
  if (!s) return;
  for (int a = 0; a < kMaxSlots; a++) {
    cudaFree(s->d_f[a]);
    cudaFree(s->d_f2[a]);
  }
  cudaFree(s->d_tbcol);
  cudaFree(s->d_tbrow);
  cudaFree(s->d_ptab);
  cudaFree(s->d_tiles);
  for (int a = 0; a < 2; a++) { cudaFree(s->d_ieps64[a]); cudaFree(s->d_ieps32[a]); }
  for (int a = 0; a < 3; a++) cudaFree(s->d_eps[a]);
  cudaFree(s->d_coef);
  for (int a = 0; a < 4; a++) { cudaFree(s->d_tab64[a]); cudaFree(s->d_tab32[a]); }
  cudaFree(s->d_ex);
  cudaFree(s->d_ey);
  cudaFree(s->d_ex32);
  cudaFree(s->d_ey32);
  cudaFree(s->d_cells);
  cudaFree(s->d_shift);
  cudaFree(s->d_vals);
  cudaFree(s->d_dg);
  cudaFree(s->d_dft_omega);
  cudaFree(s->d_dft_P);
  cudaFree(s->d_dft_S);
  cudaFree(s->d_dft_X);
  cudaFree(s->d_dft_T);
  for (int a = 0; a < 3; a++) cudaFree(s->d_ntff[a]);
  cudaFree(s->d_status);
  cudaFree(s->d_chunk);
  cudaFree(s->d_lo);
  for (cudaEvent_t e : s->ev_pool) cudaEventDestroy(e);
  cudaFree(s->d_spec);
  cudaFree(s->d_dirs);
  cudaFree(s->d_twiddle);
  cudaFree(s->d_freq);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
}

extern "C" int fdtd_create(int solver, const fdtd_config *cfg, fdtd_sim **out)
{
  if (!cfg || !out) return fail(FDTD_E_ARG, "null argument");
  *out = nullptr;
  if (solver < FDTD_TM_2D || solver > FDTD_NS_TE_2D) return fail(FDTD_E_ARG, "solver %d is not one of 0..7", solver);
  if (cfg->precision != FDTD_F64 && cfg->precision != FDTD_F32)
    return fail(FDTD_E_ARG, "precision must be FDTD_F64 or FDTD_F32");
  if (family_of(solver) && cfg->precision != FDTD_F64)
    return fail(FDTD_E_UNSUPPORTED, "the split-field and NS solvers run in FP64 only");
  if (cfg->flags & ~FDTD_CFG_NO_TIME_NTFF) return fail(FDTD_E_ARG, "unknown config flags %#x", cfg->flags);
  if (family_of(solver) && (cfg->courant_e4 || cfg->pml_order || cfg->ntff_inset))
    return fail(FDTD_E_UNSUPPORTED, "the split-field and NS solvers run with the reference's Courant number, "
                                    "sigma grading and NTFF inset only");
  fdtd_geometry geo;
  int rc = fdtd_geometry_of(cfg, &geo);
  if (rc) return rc;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(FDTD_E_CUDA, "no CUDA device is visible (the engine has no CPU path)");
  }
  fdtd_sim *s = new (std::nothrow) fdtd_sim();
  if (!s) return fail(FDTD_E_NOMEM, "host allocation failed");
  s->solver = solver;
  s->tm = is_tm(solver);
  s->mpi = is_mpi(solver);
  s->family = family_of(solver);
  s->cfg = *cfg;
  s->c0 = config_courant(*cfg);
  s->z0 = config_z0(*cfg);
  if (s->family) s->cfg.flags |= FDTD_CFG_NO_TIME_NTFF;  // these solvers have no NTFF
  s->geo = geo;
  s->f32 = cfg->precision == FDTD_F32;
  // array frame: MPI -> (N_PX+2) x (N_PY+2) halo ring, x = i-1; serial -> N_PX x N_PY, x = i
  s->ox = s->mpi ? -1 : 0;
  s->ni = s->mpi ? geo.n_px : geo.n_px - 2;
  s->nj = s->mpi ? geo.n_py : geo.n_py - 2;
  s->nxa = s->ni + 2;
  s->ncols = s->nj + 2;
  s->pitch = (s->ncols + 7) / 8 * 8;
  s->esize = s->f32 ? sizeof(float2) : sizeof(double2);
  s->nslots = s->family ? 5 : s->tm ? 7 : 8;
  if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    delete s;
    return fail(FDTD_E_CUDA, "cudaStreamCreate failed");
  }
  const size_t bytes = (size_t)s->nxa * s->pitch * s->esize;
  for (int a = 0; a < s->nslots; a++) {
    if (cudaMalloc(&s->d_f[a], bytes) != cudaSuccess) {
      cudaGetLastError();
      free_sim(s);
      return fail(FDTD_E_NOMEM, "cudaMalloc of %zu bytes for a field failed", bytes);
    }
    cudaMemsetAsync(s->d_f[a], 0, bytes, s->stream);
  }
  const int neps = s->tm ? 1 : 2;
  const size_t ecount = (size_t)s->nxa * s->pitch;
  for (int a = 0; a < neps; a++) {
    if (cudaMalloc(&s->d_ieps64[a], ecount * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&s->d_ieps32[a], ecount * sizeof(float)) != cudaSuccess) {
      cudaGetLastError();
      free_sim(s);
      return fail(FDTD_E_NOMEM, "cudaMalloc of permittivity failed");
    }
  }
  for (int a = 0; a < 3; a++) {
    if (cudaMalloc(&s->d_eps[a], ecount * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      free_sim(s);
      return fail(FDTD_E_NOMEM, "cudaMalloc of permittivity failed");
    }
  }
  if (s->family) {
    s->ncoef = solver == FDTD_NS_TE_2D ? 10 : 9;
    if (cudaMalloc(&s->d_coef, (size_t)s->ncoef * ecount * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      free_sim(s);
      return fail(FDTD_E_NOMEM, "cudaMalloc of the per-cell coefficients failed");
    }
  }
  if ((rc = build_tables(s)) || (rc = build_ntff(s)) || (rc = fdtd_fill_eps_model(s, FDTD_MODEL_NONE, nullptr, 0))) {
    std::string msg = g_err;
    free_sim(s);
    g_err = msg;
    return rc;
  }
  s->time = 0;
  *out = s;
  return FDTD_OK;
}

extern "C" int fdtd_destroy(fdtd_sim *s)
{
  if (!s) return FDTD_OK;
  cudaStreamSynchronize(s->stream);
  free_sim(s);
  return FDTD_OK;
}

extern "C" int fdtd_get_geometry(const fdtd_sim *s, fdtd_geometry *out)
{
  if (!s || !out) return fail(FDTD_E_ARG, "null argument");
  *out = s->geo;
  return FDTD_OK;
}

// ---------------------------------------------------------------- permittivity

// Permittivity lives on the device in the padded array frame (d_eps, halo
// cells 1.0).  The E components' 1/eps (FP64 and FP32 copies) are derived
// from it on the device; a non-finite or non-positive value sets
// kStatusBadEps and makes the call fail.
static int derive_inv_eps(fdtd_sim *s)
{
  if (s->family) {  // split-field / NS: per-cell coefficients from the permittivity before the next step
    s->coef_dirty = true;
    return FDTD_OK;
  }
  const size_t count = (size_t)s->nxa * s->pitch;
  const int neps = s->tm ? 1 : 2;
  CK(cudaMemsetAsync(s->d_status, 0, sizeof(unsigned int), s->stream));
  for (int a = 0; a < neps; a++)
    launch_inv_eps((const double *)s->d_eps[a], (double *)s->d_ieps64[a], (float *)s->d_ieps32[a], count,
                   s->d_status, s->stream);
  CK(cudaGetLastError());
  unsigned int st = 0;
  CK(cudaMemcpyAsync(&st, s->d_status, sizeof st, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  s->launches += neps;
  if (st & kStatusBadEps) return fail(FDTD_E_ARG, "permittivity must be finite and > 0 everywhere");
  return FDTD_OK;
}

int fdtd_derive_inv_eps(fdtd_sim *s) { return derive_inv_eps(s); }

// array offset of global cell (0,0): MPI arrays carry a one-cell halo
static size_t global_origin(const fdtd_sim *s) { return s->mpi ? (size_t)s->pitch + 1 : 0; }

extern "C" int fdtd_set_eps(fdtd_sim *s, const double *e0, const double *e1, const double *e2)
{
  if (!s) return fail(FDTD_E_ARG, "null simulation");
  if (!e0) return fail(FDTD_E_ARG, "the E-component permittivity e0 is required");
  if (!s->tm && !e1) return fail(FDTD_E_ARG, "TE needs e1 (EPS_EY) as well");
  const double *src[3] = {e0, e1, e2};
  const int n_px = s->geo.n_px, n_py = s->geo.n_py;
  for (int a = 0; a < 3; a++) {
    if (!src[a]) continue;
    double *dst = (double *)s->d_eps[a] + global_origin(s);
    CK(cudaMemcpy2DAsync(dst, (size_t)s->pitch * sizeof(double), src[a], (size_t)n_py * sizeof(double),
                         (size_t)n_py * sizeof(double), n_px, cudaMemcpyHostToDevice, s->stream));
  }
  return derive_inv_eps(s);
}

extern "C" int fdtd_fill_eps_model(fdtd_sim *s, int model, const double *params, int n_params)
{
  if (!s) return fail(FDTD_E_ARG, "null simulation");
  if (n_params < 0 || (n_params > 0 && !params)) return fail(FDTD_E_ARG, "bad parameter vector");
  mdl_params m{};
  if (model != FDTD_MODEL_NONE && model != FDTD_MODEL_CIRCLE && model != FDTD_MODEL_MORPHO &&
      model != FDTD_MODEL_ZIGZAG)
    return fail(FDTD_E_UNSUPPORTED, "model %d is not built in (none 0, circle 1, morpho 3, zigzag 5)", model);
  if (mdl_init(&m, model, params, n_params, s->geo.n_px, s->geo.n_py, s->geo.n_pml, s->cfg.h_u_nm) != 0)
    return fail(FDTD_E_ARG, "bad parameters for model %d (see mpifdtd_gb300.h)", model);
  const bool alt = s->tm ? (s->mpi || s->family != 0) : s->solver == FDTD_NS_TE_2D;
  launch_eps_model((double *)s->d_eps[0], (double *)s->d_eps[1], (double *)s->d_eps[2], s->pitch, s->nxa,
                   s->ncols, s->ox, s->geo.n_px, s->geo.n_py, s->tm, alt, m, s->stream);
  s->launches += 1;
  CK(cudaGetLastError());
  if (s->solver == FDTD_NS_TE_2D) {  // nsFdtdTE.c:116-121 sets EPS_* on the inner cells only (FOR_FOR)
    const size_t rowb = (size_t)s->pitch * sizeof(double);
    for (int a = 0; a < 3; a++) {
      char *e = (char *)s->d_eps[a];
      CK(cudaMemsetAsync(e, 0, rowb, s->stream));
      CK(cudaMemsetAsync(e + (size_t)(s->geo.n_px - 1) * rowb, 0, rowb, s->stream));
      CK(cudaMemset2DAsync(e, rowb, 0, sizeof(double), s->geo.n_px, s->stream));
      CK(cudaMemset2DAsync(e + (size_t)(s->geo.n_py - 1) * sizeof(double), rowb, 0, sizeof(double), s->geo.n_px,
                           s->stream));
    }
  }
  return derive_inv_eps(s);
}

// ---------------------------------------------------------------- NTFF windows

// Chunks of at most ntff_chunk consecutive cells of one side, and per
// (angle, chunk) the bin offsets of the E and H windows:
//   E bins m = floor(timeE + sh + 0.5) lie in floor(timeE) + [floor(sh_min+.5)-1, floor(sh_max+.5)+1]
//   H bins (timeH = timeE + 1/2) in floor(timeE) + [floor(sh_min+1)-1, floor(sh_max+1)+1]
// the taps add one bin each side; one more bin of margin on each end.
static int build_windows(fdtd_sim *s)
{
  const int n = s->ncell, ch = s->ntff_chunk;
  std::vector<int2> chunks;
  for (int c = 0; c < n;) {
    int e = c;
    while (e < n && s->h_side[e] == s->h_side[c] && e - c < ch) e++;
    chunks.push_back(make_int2(c, e - c));
    c = e;
  }
  const int nch = (int)chunks.size();
  std::vector<int2> lo((size_t)360 * nch);
  int width = 0;
  for (int ang = 0; ang < 360; ang++) {
    const double *row = &s->h_shift[(size_t)ang * n];
    for (int q = 0; q < nch; q++) {
      double mn = row[chunks[q].x], mx = mn;
      for (int c = chunks[q].x; c < chunks[q].x + chunks[q].y; c++) {
        mn = std::min(mn, row[c]);
        mx = std::max(mx, row[c]);
      }
      const int loe = (int)std::floor(mn + 0.5) - 3, loh = (int)std::floor(mn + 1.0) - 3;
      const int we = (int)std::floor(mx + 0.5) - loe + 4, wh = (int)std::floor(mx + 1.0) - loh + 4;
      lo[(size_t)ang * nch + q] = make_int2(loe, loh);
      width = std::max(width, std::max(we, wh));
    }
  }
  if ((size_t)width * 2 * sizeof(double2) > 200 * 1024)
    return fail(FDTD_E_ARG, "NTFF window of %d bins exceeds shared memory; lower FDTD_OPT_NTFF_CHUNK", width);
  cudaFree(s->d_chunk);
  cudaFree(s->d_lo);
  s->d_chunk = s->d_lo = nullptr;
  CK(cudaMalloc(&s->d_chunk, sizeof(int2) * chunks.size()));
  CK(cudaMemcpy(s->d_chunk, chunks.data(), sizeof(int2) * chunks.size(), cudaMemcpyHostToDevice));
  CK(cudaMalloc(&s->d_lo, sizeof(int2) * lo.size()));
  CK(cudaMemcpy(s->d_lo, lo.data(), sizeof(int2) * lo.size(), cudaMemcpyHostToDevice));
  s->nchunk = nch;
  s->win_width = width;
  s->window_dirty = false;
  return FDTD_OK;
}

static int flush_ntff(fdtd_sim *s);

extern "C" int fdtd_set_option(fdtd_sim *s, int key, int value)
{
  if (!s) return fail(FDTD_E_ARG, "null simulation");
  int rc = flush_ntff(s);  // buffered steps are deposited with the settings they were taken under
  if (rc) return rc;
  switch (key) {
  case FDTD_OPT_NTFF_MODE:
    if (value < 0 || value > 3) return fail(FDTD_E_ARG, "NTFF mode must be 0, 1, 2 or 3");
    if (value != 3 && (s->cfg.flags & FDTD_CFG_NO_TIME_NTFF))
      return fail(FDTD_E_STATE, "created with FDTD_CFG_NO_TIME_NTFF: NTFF mode stays 3");
    s->ntff_mode = value;
    return FDTD_OK;
  case FDTD_OPT_NTFF_CHUNK:
    if (value < 64 || value > 4096) return fail(FDTD_E_ARG, "NTFF chunk must be in [64, 4096]");
    CK(cudaStreamSynchronize(s->stream));
    s->ntff_chunk = value;
    s->window_dirty = true;
    return FDTD_OK;
  case FDTD_OPT_NTFF_BLOCK:
    if (value < 1 || value > kMaxNtffBlock) return fail(FDTD_E_ARG, "NTFF block must be in [1, %d]", kMaxNtffBlock);
    s->ntff_block = value;
    return FDTD_OK;
  case FDTD_OPT_ROWS:
    if (value != 1 && value != 2 && value != 4 && value != 8) return fail(FDTD_E_ARG, "rows must be 1, 2, 4 or 8");
    s->rows = value;
    return FDTD_OK;
  case FDTD_OPT_TBLOCK:
    if (value != 0 && value != 1 && value != 2 && value != 4 && value != 8)
      return fail(FDTD_E_ARG, "temporal blocking depth must be 0, 1, 2, 4 or 8");
    if (value == 8 && !s->f32) return fail(FDTD_E_ARG, "temporal blocking depth 8 needs FP32 fields");
    if (value > 0 && s->family != 0)
      return fail(FDTD_E_UNSUPPORTED, "temporal blocking needs a UPML solver (split-field / NS: one step per launch)");
    if (value == 8 && !s->mpi) return fail(FDTD_E_ARG, "the serial solvers block 1, 2 or 4 steps");
    s->tblock = value;
    return FDTD_OK;
  case FDTD_OPT_TBLOCK_ROWS:
    if (value < 0 || value > (1 << 20)) return fail(FDTD_E_ARG, "tile rows must be in [0, 2^20]");
    s->tb_rows = value;
    return FDTD_OK;
  case FDTD_OPT_TBLOCK_COLS:
    if (value != 1 && value != 2) return fail(FDTD_E_ARG, "columns per lane must be 1 or 2");
    if (value == 2 && !s->f32) return fail(FDTD_E_ARG, "two columns per lane need FP32 fields");
    s->tb_cols = value;
    return FDTD_OK;
  }
  return fail(FDTD_E_ARG, "unknown option %d", key);
}

extern "C" int fdtd_get_option(fdtd_sim *s, int key, int *value)
{
  if (!s || !value) return fail(FDTD_E_ARG, "null argument");
  switch (key) {
  case FDTD_OPT_NTFF_MODE: *value = s->ntff_mode; return FDTD_OK;
  case FDTD_OPT_NTFF_CHUNK: *value = s->ntff_chunk; return FDTD_OK;
  case FDTD_OPT_NTFF_BLOCK: *value = s->ntff_block; return FDTD_OK;
  case FDTD_OPT_ROWS: *value = s->rows; return FDTD_OK;
  case FDTD_OPT_TBLOCK: *value = s->tblock; return FDTD_OK;
  case FDTD_OPT_TBLOCK_ROWS: *value = s->tb_rows; return FDTD_OK;
  case FDTD_OPT_TBLOCK_COLS: *value = s->tb_cols; return FDTD_OK;
  }
  return fail(FDTD_E_ARG, "unknown option %d", key);
}

// ---------------------------------------------------------------- stepping

template <typename R>
static StencilView<R> view_of(fdtd_sim *s)
{
  StencilView<R> v{};
  for (int a = 0; a < kMaxSlots; a++) v.f[a] = (typename Cplx<R>::T *)s->d_f[a];
  for (int a = 0; a < 2; a++)
    v.inv_eps[a] = std::is_same<R, double>::value ? (const R *)s->d_ieps64[a] : (const R *)s->d_ieps32[a];
  void *const *tab = std::is_same<R, double>::value ? s->d_tab64 : s->d_tab32;
  v.tx_i = (const Coef4<R> *)tab[0];
  v.tx_h = (const Coef4<R> *)tab[1];
  v.ty_i = (const Coef4<R> *)tab[2];
  v.ty_h = (const Coef4<R> *)tab[3];
  using T = typename Cplx<R>::T;
  v.ex = (const T *)(std::is_same<R, double>::value ? s->d_ex : s->d_ex32);
  v.ey = (const T *)(std::is_same<R, double>::value ? s->d_ey : s->d_ey32);
  v.P = s->pitch;
  v.nxa = s->nxa;
  v.ni = s->ni;
  v.nj = s->nj;
  v.ox = s->ox;
  v.in_x0 = s->in_x0;
  v.in_x1 = s->in_x1;
  v.in_y0 = s->in_y0;
  v.in_y1 = s->in_y1;
  v.inv_mu = (R)s->inv_mu;
  v.rows = s->rows;
  return v;
}

template <typename R>
StencilView<R> fdtd_view_of(fdtd_sim *s)
{
  return view_of<R>(s);
}
template StencilView<double> fdtd_view_of<double>(fdtd_sim *);
template StencilView<float> fdtd_view_of<float>(fdtd_sim *);

static NtffView ntff_view(fdtd_sim *s)
{
  NtffView n{};
  for (int a = 0; a < 3; a++) n.acc[a] = (double2 *)s->d_ntff[a];
  n.shift = (const double *)s->d_shift;
  n.cells = (const SurfCell *)s->d_cells;
  n.vals = (double2 *)s->d_vals;
  n.dg = (double4 *)s->d_dg;
  n.ncell = s->ncell;
  n.array_size = s->geo.array_size;
  n.len = (long long)s->ntff_len;
  n.status = s->d_status;
  return n;
}

// field.c:224-256 per-step constants of the pulse for one component
static SourceStep pulse_step(const fdtd_sim *s, double time, double gap_x, double gap_y, double dot)
{
  SourceStep p{};
  p.kind = 2;
  const double rad = s->cfg.angle_deg * M_PI / 180.0;
  p.cos_per_c = cos(rad) / s->c0;
  p.sin_per_c = sin(rad) / s->c0;
  const double center_peak =
      (s->geo.n_px / 2.0 + gap_x) * p.cos_per_c + (s->geo.n_py / 2 + gap_y) * p.sin_per_c;
  p.t0 = -center_peak + 500;
  p.time = time;
  p.w = s->geo.omega_s;
  p.gap_x = gap_x;
  p.gap_y = gap_y;
  p.dot = dot;
  return p;
}

static DftView dft_view(const fdtd_sim *s)
{
  DftView d{};
  d.omega = (const double *)s->d_dft_omega;
  d.nfreq = 2 * (int)s->dft_lam.size();
  d.phasor = (double2 *)s->d_dft_P;
  d.S = (double2 *)s->d_dft_S;
  return d;
}

// Deposits the buffered steps of the time-blocked NTFF (and feeds the running
// DFT first, while the ring still holds them).
static void deposit_pending(fdtd_sim *s, const NtffView &n, cudaStream_t st)
{
  if (s->nb_pending == 0) return;
  if (s->d_dft_S) {
    launch_dft_accumulate(n, dft_view(s), s->nb_pending, s->pending_t0, st);
    s->launches += 2;
  }
  launch_ntff_block(n, s->nb_pending, s->pending_t0, st);
  s->nb_pending = 0;
  s->launches += 2;  // differences + deposit
}

// Records the next profiling event of the step (5 per step) when enabled.
static void mark(fdtd_sim *s)
{
  if (!s->profiling) return;
  if (s->ev_used == s->ev_pool.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) {
      cudaGetLastError();
      s->profiling = false;
      return;
    }
    s->ev_pool.push_back(e);
  }
  cudaEventRecord(s->ev_pool[s->ev_used++], s->stream);
}

static void enqueue_split(fdtd_sim *s, double time, double ray_coef);

template <typename R>
static void enqueue_step(fdtd_sim *s, double time, double ray_coef)
{
  if (s->family) {
    enqueue_split(s, time, ray_coef);
    return;
  }
  const StencilView<R> v = view_of<R>(s);
  const NtffView n = ntff_view(s);
  cudaStream_t st = s->stream;
  const double coef = s->mpi ? 1.0 / (4 * M_PI * s->c0 * 1.0e6) : 1.0;  // mpiTM_UPML.c:852-854
  mark(s);
  if (s->mpi) {
    SourceStep cw{};
    cw.kind = 1;
    const double wt = s->geo.omega_s * time;
    cw.s_re = ray_coef * cos(wt);
    cw.s_im = -ray_coef * sin(wt);
    if (s->tm) {
      launch_tm_e<R>(v, cw, st);
      mark(s);
      launch_tm_h<R>(v, st);
    } else {
      SourceStep none{};
      launch_te_e<R>(v, none, cw, st);
      mark(s);
      launch_te_h<R>(v, st);
    }
  } else if (s->tm) {  // fdtdTM_upml.c:54-66
    launch_tm_h<R>(v, st);
    mark(s);
    launch_tm_e<R>(v, pulse_step(s, time, 0, 0, 1.0), st);
  } else {             // fdtdTE_upml.c:168-192
    launch_te_h<R>(v, st);
    mark(s);
    const double co = cos((s->cfg.angle_deg + 90) * M_PI / 180.0);
    const double si = sin((s->cfg.angle_deg + 90) * M_PI / 180.0);
    SourceStep sx{}, sy{};
    if (co != 0.0) sx = pulse_step(s, time, 0.5, 0.0, co);
    if (si != 0.0) sy = pulse_step(s, time, 0.0, 0.5, si);
    launch_te_e<R>(v, sx, sy, st);
  }
  mark(s);
  s->launches += 2;
  if (s->ntff_mode == 3) {  // no time-domain NTFF
    mark(s);
    mark(s);
    if (s->profiling) s->prof_steps++;
    return;
  }
  const bool blocked = s->ntff_mode == 2;
  launch_ntff_gather<R>(v, n, coef, blocked ? s->nb_pending : 0, st);
  mark(s);
  s->launches += 1;
  if (blocked) {
    if (s->nb_pending++ == 0) s->pending_t0 = time - 1;
    if (s->nb_pending == s->ntff_block) {
      deposit_pending(s, n, st);
    }
  } else if (s->ntff_mode == 1) {
    NtffWindow w{(const int2 *)s->d_chunk, (const int2 *)s->d_lo, s->nchunk, s->win_width};
    launch_ntff_window(n, w, time - 1, time - 0.5, st);
    s->launches += 1;
  } else {
    launch_ntff_accumulate(n, time - 1, time - 0.5, st);
    s->launches += 1;
  }
  mark(s);
  if (s->profiling) s->prof_steps++;
}

// Deposits the buffered steps of the time-blocked NTFF (mode 2).  Under
// profiling the deposit is one more 5-event group whose first four events
// coincide, so fdtd_profile_read counts it as NTFF deposit time of no step.
static int flush_ntff(fdtd_sim *s)
{
  if (s->nb_pending == 0) return FDTD_OK;
  for (int q = 0; q < 4; q++) mark(s);
  deposit_pending(s, ntff_view(s), s->stream);
  mark(s);
  CK(cudaGetLastError());
  return FDTD_OK;
}

// A buffered block holds consecutive steps only: a step that does not follow
// the last buffered one first deposits the block.
static int before_step(fdtd_sim *s, double time)
{
  if (s->ntff_mode == 2 && s->nb_pending > 0 && time - 1 != s->pending_t0 + s->nb_pending) return flush_ntff(s);
  return FDTD_OK;
}

// ---------------------------------------------------------------- temporal blocking

// Columns per lane for depth K: two (FP32, K = 2 or 4) when FDTD_OPT_TBLOCK_COLS asks for them.
static int tb_cols_for(const fdtd_sim *s, int K) { return s->tb_cols == 2 && s->f32 && (K == 2 || K == 4) ? 2 : 1; }

// Tile rows when FDTD_OPT_TBLOCK_ROWS is 0: the tallest power of two in
// [16, 128] that gives at least four waves of tiles (16 resident warps per
// SM), so that the last, partly filled wave is a small share of the launch.
// On 16416² the autotuner's fastest is 128 rows (1.13 ms per FP32 TM step;
// 256: 1.17, 512: 1.29); on 4128² taller tiles gave one or two waves and a
// blocked step slower than the one-step kernels.
static int tb_auto_rows(const fdtd_sim *s, int K, int cpl)
{
  const int W = 32 * cpl - 2 * K;
  const long long nstrip = (s->nj + W - 1) / W;
  int dev = 0, nsm = 152;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev))
    cudaGetLastError();
  const long long want = 4 * 16LL * nsm;
  int L = 128;
  while (L > 16 && nstrip * ((s->ni + L - 1) / L) < want) L >>= 1;
  return L;
}

// Tiles of depth K with cpl columns per lane (strip s owns columns
// o + s W .. o + s W + W - 1, W = 32 cpl - 2K; its lanes start K columns left).  A tile whose cone -- rows r0-K .. r1+K, its 32 lane columns --
// is PML-free (x = i+ox, y = j+ox inside [in_x0,in_x1) x [in_y0,in_y1)) runs
// the interior kernel: strips [s0, s1) x rows [ra, rb) in segments of L rows.
// Everything else is a work-list tile: the row bands above ra and below rb
// (thin: the PML rows and K more), and the strips outside [s0, s1).
int fdtd_plan_tiles(const fdtd_sim *s, int K, int L, int cpl, TilePlan *plan)
{
  const int W = 32 * cpl - 2 * K;
  const int o = cpl == 1 ? 1 : (K & 1);  // first owned column (tblock_tile.cuh origin())
  const int nstrip = (s->nj + 1 - o + W - 1) / W;  // owned columns o .. o + nstrip W - 1 cover 1..nj
  const int ilo = s->in_x0 - s->ox, ihi = s->in_x1 - s->ox;  // PML-free array rows [ilo, ihi)
  const int jlo = s->in_y0 - s->ox, jhi = s->in_y1 - s->ox;  // PML-free array columns
  auto strip_in = [&](int st) {  // the lanes' 32 cpl columns
    const int c = o + st * W - K;
    return c >= jlo && c + 32 * cpl <= jhi;
  };
  int s0 = 0;
  while (s0 < nstrip && !strip_in(s0)) s0++;
  int s1 = s0;
  while (s1 < nstrip && strip_in(s1)) s1++;
  int ra = std::max(1, ilo + K), rb = std::min(s->ni + 1, ihi - 1 - K);  // r0 - K >= ilo, r1 + K < ihi
  if (rb <= ra || s1 <= s0) {
    ra = rb = 1;
    s0 = s1 = 0;
  }
  const int nseg = rb > ra ? (rb - ra + L - 1) / L : 0;
  if (nseg > 65535) return fail(FDTD_E_ARG, "tile rows %d: more than 65535 segments of %d rows", L, rb - ra);
  plan->s0 = s0;
  plan->s1 = s1;
  plan->ra = ra;
  plan->rb = rb;
  plan->L = L;
  plan->nseg = nseg;
  std::vector<int4> &gen = plan->general;
  gen.clear();
  auto band = [&](int r_lo, int r_hi) {  // all strips, rows [r_lo, r_hi) in chunks of at most L rows
    for (int r0 = r_lo; r0 < r_hi; r0 += L)
      for (int st = 0; st < nstrip; st++) gen.push_back(make_int4(st, r0, std::min(r0 + L, r_hi), 0));
  };
  band(1, ra);
  for (int g = 0; g < nseg; g++) {
    const int r0 = ra + g * L, r1 = std::min(r0 + L, rb);
    for (int st = 0; st < nstrip; st++)
      if (st < s0 || st >= s1) gen.push_back(make_int4(st, r0, r1, 0));
  }
  band(rb, s->ni + 1);
  return FDTD_OK;
}

// The spare field set, the NTFF line buffers, and the tiles of depth K and
// height L (fdtd_plan_tiles) on the device.
static int tb_prepare(fdtd_sim *s, int K, int L, int cpl)
{
  const size_t bytes = (size_t)s->nxa * s->pitch * s->esize;
  if (!s->d_f2[0])
    for (int a = 0; a < s->nslots; a++) {
      CK(cudaMalloc(&s->d_f2[a], bytes));
      CK(cudaMemsetAsync(s->d_f2[a], 0, bytes, s->stream));
    }
  if (!s->d_tbcol) {
    CK(cudaMalloc(&s->d_tbcol, (size_t)kMaxTBlock * 12 * s->nxa * s->esize));
    CK(cudaMalloc(&s->d_tbrow, (size_t)kMaxTBlock * 12 * s->pitch * s->esize));
  }
  if (!s->mpi && !s->d_ptab) CK(cudaMalloc(&s->d_ptab, sizeof(PulseRow) * 2 * kMaxTBlock * (size_t)s->nxa));
  if (s->tb_built_k == K && s->tb_built_l == L && s->tb_built_c == cpl) return FDTD_OK;
  TilePlan plan;
  if (int rc = fdtd_plan_tiles(s, K, L, cpl, &plan)) return rc;
  const std::vector<int4> &tiles = plan.general;
  if ((int)tiles.size() > s->tiles_cap) {
    CK(cudaStreamSynchronize(s->stream));
    cudaFree(s->d_tiles);
    s->d_tiles = nullptr;
    s->tiles_cap = 0;
    CK(cudaMalloc(&s->d_tiles, sizeof(int4) * tiles.size()));
    s->tiles_cap = (int)tiles.size();
  }
  if (!tiles.empty()) {
    CK(cudaStreamSynchronize(s->stream));  // the previous list may still be in use
    CK(cudaMemcpy(s->d_tiles, tiles.data(), sizeof(int4) * tiles.size(), cudaMemcpyHostToDevice));
  }
  s->ntiles = (int)tiles.size();
  s->tb_s0 = plan.s0;
  s->tb_s1 = plan.s1;
  s->tb_ra = plan.ra;
  s->tb_rb = plan.rb;
  s->tb_nseg = plan.nseg;
  s->tb_L = L;
  s->tb_built_k = K;
  s->tb_built_l = L;
  s->tb_built_c = cpl;
  return FDTD_OK;
}

template <typename R>
static TBlockView<R> tblock_view(const fdtd_sim *s, bool lines)
{
  using T = typename Cplx<R>::T;
  TBlockView<R> tb{};
  for (int a = 0; a < kMaxSlots; a++) tb.out[a] = (T *)s->d_f2[a];
  if (lines) {
    tb.col = (T *)s->d_tbcol;
    tb.row = (T *)s->d_tbrow;
  }
  const fdtd_geometry &g = s->geo;  // the path's columns / rows and their H neighbours (build_ntff)
  const int cj[4] = {g.ntff_bottom - 1, g.ntff_bottom, g.ntff_top - 1, g.ntff_top};
  const int ri[4] = {g.ntff_left - 1, g.ntff_left, g.ntff_right - 1, g.ntff_right};
  for (int q = 0; q < 4; q++) {
    tb.cj[q] = cj[q];
    tb.ri[q] = ri[q];
  }
  tb.tiles = (const int4 *)s->d_tiles;
  tb.ntiles = s->ntiles;
  tb.s0 = s->tb_s0;
  tb.s1 = s->tb_s1;
  tb.ra = s->tb_ra;
  tb.rb = s->tb_rb;
  tb.nseg = s->tb_nseg;
  tb.L = s->tb_L;
  tb.cpl = s->tb_built_c;
  return tb;
}

// K steps of an MPI solver in one blocked launch (same clock, source and NTFF
// samples as K calls of enqueue_step), then the fields swap sets.
template <typename R>
static void enqueue_block(fdtd_sim *s, int K)
{
  const StencilView<R> v = view_of<R>(s);
  const NtffView n = ntff_view(s);
  cudaStream_t st = s->stream;
  const bool lines = s->ntff_mode == 2;  // mode 3: no time-domain NTFF
  TBlockView<R> tb = tblock_view<R>(s, lines);
  double t = s->time, rc = s->ray_coef;
  const double t_first = t;
  for (int l = 0; l < K; l++) {  // field.c:312-315 per step
    const double wt = s->geo.omega_s * t;
    tb.sc[l] = make_double2(rc * cos(wt), -rc * sin(wt));
    t = t + 1.0;
    rc = 1.0 - exp(-pow(0.01 * t, 2));
  }
  if (!s->mpi) {  // serial: the pulse of the block's first step, as enqueue_step builds it
    if (s->tm) {
      tb.pulse[0] = pulse_step(s, t_first, 0, 0, 1.0);
    } else {
      const double co = cos((s->cfg.angle_deg + 90) * M_PI / 180.0);
      const double si = sin((s->cfg.angle_deg + 90) * M_PI / 180.0);
      if (co != 0.0) tb.pulse[0] = pulse_step(s, t_first, 0.5, 0.0, co);
      if (si != 0.0) tb.pulse[1] = pulse_step(s, t_first, 0.0, 0.5, si);
    }
    // at 0 degrees the pulse depends on the row only: one table per pulse and
    // block instead of a double-precision exp and sincos per cell and level
    if (s->cfg.angle_deg == 0 && s->d_ptab)
      for (int p = 0; p < 2; p++)
        if (tb.pulse[p].kind) {
          PulseRow *tab = (PulseRow *)s->d_ptab + (size_t)p * kMaxTBlock * s->nxa;
          launch_pulse_rows(tb.pulse[p], K, s->nxa, tab, st);
          s->launches += 1;
          tb.ptab[p] = tab;
        }
  }
  const double coef = s->mpi ? 1.0 / (4 * M_PI * s->c0 * 1.0e6) : 1.0;  // mpiTM_UPML.c:852-854; serial: 1
  mark(s);
  if (s->mpi) launch_tblock<R>(v, tb, K, s->tm, st);
  else launch_tblock_serial<R>(v, tb, K, s->tm, st);
  mark(s);
  mark(s);
  s->launches += (tb.s1 > tb.s0 && tb.nseg > 0 ? 1 : 0) + (tb.ntiles > 0 ? 1 : 0);
  if (lines) {
    launch_line_gather<R>(v, tb, n, coef, K, s->nb_pending, s->tm, st);
    s->launches += 1;
    if (s->nb_pending == 0) s->pending_t0 = t_first - 1;
    s->nb_pending += K;
  }
  mark(s);
  if (lines && s->nb_pending == s->ntff_block) {
    deposit_pending(s, n, st);
  }
  mark(s);
  if (s->profiling) s->prof_steps += K;
  for (int a = 0; a < kMaxSlots; a++) std::swap(s->d_f[a], s->d_f2[a]);
  s->time = t;
  s->ray_coef = rc;
}

template <typename R>
static int autotune_impl(fdtd_sim *s, int *k_out, int *rows_out, double *ms_out)
{
  cudaStream_t st = s->stream;
  if (int rc = tb_prepare(s, 1, 16, 1)) return rc;  // allocates the spare set
  cudaEvent_t a = nullptr, b = nullptr;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  auto timed = [&](auto &&fn) -> double {  // ms per call: one warm call, then >= 3 calls and >= ~20 ms
    fn();
    cudaEventRecord(a, st);
    fn();
    cudaEventRecord(b, st);
    cudaEventSynchronize(b);
    float one = 0;
    cudaEventElapsedTime(&one, a, b);
    const int reps = std::max(3, std::min(200, (int)(20.0 / std::max(one, 1e-3f))));
    cudaEventRecord(a, st);
    for (int q = 0; q < reps; q++) fn();
    cudaEventRecord(b, st);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    return ms / reps;
  };
  // one-step kernels, run in place on a copy of the fields in the spare set
  const size_t bytes = (size_t)s->nxa * s->pitch * s->esize;
  for (int q = 0; q < s->nslots; q++) CK(cudaMemcpyAsync(s->d_f2[q], s->d_f[q], bytes, cudaMemcpyDeviceToDevice, st));
  StencilView<R> vs = view_of<R>(s);
  for (int q = 0; q < kMaxSlots; q++) vs.f[q] = (typename Cplx<R>::T *)s->d_f2[q];
  SourceStep cw{};
  cw.kind = 1;
  cw.s_re = s->ray_coef;
  // the serial solvers' sources: the pulse at the current step (enqueue_step's)
  SourceStep pz{}, px{}, py{};
  if (!s->mpi) {
    if (s->tm) {
      pz = pulse_step(s, s->time, 0, 0, 1.0);
    } else {
      const double co = cos((s->cfg.angle_deg + 90) * M_PI / 180.0);
      const double si = sin((s->cfg.angle_deg + 90) * M_PI / 180.0);
      if (co != 0.0) px = pulse_step(s, s->time, 0.5, 0.0, co);
      if (si != 0.0) py = pulse_step(s, s->time, 0.0, 0.5, si);
    }
  }
  double best = timed([&] {
    if (s->mpi && s->tm) {
      launch_tm_e<R>(vs, cw, st);
      launch_tm_h<R>(vs, st);
    } else if (s->mpi) {
      launch_te_e<R>(vs, SourceStep{}, cw, st);
      launch_te_h<R>(vs, st);
    } else if (s->tm) {  // fdtdTM_upml.c:54-66
      launch_tm_h<R>(vs, st);
      launch_tm_e<R>(vs, pz, st);
    } else {             // fdtdTE_upml.c:168-192
      launch_te_h<R>(vs, st);
      launch_te_e<R>(vs, px, py, st);
    }
  });
  int best_k = 0, best_l = 0, best_c = 1;
  s->tune_table.assign({0.0, 0.0, 1.0, best});
  const int depths[4] = {1, 2, 4, 8};
  for (int K : depths) {
    if (K == 8 && (!s->f32 || !s->mpi)) continue;
    for (int cpl = 1; cpl <= 2; cpl++) {
    if (cpl == 2 && !(s->f32 && (K == 2 || K == 4))) continue;
    for (int L = 16; L <= 512; L *= 2) {
      if ((s->ni + L - 1) / L > 65535) continue;
      if (int rc = tb_prepare(s, K, L, cpl)) {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        return rc;
      }
      const StencilView<R> v = view_of<R>(s);  // reads the current set, writes the spare one
      TBlockView<R> tb = tblock_view<R>(s, false);
      tb.sc[0] = make_double2(s->ray_coef, 0.0);
      for (int l = 1; l < K; l++) tb.sc[l] = tb.sc[0];
      tb.pulse[0] = s->tm ? pz : px;
      tb.pulse[1] = s->tm ? SourceStep{} : py;
      const bool tables = !s->mpi && s->cfg.angle_deg == 0 && s->d_ptab;
      const double ms = timed([&] {
        if (s->mpi) {
          launch_tblock<R>(v, tb, K, s->tm, st);
          return;
        }
        for (int p = 0; p < 2 && tables; p++)  // enqueue_block's per-launch pulse tables
          if (tb.pulse[p].kind) {
            PulseRow *tab = (PulseRow *)s->d_ptab + (size_t)p * kMaxTBlock * s->nxa;
            launch_pulse_rows(tb.pulse[p], K, s->nxa, tab, st);
            tb.ptab[p] = tab;
          }
        launch_tblock_serial<R>(v, tb, K, s->tm, st);
      }) / K;
      s->tune_table.insert(s->tune_table.end(), {(double)K, (double)L, (double)cpl, ms});
      if (ms < best) {
        best = ms;
        best_k = K;
        best_l = L;
        best_c = cpl;
      }
    }
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  CK(cudaGetLastError());
  s->tblock = best_k;
  s->tb_rows = best_l;
  s->tb_cols = best_c;
  if (k_out) *k_out = best_k;
  if (rows_out) *rows_out = best_l;
  if (ms_out) *ms_out = best;
  return FDTD_OK;
}

extern "C" int fdtd_autotune(fdtd_sim *s, int *k_out, int *rows_out, double *ms_per_step_out)
{
  if (!s) return fail(FDTD_E_ARG, "null simulation");
  if (s->family != 0) return fail(FDTD_E_UNSUPPORTED, "temporal blocking needs a UPML solver");
  if (int rc = flush_ntff(s)) return rc;
  return s->f32 ? autotune_impl<float>(s, k_out, rows_out, ms_per_step_out)
                : autotune_impl<double>(s, k_out, rows_out, ms_per_step_out);
}

extern "C" int fdtd_autotune_report(const fdtd_sim *s, double *out, int cap)
{
  if (!s) return -fail(FDTD_E_ARG, "null simulation");
  const int n = (int)(s->tune_table.size() / 4);
  if (out)
    for (int q = 0; q < std::min(n, cap) * 4; q++) out[q] = s->tune_table[q];
  return n;
}

extern "C" int fdtd_profile_enable(fdtd_sim *s, int on)
{
  if (!s) return fail(FDTD_E_ARG, "null simulation");
  CK(cudaStreamSynchronize(s->stream));
  s->profiling = on != 0;
  s->ev_used = 0;
  s->prof_steps = 0;
  return FDTD_OK;
}

extern "C" int fdtd_profile_read(fdtd_sim *s, double *ms_out, long long *steps)
{
  if (!s || !ms_out) return fail(FDTD_E_ARG, "null argument");
  CK(cudaStreamSynchronize(s->stream));
  double acc[4] = {0, 0, 0, 0};
  // event order per step: start, after 1st stencil, after 2nd stencil, after gather, after deposit
  const int first = s->mpi ? 0 : 1, second = s->mpi ? 1 : 0;
  const int cls[4] = {first, second, 2, 3};
  for (size_t q = 0; q + 5 <= s->ev_used; q += 5)
    for (int c = 0; c < 4; c++) {
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, s->ev_pool[q + c], s->ev_pool[q + c + 1]));
      acc[cls[c]] += ms;
    }
  for (int c = 0; c < 4; c++) ms_out[c] = acc[c];
  if (steps) *steps = s->prof_steps;
  s->ev_used = 0;
  s->prof_steps = 0;
  return FDTD_OK;
}

// ------------------------------------------------- split-field / NS solvers

// Per-cell coefficients of the split-field PML solvers (fdtdTM.c:167-242,
// fdtdTE.c:170-238) and the NS-FDTD solvers (nsFdtdTM.c:231-307,
// nsFdtdTE.c:100-181), from the permittivity as it is now, in the reference's
// expression order (this file is compiled without contraction).  Layout:
// fdtd_split.cu.
static int split_coefficients(fdtd_sim *s)
{
  const fdtd_geometry &g = s->geo;
  const int NX = g.n_px, NY = g.n_py, P = s->pitch, npml = g.n_pml;
  const size_t plane = (size_t)s->nxa * P;
  std::vector<double> eps[3];
  for (int a = 0; a < 3; a++) {
    eps[a].resize((size_t)NX * NY);
    if (int rc = fdtd_get_eps(s, a, FDTD_LAYOUT_GLOBAL, eps[a].data())) return rc;
  }
  for (int a = 0; a < 3; a++)
    for (int x = 1; x < NX - 1; x++)
      for (int y = 1; y < NY - 1; y++) {
        const double e = eps[a][(size_t)x * NY + y];
        if (!(e > 0.0) || !std::isfinite(e)) return fail(FDTD_E_ARG, "permittivity must be finite and > 0 inside");
      }
  std::vector<double> c((size_t)s->ncoef * plane, 0.0);
  auto C = [&](int q, int x, int y) -> double & { return c[q * plane + (size_t)x * P + y]; };
  auto sx = [&](double x) { return sigma_axis(x, npml, g.n_x, NX); };  // field_sigmaX (field.c:259-270)
  auto sy = [&](double y) { return sigma_axis(y, npml, g.n_y, NY); };  // field_sigmaY (field.c:272-283)
  const double EPS0 = 1.0, C0 = kC, MU0 = 1.0 / kC / kC, LIGHT = kC;   // field.h:70-74
  const double R = 1.0e-8, M = 2.0;
  // field.c:288-295 pmlCoef / pmlCoef_LXY
  auto pml = [](double ep, double sig) { return (1.0 - sig / ep) / (1.0 + sig / ep); };
  auto lxy = [](double ep, double sig) { return 1.0 / (ep + sig); };
  // nsFdtdTM.c:221-229 beta / coef1
  auto beta = [](double a) { return tanh(a) / (1 + pow(tanh(a), 2)); };
  auto coef1 = [](double a, double b) { return (1 - b) / (1 + b); };
  const double w_s = g.omega_s, k_s = g.k_s;
  // source amplitude of field_nsScatteredWaveNotUPML (field.c:168-174) at permittivity e
  auto ns_amp = [&](double e) {
    const double n = sqrt(e / EPS0);
    const double u0 = sin(w_s * 0.5) / sin(k_s * 0.5);
    const double u1 = sin(w_s * 0.5) / sin(n * k_s * 0.5);
    const double _n = u0 / u1;
    return 1.0 / (_n * n) - 1.0;
  };
  // u z / (1 + b) style factors of the NS coefficients: u = sin(w/2) / sin(k n / 2)
  auto ns_u = [&](double e) {
    const double n = sqrt(e / EPS0);
    const double kk = k_s * n;
    return sin(w_s * 0.5) / sin(kk * 0.5);
  };
  switch (s->solver) {
  case FDTD_TM_2D: {
    const double sig_max = -(M + 1.0) * EPS0 * LIGHT / 2.0 / npml * log(R);
    for (int x = 0; x < NX; x++)
      for (int y = 0; y < NY; y++) {
        const double eez = eps[0][(size_t)x * NY + y];
        const double sig_ez_x = sig_max * sx(x), sig_ez_y = sig_max * sy(y);
        const double sig_hx_yy = MU0 / EPS0 * (sig_max * sy(y + 0.5));
        const double sig_hy_xx = MU0 / EPS0 * (sig_max * sx(x + 0.5));
        C(0, x, y) = pml(eez, sig_ez_x);
        C(1, x, y) = lxy(eez, sig_ez_x);
        C(2, x, y) = pml(eez, sig_ez_y);
        C(3, x, y) = lxy(eez, sig_ez_y);
        C(4, x, y) = pml(MU0, sig_hx_yy);
        C(5, x, y) = lxy(MU0, sig_hx_yy);
        C(6, x, y) = pml(MU0, sig_hy_xx);
        C(7, x, y) = lxy(MU0, sig_hy_xx);
        C(8, x, y) = EPS0 / eez - 1.0;
      }
    break;
  }
  case FDTD_TE_2D: {
    const double sig_max = -(M + 1.0) * EPS0 * LIGHT / 2.0 / npml * log(R);
    for (int x = 0; x < NX; x++)
      for (int y = 0; y < NY; y++) {
        const double eex = eps[0][(size_t)x * NY + y], eey = eps[1][(size_t)x * NY + y];
        const double sig_ex_y = sig_max * sy(y), sig_ey_x = sig_max * sx(x);
        const double sig_hz_xx = MU0 / EPS0 * (sig_max * sx(x + 0.5));
        const double sig_hz_yy = MU0 / EPS0 * (sig_max * sy(y + 0.5));
        C(0, x, y) = pml(eex, sig_ex_y);
        C(1, x, y) = lxy(eex, sig_ex_y);
        C(2, x, y) = pml(eey, sig_ey_x);
        C(3, x, y) = lxy(eey, sig_ey_x);
        C(4, x, y) = pml(MU0, sig_hz_xx);
        C(5, x, y) = lxy(MU0, sig_hz_xx);
        C(6, x, y) = pml(MU0, sig_hz_yy);
        C(7, x, y) = lxy(MU0, sig_hz_yy);
        C(8, x, y) = EPS0 / eey - 1.0;
      }
    break;
  }
  case FDTD_NS_TM_2D: {
    const double sig_max = -(M + 1.0) * EPS0 * C0 / npml * log(R);
    for (int x = 0; x < NX; x++)
      for (int y = 0; y < NY; y++) {
        const size_t k = (size_t)x * NY + y;
        const double eez = eps[0][k], ehx = eps[1][k], ehy = eps[2][k];
        const double sig_ez_x = sig_max * sx(x), sig_ez_y = sig_max * sy(y);
        const double sig_hx_y = sig_max * sy(y + 0.5), sig_hy_x = sig_max * sx(x + 0.5);
        const double a_hx_y = sig_hx_y / (2 * EPS0), a_hy_x = sig_hy_x / (2 * EPS0);
        const double a_ez_x = sig_ez_x / (2 * EPS0), a_ez_y = sig_ez_y / (2 * EPS0);
        const double b_hx_y = beta(a_hx_y), b_hy_x = beta(a_hy_x), b_ez_x = beta(a_ez_x), b_ez_y = beta(a_ez_y);
        const double z_ez = sqrt(MU0 / eez), u_ez = ns_u(eez);
        C(0, x, y) = coef1(a_ez_x, b_ez_x);
        C(1, x, y) = u_ez * z_ez / (1 + b_ez_x);
        C(2, x, y) = coef1(a_ez_y, b_ez_y);
        C(3, x, y) = u_ez * z_ez / (1.0 + b_ez_x);  // nsFdtdTM.c:287: b_ez_x, as written
        const double z_hx = sqrt(MU0 / ehx), u_hx = ns_u(ehx);
        C(4, x, y) = coef1(a_hx_y, b_hx_y);
        C(5, x, y) = u_hx / z_hx / (1.0 + b_hx_y);
        const double z_hy = sqrt(MU0 / ehy), u_hy = ns_u(ehy);
        C(6, x, y) = coef1(a_hy_x, b_hy_x);
        C(7, x, y) = u_hy / z_hy / (1.0 + b_hy_x);
        C(8, x, y) = ns_amp(eez);
      }
    break;
  }
  default: {  // FDTD_NS_TE_2D, inner cells only (FOR_FOR)
    const double sig_max = -(M + 1.0) * EPS0 * C0 / npml * log(R);
    for (int x = 1; x < NX - 1; x++)
      for (int y = 1; y < NY - 1; y++) {
        const size_t k = (size_t)x * NY + y;
        const double eex = eps[0][k], eey = eps[1][k], ehz = eps[2][k];
        const double sig_ex_y = sig_max * sy(y), sig_ey_x = sig_max * sx(x);
        const double sig_hz_x = sig_max * sx(x + 0.5), sig_hz_y = sig_max * sy(y + 0.5);
        const double a_ex_y = sig_ex_y / (2 * eex), a_ey_x = sig_ey_x / (2 * eey);
        const double a_hz_x = sig_hz_x / (2 * ehz), a_hz_y = sig_hz_y / (2 * ehz);
        const double b_ex_y = beta(a_ex_y), b_ey_x = beta(a_ey_x), b_hz_x = beta(a_hz_x), b_hz_y = beta(a_hz_y);
        const double z_hz = sqrt(MU0 / ehz), u_hz = ns_u(ehz);
        C(4, x, y) = coef1(a_hz_x, b_hz_x);
        C(5, x, y) = u_hz / z_hz / (1.0 + b_hz_x);
        C(6, x, y) = coef1(a_hz_y, b_hz_y);
        C(7, x, y) = u_hz / z_hz / (1.0 + b_hz_y);
        const double z_ex = sqrt(MU0 / eex), u_ex = ns_u(eex);
        C(0, x, y) = coef1(a_ex_y, b_ex_y);
        C(1, x, y) = u_ex * z_ex / (1.0 + b_ex_y);
        const double z_ey = sqrt(MU0 / eey), u_ey = ns_u(eey);
        C(2, x, y) = coef1(a_ey_x, b_ey_x);
        C(3, x, y) = u_ey * z_ey / (1.0 + b_ey_x);
        C(8, x, y) = ns_amp(eex);
        C(9, x, y) = ns_amp(eey);
      }
    break;
  }
  }
  CK(cudaMemcpy(s->d_coef, c.data(), c.size() * sizeof(double), cudaMemcpyHostToDevice));
  s->coef_dirty = false;
  return FDTD_OK;
}

// One update() of a split-field / NS solver at (time, ray_coef).
static void enqueue_split(fdtd_sim *s, double time, double ray_coef)
{
  SplitView v{};
  for (int a = 0; a < 5; a++) v.f[a] = (double2 *)s->d_f[a];
  const size_t plane = (size_t)s->nxa * s->pitch;
  for (int q = 0; q < s->ncoef; q++) v.c[q] = (const double *)s->d_coef + q * plane;
  v.P = s->pitch;
  v.n_px = s->geo.n_px;
  v.n_py = s->geo.n_py;
  v.ray = ray_coef;
  v.t = time;
  v.w_s = s->geo.omega_s;
  const double k_s = s->geo.k_s;
  const double rad = s->cfg.angle_deg * M_PI / 180.0;  // field.c:162-163, 186-187
  v.ks_cos = cos(rad) * k_s;
  v.ks_sin = sin(rad) * k_s;
  const double r = 1.0 / 6.0 + k_s * k_s / 180.0 - pow(k_s, 4) / 23040;  // nsFdtdTM.c:117
  v.r_2 = r / 2.0;
  v.co = cos((s->cfg.angle_deg + 90) * M_PI / 180.0);  // nsFdtdTE.c:244-245
  v.si = sin((s->cfg.angle_deg + 90) * M_PI / 180.0);
  mark(s);
  launch_split_step(v, s->solver, s->stream);
  mark(s);
  mark(s);
  mark(s);
  mark(s);
  s->launches += 2;
  if (s->profiling) s->prof_steps++;
}

static int prepare_step(fdtd_sim *s)
{
  if (s->family && s->coef_dirty) return split_coefficients(s);
  if (s->ntff_mode == 1 && s->window_dirty) return build_windows(s);
  return FDTD_OK;
}

// The reference steps only while time < maxTime (field.c:317-319); past it
// the flat NTFF index leaves its allocation, so the engine refuses.
static int check_clock(const fdtd_sim *s, double time)
{
  if (!(time >= 0) || time > (double)s->cfg.step_num - 1)
    return fail(FDTD_E_STATE, "time %g outside [0, step_num-1 = %d]", time, s->cfg.step_num - 1);
  return FDTD_OK;
}

extern "C" int fdtd_update(fdtd_sim *s, double time, double ray_coef)
{
  if (!s) return fail(FDTD_E_ARG, "null simulation");
  if (int rc = check_clock(s, time)) return rc;
  if (int rc = prepare_step(s)) return rc;
  if (int rc = before_step(s, time)) return rc;
  if (s->f32) enqueue_step<float>(s, time, ray_coef);
  else enqueue_step<double>(s, time, ray_coef);
  CK(cudaGetLastError());
  return FDTD_OK;
}

extern "C" int fdtd_run(fdtd_sim *s, int n_steps)
{
  if (!s) return fail(FDTD_E_ARG, "null simulation");
  if (n_steps < 0) return fail(FDTD_E_ARG, "n_steps < 0");
  if (n_steps > 0)
    if (int rc = check_clock(s, s->time + (n_steps - 1))) return rc;
  if (int rc = prepare_step(s)) return rc;
  if (n_steps > 0)
    if (int rc = before_step(s, s->time)) return rc;
  const int K = s->tblock;
  const bool blocked = K > 0 && s->family == 0 &&
                       (s->ntff_mode == 3 || (s->ntff_mode == 2 && K <= s->ntff_block)) && n_steps >= K;
  if (blocked)
    if (int rc = tb_prepare(s, K, s->tb_rows > 0 ? s->tb_rows : tb_auto_rows(s, K, tb_cols_for(s, K)),
                            tb_cols_for(s, K)))
      return rc;
  for (int q = 0; q < n_steps; q++) {
    if (blocked && n_steps - q >= K) {
      if (s->nb_pending + K > s->ntff_block)
        if (int rc = flush_ntff(s)) return rc;
      if (s->f32) enqueue_block<float>(s, K);
      else enqueue_block<double>(s, K);
      q += K - 1;
      continue;
    }
    const double t = s->time;
    const double rc = s->ray_coef;
    if (s->f32) enqueue_step<float>(s, t, rc);
    else enqueue_step<double>(s, t, rc);
    // field.c:312-315
    s->time = t + 1.0;
    s->ray_coef = 1.0 - exp(-pow(0.01 * s->time, 2));
  }
  CK(cudaGetLastError());
  return FDTD_OK;
}

extern "C" int fdtd_get_time(const fdtd_sim *s, double *t)
{
  if (!s || !t) return fail(FDTD_E_ARG, "null argument");
  *t = s->time;
  return FDTD_OK;
}

extern "C" int fdtd_set_time(fdtd_sim *s, double t)
{
  if (!s) return fail(FDTD_E_ARG, "null simulation");
  s->time = t;
  s->ray_coef = t == 0 ? 0.0 : 1.0 - exp(-pow(0.01 * t, 2));
  return FDTD_OK;
}

extern "C" int fdtd_flush(fdtd_sim *s)
{
  if (!s) return fail(FDTD_E_ARG, "null simulation");
  return flush_ntff(s);
}

extern "C" int fdtd_synchronize(fdtd_sim *s)
{
  if (!s) return fail(FDTD_E_ARG, "null simulation");
  if (int rc = flush_ntff(s)) return rc;
  CK(cudaStreamSynchronize(s->stream));
  return FDTD_OK;
}

extern "C" long long fdtd_launch_count(const fdtd_sim *s) { return s ? s->launches : 0; }

extern "C" int fdtd_get_status(fdtd_sim *s, unsigned int *flags)
{
  if (!s || !flags) return fail(FDTD_E_ARG, "null argument");
  if (int rc = flush_ntff(s)) return rc;
  CK(cudaStreamSynchronize(s->stream));
  CK(cudaMemcpy(flags, s->d_status, sizeof(unsigned int), cudaMemcpyDeviceToHost));
  return FDTD_OK;
}

// ---------------------------------------------------------------- copy-out

static int field_slot(const fdtd_sim *s, int which)
{
  static const int tm_slot[3] = {0, 3, 4}, te_slot[3] = {0, 1, 6};
  // split-field / NS: 3, 4 are the split parts (TM Ezx, Ezy; TE Hzx, Hzy)
  static const int split_tm_slot[5] = {0, 3, 4, 1, 2}, split_te_slot[5] = {0, 1, 2, 3, 4};
  if (s->family) {
    if (which < 0 || which > 4) return -1;
    return s->tm ? split_tm_slot[which] : split_te_slot[which];
  }
  if (which < 0 || which > 2) return -1;
  return s->tm ? tm_slot[which] : te_slot[which];
}

extern "C" int fdtd_get_field(fdtd_sim *s, int which, int layout, double *out)
{
  if (!s || !out) return fail(FDTD_E_ARG, "null argument");
  const int slot = field_slot(s, which);
  if (slot < 0) return fail(FDTD_E_ARG, "field index %d out of range", which);
  if (layout != FDTD_LAYOUT_GLOBAL && layout != FDTD_LAYOUT_SOLVER) return fail(FDTD_E_ARG, "bad layout");
  // rows/cols of the array to copy, in array coordinates
  int r0, c0, nr, nc;
  if (s->mpi && layout == FDTD_LAYOUT_GLOBAL) { r0 = 1; c0 = 1; nr = s->geo.n_px; nc = s->geo.n_py; }
  else { r0 = 0; c0 = 0; nr = s->nxa; nc = s->ncols; }
  CK(cudaStreamSynchronize(s->stream));
  const char *src = (const char *)s->d_f[slot] + ((size_t)r0 * s->pitch + c0) * s->esize;
  if (!s->f32) {
    CK(cudaMemcpy2D(out, (size_t)nc * 16, src, (size_t)s->pitch * 16, (size_t)nc * 16, nr, cudaMemcpyDeviceToHost));
  } else {
    std::vector<float2> tmp((size_t)nr * nc);
    CK(cudaMemcpy2D(tmp.data(), (size_t)nc * 8, src, (size_t)s->pitch * 8, (size_t)nc * 8, nr,
                    cudaMemcpyDeviceToHost));
    for (size_t q = 0; q < tmp.size(); q++) { out[2 * q] = tmp[q].x; out[2 * q + 1] = tmp[q].y; }
  }
  return FDTD_OK;
}

extern "C" int fdtd_get_eps(fdtd_sim *s, int which, int layout, double *out)
{
  if (!s || !out) return fail(FDTD_E_ARG, "null argument");
  if (which < 0 || which > 2) return fail(FDTD_E_ARG, "eps index %d out of range", which);
  if (layout != FDTD_LAYOUT_GLOBAL && layout != FDTD_LAYOUT_SOLVER) return fail(FDTD_E_ARG, "bad layout");
  // SOLVER layout of an MPI solver includes the halo ring (1.0 there)
  const bool halo = s->mpi && layout == FDTD_LAYOUT_SOLVER;
  const int nr = halo ? s->nxa : s->geo.n_px, nc = halo ? s->ncols : s->geo.n_py;
  const double *src = (const double *)s->d_eps[which] + (halo ? 0 : global_origin(s));
  CK(cudaStreamSynchronize(s->stream));
  CK(cudaMemcpy2D(out, (size_t)nc * sizeof(double), src, (size_t)s->pitch * sizeof(double),
                  (size_t)nc * sizeof(double), nr, cudaMemcpyDeviceToHost));
  return FDTD_OK;
}

extern "C" int fdtd_get_ntff(fdtd_sim *s, int which, double *out)
{
  if (!s || !out) return fail(FDTD_E_ARG, "null argument");
  if (!s->d_ntff[0]) return fail(FDTD_E_STATE, "no time-domain NTFF (FDTD_CFG_NO_TIME_NTFF)");
  if (which < 0 || which > 2) return fail(FDTD_E_ARG, "ntff index %d out of range", which);
  if (int rc = flush_ntff(s)) return rc;
  CK(cudaStreamSynchronize(s->stream));
  CK(cudaMemcpy(out, (const double2 *)s->d_ntff[which] + kGuard, sizeof(double2) * 360 * s->geo.array_size,
                cudaMemcpyDeviceToHost));
  return FDTD_OK;
}

extern "C" int fdtd_get_ntff_guard(fdtd_sim *s, int which, double *out, int *guard)
{
  if (!s || !out) return fail(FDTD_E_ARG, "null argument");
  if (!s->d_ntff[0]) return fail(FDTD_E_STATE, "no time-domain NTFF (FDTD_CFG_NO_TIME_NTFF)");
  if (which < 0 || which > 2) return fail(FDTD_E_ARG, "ntff index %d out of range", which);
  if (int rc = flush_ntff(s)) return rc;
  CK(cudaStreamSynchronize(s->stream));
  const double2 *base = (const double2 *)s->d_ntff[which];
  CK(cudaMemcpy(out, base, sizeof(double2) * kGuard, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(out + 2 * kGuard, base + kGuard + (size_t)360 * s->geo.array_size, sizeof(double2) * kGuard,
                cudaMemcpyDeviceToHost));
  if (guard) *guard = kGuard;
  return FDTD_OK;
}

extern "C" int fdtd_reset(fdtd_sim *s)
{
  if (!s) return fail(FDTD_E_ARG, "null simulation");
  if (int rc = flush_ntff(s)) return rc;
  const size_t bytes = (size_t)s->nxa * s->pitch * s->esize;
  for (int a = 0; a < s->nslots; a++) CK(cudaMemsetAsync(s->d_f[a], 0, bytes, s->stream));
  if (s->d_dft_S)
    CK(cudaMemsetAsync(s->d_dft_S, 0, sizeof(double2) * 2 * (size_t)s->ncell * 2 * s->dft_lam.size(), s->stream));
  if (!s->mpi && s->d_ntff[0])
    for (int a = 0; a < 3; a++) CK(cudaMemsetAsync(s->d_ntff[a], 0, sizeof(double2) * s->ntff_len, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  s->time = 0;
  s->ray_coef = 0;
  return FDTD_OK;
}

extern "C" int fdtd_get_stream(fdtd_sim *s, void **stream)
{
  if (!s || !stream) return fail(FDTD_E_ARG, "null argument");
  *stream = (void *)s->stream;
  return FDTD_OK;
}

extern "C" int fdtd_device_field(fdtd_sim *s, int which, void **dptr, int *pitch, int *rows)
{
  if (!s || !dptr) return fail(FDTD_E_ARG, "null argument");
  const int slot = field_slot(s, which);
  if (slot < 0) return fail(FDTD_E_ARG, "field index %d out of range", which);
  *dptr = s->d_f[slot];
  if (pitch) *pitch = s->pitch;
  if (rows) *rows = s->nxa;
  return FDTD_OK;
}

// ---------------------------------------------------------------- far field

static int ensure_farfield(fdtd_sim *s)
{
  if (s->d_spec) return FDTD_OK;
  CK(cudaMalloc(&s->d_spec, sizeof(double) * 321 * 360));
  CK(cudaMalloc(&s->d_dirs, sizeof(double2) * 2 * 360));
  CK(cudaMalloc(&s->d_twiddle, sizeof(double2) * (kNfft / 2)));
  CK(cudaMalloc(&s->d_freq, sizeof(double2) * 360));
  std::vector<double2> dirs(2 * 360), tw(kNfft / 2);
  for (int ang = 0; ang < 360; ang++) {
    // [0..359] the spectrum's phi: ntffTM.c:169-173 ang*(M_PI/180.0) (TM), ntffTE.c:33 ang*M_PI/180.0 (TE)
    const double phi = s->tm ? ang * (M_PI / 180.0) : ang * M_PI / 180.0;
    dirs[ang] = make_double2(cos(phi), sin(phi));
    // [360..719] ntffTM_Frequency's direction (ntffTM.c:89-91)
    const double rad = ang * M_PI / 180.0;
    dirs[360 + ang] = make_double2(cos(rad), sin(rad));
  }
  for (int k = 0; k < kNfft / 2; k++) {
    const double arg = 2 * M_PI * k / kNfft;
    tw[k] = make_double2(cos(arg), sin(arg));
  }
  CK(cudaMemcpy(s->d_dirs, dirs.data(), sizeof(double2) * dirs.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(s->d_twiddle, tw.data(), sizeof(double2) * tw.size(), cudaMemcpyHostToDevice));
  return FDTD_OK;
}

extern "C" int fdtd_spectrum(fdtd_sim *s, double *out)
{
  if (!s || !out) return fail(FDTD_E_ARG, "null argument");
  if (!s->d_ntff[0]) return fail(FDTD_E_STATE, "no time-domain NTFF (FDTD_CFG_NO_TIME_NTFF)");
  if (s->cfg.step_num > kNfft)
    return fail(FDTD_E_UNSUPPORTED, "step_num %d > %d: the reference's FFT buffer overflows (ntffTM.c:214-221)",
                s->cfg.step_num, kNfft);
  if (int rc = flush_ntff(s)) return rc;
  if (int rc = ensure_farfield(s)) return rc;
  SpectrumView v{};
  for (int a = 0; a < 3; a++) v.acc[a] = (const double2 *)s->d_ntff[a];
  v.array_size = s->geo.array_size;
  v.max_time = s->cfg.step_num;
  v.tm = s->tm ? 1 : 0;
  v.h_u_nm = s->cfg.h_u_nm;
  v.c0 = s->c0;
  v.z0 = s->z0;
  v.dir = (const double2 *)s->d_dirs;
  v.twiddle = (const double2 *)s->d_twiddle;
  // ntffTM.c:165 / ntffTE.c:25: 1/(4 pi C) * csqrt(2 pi C / (i w))
  const std::complex<double> q = std::complex<double>(2 * M_PI * s->c0, 0.0) /
                                 std::complex<double>(0.0, s->geo.omega_s);
  const std::complex<double> c = (1.0 / (4 * M_PI * s->c0)) * std::sqrt(q);
  v.coef = make_double2(c.real(), c.imag());
  v.out = (double *)s->d_spec;
  launch_spectrum(v, s->stream);
  s->launches += 1;
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, s->d_spec, sizeof(double) * 321 * 360, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return FDTD_OK;
}

// ---------------------------------------------------------------- running DFT

static std::complex<double> spectrum_coef(const fdtd_sim *s)
{
  // ntffTM.c:165 / ntffTE.c:25: 1/(4 pi C) * csqrt(2 pi C / (i w))
  const std::complex<double> q = std::complex<double>(2 * M_PI * s->c0, 0.0) /
                                 std::complex<double>(0.0, s->geo.omega_s);
  return (1.0 / (4 * M_PI * s->c0)) * std::sqrt(q);
}

extern "C" int fdtd_dft_enable(fdtd_sim *s, int nlam, const int *lambda_nm)
{
  if (!s || nlam <= 0 || !lambda_nm) return fail(FDTD_E_ARG, "bad wavelength list");
  if (!s->d_ntff[0]) return fail(FDTD_E_STATE, "no NTFF path (FDTD_CFG_NO_TIME_NTFF)");
  if (s->ntff_mode != 2) return fail(FDTD_E_STATE, "the running DFT reads the time-blocked NTFF ring (mode 2)");
  if (int rc = flush_ntff(s)) return rc;
  std::vector<double> omega;
  s->dft_lam.assign(lambda_nm, lambda_nm + nlam);
  s->dft_frac.clear();
  for (int l : s->dft_lam) {
    if (l <= 0) return fail(FDTD_E_ARG, "wavelength %d nm", l);
    const double p = s->c0 * s->cfg.h_u_nm * kNfft / l;  // the spectrum's fractional bin (ntffTM.c:227)
    const double idx = floor(p);
    s->dft_frac.push_back(p - idx);
    omega.push_back(2 * M_PI * idx / kNfft);
    omega.push_back(2 * M_PI * (idx + 1) / kNfft);
  }
  const int nfreq = (int)omega.size();
  cudaFree(s->d_dft_omega);
  cudaFree(s->d_dft_P);
  cudaFree(s->d_dft_S);
  cudaFree(s->d_dft_X);
  s->d_dft_omega = s->d_dft_P = s->d_dft_S = s->d_dft_X = nullptr;
  CK(cudaMalloc(&s->d_dft_omega, sizeof(double) * nfreq));
  CK(cudaMemcpy(s->d_dft_omega, omega.data(), sizeof(double) * nfreq, cudaMemcpyHostToDevice));
  CK(cudaMalloc(&s->d_dft_P, sizeof(double2) * (size_t)kMaxNtffBlock * nfreq));
  CK(cudaMalloc(&s->d_dft_S, sizeof(double2) * 2 * (size_t)s->ncell * nfreq));
  CK(cudaMemsetAsync(s->d_dft_S, 0, sizeof(double2) * 2 * (size_t)s->ncell * nfreq, s->stream));
  CK(cudaMalloc(&s->d_dft_X, sizeof(double2) * 360 * (size_t)nfreq));
  return FDTD_OK;
}

// The far field's table of e^{i w m} over the retarded bins m = floor(shift +
// 1/2) (E) and floor(shift + 1) (H) of the path, in the simulation's buffer.
static int dft_bins(fdtd_sim *s, int nfreq, DftBins *bins)
{
  if (s->bin_nm < 0) {
    double lo = 0, hi = 0;
    if (!s->h_shift.empty()) {
      const auto mm = std::minmax_element(s->h_shift.begin(), s->h_shift.end());
      lo = *mm.first;
      hi = *mm.second;
    }
    s->bin_mlo = (int)floor(lo) - 1;
    s->bin_nm = (int)floor(hi) + 2 - s->bin_mlo + 1;
  }
  const size_t bytes = sizeof(double2) * (size_t)s->bin_nm * nfreq;
  if (bytes > s->d_dft_T_bytes) {
    CK(cudaStreamSynchronize(s->stream));  // the previous table may still be read
    cudaFree(s->d_dft_T);
    s->d_dft_T = nullptr;
    s->d_dft_T_bytes = 0;
    CK(cudaMalloc(&s->d_dft_T, bytes));
    s->d_dft_T_bytes = bytes;
  }
  bins->T = (double2 *)s->d_dft_T;
  bins->mlo = s->bin_mlo;
  bins->nm = s->bin_nm;
  return FDTD_OK;
}

int fdtd_far_field_of_sums(fdtd_sim *s, const double *d_omega, int nfreq, const double2 *d_S, double2 *d_X,
                           double scale)
{
  if (!s->d_cells) return fail(FDTD_E_STATE, "no NTFF path (FDTD_CFG_NO_TIME_NTFF)");
  if (int rc = ensure_farfield(s)) return rc;
  const std::complex<double> c = spectrum_coef(s) * scale;
  DftView d{};
  d.omega = d_omega;
  d.nfreq = nfreq;
  d.S = const_cast<double2 *>(d_S);
  DftBins bins{};
  if (int rc = dft_bins(s, nfreq, &bins)) return rc;
  launch_dft_farfield(ntff_view(s), d, s->tm ? 1 : 0, s->z0, (const double2 *)s->d_dirs,
                      make_double2(c.real(), c.imag()), bins, d_X, s->stream);
  s->launches += 1;
  CK(cudaGetLastError());
  return FDTD_OK;
}

int fdtd_far_field_of_sums_group(fdtd_sim *s, const double *d_omega, int nfreq, const double2 *const *d_S,
                                 const int *d_idx, int nmaps, double2 *d_X, size_t x_stride, double scale,
                                 cudaStream_t st)
{
  if (!s->d_cells) return fail(FDTD_E_STATE, "no NTFF path (FDTD_CFG_NO_TIME_NTFF)");
  if (int rc = ensure_farfield(s)) return rc;
  const std::complex<double> c = spectrum_coef(s) * scale;
  DftBins bins{};
  if (int rc = dft_bins(s, nfreq, &bins)) return rc;
  launch_dft_farfield_group(ntff_view(s), d_S, d_idx, nmaps, d_omega, nfreq, s->tm ? 1 : 0, s->z0,
                            (const double2 *)s->d_dirs, make_double2(c.real(), c.imag()), bins, d_X, x_stride, st);
  s->launches += 2;
  CK(cudaGetLastError());
  return FDTD_OK;
}

// X[360][2 nlam]: the far-field component's Fourier sum at the two bins of each wavelength
extern "C" int fdtd_dft_far_field(fdtd_sim *s, double *out_complex)
{
  if (!s || !out_complex) return fail(FDTD_E_ARG, "null argument");
  if (!s->d_dft_S) return fail(FDTD_E_STATE, "running DFT not enabled (fdtd_dft_enable)");
  if (int rc = flush_ntff(s)) return rc;
  if (int rc = ensure_farfield(s)) return rc;
  const std::complex<double> c = spectrum_coef(s);
  const DftView d = dft_view(s);
  DftBins bins{};
  if (int rc = dft_bins(s, d.nfreq, &bins)) return rc;
  launch_dft_farfield(ntff_view(s), d, s->tm ? 1 : 0, s->z0, (const double2 *)s->d_dirs, make_double2(c.real(), c.imag()),
                      bins, (double2 *)s->d_dft_X, s->stream);
  s->launches += 1;
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out_complex, s->d_dft_X, sizeof(double2) * 360 * (size_t)d.nfreq, cudaMemcpyDeviceToHost,
                     s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return FDTD_OK;
}

// out[nlam][360]: |E|^2 per wavelength, the spectrum's interpolation between the two bins
extern "C" int fdtd_dft_spectrum(fdtd_sim *s, double *out)
{
  if (!s || !out) return fail(FDTD_E_ARG, "null argument");
  const int nlam = (int)s->dft_lam.size();
  std::vector<double2> X(360 * (size_t)2 * nlam);
  if (int rc = fdtd_dft_far_field(s, (double *)X.data())) return rc;
  for (int l = 0; l < nlam; l++) {
    const double p = s->dft_frac[l];
    for (int ang = 0; ang < 360; ang++) {
      const double2 a = X[(size_t)ang * 2 * nlam + 2 * l], b = X[(size_t)ang * 2 * nlam + 2 * l + 1];
      const double na = a.x * a.x + a.y * a.y, nb = b.x * b.x + b.y * b.y;
      out[(size_t)l * 360 + ang] = ((1 - p) * na + p * nb) / kNfft;
    }
  }
  return FDTD_OK;
}

extern "C" int fdtd_frequency(fdtd_sim *s, double *out)
{
  if (!s || !out) return fail(FDTD_E_ARG, "null argument");
  if (s->family) return fail(FDTD_E_UNSUPPORTED, "the split-field and NS solvers have no NTFF");
  if (int rc = ensure_farfield(s)) return rc;
  FrequencyView f{};
  f.tm = s->tm ? 1 : 0;
  if (s->tm) {  // slots: 0 Ez, 3 Hx, 4 Hy
    f.e[0] = f.e[1] = s->d_f[0];
    f.h[0] = s->d_f[3];
    f.h[1] = s->d_f[4];
  } else {      // slots: 0 Ex, 1 Ey, 6 Hz
    f.e[0] = s->d_f[0];
    f.e[1] = s->d_f[1];
    f.h[0] = f.h[1] = s->d_f[6];
  }
  f.f32 = s->f32 ? 1 : 0;   // FP32 fields are widened; the transform stays FP64
  f.P = s->pitch;
  f.ox = s->ox;
  f.lt = s->geo.ntff_left;
  f.rt = s->geo.ntff_right;
  f.bm = s->geo.ntff_bottom;
  f.tp = s->geo.ntff_top;
  f.cx = s->geo.ntff_cx;
  f.cy = s->geo.ntff_cy;
  f.k_s = s->geo.k_s;
  f.scale = s->tm ? sqrt((double)s->cfg.h_u_nm) : (double)s->cfg.h_u_nm;  // ntffTM.c:156, ntffTE.c:329
  f.z0 = s->z0;
  f.dir = (const double2 *)s->d_dirs + 360;
  // ntffTM.c:31 R0 = 1e6 * field_toCellUnit(500); ntffTM.c:82 / ntffTE.c:256 coef
  const double R0 = 1.0e6 * (500.0 / s->cfg.h_u_nm);
  const std::complex<double> i_k(0.0, s->geo.k_s);
  const std::complex<double> c = std::sqrt(i_k / (8 * M_PI * R0)) * std::exp(i_k * R0);
  f.coef = make_double2(c.real(), c.imag());
  f.out = (double2 *)s->d_freq;
  launch_frequency(f, s->stream);
  s->launches += 1;
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, s->d_freq, sizeof(double2) * 360, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return FDTD_OK;
}

// field_outputElliptic (field.c:322-343): |E|^2 of field `which`, bilinearly
// interpolated as cbilinear does (myComplex.c:40-52) on the circle of radius
// 1.2 lambda_s about (N_PX/2, N_PY/2), for ang = 180 down to 0; out[q] is the
// line the reference prints as "q norm" with q = 180 - ang.  Points whose
// 2 x 2 corner cells leave the grid are refused (the reference reads outside
// its array there).
extern "C" int fdtd_elliptic(fdtd_sim *s, int which, double *out)
{
  if (!s || !out) return fail(FDTD_E_ARG, "null argument");
  const int slot = field_slot(s, which);
  if (slot < 0) return fail(FDTD_E_ARG, "field index %d out of range", which);
  const int NX = s->geo.n_px, NY = s->geo.n_py, n = 181;
  const double lambda_s = s->geo.lambda_s;
  std::vector<long long> idx(4 * n);
  std::vector<double> wx(n), wy(n);
  for (int ang = 180; ang >= 0; ang--) {
    const int q = 180 - ang;
    const double rad = ang * M_PI / 180.0;
    const double x = 1.2 * lambda_s * cos(rad) + NX / 2.0;
    const double y = 1.2 * lambda_s * sin(rad) + NY / 2.0;
    const int i = (int)floor(x), j = (int)floor(y);
    if (i < 0 || j < 0 || i + 1 >= NX || j + 1 >= NY)
      return fail(FDTD_E_ARG, "elliptic ring point (%.3f, %.3f) at %d deg leaves the %d x %d grid", x, y, ang, NX, NY);
    wx[q] = x - i;
    wy[q] = y - j;
    const long long k = (long long)(i - s->ox) * s->pitch + (j - s->ox);  // p[index] of global (i, j)
    idx[4 * q + 0] = k;                 // p[index]
    idx[4 * q + 1] = k + s->pitch;      // p[index + height]
    idx[4 * q + 2] = k + 1;             // p[index + 1]
    idx[4 * q + 3] = k + s->pitch + 1;  // p[index + height + 1]
  }
  void *d_idx = nullptr, *d_val = nullptr;
  std::vector<double2> val(4 * n);
  cudaError_t e = cudaMalloc(&d_idx, sizeof(long long) * idx.size());
  if (e == cudaSuccess) e = cudaMalloc(&d_val, sizeof(double2) * val.size());
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_idx, idx.data(), sizeof(long long) * idx.size(), cudaMemcpyHostToDevice, s->stream);
  if (e == cudaSuccess) {
    launch_point_gather(s->d_f[slot], s->f32 ? 1 : 0, (const long long *)d_idx, 4 * n, (double2 *)d_val, s->stream);
    s->launches += 1;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(val.data(), d_val, sizeof(double2) * val.size(), cudaMemcpyDeviceToHost, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  cudaFree(d_idx);
  cudaFree(d_val);
  if (e != cudaSuccess) return fail(FDTD_E_CUDA, "elliptic ring: %s", cudaGetErrorString(e));
  for (int q = 0; q < n; q++) {
    const double dx = wx[q], dy = wy[q];
    const double2 *p = &val[4 * q];
    // p[index]*(1-dx)*(1-dy) + p[index+height]*dx*(1-dy) + p[index+1]*(1-dx)*dy + p[index+height+1]*dx*dy
    const double re = p[0].x * (1.0 - dx) * (1.0 - dy) + p[1].x * dx * (1.0 - dy) + p[2].x * (1.0 - dx) * dy + p[3].x * dx * dy;
    const double im = p[0].y * (1.0 - dx) * (1.0 - dy) + p[1].y * dx * (1.0 - dy) + p[2].y * (1.0 - dx) * dy + p[3].y * dx * dy;
    out[q] = re * re + im * im;  // cnorm (myComplex.c:33-38)
  }
  return FDTD_OK;
}

// The text file field_outputElliptic writes: "%d %lf \n" per angle.
extern "C" int fdtd_write_elliptic(fdtd_sim *s, int which, const char *path)
{
  if (!path) return fail(FDTD_E_ARG, "null path");
  double norm[181];
  if (int rc = fdtd_elliptic(s, which, norm)) return rc;
  FILE *fp = fopen(path, "w");
  if (!fp) return fail(FDTD_E_ARG, "cannot open file %s", path);
  for (int q = 0; q < 181; q++) fprintf(fp, "%d %lf \n", q, norm[q]);
  if (fclose(fp) != 0) return fail(FDTD_E_ARG, "cannot write file %s", path);
  return FDTD_OK;
}

namespace {
// modelColorTransform over colorTransform(0) (drawer.c:230-251): green 1 less
// (1 - 1/n^2) on every channel, channels kept as float like the reference's colorf.
struct ColorF { float r, g, b; };
ColorF model_color(double n)
{
  ColorF c{0.0f, 1.0f, 0.0f};  // colorTransform(0): a = 0, g = min(1, max(0, 2)) = 1
  c.r = (float)(c.r - (1 - 1.0 / n / n));
  c.g = (float)(c.g - (1 - 1.0 / n / n));
  c.b = (float)(c.b - (1 - 1.0 / n / n));
  return c;
}
// max(0, min(255, v*255)) with the reference's macros (function.h:7-8), stored to a byte
unsigned char bmp_channel(float v)
{
  const float x = v * 255;
  const float m = 255 < x ? 255.0f : x;
  return (unsigned char)(0 > m ? 0.0f : m);
}
void put_le(std::vector<unsigned char> &b, unsigned long d, int bytes)
{
  for (int q = 0; q < bytes; q++) b.push_back((unsigned char)((d >> (8 * q)) & 0xFF));
}
}  // namespace

// drawer_outputImage (drawer.c:253-298) with putBmpHeader (drawer.c:312-395):
// a 24-bit BMP of permittivity `which` in the global frame, (N_PX & ~3) x N_PY
// pixels, rows of constant y, colour from modelColorTransform.  The header
// keeps the reference's bfSize = 54 + width * height.  (main.c:146 passes the
// solver's own eps array, which for the MPI solvers carries the halo ring;
// this writes the global frame the image is meant to show.)
extern "C" int fdtd_write_model_image(fdtd_sim *s, int which, const char *path)
{
  if (!s || !path) return fail(FDTD_E_ARG, "null argument");
  const int width = s->geo.n_px, height = s->geo.n_py;
  const int data_width = (width >> 2) << 2;
  if (data_width <= 0 || height <= 0) return fail(FDTD_E_ARG, "image of %d x %d cells has no 4-pixel column", width, height);
  std::vector<double> model((size_t)width * height);
  if (int rc = fdtd_get_eps(s, which, FDTD_LAYOUT_GLOBAL, model.data())) return rc;
  std::vector<unsigned char> out;
  out.reserve(54 + (size_t)height * data_width * 3);
  out.push_back('B');
  out.push_back('M');
  put_le(out, 54 + (unsigned long)data_width * height, 4);  // bfSize
  put_le(out, 0, 2);
  put_le(out, 0, 2);
  put_le(out, 54, 4);          // bfOffBits
  put_le(out, 40, 4);          // biSize
  put_le(out, data_width, 4);
  put_le(out, height, 4);
  put_le(out, 1, 2);           // planes
  put_le(out, 24, 2);          // bits per pixel
  for (int q = 0; q < 6; q++) put_le(out, 0, 4);
  for (int j = 0; j < height; j++)
    for (int i = 0; i < data_width; i++) {
      const ColorF c = model_color(model[(size_t)i * height + j]);
      out.push_back(bmp_channel(c.b));
      out.push_back(bmp_channel(c.g));
      out.push_back(bmp_channel(c.r));
    }
  FILE *fp = fopen(path, "wb");
  if (!fp) return fail(FDTD_E_ARG, "can not open file %s", path);
  const size_t w = fwrite(out.data(), 1, out.size(), fp);
  if (fclose(fp) != 0 || w != out.size()) return fail(FDTD_E_ARG, "can not write file %s", path);
  return FDTD_OK;
}
