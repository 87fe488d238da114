// ntff_noalloc.cu -- fdtd_ntff_step_noalloc(): the NTFF step of the MPI UPML
// solvers for callers that may not allocate device memory (see the comment
// above its declaration in include/mpifdtd_gb300.h).
//
// Same arithmetic as the engine's ntff_gather_kernel + ntff_accumulate_kernel
// (mode 0), but the path is derived from the grid on the fly, the
// retarded-time shift of every (angle, cell) pair is evaluated in the kernel
// with IEEE-rounded operations in the reference's order (bit-identical to the
// engine's host-built shift table), and the path samples live in a file-scope
// __device__ array instead of engine-allocated memory.
#include <cuda.h>  // CUcontext / CUresult types only: the two driver calls are looked up at run time
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "fdtd_internal.cuh"

namespace fdtd {
namespace {

// Scratch: the signed, scaled E and H samples of every path cell of one step
// ([0, ncell) E, [ncell, 2 ncell) H).  Every call writes the 2 ncell entries
// it reads before reading them, so nothing has to be cleared between calls.
__device__ __align__(256) double2 g_noalloc_samples[2 * FDTD_NOALLOC_MAX_PATH];
// (cos, sin) of each of the 360 observation angles, from the host libm
// (mpiTM_UPML.c:875-876), uploaded once per device.
__constant__ double2 g_noalloc_dir[360];

struct NoAllocPath {
  int tm, P;
  int i0, i1, j0, j1;        // path ranges clipped as mpiTM_UPML.c:886-887, :926-927
  int bm, tp, lt, rt, cx, cy;
  int nb, nr, ncell;         // cells on the bottom (= top) and right (= left) sides
  double rf, coef, c0;       // RFperC, 1/(4 pi C R), Courant number
  long long array_size, lo, hi;  // valid accumulator indices [lo, hi) around element 0
};

// side and array cell of path cell c, in the reference's order bottom, right, top, left
__device__ __forceinline__ void path_cell(const NoAllocPath &p, int c, int &side, int &i, int &j)
{
  if (c < p.nb) { side = 0; i = p.i0 + c; j = p.bm; return; }
  c -= p.nb;
  if (c < p.nr) { side = 1; i = p.rt; j = p.j0 + c; return; }
  c -= p.nr;
  if (c < p.nb) { side = 2; i = p.i0 + c; j = p.tp; return; }
  c -= p.nb;
  side = 3; i = p.lt; j = p.j0 + c;
}

__global__ void noalloc_gather_kernel(NoAllocPath p, const double2 *e0, const double2 *e1, const double2 *h0,
                                      const double2 *h1, double2 *samples)
{
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= p.ncell) return;
  int side, i, j;
  path_cell(p, c, side, i, j);
  const bool horiz = side == 0 || side == 2;  // bottom / top
  const long long k = (long long)i * p.P + j;
  const long long hoff = horiz ? -1 : -(long long)p.P;
  const double2 *E, *H;
  double sg;
  if (p.tm) {  // mpiTM_UPML.c:899-1017
    E = e0;
    H = horiz ? h0 : h1;
    sg = (side < 2) ? 1.0 : -1.0;
  } else {     // mpiTE_UPML.c:659-774
    E = horiz ? e0 : e1;
    H = h0;
    sg = (side < 2) ? -1.0 : 1.0;
  }
  const double2 e = E[k], ha = H[k], hb = H[k + hoff];
  double2 ev, hv;
  ev.x = sg * e.x * p.coef;
  ev.y = sg * e.y * p.coef;
  hv.x = (sg * 0.5) * (ha.x + hb.x) * p.coef;
  hv.y = (sg * 0.5) * (ha.y + hb.y) * p.coef;
  samples[c] = ev;
  samples[p.ncell + c] = hv;
}

__device__ __forceinline__ void noalloc_deposit(const NoAllocPath &p, double2 *acc, long long row, double t,
                                                double2 v)
{
  const double u = t + 0.5;
  const double mf = floor(u);
  if (!(mf > -1e15 && mf < 1e15)) return;
  const double a = u - mf, b = 1.0 - a, ab = a - b;
  const long long at = row + (long long)mf;
  if (at - 1 < p.lo || at + 1 >= p.hi) return;  // beyond the caller's guard cells: dropped
  double2 *q = acc + at;
  atomicAdd(&q[-1].x, v.x * b);
  atomicAdd(&q[-1].y, v.y * b);
  atomicAdd(&q[0].x, v.x * ab);
  atomicAdd(&q[0].y, v.y * ab);
  atomicAdd(&q[1].x, -(v.x * a));
  atomicAdd(&q[1].y, -(v.y * a));
}

__global__ void __launch_bounds__(256) noalloc_deposit_kernel(NoAllocPath p, const double2 *samples, double2 *u0,
                                                              double2 *u1, double2 *u2, double timeE)
{
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int ang = blockIdx.y;
  if (c >= p.ncell) return;
  int side, i, j;
  path_cell(p, c, side, i, j);
  const bool horiz = side == 0 || side == 2;
  const double half = p.tm ? 0.0 : 0.5;  // TE samples sit half a cell along the side
  double r2x, r2y;
  switch (side) {
  case 0: r2x = (double)(i - p.cx) + half; r2y = (double)(p.bm - p.cy); break;
  case 1: r2x = (double)(p.rt - p.cx); r2y = (double)(j - p.cy) + half; break;
  case 2: r2x = (double)(i - p.cx) + half; r2y = (double)(p.tp - p.cy); break;
  default: r2x = (double)(p.lt - p.cx); r2y = (double)(j - p.cy) + half; break;
  }
  // -(r1x r2x + r1y r2y) / C + RFperC, rounded step by step as the reference
  const double2 d = g_noalloc_dir[ang];
  const double dot = __dadd_rn(__dmul_rn(d.x, r2x), __dmul_rn(d.y, r2y));
  const double sh = __dadd_rn(-__ddiv_rn(dot, p.c0), p.rf);
  double2 *acc[3] = {u0, u1, u2};
  const int uid = p.tm ? (horiz ? 0 : 1) : 2;
  const int wid = p.tm ? 2 : (horiz ? 0 : 1);
  const long long row = (long long)ang * p.array_size;
  noalloc_deposit(p, acc[uid], row, timeE + sh, samples[c]);
  noalloc_deposit(p, acc[wid], row, (timeE + 0.5) + sh, samples[p.ncell + c]);
}

std::mutex g_setup_mutex;
constexpr int kMaxDevices = 64;
double2 *g_scratch_addr[kMaxDevices];  // device address of g_noalloc_samples per device
bool g_ready[kMaxDevices];
unsigned long long g_ctx_id[kMaxDevices];  // the context the set-up was made in (0: unknown)

// Unique id of the calling thread's current CUDA context (cuCtxGetId), or 0
// when the driver does not offer it.  A cudaDeviceReset destroys the primary
// context, with it the module's __device__ / __constant__ storage; the next
// context has another id, which tells the set-up to run again.
unsigned long long current_context_id()
{
  using GetCurrent = CUresult (*)(CUcontext *);
  using GetId = CUresult (*)(CUcontext, unsigned long long *);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {  // under g_setup_mutex
    void *f0 = nullptr, *f1 = nullptr;
    cudaDriverEntryPointQueryResult q0, q1;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000, cudaEnableDefault, &q0) == cudaSuccess &&
        q0 == cudaDriverEntryPointSuccess &&
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
        q1 == cudaDriverEntryPointSuccess) {
      get_current = (GetCurrent)f0;
      get_id = (GetId)f1;
    }
    cudaGetLastError();
    looked_up = true;
  }
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS)
    return 0;
  return id;
}

}  // namespace
}  // namespace fdtd

using namespace fdtd;

extern "C" int fdtd_ntff_step_noalloc(const fdtd_ntff_step_args *a, void *stream)
{
  if (!a) return set_error(FDTD_E_ARG, "null argument");
  if (a->solver != FDTD_MPI_TM_UPML && a->solver != FDTD_MPI_TE_UPML)
    return set_error(FDTD_E_ARG, "the allocation-free NTFF step supports the MPI UPML solvers (4, 5)");
  if (a->cfg.precision != FDTD_F64) return set_error(FDTD_E_ARG, "FP64 fields only");
  fdtd_geometry g;
  if (int rc = fdtd_geometry_of(&a->cfg, &g)) return rc;
  const bool tm = a->solver == FDTD_MPI_TM_UPML;
  if (!a->e0 || !a->h0 || (tm ? !a->h1 : !a->e1) || !a->acc[0] || !a->acc[1] || !a->acc[2])
    return set_error(FDTD_E_ARG, "null field or accumulator pointer");
  if (a->pitch < g.n_py + 2) return set_error(FDTD_E_ARG, "pitch %d < N_PY + 2 = %d", a->pitch, g.n_py + 2);
  if (!(a->time >= 0) || a->time > (double)a->cfg.step_num - 1)
    return set_error(FDTD_E_STATE, "time %g outside [0, step_num-1 = %d]", a->time, a->cfg.step_num - 1);

  NoAllocPath p{};
  p.tm = tm ? 1 : 0;
  p.P = a->pitch;
  const int nrow = g.n_px + 2, ncol = g.n_py + 2;
  p.bm = g.ntff_bottom; p.tp = g.ntff_top; p.lt = g.ntff_left; p.rt = g.ntff_right;
  p.cx = g.ntff_cx; p.cy = g.ntff_cy;
  p.i0 = p.lt > 1 ? p.lt : 1;
  p.i1 = p.rt < nrow ? p.rt : nrow;
  p.j0 = p.bm > 1 ? p.bm : 1;
  p.j1 = p.tp < ncol ? p.tp : ncol;
  p.nb = p.i1 - p.i0;
  p.nr = p.j1 - p.j0;
  p.ncell = 2 * p.nb + 2 * p.nr;
  if (p.ncell > FDTD_NOALLOC_MAX_PATH)
    return set_error(FDTD_E_ARG, "NTFF path of %d cells exceeds the static scratch (%d cells)", p.ncell,
                     FDTD_NOALLOC_MAX_PATH);
  p.rf = g.rf_per_c;
  p.c0 = config_courant(a->cfg);
  p.coef = 1.0 / (4 * M_PI * p.c0 * 1.0e6);  // mpiTM_UPML.c:852-854
  p.array_size = g.array_size;
  p.lo = -FDTD_NTFF_GUARD;
  p.hi = 360LL * g.array_size + FDTD_NTFF_GUARD;

  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_error(FDTD_E_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return set_error(FDTD_E_CUDA, "device %d out of range", dev);
  double2 *scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    const unsigned long long ctx = current_context_id();
    if (g_ready[dev] && ctx != 0 && ctx != g_ctx_id[dev]) g_ready[dev] = false;  // a new context: set up again
    if (!g_ready[dev]) {  // once per device context, with that device current
      void *addr = nullptr;
      e = cudaGetSymbolAddress(&addr, g_noalloc_samples);
      if (e != cudaSuccess) return set_error(FDTD_E_CUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
      double2 dir[360];
      for (int ang = 0; ang < 360; ang++) {
        const double rad = ang * M_PI / 180.0;
        dir[ang] = make_double2(cos(rad), sin(rad));
      }
      e = cudaMemcpyToSymbol(g_noalloc_dir, dir, sizeof dir);
      if (e != cudaSuccess) return set_error(FDTD_E_CUDA, "cudaMemcpyToSymbol: %s", cudaGetErrorString(e));
      g_scratch_addr[dev] = (double2 *)addr;
      g_ctx_id[dev] = ctx;
      g_ready[dev] = true;
    }
    scratch = g_scratch_addr[dev];
  }
  cudaStream_t st = (cudaStream_t)stream;
  noalloc_gather_kernel<<<(p.ncell + 255) / 256, 256, 0, st>>>(p, (const double2 *)a->e0, (const double2 *)a->e1,
                                                                (const double2 *)a->h0, (const double2 *)a->h1,
                                                                scratch);
  dim3 grid((unsigned)((p.ncell + 255) / 256), 360);
  noalloc_deposit_kernel<<<grid, 256, 0, st>>>(p, scratch, (double2 *)a->acc[0], (double2 *)a->acc[1],
                                               (double2 *)a->acc[2], a->time - 1);
  e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(FDTD_E_CUDA, "launch: %s", cudaGetErrorString(e));
  return FDTD_OK;
}
