// fdtd_setup.cu -- one-time device kernels: permittivity fill from the
// built-in models and the 1/eps tables the E updates read.
//
// The model is evaluated at exactly the staggered points and sub-cell modes
// of the solvers' setCoefficient():
//   MPI TM   EZ (x,y,D_XY)  HX (x,y+.5,D_Y)  HY (x+.5,y,D_X)    mpiTM_UPML.c:680-682
//   serial TM  EZ (x,y,D_XY)  HX (x,y+.5,D_XY) HY (x+.5,y,D_XY) fdtdTM_upml.c:237-239
//   TE       EX (x+.5,y,D_Y)  EY (x,y+.5,D_X)
//            HZ 0.5*(eps(x+.5,y+.5,D_X) + eps(x+.5,y+.5,D_Y))  mpiTE_UPML.c:503-505
//   split-field and NS TM as MPI TM (fdtdTM.c:209-211, nsFdtdTM.c:244-246),
//   split-field TE as TE (fdtdTE.c:210-212), NS TE with HZ (x+.5,y+.5,D_XY)
//   (nsFdtdTE.c:119-121)
#include <cuda_runtime.h>

#include "fdtd_internal.cuh"
#include "models_eval.h"

namespace fdtd {

__global__ void eps_model_kernel(double *e0, double *e1, double *e2, int P, int nxa, int ncols, int ox, int n_px,
                                 int n_py, int tm, int alt, mdl_params m)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  // every column of the pitch is written (padding and halo get 1.0) so the
  // 1/eps pass over the whole allocation never reads unset memory
  if (i >= nxa || j >= P) return;
  const size_t k = (size_t)i * P + j;
  const int x = i + ox, y = j + ox;
  double a = 1.0, b = 1.0, c = 1.0;
  if (x >= 0 && x < n_px && y >= 0 && y < n_py) {
    if (tm) {
      a = mdl_eps(&m, x, y, 1, 1);
      b = alt ? mdl_eps(&m, x, y + 0.5, 0, 1) : mdl_eps(&m, x, y + 0.5, 1, 1);
      c = alt ? mdl_eps(&m, x + 0.5, y, 1, 0) : mdl_eps(&m, x + 0.5, y, 1, 1);
    } else {
      a = mdl_eps(&m, x + 0.5, y, 0, 1);
      b = mdl_eps(&m, x, y + 0.5, 1, 0);
      c = alt ? mdl_eps(&m, x + 0.5, y + 0.5, 1, 1)
              : 0.5 * (mdl_eps(&m, x + 0.5, y + 0.5, 1, 0) + mdl_eps(&m, x + 0.5, y + 0.5, 0, 1));
    }
  }
  e0[k] = a;
  e1[k] = b;
  e2[k] = c;
}

__global__ void inv_eps_kernel(const double *eps, double *ie64, float *ie32, size_t count, unsigned int *status)
{
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < count; k += (size_t)gridDim.x * blockDim.x) {
    const double e = eps[k];
    if (!(e > 0.0) || !isfinite(e)) atomicOr(status, kStatusBadEps);
    const double v = 1.0 / e;  // EPSILON_0_S / eps (mpiTM_UPML.c:370), IEEE division
    ie64[k] = v;
    ie32[k] = (float)v;
  }
}

__global__ void fill_kernel(double *p, double v, size_t count)
{
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < count; k += (size_t)gridDim.x * blockDim.x)
    p[k] = v;
}

void launch_eps_model(double *e0, double *e1, double *e2, int P, int nxa, int ncols, int ox, int n_px, int n_py,
                      bool tm, bool alt, const mdl_params &m, cudaStream_t st)
{
  (void)ncols;
  dim3 b(32, 8), g((unsigned)((P + 31) / 32), (unsigned)((nxa + 7) / 8));
  eps_model_kernel<<<g, b, 0, st>>>(e0, e1, e2, P, nxa, ncols, ox, n_px, n_py, tm ? 1 : 0, alt ? 1 : 0, m);
}

void launch_inv_eps(const double *eps, double *ie64, float *ie32, size_t count, unsigned int *status,
                    cudaStream_t st)
{
  inv_eps_kernel<<<152 * 8, 256, 0, st>>>(eps, ie64, ie32, count, status);
}

void launch_fill(double *p, double v, size_t count, cudaStream_t st)
{
  fill_kernel<<<152 * 8, 256, 0, st>>>(p, v, count);
}

}  // namespace fdtd
