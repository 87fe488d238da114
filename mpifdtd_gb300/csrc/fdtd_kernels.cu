// fdtd_kernels.cu -- sm_103a kernels of the 2-D UPML FDTD time step.
//
// One time step of the MPI solvers (mpiTM_UPML.c:196-217, mpiTE_UPML.c:290-304)
// is four launches:
//   e-half  : calcJD + calcE + scatteredWave fused (one sweep over the grid)
//   h-half  : calcMB + calcH fused
//   gather  : the tangential E/H samples of the NTFF surface
//   accum   : the 360-angle retarded-time deposit (mpiTM_UPML.c:849-1037)
// The serial solvers run h-half, e-half (+ pulse), gather, accum
// (fdtdTM_upml.c:54-66, fdtdTE_upml.c:168-192).
//
// Interior cells (sigma_x = sigma_y = 0 at every stagger) have every UPML
// coefficient exactly 1, so the J/M auxiliaries drop out algebraically:
//   TM: Dz += curl H ; Hx -= dEz/dy / mu0 ; Hy += dEz/dx / mu0
// which is the reference's update with C_* = 1 up to rounding (the reference
// computes (Dz + Jz') - Jz where this computes Dz + (Jz' - Jz)).  PML cells run
// the full Gedney update with coefficients from the 1-D tables.  H is stored
// instead of B (B/mu0, mpiTM_UPML.c:526-527) and M is stored scaled by 1/mu0,
// which turns every H update into one FMA per component.
#include <cuda_runtime.h>

#include "fdtd_internal.cuh"
#include "stencil_ops.cuh"

namespace fdtd {

// ------------------------------------------------------------------ TM
//
// Each thread owns one column j and ROWS consecutive rows i (x).  Walking the
// rows in order lets a thread reuse the neighbour row it loaded for the
// previous cell (Hy[k-P] of row i is Hy[k] of row i-1; Ez[k+P] of row i is
// Ez[k] of row i+1) and gives the scheduler ROWS independent cell updates to
// overlap with the FP64 pipe.

// calcJD + calcE + scatteredWave (mpiTM_UPML.c:431-458, :337-374)
template <typename R, int ROWS>
__global__ void __launch_bounds__(256) tm_e_kernel(StencilView<R> v, SourceStep s)
{
  using T = typename Cplx<R>::T;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i0 = (blockIdx.y * blockDim.y + threadIdx.y) * ROWS + 1;
  if (j < 1 || j > v.nj || i0 > v.ni) return;
  T *Ez = v.f[0], *Dz = v.f[1], *Jz = v.f[2];
  const T *Hx = v.f[3], *Hy = v.f[4];
  size_t k = (size_t)i0 * v.P + j;
  T hyl = ldro(Hy + k - v.P);
#pragma unroll
  for (int r = 0; r < ROWS; r++, k += v.P) {
    const int i = i0 + r;
    if (i > v.ni) break;
    const T hyk = ldro(Hy + k), hxk = ldro(Hx + k), hxb = ldro(Hx + k - 1);
    T curl;
    curl.x = ((hyk.x - hyl.x) - hxk.x) + hxb.x;
    curl.y = ((hyk.y - hyl.y) - hxk.y) + hxb.y;
    hyl = hyk;
    T dz = Dz[k];
    if (interior(v, i, j)) {
      dz = cadd(dz, curl);
    } else {
      T jz = Jz[k];
      tm_e_pml(v, i, j, curl, dz, jz);
      Jz[k] = jz;
    }
    Dz[k] = dz;
    const R ie = v.inv_eps[0][k];
    T ez = dz;
    if (!is_one(ie)) {
      ez = cscale(dz, ie);
      apply_source<R>(v, s, i, j, ie, ez);
    }
    Ez[k] = ez;
  }
}

// calcMB + calcH (mpiTM_UPML.c:491-530)
template <typename R, int ROWS>
__global__ void __launch_bounds__(256) tm_h_kernel(StencilView<R> v)
{
  using T = typename Cplx<R>::T;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i0 = (blockIdx.y * blockDim.y + threadIdx.y) * ROWS + 1;
  if (j < 1 || j > v.nj || i0 > v.ni) return;
  const T *Ez = v.f[0];
  T *Hx = v.f[3], *Hy = v.f[4], *Mx = v.f[5], *My = v.f[6];
  size_t k = (size_t)i0 * v.P + j;
  T ek = ldro(Ez + k);
#pragma unroll
  for (int r = 0; r < ROWS; r++, k += v.P) {
    const int i = i0 + r;
    if (i > v.ni) break;
    const T et = ldro(Ez + k + 1), er = ldro(Ez + k + v.P);
    const T dEx = csub(et, ek);           // Ez[k_top] - Ez[k]
    const T dEy = csub(ek, er);           // -Ez[k_rht] + Ez[k]
    ek = er;
    T hx = Hx[k], hy = Hy[k];
    if (interior(v, i, j)) {
      hx.x -= v.inv_mu * dEx.x; hx.y -= v.inv_mu * dEx.y;
      hy.x -= v.inv_mu * dEy.x; hy.y -= v.inv_mu * dEy.y;
    } else {
      T mx = Mx[k], my = My[k];
      tm_h_pml(v, i, j, dEx, dEy, hx, hy, mx, my);
      Mx[k] = mx;
      My[k] = my;
    }
    Hx[k] = hx;
    Hy[k] = hy;
  }
}

// ------------------------------------------------------------------ TE

// calcJD + calcE + scatteredWave on Ey (mpiTE_UPML.c:337-375, :250-281)
template <typename R, int ROWS>
__global__ void __launch_bounds__(256) te_e_kernel(StencilView<R> v, SourceStep sx, SourceStep sy)
{
  using T = typename Cplx<R>::T;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i0 = (blockIdx.y * blockDim.y + threadIdx.y) * ROWS + 1;
  if (j < 1 || j > v.nj || i0 > v.ni) return;
  T *Ex = v.f[0], *Ey = v.f[1], *Dx = v.f[2], *Dy = v.f[3], *Jx = v.f[4], *Jy = v.f[5];
  const T *Hz = v.f[6];
  size_t k = (size_t)i0 * v.P + j;
  T hzl = ldro(Hz + k - v.P);
#pragma unroll
  for (int r = 0; r < ROWS; r++, k += v.P) {
    const int i = i0 + r;
    if (i > v.ni) break;
    const T hzk = ldro(Hz + k), hzb = ldro(Hz + k - 1);
    const T cxv = csub(hzk, hzb);          // Hz[k] - Hz[k_btm]
    T cyv;                                 // -Hz[k] + Hz[k_lft]
    cyv.x = -hzk.x + hzl.x;
    cyv.y = -hzk.y + hzl.y;
    hzl = hzk;
    T dx = Dx[k], dy = Dy[k];
    if (interior(v, i, j)) {
      dx = cadd(dx, cxv);
      dy = cadd(dy, cyv);
    } else {
      T jx = Jx[k], jy = Jy[k];
      te_e_pml(v, i, j, cxv, cyv, dx, dy, jx, jy);
      Jx[k] = jx;
      Jy[k] = jy;
    }
    Dx[k] = dx;
    Dy[k] = dy;
    const R iex = v.inv_eps[0][k], iey = v.inv_eps[1][k];
    T ex = dx, ey = dy;
    if (!is_one(iex)) {
      ex = cscale(dx, iex);
      if (sx.kind) apply_source<R>(v, sx, i, j, iex, ex);
    }
    if (!is_one(iey)) {
      ey = cscale(dy, iey);
      apply_source<R>(v, sy, i, j, iey, ey);
    }
    Ex[k] = ex;
    Ey[k] = ey;
  }
}

// calcMB + calcH (mpiTE_UPML.c:377-399)
template <typename R, int ROWS>
__global__ void __launch_bounds__(256) te_h_kernel(StencilView<R> v)
{
  using T = typename Cplx<R>::T;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i0 = (blockIdx.y * blockDim.y + threadIdx.y) * ROWS + 1;
  if (j < 1 || j > v.nj || i0 > v.ni) return;
  const T *Ex = v.f[0], *Ey = v.f[1];
  T *Hz = v.f[6], *Mz = v.f[7];
  size_t k = (size_t)i0 * v.P + j;
  T eyk = ldro(Ey + k);
#pragma unroll
  for (int r = 0; r < ROWS; r++, k += v.P) {
    const int i = i0 + r;
    if (i > v.ni) break;
    const T eyr = ldro(Ey + k + v.P), ext = ldro(Ex + k + 1), exk = ldro(Ex + k);
    T ce;                                  // Ey[k_rht] - Ey[k] - Ex[k_top] + Ex[k]
    ce.x = ((eyr.x - eyk.x) - ext.x) + exk.x;
    ce.y = ((eyr.y - eyk.y) - ext.y) + exk.y;
    eyk = eyr;
    T hz = Hz[k];
    if (interior(v, i, j)) {
      hz.x -= v.inv_mu * ce.x;
      hz.y -= v.inv_mu * ce.y;
    } else {
      T mz = Mz[k];
      te_h_pml(v, i, j, ce, hz, mz);
      Mz[k] = mz;
    }
    Hz[k] = hz;
  }
}

// ------------------------------------------------------------------ NTFF

// Tangential samples of the NTFF path, already signed and scaled:
//   e = sign * E[k] * coef,  h = sign * 0.5 * (H[k] + H[k+hoff]) * coef
template <typename R>
__global__ void ntff_gather_kernel(StencilView<R> v, NtffView n, double coef, int slot)
{
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n.ncell) return;
  n.vals += (size_t)slot * 2 * n.ncell;
  const SurfCell sc = n.cells[c];
  const typename Cplx<R>::T *E = v.f[sc.e_slot], *H = v.f[sc.h_slot];
  const auto e = E[sc.k];
  const auto h0 = H[sc.k], h1 = H[sc.k + sc.hoff];
  const double sg = sc.sign;
  double2 ev, hv;
  ev.x = sg * (double)e.x * coef;
  ev.y = sg * (double)e.y * coef;
  hv.x = (sg * 0.5) * ((double)h0.x + (double)h1.x) * coef;
  hv.y = (sg * 0.5) * ((double)h0.y + (double)h1.y) * coef;
  n.vals[c] = ev;
  n.vals[n.ncell + c] = hv;
}

// Three-tap deposit of mpiTM_UPML.c:840-847 (and ntffTM.c:279-288):
//   m = floor(t+0.5), a = 0.5+t-m, b = 1-a:  U[m-1] += v b, U[m] += v (a-b), U[m+1] -= v a
__device__ __forceinline__ void deposit(const NtffView &n, double2 *acc, long long row, double t, double2 val)
{
  const double u = t + 0.5;
  const double mf = floor(u);
  const double a = u - mf, b = 1.0 - a, ab = a - b;
  const long long at = row + (long long)mf;
  if (!(mf > -1e15 && mf < 1e15) || at - 1 < 0 || at + 1 >= n.len) {  // never write outside
    atomicOr(n.status, kStatusNtffRange);
    return;
  }
  double2 *p = acc + at;
  atomicAdd(&p[-1].x, val.x * b);
  atomicAdd(&p[-1].y, val.y * b);
  atomicAdd(&p[0].x, val.x * ab);
  atomicAdd(&p[0].y, val.y * ab);
  atomicAdd(&p[1].x, -(val.x * a));
  atomicAdd(&p[1].y, -(val.y * a));
}

__global__ void __launch_bounds__(256) ntff_accumulate_kernel(NtffView n, double timeE, double timeH)
{
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int ang = blockIdx.y;
  if (c >= n.ncell) return;
  const double sh = n.shift[(size_t)ang * n.ncell + c];
  const unsigned char uw = (unsigned char)n.cells[c].uid_wid;
  const long long row = (long long)kGuard + (long long)ang * n.array_size;
  deposit(n, n.acc[uw & 15], row, timeE + sh, n.vals[c]);
  deposit(n, n.acc[uw >> 4], row, timeH + sh, n.vals[n.ncell + c]);
}

// Three-tap deposit into a shared-memory window [base, base+W) of bins, with
// v b written as v - p and v (a-b) as 2p - v (p = v a): the same taps as
// deposit() up to one rounding.  Taps outside the window go to global memory.
__device__ __forceinline__ void window_deposit(const NtffView &n, double2 *win, int W, double2 *acc,
                                               long long row, long long base, double t, double2 v)
{
  const double u = t + 0.5;
  const double mf = floor(u);
  if (!(mf > -1e15 && mf < 1e15)) {
    atomicOr(n.status, kStatusNtffRange);
    return;
  }
  const double a = u - mf;
  const long long rel = (long long)mf - base;
  const double px = v.x * a, py = v.y * a;
  const double t0x = v.x - px, t0y = v.y - py;            // v b
  const double t1x = 2.0 * px - v.x, t1y = 2.0 * py - v.y;  // v (a - b)
  if (rel >= 1 && rel + 1 < W) {
    double2 *p = win + rel;
    atomicAdd(&p[-1].x, t0x);
    atomicAdd(&p[-1].y, t0y);
    atomicAdd(&p[0].x, t1x);
    atomicAdd(&p[0].y, t1y);
    atomicAdd(&p[1].x, -px);
    atomicAdd(&p[1].y, -py);
    return;
  }
  const long long at = row + (long long)mf;
  if (at - 1 < 0 || at + 1 >= n.len) {
    atomicOr(n.status, kStatusNtffRange);
    return;
  }
  double2 *p = acc + at;
  atomicAdd(&p[-1].x, t0x);
  atomicAdd(&p[-1].y, t0y);
  atomicAdd(&p[0].x, t1x);
  atomicAdd(&p[0].y, t1y);
  atomicAdd(&p[1].x, -px);
  atomicAdd(&p[1].y, -py);
}

__device__ __forceinline__ void window_flush(const NtffView &n, double2 *acc, long long at, double2 v)
{
  if (v.x == 0.0 && v.y == 0.0) return;
  if (at < 0 || at >= n.len) {
    atomicOr(n.status, kStatusNtffRange);
    return;
  }
  atomicAdd(&acc[at].x, v.x);
  atomicAdd(&acc[at].y, v.y);
}

// One block per (chunk of a side, angle): deposit into shared memory, then
// add the window to the flat [360][arraySize] accumulators.
__global__ void __launch_bounds__(256) ntff_window_kernel(NtffView n, NtffWindow w, double timeE, double timeH)
{
  extern __shared__ double2 win[];
  double2 *winE = win, *winH = win + w.width;
  const int ch = blockIdx.x, ang = blockIdx.y;
  const int2 cr = w.chunk[ch];
  const int2 lo = w.lo[(size_t)ang * w.nchunk + ch];
  const long long t0 = (long long)floor(timeE);
  const long long row = (long long)kGuard + (long long)ang * n.array_size;
  const long long baseE = t0 + lo.x, baseH = t0 + lo.y;
  for (int r = threadIdx.x; r < 2 * w.width; r += blockDim.x) win[r] = make_double2(0.0, 0.0);
  __syncthreads();
  const unsigned char uw = (unsigned char)n.cells[cr.x].uid_wid;  // one side per chunk
  double2 *U = n.acc[uw & 15], *Wa = n.acc[uw >> 4];
  const double *sh = n.shift + (size_t)ang * n.ncell;
  for (int q = threadIdx.x; q < cr.y; q += blockDim.x) {
    const int c = cr.x + q;
    const double s = sh[c];
    window_deposit(n, winE, w.width, U, row, baseE, timeE + s, n.vals[c]);
    window_deposit(n, winH, w.width, Wa, row, baseH, timeH + s, n.vals[n.ncell + c]);
  }
  __syncthreads();
  for (int r = threadIdx.x; r < w.width; r += blockDim.x) {
    window_flush(n, U, row + baseE + r, winE[r]);
    window_flush(n, Wa, row + baseH + r, winH[r]);
  }
}

// Time-blocked deposit.  One thread owns one (angle, path cell) pair and walks
// nb buffered steps.  With timeE integer and t = timeE + sh, the reference's
// rounding gives fl(timeE + sh) = timeE + R(sh) for every step whose t and
// t + 1/2 stay inside one binade (timeE is then a multiple of the ulp), so
// m = floor(t + 1/2) advances by exactly one per step and a = 1/2 + t - m is
// the same every step.  Bin m0 + j - 1 (j = 0 .. nb+1) then collects
//   b v_j + (a - b) v_{j-1} - a v_{j-2} = d_j - a e_j,
//   d_j = v_j - v_{j-1},  e_j = d_j - d_{j-1}   (v outside 0..nb-1 is zero),
// i.e. one complex FMA per bin on differences that ntff_diff_kernel computes
// once per path cell for all 360 angles (the first bin, d_0 - a e_0 =
// fma(-a, v_0, v_0), rounds exactly as v_0 b).  A block whose t range crosses a
// binade, or a non-integer clock, takes the exact per-step path (deposit()).
__device__ __forceinline__ int binade(double x) { return (int)((__double_as_longlong(x) >> 52) & 0x7ff); }

__device__ __forceinline__ void red_c(const NtffView &n, double2 *acc, long long at, double2 v)
{
  if (at < 0 || at >= n.len) {
    atomicOr(n.status, kStatusNtffRange);
    return;
  }
  atomicAdd(&acc[at].x, v.x);
  atomicAdd(&acc[at].y, v.y);
}

// (d_j, e_j) of every path cell and field, j = 0 .. nb+1
__global__ void ntff_diff_kernel(NtffView n, int nb)
{
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int f = blockIdx.y;  // 0: E samples, 1: H samples
  if (c >= n.ncell) return;
  double2 vp = make_double2(0.0, 0.0), dp = make_double2(0.0, 0.0);
  for (int j = 0; j <= nb + 1; j++) {
    const double2 v = j < nb ? n.vals[(size_t)j * 2 * n.ncell + (size_t)f * n.ncell + c] : make_double2(0.0, 0.0);
    const double2 d = make_double2(v.x - vp.x, v.y - vp.y);
    n.dg[((size_t)j * 2 + f) * n.ncell + c] = make_double4(d.x, d.y, d.x - dp.x, d.y - dp.y);
    vp = v;
    dp = d;
  }
}

__device__ __forceinline__ void block_field(const NtffView &n, double2 *acc, long long row, const double2 *vals,
                                            const double4 *dg, int nb, double base, double sh, bool t0_integer)
{
  const double tf = base + sh;
  const double ul = (base + (double)(nb - 1) + sh) + 0.5;
  const int e = binade(tf);
  if (t0_integer && tf >= 1.0 && e == binade(ul) && e <= 1023 + 50) {
    const double uf = tf + 0.5;
    const double mf = floor(uf);
    const double a = uf - mf;
    const long long m0 = row + (long long)mf;
    for (int j = 0; j <= nb + 1; j++) {
      const double4 q = dg[(size_t)j * 2 * n.ncell];
      const double2 f = make_double2(fma(-a, q.z, q.x), fma(-a, q.w, q.y));
      // skip (+-)0 + (+-)0i: tested on the bit patterns (integer ALU), not with two
      // FP64 compares, which would double the FP64 work of the loop
      const unsigned long long bits =
          (unsigned long long)__double_as_longlong(f.x) | (unsigned long long)__double_as_longlong(f.y);
      if (bits << 1) red_c(n, acc, m0 + j - 1, f);
    }
    return;
  }
  for (int s = 0; s < nb; s++) deposit(n, acc, row, (base + (double)s) + sh, vals[(size_t)s * 2 * n.ncell]);
}

// blockIdx.x = angle (fastest, so the 360 blocks of one cell chunk find its
// differences in L2), blockIdx.y = chunk of 256 path cells
__global__ void __launch_bounds__(256) ntff_block_kernel(NtffView n, int nb, double t0)
{
  const int ang = blockIdx.x;
  const int c = blockIdx.y * blockDim.x + threadIdx.x;
  if (c >= n.ncell) return;
  const double sh = n.shift[(size_t)ang * n.ncell + c];
  const unsigned char uw = (unsigned char)n.cells[c].uid_wid;
  const long long row = (long long)kGuard + (long long)ang * n.array_size;
  const bool integer_clock = t0 == floor(t0);
  block_field(n, n.acc[uw & 15], row, n.vals + c, n.dg + c, nb, t0, sh, integer_clock);  // E, timeE
  block_field(n, n.acc[uw >> 4], row, n.vals + n.ncell + c, n.dg + n.ncell + c, nb, t0 + 0.5, sh,
              integer_clock);  // H, timeH
}

// ------------------------------------------------------------------ launchers

static const dim3 kBlock(32, 8);

// columns 1..nj and rows 1..ni, ROWS rows per thread
template <typename R>
static dim3 grid_of(const StencilView<R> &v, int rows)
{
  const int span = (int)kBlock.y * rows;
  return dim3((unsigned)((v.nj + 1 + kBlock.x - 1) / kBlock.x), (unsigned)((v.ni + span - 1) / span));
}

// dispatch on the run-time rows-per-thread setting (1, 2, 4 or 8)
#define ROWS_DISPATCH(KERNEL, ...)                                                                   \
  switch (v.rows) {                                                                                \
  case 1: KERNEL<R, 1><<<grid_of(v, 1), kBlock, 0, st>>>(__VA_ARGS__); break;                     \
  case 2: KERNEL<R, 2><<<grid_of(v, 2), kBlock, 0, st>>>(__VA_ARGS__); break;                     \
  case 8: KERNEL<R, 8><<<grid_of(v, 8), kBlock, 0, st>>>(__VA_ARGS__); break;                     \
  default: KERNEL<R, 4><<<grid_of(v, 4), kBlock, 0, st>>>(__VA_ARGS__); break;                    \
  }

template <typename R>
void launch_tm_e(const StencilView<R> &v, const SourceStep &s, cudaStream_t st)
{
  ROWS_DISPATCH(tm_e_kernel, v, s)
}
template <typename R>
void launch_tm_h(const StencilView<R> &v, cudaStream_t st)
{
  ROWS_DISPATCH(tm_h_kernel, v)
}
template <typename R>
void launch_te_e(const StencilView<R> &v, const SourceStep &sx, const SourceStep &sy, cudaStream_t st)
{
  ROWS_DISPATCH(te_e_kernel, v, sx, sy)
}
template <typename R>
void launch_te_h(const StencilView<R> &v, cudaStream_t st)
{
  ROWS_DISPATCH(te_h_kernel, v)
}
#undef ROWS_DISPATCH
template <typename R>
void launch_ntff_gather(const StencilView<R> &v, const NtffView &n, double coef, int slot, cudaStream_t st)
{
  ntff_gather_kernel<R><<<(n.ncell + 255) / 256, 256, 0, st>>>(v, n, coef, slot);
}
void launch_ntff_block(const NtffView &n, int nb, double t0, cudaStream_t st)
{
  const unsigned chunks = (unsigned)((n.ncell + 255) / 256);
  ntff_diff_kernel<<<dim3(chunks, 2), 256, 0, st>>>(n, nb);
  ntff_block_kernel<<<dim3(360, chunks), 256, 0, st>>>(n, nb, t0);
}
void launch_ntff_accumulate(const NtffView &n, double timeE, double timeH, cudaStream_t st)
{
  dim3 g((unsigned)((n.ncell + 255) / 256), 360);
  ntff_accumulate_kernel<<<g, 256, 0, st>>>(n, timeE, timeH);
}
void launch_ntff_window(const NtffView &n, const NtffWindow &w, double timeE, double timeH, cudaStream_t st)
{
  const size_t smem = sizeof(double2) * 2 * (size_t)w.width;
  static size_t configured = 0;  // raise the dynamic shared-memory cap once per size
  if (smem > 48 * 1024 && smem > configured) {
    cudaFuncSetAttribute(ntff_window_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    configured = smem;
  }
  dim3 g((unsigned)w.nchunk, 360);
  ntff_window_kernel<<<g, 256, smem, st>>>(n, w, timeE, timeH);
}

#define INST(R)                                                                                    \
  template void launch_tm_e<R>(const StencilView<R> &, const SourceStep &, cudaStream_t);        \
  template void launch_tm_h<R>(const StencilView<R> &, cudaStream_t);                            \
  template void launch_te_e<R>(const StencilView<R> &, const SourceStep &, const SourceStep &,   \
                               cudaStream_t);                                                    \
  template void launch_te_h<R>(const StencilView<R> &, cudaStream_t);                            \
  template void launch_ntff_gather<R>(const StencilView<R> &, const NtffView &, double, int, cudaStream_t);
INST(double)
INST(float)
#undef INST

}  // namespace fdtd
