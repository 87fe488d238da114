// surrogate_ops.cu -- the far-field surrogate's non-GEMM kernels (forward,
// backward, optimizer).  Every contraction of the model runs in the tcgen05
// GEMM (surrogate_gemm.cu); these kernels do the layout permutations,
// pooling, the point-wise channel mixing, activations, reductions, the loss
// and the Adam update.  Tensors are row-major; shapes are given per call.
//
// Notation: B structures, C = 64 channels, S = 1024 points of the 32 x 32 grid,
// Q = 256 retained Fourier modes (2 real components each: 2Q = 512).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace sgo {

using bf16 = __nv_bfloat16;

__device__ __forceinline__ float gelu_f(float x)  // tanh form, Hendrycks & Gimpel (2016)
{
  const float k0 = 0.7978845608f, k1 = 0.044715f;
  return 0.5f * x * (1.0f + tanhf(k0 * (x + k1 * x * x * x)));
}

__device__ __forceinline__ float gelu_grad(float x)
{
  const float k0 = 0.7978845608f, k1 = 0.044715f;
  const float u = k0 * (x + k1 * x * x * x);
  const float t = tanhf(u);
  return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * k0 * (1.0f + 3.0f * k1 * x * x);
}

// map [B][256][256] u8 -> x [B][32*32] f32: mean of each 8 x 8 block
__global__ void pool_map_kernel(const uint8_t *map, float *x, int B)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B * 1024) return;
  const int b = i / 1024, p = i % 1024, px = p / 32, py = p % 32;
  const uint8_t *m = map + (size_t)b * 65536 + (size_t)(px * 8) * 256 + py * 8;
  int s = 0;
  for (int r = 0; r < 8; r++)
    for (int c = 0; c < 8; c++) s += m[r * 256 + c] ? 1 : 0;
  x[i] = s * (1.0f / 64.0f);
}

// h0[b][c][s] = x[b][s] wl[c] + bl[c]
__global__ void lift_kernel(const float *x, const float *wl, const float *bl, bf16 *h, int B, int C)
{
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)B * C * 1024) return;
  const int s = i % 1024, c = (i / 1024) % C, b = (int)(i / (1024 * (size_t)C));
  h[i] = __float2bfloat16(x[(size_t)b * 1024 + s] * wl[c] + bl[c]);
}

// lift backward: dwl[c] = sum_{b,s} dh x, dbl[c] = sum dh (one block per c)
__global__ void lift_bwd_kernel(const float *x, const float *dh, float *dwl, float *dbl, int B, int C)
{
  const int c = blockIdx.x;
  float sw = 0, sb = 0;
  for (int i = threadIdx.x; i < B * 1024; i += blockDim.x) {
    const int b = i / 1024, s = i % 1024;
    const float g = dh[((size_t)b * C + c) * 1024 + s];
    sw += g * x[(size_t)b * 1024 + s];
    sb += g;
  }
  __shared__ float rw[256], rb[256];
  rw[threadIdx.x] = sw;
  rb[threadIdx.x] = sb;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      rw[threadIdx.x] += rw[threadIdx.x + w];
      rb[threadIdx.x] += rb[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    dwl[c] = rw[0];
    dbl[c] = rb[0];
  }
}

// F[b][c][2q+r] <-> Fm[q][b][r*C + c]  (dir 0: F -> Fm, 1: Fm -> F)
__global__ void mode_permute_kernel(const bf16 *in, bf16 *out, int B, int C, int Q, int dir)
{
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t n = (size_t)B * C * 2 * Q;
  if (i >= n) return;
  // i indexes the output
  if (dir == 0) {  // out = Fm[q][b][r*C+c]
    const int rc = i % (2 * C), b = (i / (2 * C)) % B, q = (int)(i / ((size_t)2 * C * B));
    const int r = rc / C, c = rc % C;
    out[i] = in[((size_t)b * C + c) * (2 * Q) + 2 * q + r];
  } else {  // out = F[b][c][2q+r]
    const int k = i % (2 * Q), c = (i / (2 * Q)) % C, b = (int)(i / ((size_t)2 * Q * C));
    const int q = k / 2, r = k % 2;
    out[i] = in[((size_t)q * B + b) * (2 * C) + r * C + c];
  }
}

// z[b][c][s] = hs[b][c][s] + sum_c' wp[c][c'] h[b][c'][s] + bp[c]; hn = act(z)
// block: one (b, 32 points); thread: point s, all C outputs
__global__ void pointwise_fwd_kernel(const bf16 *h, const float *hs, const float *wp, const float *bp, float *z,
                                     bf16 *hn, int B, int C, int act)
{
  __shared__ float w[64 * 64];
  for (int q = threadIdx.x; q < C * C; q += blockDim.x) w[q] = wp[q];
  __syncthreads();
  const int b = blockIdx.y, s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= 1024) return;
  float hv[64];
  for (int c = 0; c < C; c++) hv[c] = __bfloat162float(h[((size_t)b * C + c) * 1024 + s]);
  for (int c = 0; c < C; c++) {
    float acc = bp[c];
    for (int k = 0; k < C; k++) acc += w[c * C + k] * hv[k];
    const size_t o = ((size_t)b * C + c) * 1024 + s;
    const float zz = hs[o] + acc;
    z[o] = zz;
    hn[o] = __float2bfloat16(act ? gelu_f(zz) : zz);
  }
}

// dz = dh * act'(z) (FP32, in place in dz); dhs_bf = bf16(dz) for the spectral GEMMs
__global__ void act_bwd_kernel(const float *dh, const float *z, float *dz, bf16 *dz_bf, size_t n, int act)
{
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float g = act ? dh[i] * gelu_grad(z[i]) : dh[i];
  dz[i] = g;
  dz_bf[i] = __float2bfloat16(g);
}

// dh_prev[b][c'][s] = sum_c wp[c][c'] dz[b][c][s] + dspec[b][c'][s]
__global__ void pointwise_bwd_x_kernel(const float *dz, const float *wp, const float *dspec, float *dh, int B, int C)
{
  __shared__ float w[64 * 64];
  for (int q = threadIdx.x; q < C * C; q += blockDim.x) w[q] = wp[q];
  __syncthreads();
  const int b = blockIdx.y, s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= 1024) return;
  float g[64];
  for (int c = 0; c < C; c++) g[c] = dz[((size_t)b * C + c) * 1024 + s];
  for (int k = 0; k < C; k++) {
    float acc = 0;
    for (int c = 0; c < C; c++) acc += w[c * C + k] * g[c];
    const size_t o = ((size_t)b * C + k) * 1024 + s;
    dh[o] = acc + dspec[o];
  }
}

// dwp[c][c'] = sum_{b,s} dz[b][c][s] h[b][c'][s]; dbp[c] = sum dz  (one block per (c, c'))
__global__ void pointwise_bwd_w_kernel(const float *dz, const bf16 *h, float *dwp, float *dbp, int B, int C)
{
  const int c = blockIdx.x / C, k = blockIdx.x % C;
  float acc = 0, accb = 0;
  for (int i = threadIdx.x; i < B * 1024; i += blockDim.x) {
    const int b = i / 1024, s = i % 1024;
    const float g = dz[((size_t)b * C + c) * 1024 + s];
    acc += g * __bfloat162float(h[((size_t)b * C + k) * 1024 + s]);
    if (k == 0) accb += g;
  }
  __shared__ float r[256], rb[256];
  r[threadIdx.x] = acc;
  rb[threadIdx.x] = accb;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      r[threadIdx.x] += r[threadIdx.x + w];
      rb[threadIdx.x] += rb[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    dwp[c * C + k] = r[0];
    if (k == 0) dbp[c] = rb[0];
  }
}

// head pooling: h [B][C][32][32] -> flat [B][C*64] (mean of 4 x 4 blocks); backward broadcasts /16
__global__ void head_pool_kernel(const bf16 *h, bf16 *flat, int B, int C)
{
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)B * C * 64) return;
  const int p = i % 64, c = (i / 64) % C, b = (int)(i / (64 * (size_t)C));
  const int px = p / 8, py = p % 8;
  const bf16 *src = h + ((size_t)b * C + c) * 1024 + (px * 4) * 32 + py * 4;
  float s = 0;
  for (int r = 0; r < 4; r++)
    for (int q = 0; q < 4; q++) s += __bfloat162float(src[r * 32 + q]);
  flat[i] = __float2bfloat16(s * (1.0f / 16.0f));
}

__global__ void head_unpool_kernel(const float *dflat, float *dh, int B, int C)
{
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)B * C * 1024) return;
  const int s = i % 1024, c = (i / 1024) % C, b = (int)(i / (1024 * (size_t)C));
  const int px = (s / 32) / 4, py = (s % 32) / 4;
  dh[i] = dflat[((size_t)b * C + c) * 64 + px * 8 + py] * (1.0f / 16.0f);
}

// squared error against targets of width nt inside rows of width n (the rest
// is padding with zero gradient); loss[b] per row; dout = 2 (out - y) / (B nt) in bf16
__global__ void mse_kernel(const float *out, const float *y, bf16 *dout, float *loss, int B, int n, int nt)
{
  const int b = blockIdx.x;
  float acc = 0;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    float g = 0;
    if (j < nt) {
      const float d = out[(size_t)b * n + j] - y[(size_t)b * nt + j];
      acc += d * d;
      g = 2.0f * d / ((float)B * nt);
    }
    if (dout) dout[(size_t)b * n + j] = __float2bfloat16(g);
  }
  __shared__ float r[256];
  r[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) r[threadIdx.x] += r[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) loss[b] = r[0] / nt;
}

// dpre = du * gelu'(pre)  -> bf16
__global__ void gelu_bwd_kernel(const float *du, const float *pre, bf16 *dpre, size_t n)
{
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dpre[i] = __float2bfloat16(du[i] * gelu_grad(pre[i]));
}

// column sums of a bf16 [R][N] matrix -> FP32 [N]
__global__ void colsum_kernel(const bf16 *a, float *out, int R, int N)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  float s = 0;
  for (int r = 0; r < R; r++) s += __bfloat162float(a[(size_t)r * N + j]);
  out[j] = s;
}

// batched transpose of bf16 [Z][R][Cc] -> [Z][Cc][R] through 32 x 33 shared tiles
__global__ void transpose_kernel(const bf16 *in, bf16 *out, int R, int Cc)
{
  __shared__ bf16 t[32][33];
  const size_t zoff = (size_t)blockIdx.z * R * Cc;
  const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int r = r0 + k, c = c0 + threadIdx.x;
    if (r < R && c < Cc) t[k][threadIdx.x] = in[zoff + (size_t)r * Cc + c];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int c = c0 + k, r = r0 + threadIdx.x;
    if (r < R && c < Cc) out[zoff + (size_t)c * R + r] = t[threadIdx.x][k];
  }
}

__global__ void cast_bf16_kernel(const float *in, bf16 *out, size_t n)
{
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = __float2bfloat16(in[i]);
}

// Adam (Kingma & Ba 2015) on FP32 master weights, refreshing the BF16 copy
__global__ void adam_kernel(float *w, const float *g, float *m, float *v, bf16 *w_bf, size_t n, float lr, float b1,
                            float b2, float eps, float c1, float c2, float wd)
{
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i] + wd * w[i];
  const float mi = b1 * m[i] + (1 - b1) * gi;
  const float vi = b2 * v[i] + (1 - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  w[i] = wi;
  if (w_bf) w_bf[i] = __float2bfloat16(wi);
}

inline unsigned nb(size_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace sgo

using namespace sgo;

#define ST ((cudaStream_t)stream)
#define RET return cudaGetLastError() == cudaSuccess ? 0 : 2

extern "C" {

int sg_pool_map(const void *map, float *x, int B, void *stream)
{
  pool_map_kernel<<<nb((size_t)B * 1024, 256), 256, 0, ST>>>((const uint8_t *)map, x, B);
  RET;
}
int sg_lift(const float *x, const float *wl, const float *bl, void *h, int B, int C, void *stream)
{
  lift_kernel<<<nb((size_t)B * C * 1024, 256), 256, 0, ST>>>(x, wl, bl, (bf16 *)h, B, C);
  RET;
}
int sg_lift_bwd(const float *x, const float *dh, float *dwl, float *dbl, int B, int C, void *stream)
{
  lift_bwd_kernel<<<C, 256, 0, ST>>>(x, dh, dwl, dbl, B, C);
  RET;
}
int sg_mode_permute(const void *in, void *out, int B, int C, int Q, int dir, void *stream)
{
  mode_permute_kernel<<<nb((size_t)B * C * 2 * Q, 256), 256, 0, ST>>>((const bf16 *)in, (bf16 *)out, B, C, Q, dir);
  RET;
}
int sg_pointwise_fwd(const void *h, const float *hs, const float *wp, const float *bp, float *z, void *hn, int B,
                     int C, int act, void *stream)
{
  if (C > 64) return 1;
  pointwise_fwd_kernel<<<dim3(32, B), 32, 0, ST>>>((const bf16 *)h, hs, wp, bp, z, (bf16 *)hn, B, C, act);
  RET;
}
int sg_act_bwd(const float *dh, const float *z, float *dz, void *dz_bf, long long n, int act, void *stream)
{
  act_bwd_kernel<<<nb((size_t)n, 256), 256, 0, ST>>>(dh, z, dz, (bf16 *)dz_bf, (size_t)n, act);
  RET;
}
int sg_pointwise_bwd_x(const float *dz, const float *wp, const float *dspec, float *dh, int B, int C, void *stream)
{
  if (C > 64) return 1;
  pointwise_bwd_x_kernel<<<dim3(32, B), 32, 0, ST>>>(dz, wp, dspec, dh, B, C);
  RET;
}
int sg_pointwise_bwd_w(const float *dz, const void *h, float *dwp, float *dbp, int B, int C, void *stream)
{
  pointwise_bwd_w_kernel<<<C * C, 256, 0, ST>>>(dz, (const bf16 *)h, dwp, dbp, B, C);
  RET;
}
int sg_head_pool(const void *h, void *flat, int B, int C, void *stream)
{
  head_pool_kernel<<<nb((size_t)B * C * 64, 256), 256, 0, ST>>>((const bf16 *)h, (bf16 *)flat, B, C);
  RET;
}
int sg_head_unpool(const float *dflat, float *dh, int B, int C, void *stream)
{
  head_unpool_kernel<<<nb((size_t)B * C * 1024, 256), 256, 0, ST>>>(dflat, dh, B, C);
  RET;
}
int sg_mse(const float *out, const float *y, void *dout, float *loss, int B, int n, int nt, void *stream)
{
  mse_kernel<<<B, 256, 0, ST>>>(out, y, (bf16 *)dout, loss, B, n, nt);
  RET;
}
int sg_gelu_bwd(const float *du, const float *pre, void *dpre, long long n, void *stream)
{
  gelu_bwd_kernel<<<nb((size_t)n, 256), 256, 0, ST>>>(du, pre, (bf16 *)dpre, (size_t)n);
  RET;
}
int sg_colsum(const void *a, float *out, int R, int N, void *stream)
{
  colsum_kernel<<<nb((size_t)N, 256), 256, 0, ST>>>((const bf16 *)a, out, R, N);
  RET;
}
int sg_transpose(const void *in, void *out, int Z, int R, int Cc, void *stream)
{
  transpose_kernel<<<dim3((Cc + 31) / 32, (R + 31) / 32, Z), dim3(32, 8), 0, ST>>>((const bf16 *)in, (bf16 *)out, R,
                                                                                      Cc);
  RET;
}
int sg_cast_bf16(const float *in, void *out, long long n, void *stream)
{
  cast_bf16_kernel<<<nb((size_t)n, 256), 256, 0, ST>>>(in, (bf16 *)out, (size_t)n);
  RET;
}
int sg_adam(float *w, const float *g, float *m, float *v, void *w_bf, long long n, float lr, float b1, float b2,
            float eps, float c1, float c2, float wd, void *stream)
{
  adam_kernel<<<nb((size_t)n, 256), 256, 0, ST>>>(w, g, m, v, (bf16 *)w_bf, (size_t)n, lr, b1, b2, eps, c1, c2, wd);
  RET;
}

}  // extern "C"
