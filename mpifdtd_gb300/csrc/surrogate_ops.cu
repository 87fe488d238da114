// surrogate_ops.cu -- the far-field surrogate's non-GEMM kernels (forward,
// backward, optimizer).  Every contraction of the model, the point-wise
// channel mixing included, runs in the tcgen05 GEMM (surrogate_gemm.cu); these
// kernels do the layout permutations, pooling, activations, reductions, the
// loss and the Adam update.  Tensors are row-major; shapes are given per call.
//
// Notation: B structures, C = 64 channels, S = 1024 points of the 32 x 32 grid,
// Q = 256 retained Fourier modes (2 real components each: 2Q = 512).
// Activations exist in two layouts: channels-first [B][C][S] (rows of S points,
// the operand of the truncated-DFT GEMMs) and channels-last [B][S][C] (rows of
// C channels, the operand and output of the point-wise mixing GEMM).
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

// map [B][256][256] u8 -> x [kNin][B][32*32] f32: per 8 x 8 block the
// dielectric's fill fraction and its first and second moments about the
// block centre, u = (p - 3.5) / 4 along x and y (where in the block the
// material sits, which the fill fraction alone loses):
//   x0 = mean e, x1 = mean e u_x, x2 = mean e u_y, x3 = mean e u_x^2, x4 = mean e u_y^2
constexpr int kNin = 5;
__global__ void pool_map_kernel(const uint8_t *map, float *x, int B)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B * 1024) return;
  const int b = i / 1024, p = i % 1024, px = p / 32, py = p % 32;
  const uint8_t *m = map + (size_t)b * 65536 + (size_t)(px * 8) * 256 + py * 8;
  int s = 0, sx = 0, sy = 0, sxx = 0, syy = 0;  // in units of (2u)*4 = 2r - 7: integers
  for (int r = 0; r < 8; r++)
    for (int c = 0; c < 8; c++)
      if (m[r * 256 + c]) {
        const int ux = 2 * r - 7, uy = 2 * c - 7;
        s += 1;
        sx += ux;
        sy += uy;
        sxx += ux * ux;
        syy += uy * uy;
      }
  const size_t n = (size_t)B * 1024;
  x[i] = s * (1.0f / 64.0f);
  x[n + i] = sx * (1.0f / (64.0f * 8.0f));
  x[2 * n + i] = sy * (1.0f / (64.0f * 8.0f));
  x[3 * n + i] = sxx * (1.0f / (64.0f * 64.0f));
  x[4 * n + i] = syy * (1.0f / (64.0f * 64.0f));
}

// h0[b][c][s] = sum_i x[i][b][s] wl[i][c] + bl[c] in both layouts: idx < n
// writes the channels-first copy, n <= idx < 2n the channels-last one
// (each coalesced)
__device__ __forceinline__ float lift_value(const float *x, const float *wl, const float *bl, int B, int C, int b,
                                            int c, int s)
{
  const size_t n = (size_t)B * 1024, o = (size_t)b * 1024 + s;
  float v = bl[c];
#pragma unroll
  for (int q = 0; q < kNin; q++) v += x[q * n + o] * wl[q * C + c];
  return v;
}
__global__ void lift_kernel(const float *x, const float *wl, const float *bl, bf16 *h_cf, bf16 *h_cl, int B, int C)
{
  const size_t n = (size_t)B * C * 1024;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 2 * n) return;
  if (i < n) {
    const int s = i % 1024, c = (i / 1024) % C, b = (int)(i / (1024 * (size_t)C));
    h_cf[i] = __float2bfloat16(lift_value(x, wl, bl, B, C, b, c, s));
  } else {
    const size_t k = i - n;
    const int c = k % C, s = (k / C) % 1024, b = (int)(k / ((size_t)C * 1024));
    h_cl[k] = __float2bfloat16(lift_value(x, wl, bl, B, C, b, c, s));
  }
}

// column sums of a tall FP32 [R][64] matrix, plain and weighted by w[r]:
// out[c] += sum_r a[r][c] (out may be null), out_w[c] += sum_r a[r][c] w[r]
// (both zeroed by the caller); 4 row lanes x 64 columns per block, one atomic
// per column and block
__global__ void colsum_tall_kernel(const float *a, const float *w, float *out, float *out_w, long long R)
{
  const int c = threadIdx.x & 63, rl = threadIdx.x >> 6;
  float s = 0, sw = 0;
  for (long long r = (long long)blockIdx.x * 4 + rl; r < R; r += (long long)gridDim.x * 4) {
    const float v = a[r * 64 + c];
    s += v;
    if (w) sw += v * w[r];
  }
  __shared__ float rs[4][64], rw[4][64];
  rs[rl][c] = s;
  rw[rl][c] = sw;
  __syncthreads();
  if (rl == 0) {
    if (out) atomicAdd(&out[c], rs[0][c] + rs[1][c] + rs[2][c] + rs[3][c]);
    if (w) atomicAdd(&out_w[c], rw[0][c] + rw[1][c] + rw[2][c] + rw[3][c]);
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

// Activation of the mixed layer, one tile of 32 points x 64 channels of one
// structure per block: z (FP32, channels-last, the pre-activation the backward
// keeps) -> hn = act(z) in BF16, channels-last (next point-wise GEMM) and
// channels-first (next DFT GEMM, transposed through shared memory).
__global__ void __launch_bounds__(256) act_fwd_kernel(const float *z, bf16 *hn_cf, bf16 *hn_cl, int act)
{
  __shared__ bf16 t[64][34];
  const int b = blockIdx.y, s0 = blockIdx.x * 32;
  const size_t base = ((size_t)b * 1024 + s0) * 64;
  for (int e = threadIdx.x; e < 32 * 64; e += 256) {
    const float v = z[base + e];
    const bf16 h = __float2bfloat16(act ? gelu_f(v) : v);
    hn_cl[base + e] = h;
    t[e & 63][e >> 6] = h;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < 32 * 64; e += 256) {
    const int c = e >> 5, r = e & 31;
    hn_cf[((size_t)b * 64 + c) * 1024 + s0 + r] = t[c][r];
  }
}

// Backward of the activation on the same tiles: dz = dh act'(z) from
// channels-last dh and z; writes BF16 dz channels-last (point-wise GEMMs) and
// channels-first (DFT GEMMs), and adds the column sums of the FP32 dz into
// dbp[c] (the bias gradient, zeroed by the caller).
__global__ void __launch_bounds__(256) act_bwd_kernel(const float *dh, const float *z, bf16 *dz_cl, bf16 *dz_cf,
                                                      float *dbp, int act)
{
  __shared__ float t[64][33];
  const int b = blockIdx.y, s0 = blockIdx.x * 32;
  const size_t base = ((size_t)b * 1024 + s0) * 64;
  for (int e = threadIdx.x; e < 32 * 64; e += 256) {
    const float g = act ? dh[base + e] * gelu_grad(z[base + e]) : dh[base + e];
    dz_cl[base + e] = __float2bfloat16(g);
    t[e & 63][e >> 6] = g;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < 32 * 64; e += 256) {
    const int c = e >> 5, r = e & 31;
    dz_cf[((size_t)b * 64 + c) * 1024 + s0 + r] = __float2bfloat16(t[c][r]);
  }
  if (threadIdx.x < 64) {
    float sum = 0;
    for (int r = 0; r < 32; r++) sum += t[threadIdx.x][r];
    atomicAdd(&dbp[threadIdx.x], sum);
  }
}

// head pooling: h [B][C][32][32] -> flat [B][C*g*g] (mean of hp x hp blocks, g = 32 / hp);
// backward broadcasts / hp^2
__global__ void head_pool_kernel(const bf16 *h, bf16 *flat, int B, int C, int hp)
{
  const int g = 32 / hp, gg = g * g;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)B * C * gg) return;
  const int p = i % gg, c = (i / gg) % C, b = (int)(i / (gg * (size_t)C));
  const int px = p / g, py = p % g;
  const bf16 *src = h + ((size_t)b * C + c) * 1024 + (px * hp) * 32 + py * hp;
  float s = 0;
  for (int r = 0; r < hp; r++)
    for (int q = 0; q < hp; q++) s += __bfloat162float(src[r * 32 + q]);
  flat[i] = __float2bfloat16(s / (float)(hp * hp));
}

// the backward of head_pool into channels-last dh [B][S][C]
__global__ void head_unpool_kernel(const float *dflat, float *dh, int B, int C, int hp)
{
  const int g = 32 / hp;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)B * C * 1024) return;
  const int c = i % C, s = (i / C) % 1024, b = (int)(i / ((size_t)C * 1024));
  const int px = (s / 32) / hp, py = (s % 32) / hp;
  dh[i] = dflat[((size_t)b * C + c) * g * g + px * g + py] / (float)(hp * hp);
}

// Amplitude head: row b of out holds the far-field amplitude, real parts in
// columns [0, nt) and imaginary parts in [nt, 2 nt) (the rest is padding with
// zero gradient); the predicted intensity is I_j = re_j^2 + im_j^2.  Squared
// error of I against targets y [B][nt], row b weighted by w[b] (null: 1):
// loss[b] = w[b] mean_j (I_j - y_j)^2; dout = dL/d(re, im) = 2 g (re, im)
// with g = 2 w[b] (I - y) / (B nt), in bf16.
__global__ void amp_mse_kernel(const float *out, const float *y, const float *w, bf16 *dout, float *loss, int B,
                               int n, int nt)
{
  const int b = blockIdx.x;
  const float wb = w ? w[b] : 1.0f;
  const float *o = out + (size_t)b * n;
  bf16 *dz = dout ? dout + (size_t)b * n : nullptr;
  float acc = 0;
  for (int j = threadIdx.x; j < nt; j += blockDim.x) {
    const float re = o[j], im = o[nt + j];
    const float d = (re * re + im * im) - y[(size_t)b * nt + j];
    acc += d * d;
    if (dz) {
      const float g = 2.0f * wb * d / ((float)B * nt);
      dz[j] = __float2bfloat16(2.0f * g * re);
      dz[nt + j] = __float2bfloat16(2.0f * g * im);
    }
  }
  if (dz)
    for (int j = 2 * nt + threadIdx.x; j < n; j += blockDim.x) dz[j] = __float2bfloat16(0.0f);
  __shared__ float r[256];
  r[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) r[threadIdx.x] += r[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) loss[b] = wb * r[0] / nt;
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

// column sums of an FP32 [R][N] matrix -> [N] (the dW partials of the point-wise GEMM, R = B)
__global__ void colsum_f32_kernel(const float *a, float *out, int R, int N)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  float s = 0;
  for (int r = 0; r < R; r++) s += a[(size_t)r * N + j];
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
int sg_lift(const float *x, const float *wl, const float *bl, void *h_cf, void *h_cl, int B, int C, void *stream)
{
  lift_kernel<<<nb(2 * (size_t)B * C * 1024, 256), 256, 0, ST>>>(x, wl, bl, (bf16 *)h_cf, (bf16 *)h_cl, B, C);
  RET;
}
// dwl[i][c] = sum_{b,s} dh[b][s][c] x[i][b][s], dbl[c] = sum dh[b][s][c]  (dh channels-last)
int sg_lift_bwd(const float *x, const float *dh, float *dwl, float *dbl, int B, int C, void *stream)
{
  if (C != 64) return 1;
  if (cudaMemsetAsync(dwl, 0, kNin * 64 * sizeof(float), ST) != cudaSuccess ||
      cudaMemsetAsync(dbl, 0, 64 * sizeof(float), ST) != cudaSuccess)
    return 2;
  const long long R = (long long)B * 1024;
  for (int q = 0; q < kNin; q++)
    colsum_tall_kernel<<<304, 256, 0, ST>>>(dh, x + q * R, q == 0 ? dbl : nullptr, dwl + q * 64, R);
  RET;
}
int sg_input_channels(void) { return kNin; }
int sg_mode_permute(const void *in, void *out, int B, int C, int Q, int dir, void *stream)
{
  mode_permute_kernel<<<nb((size_t)B * C * 2 * Q, 256), 256, 0, ST>>>((const bf16 *)in, (bf16 *)out, B, C, Q, dir);
  RET;
}
int sg_act_fwd(const float *z, void *hn_cf, void *hn_cl, int B, int C, int act, void *stream)
{
  if (C != 64) return 1;
  act_fwd_kernel<<<dim3(32, B), 256, 0, ST>>>(z, (bf16 *)hn_cf, (bf16 *)hn_cl, act);
  RET;
}
int sg_act_bwd(const float *dh, const float *z, void *dz_cl, void *dz_cf, float *dbp, int B, int C, int act,
               void *stream)
{
  if (C != 64) return 1;
  if (cudaMemsetAsync(dbp, 0, 64 * sizeof(float), ST) != cudaSuccess) return 2;
  act_bwd_kernel<<<dim3(32, B), 256, 0, ST>>>(dh, z, (bf16 *)dz_cl, (bf16 *)dz_cf, dbp, act);
  RET;
}
int sg_head_pool(const void *h, void *flat, int B, int C, int hp, void *stream)
{
  if (hp != 1 && hp != 2 && hp != 4) return 1;
  head_pool_kernel<<<nb((size_t)B * C * (1024 / (hp * hp)), 256), 256, 0, ST>>>((const bf16 *)h, (bf16 *)flat, B, C,
                                                                                 hp);
  RET;
}
int sg_head_unpool(const float *dflat, float *dh, int B, int C, int hp, void *stream)
{
  if (hp != 1 && hp != 2 && hp != 4) return 1;
  head_unpool_kernel<<<nb((size_t)B * C * 1024, 256), 256, 0, ST>>>(dflat, dh, B, C, hp);
  RET;
}
int sg_amp_mse(const float *out, const float *y, const float *w, void *dout, float *loss, int B, int n, int nt,
               void *stream)
{
  if (n < 2 * nt) return 1;
  amp_mse_kernel<<<B, 256, 0, ST>>>(out, y, w, (bf16 *)dout, loss, B, n, nt);
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
int sg_colsum_f32(const float *a, float *out, int R, int N, void *stream)
{
  colsum_f32_kernel<<<nb((size_t)N, 256), 256, 0, ST>>>(a, out, R, N);
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
