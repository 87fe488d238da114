// surrogate_gemm.cu -- BF16 tensor-core GEMM for sm_103a (tcgen05 + TMA +
// TMEM), the contraction kernel of the far-field surrogate's forward and
// backward passes.
//
//   C[M,N] (FP32 or BF16, row-major, ldc) = A[M,K] . B[N,K]^T (+ bias[N])
//   (+ C if accumulate), optional GELU, with A, B BF16 row-major ("K-major").
//
// One CTA computes one 128 x BN output tile with 128 threads, two CTAs per SM
// (so that one CTA's epilogue runs under the other's MMAs):
//   thread 0 (warp 0)  TMA producer: 128 x 64 and BN x 64 operand tiles, 128-byte
//                      swizzled, into a 3-stage shared-memory ring (mbarrier
//                      full[s] with the transaction byte count);
//   thread 32 (warp 1) MMA issuer: four tcgen05.mma.kind::f16 (K = 16 each) per
//                      stage into an FP32 accumulator in TMEM, tcgen05.commit
//                      frees the stage (mbarrier empty[s]); a last commit
//                      signals `done`;
//   warp 2             allocates / frees the BN TMEM columns;
//   all four warps     epilogue: tcgen05.ld of their 32 accumulator lanes
//                      (rows), bias / accumulate / GELU, stores.
// Every mbarrier wait is bounded: on timeout the kernel sets *err and leaves
// the loop (results are then invalid and the host reports the error).
// Batched: grid.z runs independent products (3-D tensor maps); A or B may be
// shared by every batch entry.
// Shapes: M % 64 == 0, N % 64 == 0, K % 64 == 0, leading dims % 8 == 0.  A row
// tile reaching past M (M = 64, or M % 128 == 64) is loaded with the tensor
// map's zero fill and its rows past M are not stored.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>

namespace sg {

constexpr int BM = 128, BK = 64, STAGES = 3;  // 3 x 32 KB (BN = 128): two CTAs fit in an SM
constexpr int GROUP_M = 8;  // tile raster: GROUP_M row tiles share their column tiles' B panels in L2
constexpr unsigned kSpinLimit = 1u << 26;  // ~ seconds of polling, then give up

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity)
{
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait; returns false (and flags err) on timeout
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity, unsigned *err, unsigned code)
{
  for (unsigned it = 0; it < kSpinLimit; it++) {
    if (mbar_try_wait(bar, parity)) return true;
    if (it > 1024) __nanosleep(64);
  }
  atomicOr(err, code);
  return false;
}

// 3-D tile (K, rows, batch entry) into shared memory, completing on bar
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int c0, int c1, int c2, uint64_t *bar)
{
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_u32(dst)),
      "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
      : "memory");
}

// shared-memory matrix descriptor: K-major operand, 128-byte swizzle, 8-row
// groups 1024 bytes apart (SBO), version 1 (sm_100 family)
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr)
{
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);  // start address
  d |= (uint64_t)1 << 16;                   // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;         // stride byte offset
  d |= (uint64_t)1 << 46;                   // descriptor version
  d |= (uint64_t)2 << 61;                   // swizzle: 128 B
  return d;
}

// instruction descriptor, kind::f16: FP32 D, BF16 A and B, both K-major
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n)
{
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool acc)
{
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)acc));
}

__device__ __forceinline__ void mma_commit(uint64_t *bar)
{
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float *v)
{
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int q = 0; q < 32; q++) v[q] = __uint_as_float(r[q]);
}

// GELU with the tanh form of Hendrycks & Gimpel (2016)
__device__ __forceinline__ float gelu(float x)
{
  const float k0 = 0.7978845608f, k1 = 0.044715f;
  return 0.5f * x * (1.0f + tanhf(k0 * (x + k1 * x * x * x)));
}

struct Epilogue {
  void *c;            // output
  int M;              // rows of C: accumulator lanes at or past M are not stored
  long long c_bstride;  // elements between batch entries of C (and pre)
  int ldc;
  int c_bf16;         // 1: BF16 output, 0: FP32
  int accumulate;     // add into C (FP32 output only)
  const float *bias;  // per output column, or null
  int act;            // 0 none, 1 GELU
  float *pre;         // optional FP32 copy of the pre-activation (for the GELU backward)
};

template <int BN>
__global__ void __launch_bounds__(128, 2)
    gemm_bf16_tn_kernel(const __grid_constant__ CUtensorMap tA, const __grid_constant__ CUtensorMap tB, Epilogue ep,
                        int K, int a_batched, int b_batched, unsigned *err)
{
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  constexpr int A_BYTES = BM * BK * 2, B_BYTES = BN * BK * 2;
  uint8_t *sA = smem;
  uint8_t *sB = smem + STAGES * A_BYTES;
  uint64_t *full = (uint64_t *)(sB + STAGES * B_BYTES);
  uint64_t *empty = full + STAGES;
  uint64_t *done = empty + STAGES;
  uint32_t *tmem_slot = (uint32_t *)(done + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // grouped raster of the (column, row) tiles: consecutive CTAs walk GROUP_M
  // row tiles for each column tile, so the A and B panels of the CTAs in
  // flight stay in L2
  const int n_tiles = gridDim.x, m_tiles = gridDim.y;
  const int id = blockIdx.y * n_tiles + blockIdx.x;
  const int group = id / (GROUP_M * n_tiles);
  const int first_m = group * GROUP_M;
  const int gm = min(GROUP_M, m_tiles - first_m);
  const int in_group = id - group * GROUP_M * n_tiles;
  const int m0 = (first_m + in_group % gm) * BM, n0 = (in_group / gm) * BN, z = blockIdx.z;
  const int nk = K / BK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 2) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"((uint32_t)BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (threadIdx.x == 0) {  // TMA producer
    for (int kb = 0; kb < nk; kb++) {
      const int s = kb % STAGES;
      if (kb >= STAGES && !mbar_wait(&empty[s], ((kb / STAGES) - 1) & 1, err, 1u)) break;
      mbar_expect_tx(&full[s], A_BYTES + B_BYTES);
      tma_load_3d(sA + s * A_BYTES, &tA, kb * BK, m0, a_batched ? z : 0, &full[s]);
      tma_load_3d(sB + s * B_BYTES, &tB, kb * BK, n0, b_batched ? z : 0, &full[s]);
    }
  } else if (threadIdx.x == 32) {  // MMA issuer
    constexpr uint32_t idesc = idesc_bf16(BM, BN);
    bool ok = true;
    for (int kb = 0; kb < nk && ok; kb++) {
      const int s = kb % STAGES;
      ok = mbar_wait(&full[s], (kb / STAGES) & 1, err, 2u);
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint64_t ad = sw128_desc(smem_u32(sA + s * A_BYTES));
      const uint64_t bd = sw128_desc(smem_u32(sB + s * B_BYTES));
#pragma unroll
      for (int k = 0; k < BK / 16; k++)  // 16 BF16 = 32 bytes = 2 descriptor units per step
        mma_bf16(tmem, ad + 2 * k, bd + 2 * k, idesc, (kb | k) != 0);
      mma_commit(&empty[s]);
    }
    mma_commit(done);
  }
  __syncwarp();
  // epilogue
  const bool have = __all_sync(0xffffffffu, mbar_wait(done, 0, err, 4u));  // tcgen05.ld is warp-aligned
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const int row = m0 + warp * 32 + lane;
  if (have && m0 + warp * 32 < ep.M) {  // tcgen05.ld stays warp-uniform; lanes past M skip their stores
#pragma unroll 1
    for (int c = 0; c < BN; c += 32) {
      float v[32];
      tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
      const int col = n0 + c;
      if (ep.bias)
#pragma unroll
        for (int q = 0; q < 32; q++) v[q] += ep.bias[col + q];
      if (ep.c_bf16) {
        __nv_bfloat16 *out = (__nv_bfloat16 *)ep.c + z * ep.c_bstride + (size_t)row * ep.ldc + col;
        if (ep.pre) {
          float *pp = ep.pre + z * ep.c_bstride + (size_t)row * ep.ldc + col;
#pragma unroll
          for (int q = 0; q < 32; q += 4) *(float4 *)(pp + q) = make_float4(v[q], v[q + 1], v[q + 2], v[q + 3]);
        }
        if (ep.act == 1)
#pragma unroll
          for (int q = 0; q < 32; q++) v[q] = gelu(v[q]);
#pragma unroll
        for (int q = 0; q < 32; q += 8) {
          __align__(16) __nv_bfloat162 h[4];
#pragma unroll
          for (int e = 0; e < 4; e++) h[e] = __floats2bfloat162_rn(v[q + 2 * e], v[q + 2 * e + 1]);
          *(uint4 *)(out + q) = *(const uint4 *)h;
        }
      } else {
        float *out = (float *)ep.c + z * ep.c_bstride + (size_t)row * ep.ldc + col;
        if (ep.pre)
#pragma unroll
          for (int q = 0; q < 32; q += 4)
            *(float4 *)(ep.pre + z * ep.c_bstride + (size_t)row * ep.ldc + col + q) =
                make_float4(v[q], v[q + 1], v[q + 2], v[q + 3]);
        if (ep.act == 1)
#pragma unroll
          for (int q = 0; q < 32; q++) v[q] = gelu(v[q]);
#pragma unroll
        for (int q = 0; q < 32; q += 4) {
          float4 o = make_float4(v[q], v[q + 1], v[q + 2], v[q + 3]);
          if (ep.accumulate) {
            const float4 p = *(const float4 *)(out + q);
            o.x += p.x;
            o.y += p.y;
            o.z += p.z;
            o.w += p.w;
          }
          *(float4 *)(out + q) = o;
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 2) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)BN));
}

// ---------------------------------------------------------------- host

static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
static std::mutex g_mu;
static char g_err[256];

static int set_err(int code, const char *msg)
{
  snprintf(g_err, sizeof g_err, "%s", msg);
  return code;
}

static int encoder()
{
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_encode) return 0;
  cudaDriverEntryPointQueryResult q;
  void *fn = nullptr;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !fn) {
    cudaGetLastError();
    return set_err(2, "cuTensorMapEncodeTiled not available");
  }
  g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  return 0;
}

// batch x rows x K BF16 row-major matrices (ld elements between rows, bstride
// between batch entries), boxes of box_rows x 64, 128-byte swizzle
static int make_map(CUtensorMap *map, const void *ptr, int rows, int K, int ld, int box_rows, int batch,
                    long long bstride)
{
  const cuuint64_t dims[3] = {(cuuint64_t)K, (cuuint64_t)rows, (cuuint64_t)batch};
  const cuuint64_t strides[2] = {(cuuint64_t)ld * 2, (cuuint64_t)(batch > 1 ? bstride : (long long)ld * rows) * 2};
  const cuuint32_t box[3] = {(cuuint32_t)BK, (cuuint32_t)box_rows, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void *>(ptr), dims, strides, box,
                              estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : set_err(1, "cuTensorMapEncodeTiled rejected the operand");
}

template <int BN>
static size_t smem_bytes()
{
  return 1024 + STAGES * (BM * BK * 2 + BN * BK * 2) + (2 * STAGES + 1) * 8 + 16;
}

}  // namespace sg

using namespace sg;

extern "C" const char *sg_last_error(void) { return g_err; }

// C[z] = A[z] . B[z]^T (+bias) (+C[z]) (GELU) for z < batch.  c_bf16: BF16
// output; pre: optional FP32 copy of the pre-activation (same layout as C).
// *_bstride: elements between batch entries (0 for an operand shared by all).
// err: device word, OR-ed with 1/2/4 when a wait timed out.  stream: cudaStream_t.
extern "C" int sg_gemm_bf16_tn_batched(const void *A, int lda, long long a_bstride, const void *B, int ldb,
                                       long long b_bstride, void *C, int ldc, long long c_bstride, int M, int N,
                                       int K, int batch, int c_bf16, int accumulate, const float *bias, int act,
                                       float *pre, unsigned *err, void *stream)
{
  if (!A || !B || !C || !err) return set_err(1, "null pointer");
  if (M <= 0 || N <= 0 || K <= 0 || M % 64 || K % BK || N % 64) return set_err(1, "shape: M%64, N%64, K%64");
  if (batch < 1 || batch > 65535) return set_err(1, "batch must be in [1, 65535]");
  if (lda % 8 || ldb % 8 || ldc % 8 || a_bstride % 8 || b_bstride % 8 || c_bstride % 8 || ((uintptr_t)A & 15) ||
      ((uintptr_t)B & 15) || ((uintptr_t)C & 15))
    return set_err(1, "alignment");
  if (c_bf16 && accumulate) return set_err(1, "accumulate needs FP32 output");
  if (int rc = encoder()) return rc;
  const bool wide = N % 128 == 0;
  CUtensorMap ta, tb;
  // A or B may be shared by every batch entry (bstride 0: a one-entry map always read at z = 0)
  if (make_map(&ta, A, M, K, lda, BM, a_bstride ? batch : 1, a_bstride) ||
      make_map(&tb, B, N, K, ldb, wide ? 128 : 64, b_bstride ? batch : 1, b_bstride))
    return 1;
  Epilogue ep{C, M, c_bstride, ldc, c_bf16, accumulate, bias, act, pre};
  cudaStream_t st = (cudaStream_t)stream;
  const dim3 grid((unsigned)(N / (wide ? 128 : 64)), (unsigned)((M + BM - 1) / BM), (unsigned)batch);
  if (wide) {
    static bool cfg = false;
    if (!cfg) {
      cudaFuncSetAttribute(gemm_bf16_tn_kernel<128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem_bytes<128>());
      cfg = true;
    }
    gemm_bf16_tn_kernel<128><<<grid, 128, smem_bytes<128>(), st>>>(ta, tb, ep, K, a_bstride ? 1 : 0,
                                                                   b_bstride ? 1 : 0, err);
  } else {
    static bool cfg = false;
    if (!cfg) {
      cudaFuncSetAttribute(gemm_bf16_tn_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem_bytes<64>());
      cfg = true;
    }
    gemm_bf16_tn_kernel<64><<<grid, 128, smem_bytes<64>(), st>>>(ta, tb, ep, K, a_bstride ? 1 : 0,
                                                                 b_bstride ? 1 : 0, err);
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_err(2, cudaGetErrorString(e));
  return 0;
}

extern "C" int sg_gemm_bf16_tn(const void *A, int lda, const void *B, int ldb, void *C, int ldc, int M, int N, int K,
                               int c_bf16, int accumulate, const float *bias, int act, float *pre, unsigned *err,
                               void *stream)
{
  return sg_gemm_bf16_tn_batched(A, lda, 0, B, ldb, 0, C, ldc, 0, M, N, K, 1, c_bf16, accumulate, bias, act, pre,
                                 err, stream);
}
