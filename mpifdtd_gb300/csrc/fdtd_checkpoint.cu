// fdtd_checkpoint.cu -- checkpoint / resume and the finite-value check of one
// simulation.
//
// The reference has neither: its reset only zeroes the fields
// (mpiTM_UPML.c:219-232) and an error is a printf + exit (function.c:27-32).
// A checkpoint image is the simulation's whole time-stepping state in one
// byte image:
//
//   header (CkptHeader, then the running-DFT wavelengths as int32)
//   permittivity as given, 3 arrays of nxa x pitch doubles (halo included)
//   every field slot of the solver, nxa x pitch elements of the field precision
//   the three time-domain NTFF accumulators with their guard bins (if any)
//   the running-DFT sums [2][ncell][2 nlam] complex (if enabled)
//
// The derived state (1/eps, the per-cell coefficients of the split / NS
// solvers, the PML tables, the source tables, the NTFF path) is rebuilt from
// the configuration and the permittivity; the buffered NTFF steps are
// deposited before saving, so an image holds no pending work.  The tuning
// options are stored and restored, so a resumed run's fields and DFT sums
// round exactly as the saved simulation's would have (the NTFF accumulators
// only to the order of their atomic adds, which no two runs share).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "fdtd_internal.cuh"
#include "fdtd_sim.h"

using namespace fdtd;

namespace {

#define KCK(call)                                                                                  \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) {                                                                       \
      cudaGetLastError();                                                                          \
      return set_error(FDTD_E_CUDA, "%s: %s", #call, cudaGetErrorString(e_));                     \
    }                                                                                              \
  } while (0)

constexpr char kMagic[8] = {'M', 'F', 'D', 'T', 'D', 'C', 'K', '1'};
constexpr uint32_t kVersion = 1;
constexpr int kNumOptions = 7;  // FDTD_OPT_NTFF_MODE .. FDTD_OPT_TBLOCK_COLS

// Fixed-width, 8-byte aligned members only: the image is the same on x86-64
// and aarch64 hosts (both little-endian).
struct CkptHeader {
  char magic[8];
  uint32_t version, header_bytes;        // header_bytes: this struct + 4 nlam
  int32_t solver, nslots, esize, nxa, pitch, nlam;
  fdtd_config cfg;                       // 16 int32
  int32_t has_ntff, has_dft;
  int32_t options[8];                    // values of options 1..7, [7] unused
  uint64_t ntff_len, ncell, payload_bytes, reserved;
  double time, ray_coef;
};
static_assert(sizeof(fdtd_config) == 16 * sizeof(int32_t), "fdtd_config is 16 ints");
static_assert(sizeof(CkptHeader) == 8 + 8 + 24 + 64 + 8 + 32 + 32 + 16, "checkpoint header layout");

struct Segment {
  void *dev;
  size_t bytes;
};

std::vector<Segment> segments_of(const fdtd_sim *s)
{
  std::vector<Segment> seg;
  const size_t cells = (size_t)s->nxa * s->pitch;
  for (int a = 0; a < 3; a++) seg.push_back({s->d_eps[a], cells * sizeof(double)});
  for (int a = 0; a < s->nslots; a++) seg.push_back({s->d_f[a], cells * s->esize});
  if (s->d_ntff[0])
    for (int a = 0; a < 3; a++) seg.push_back({s->d_ntff[a], s->ntff_len * sizeof(double2)});
  if (s->d_dft_S) seg.push_back({s->d_dft_S, 2 * (size_t)s->ncell * 2 * s->dft_lam.size() * sizeof(double2)});
  return seg;
}

size_t payload_of(const std::vector<Segment> &seg)
{
  size_t n = 0;
  for (const Segment &g : seg) n += g.bytes;
  return n;
}

int header_of(fdtd_sim *s, CkptHeader *h)
{
  std::memset(h, 0, sizeof *h);
  std::memcpy(h->magic, kMagic, sizeof kMagic);
  h->version = kVersion;
  h->nlam = (int32_t)s->dft_lam.size();
  h->header_bytes = (uint32_t)(sizeof(CkptHeader) + 4 * (size_t)h->nlam);
  h->solver = s->solver;
  h->nslots = s->nslots;
  h->esize = (int32_t)s->esize;
  h->nxa = s->nxa;
  h->pitch = s->pitch;
  h->cfg = s->cfg;
  h->has_ntff = s->d_ntff[0] != nullptr;
  h->has_dft = s->d_dft_S != nullptr;
  for (int k = 0; k < kNumOptions; k++)
    if (int rc = fdtd_get_option(s, k + 1, &h->options[k])) return rc;
  h->ntff_len = s->d_ntff[0] ? s->ntff_len : 0;
  h->ncell = (uint64_t)s->ncell;
  h->payload_bytes = payload_of(segments_of(s));
  h->time = s->time;
  h->ray_coef = s->ray_coef;
  return FDTD_OK;
}

// The image's header against the simulation it is loaded into.
int check_header(const fdtd_sim *s, const CkptHeader &h, const int32_t *lam, size_t bytes)
{
  if (std::memcmp(h.magic, kMagic, sizeof kMagic) != 0) return set_error(FDTD_E_ARG, "not a checkpoint image");
  if (h.version != kVersion) return set_error(FDTD_E_ARG, "checkpoint version %u (this library reads %u)", h.version, kVersion);
  if (h.nlam < 0 || h.header_bytes != sizeof(CkptHeader) + 4 * (size_t)h.nlam)
    return set_error(FDTD_E_ARG, "checkpoint header is corrupt");
  if (bytes != h.header_bytes + h.payload_bytes)
    return set_error(FDTD_E_ARG, "checkpoint image is %zu bytes, its header says %llu", bytes,
                     (unsigned long long)(h.header_bytes + h.payload_bytes));
  if (h.solver != s->solver) return set_error(FDTD_E_ARG, "checkpoint of solver %d, simulation is %d", h.solver, s->solver);
  if (std::memcmp(&h.cfg, &s->cfg, sizeof(fdtd_config)) != 0)
    return set_error(FDTD_E_ARG, "checkpoint was taken with another fdtd_config");
  if (h.nslots != s->nslots || h.esize != (int32_t)s->esize || h.nxa != s->nxa || h.pitch != s->pitch ||
      h.ncell != (uint64_t)s->ncell || h.has_ntff != (s->d_ntff[0] != nullptr) ||
      (h.has_ntff && h.ntff_len != s->ntff_len))
    return set_error(FDTD_E_ARG, "checkpoint layout differs from the simulation's");
  if (h.has_dft != (h.nlam > 0)) return set_error(FDTD_E_ARG, "checkpoint header is corrupt");
  // a simulation without a running DFT gets the image's (prepare_load)
  if (s->d_dft_S && ((size_t)h.nlam != s->dft_lam.size() || !std::equal(s->dft_lam.begin(), s->dft_lam.end(), lam)))
    return set_error(FDTD_E_ARG, "the simulation's running-DFT wavelengths differ from the checkpoint's");
  return FDTD_OK;
}

// Before the device arrays are written: the buffered NTFF steps of the old
// state are deposited (nothing of it may land after the image), the image's
// options are set, and its running DFT is enabled on a simulation without one.
int prepare_load(fdtd_sim *s, const CkptHeader &h, const int32_t *lam)
{
  if (int rc = fdtd_flush(s)) return rc;
  for (int k = 0; k < kNumOptions; k++)
    if (int rc = fdtd_set_option(s, k + 1, h.options[k])) return rc;
  if (h.nlam > 0 && !s->d_dft_S) {
    std::vector<int> l(lam, lam + h.nlam);
    if (int rc = fdtd_dft_enable(s, h.nlam, l.data())) return rc;
  }
  if (payload_of(segments_of(s)) != h.payload_bytes) return set_error(FDTD_E_ARG, "checkpoint payload size differs");
  return FDTD_OK;
}

// After: 1/eps (or the per-cell coefficients) from the permittivity, and the clock.
int finish_load(fdtd_sim *s, const CkptHeader &h)
{
  if (int rc = fdtd_derive_inv_eps(s)) return rc;
  s->time = h.time;
  s->ray_coef = h.ray_coef;
  return FDTD_OK;
}

constexpr size_t kStage = 64u << 20;  // pinned staging chunk of the file route

// ---------------------------------------------------------------- finite check

__device__ __forceinline__ bool nonfinite(double v)
{
  return ((__double_as_longlong(v) >> 52) & 0x7ff) == 0x7ff;  // exponent all ones: Inf or NaN
}
__device__ __forceinline__ bool nonfinite(float v) { return ((__float_as_uint(v) >> 23) & 0xff) == 0xff; }

// Counts the complex elements of a[0..n) with a non-finite part; the bit
// patterns are tested on the integer ALU.
template <typename T>
__global__ void __launch_bounds__(256) nonfinite_kernel(const T *__restrict__ a, size_t n,
                                                        unsigned long long *count, unsigned int *status)
{
  unsigned long long c = 0;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    const T v = a[k];
    c += (nonfinite(v.x) || nonfinite(v.y)) ? 1 : 0;
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) {
    atomicAdd(count, c);
    atomicOr(status, kStatusNonFinite);
  }
}

}  // namespace

extern "C" int fdtd_checkpoint_size(fdtd_sim *s, size_t *bytes)
{
  if (!s || !bytes) return set_error(FDTD_E_ARG, "null argument");
  *bytes = sizeof(CkptHeader) + 4 * s->dft_lam.size() + payload_of(segments_of(s));
  return FDTD_OK;
}

extern "C" int fdtd_checkpoint_save(fdtd_sim *s, void *buf, size_t bytes)
{
  if (!s || !buf) return set_error(FDTD_E_ARG, "null argument");
  if (int rc = fdtd_flush(s)) return rc;
  CkptHeader h;
  if (int rc = header_of(s, &h)) return rc;
  if (bytes != h.header_bytes + h.payload_bytes)
    return set_error(FDTD_E_ARG, "checkpoint buffer is %zu bytes, the image %llu (fdtd_checkpoint_size)", bytes,
                     (unsigned long long)(h.header_bytes + h.payload_bytes));
  char *p = (char *)buf;
  std::memcpy(p, &h, sizeof h);
  for (size_t k = 0; k < s->dft_lam.size(); k++) {
    const int32_t l = s->dft_lam[k];
    std::memcpy(p + sizeof h + 4 * k, &l, 4);
  }
  p += h.header_bytes;
  for (const Segment &g : segments_of(s)) {
    KCK(cudaMemcpyAsync(p, g.dev, g.bytes, cudaMemcpyDeviceToHost, s->stream));
    p += g.bytes;
  }
  KCK(cudaStreamSynchronize(s->stream));
  return FDTD_OK;
}

extern "C" int fdtd_checkpoint_load(fdtd_sim *s, const void *buf, size_t bytes)
{
  if (!s || !buf) return set_error(FDTD_E_ARG, "null argument");
  if (bytes < sizeof(CkptHeader)) return set_error(FDTD_E_ARG, "checkpoint image of %zu bytes is too short", bytes);
  CkptHeader h;
  std::memcpy(&h, buf, sizeof h);
  const char *p = (const char *)buf;
  std::vector<int32_t> lam(h.nlam > 0 && bytes >= sizeof h + 4 * (size_t)h.nlam ? h.nlam : 0);
  if (!lam.empty()) std::memcpy(lam.data(), p + sizeof h, 4 * lam.size());
  if ((size_t)std::max(h.nlam, 0) != lam.size()) return set_error(FDTD_E_ARG, "checkpoint header is corrupt");
  if (int rc = check_header(s, h, lam.data(), bytes)) return rc;
  if (int rc = prepare_load(s, h, lam.data())) return rc;
  p += h.header_bytes;
  for (const Segment &g : segments_of(s)) {
    KCK(cudaMemcpyAsync(g.dev, p, g.bytes, cudaMemcpyHostToDevice, s->stream));
    p += g.bytes;
  }
  KCK(cudaStreamSynchronize(s->stream));
  return finish_load(s, h);
}

extern "C" int fdtd_checkpoint_write(fdtd_sim *s, const char *path)
{
  if (!s || !path) return set_error(FDTD_E_ARG, "null argument");
  if (int rc = fdtd_flush(s)) return rc;
  CkptHeader h;
  if (int rc = header_of(s, &h)) return rc;
  FILE *f = std::fopen(path, "wb");
  if (!f) return set_error(FDTD_E_ARG, "cannot open %s for writing", path);
  std::vector<int32_t> lam(s->dft_lam.begin(), s->dft_lam.end());
  bool ok = std::fwrite(&h, sizeof h, 1, f) == 1 && (lam.empty() || std::fwrite(lam.data(), 4, lam.size(), f) == lam.size());
  void *stage = nullptr;
  if (ok && cudaMallocHost(&stage, kStage) != cudaSuccess) {
    cudaGetLastError();
    std::fclose(f);
    return set_error(FDTD_E_NOMEM, "pinned staging buffer of %zu bytes", kStage);
  }
  int rc = FDTD_OK;
  for (const Segment &g : segments_of(s)) {
    for (size_t off = 0; ok && rc == FDTD_OK && off < g.bytes; off += kStage) {
      const size_t n = std::min(kStage, g.bytes - off);
      cudaError_t e = cudaMemcpyAsync(stage, (const char *)g.dev + off, n, cudaMemcpyDeviceToHost, s->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
      if (e != cudaSuccess) {
        cudaGetLastError();
        rc = set_error(FDTD_E_CUDA, "checkpoint copy: %s", cudaGetErrorString(e));
      } else {
        ok = std::fwrite(stage, 1, n, f) == n;
      }
    }
  }
  if (stage) cudaFreeHost(stage);
  if (std::fclose(f) != 0) ok = false;
  if (rc) return rc;
  if (!ok) return set_error(FDTD_E_ARG, "writing %s failed", path);
  return FDTD_OK;
}

extern "C" int fdtd_checkpoint_read(fdtd_sim *s, const char *path)
{
  if (!s || !path) return set_error(FDTD_E_ARG, "null argument");
  FILE *f = std::fopen(path, "rb");
  if (!f) return set_error(FDTD_E_ARG, "cannot open %s", path);
  CkptHeader h;
  std::vector<int32_t> lam;
  bool ok = std::fread(&h, sizeof h, 1, f) == 1 && h.nlam >= 0 && h.nlam < (1 << 20);
  if (ok && h.nlam > 0) {
    lam.resize(h.nlam);
    ok = std::fread(lam.data(), 4, lam.size(), f) == lam.size();
  }
  long long size = -1;
  if (ok && std::fseek(f, 0, SEEK_END) == 0) size = std::ftell(f);
  if (!ok || size < 0 || std::fseek(f, (long)(sizeof h + 4 * lam.size()), SEEK_SET) != 0) {
    std::fclose(f);
    return set_error(FDTD_E_ARG, "%s is not a checkpoint image", path);
  }
  int rc = check_header(s, h, lam.data(), (size_t)size);
  if (!rc) rc = prepare_load(s, h, lam.data());
  void *stage = nullptr;
  if (!rc && cudaMallocHost(&stage, kStage) != cudaSuccess) {
    cudaGetLastError();
    rc = set_error(FDTD_E_NOMEM, "pinned staging buffer of %zu bytes", kStage);
  }
  if (!rc) {
    for (const Segment &g : segments_of(s)) {
      for (size_t off = 0; rc == FDTD_OK && off < g.bytes; off += kStage) {
        const size_t n = std::min(kStage, g.bytes - off);
        if (std::fread(stage, 1, n, f) != n) {
          rc = set_error(FDTD_E_ARG, "%s ends early", path);
          break;
        }
        cudaError_t e = cudaMemcpyAsync((char *)g.dev + off, stage, n, cudaMemcpyHostToDevice, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);  // the stage is reused
        if (e != cudaSuccess) {
          cudaGetLastError();
          rc = set_error(FDTD_E_CUDA, "checkpoint copy: %s", cudaGetErrorString(e));
        }
      }
    }
  }
  if (stage) cudaFreeHost(stage);
  std::fclose(f);
  if (rc) return rc;
  return finish_load(s, h);
}

extern "C" int fdtd_check_finite(fdtd_sim *s, long long *count)
{
  if (!s || !count) return set_error(FDTD_E_ARG, "null argument");
  if (int rc = fdtd_flush(s)) return rc;
  unsigned long long *d_count = nullptr;
  KCK(cudaMallocAsync((void **)&d_count, sizeof *d_count, s->stream));
  cudaError_t e = cudaMemsetAsync(d_count, 0, sizeof *d_count, s->stream);
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const size_t cells = (size_t)s->nxa * s->pitch;
  const unsigned grid = (unsigned)std::max(1, nsm) * 8;
  for (int a = 0; e == cudaSuccess && a < s->nslots; a++) {
    if (s->f32)
      nonfinite_kernel<float2><<<grid, 256, 0, s->stream>>>((const float2 *)s->d_f[a], cells, d_count, s->d_status);
    else
      nonfinite_kernel<double2><<<grid, 256, 0, s->stream>>>((const double2 *)s->d_f[a], cells, d_count,
                                                              s->d_status);
    s->launches++;
    e = cudaGetLastError();
  }
  unsigned long long h = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d_count, sizeof h, cudaMemcpyDeviceToHost, s->stream);
  cudaFreeAsync(d_count, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(FDTD_E_CUDA, "finite check: %s", cudaGetErrorString(e));
  }
  *count = (long long)h;
  return FDTD_OK;
}
