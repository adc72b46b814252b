// SPDX-License-Identifier: MPL-2.0
// Allocation-free variant of the curvature-ratio prune (the second half of
// the reference's select(), src/cpu/selection.cpp:20-27, and of its CUDA
// prune + compaction, src/cuda/backend.cu:21-30 and :375-407).
//
// The regular entry point (sym_select) draws its scratch (keep flags, per
// sample counts, scan partials) from the context's workspace, which grows by
// cudaMalloc when a call needs more.  Callers that may not allocate device
// memory at call time -- a service that pre-sizes every buffer at start-up,
// or code that runs between allocator checkpoints -- use sym_prune_static
// instead: the caller owns every input and output buffer, and the only
// scratch is one fixed array of per-tile counters in this module's static
// device memory.
//
// Three kernels on the caller's stream, order-preserving (the kept samples
// come out in sample order, like the reference's push_back loop):
//   1. prune_tile_counts  each block of kPruneTile samples counts its kept
//                         samples -> scratch counts[tile]; samples outside
//                         [0, vertex_count) set the scratch status word
//   2. prune_tile_offsets one block scans counts[] in place (exclusive) and
//                         writes the total (or UINT64_MAX on a bad index)
//   3. prune_scatter      each block re-evaluates its samples, ranks the kept
//                         ones inside the block and writes them at
//                         offsets[tile] + rank (it leaves the status word to
//                         prune_tile_counts, which already reported any bad
//                         index before the scan read the word)
#include "common.cuh"

#include <cstring>
#include <mutex>

namespace {

constexpr uint32_t kPruneThreads = 256;
constexpr uint32_t kPrunePerThread = 4;
constexpr uint32_t kPruneTile = kPruneThreads * kPrunePerThread;  // 1024 samples
constexpr uint64_t kPruneMaxSamples = uint64_t(1) << 24;           // 16,777,216
constexpr uint32_t kPruneMaxTiles = uint32_t(kPruneMaxSamples / kPruneTile);  // 16,384
constexpr uint32_t kScanThreads = 1024;
static_assert(kPruneMaxTiles % kScanThreads == 0, "scan assigns whole runs to threads");

// Scratch: kPruneMaxTiles per-tile counters (overwritten by every call
// before they are read), then one status word (cleared at the start of
// every call).  64 KiB + 256 bytes of static device memory.
constexpr uint32_t kStatusWord = kPruneMaxTiles;
static __device__ __align__(256) uint32_t g_prune_scratch[kPruneMaxTiles + 64];

// Keep rule of the reference's select(): valid, not flat, and the principal
// curvatures differ by more than `threshold` (= 1 - prune) relative to the
// larger magnitude.
__device__ __forceinline__ bool keep_vertex(int32_t v, const double *kmin, const double *kmax,
                                            const uint8_t *valid, double threshold) {
  double a = kmin[v], b = kmax[v];
  double maximum = fabs(a) < fabs(b) ? fabs(b) : fabs(a);
  return valid[v] && maximum > 1e-10 && fabs(a - b) / maximum > threshold;
}

// Keep flags of this thread's kPrunePerThread consecutive samples (bit j =
// sample base + j); an index outside [0, vertex_count) is not kept and, when
// `report` is set, raises the status word.
__device__ __forceinline__ uint32_t thread_flags(const int32_t *sample, uint64_t count,
                                                 const double *kmin, const double *kmax,
                                                 const uint8_t *valid, uint64_t vertex_count,
                                                 double threshold, uint32_t *scratch,
                                                 bool report) {
  uint64_t base = uint64_t(blockIdx.x) * kPruneTile + uint64_t(threadIdx.x) * kPrunePerThread;
  uint32_t bits = 0;
  for (uint32_t j = 0; j < kPrunePerThread; ++j) {
    uint64_t i = base + j;
    if (i >= count) break;
    int32_t v = sample[i];
    if (v < 0 || uint64_t(v) >= vertex_count) {
      if (report) atomicOr(&scratch[kStatusWord], 1u);
      continue;
    }
    if (keep_vertex(v, kmin, kmax, valid, threshold)) bits |= 1u << j;
  }
  return bits;
}

// Exclusive block-wide prefix of `value` over kPruneThreads threads; the
// block total is returned through *total.
__device__ __forceinline__ uint32_t block_exclusive(uint32_t value, uint32_t *total) {
  __shared__ uint32_t warp_sums[kPruneThreads / 32];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = value;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t n = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= uint32_t(o)) incl += n;
  }
  if (lane == 31) warp_sums[warp] = incl;
  __syncthreads();
  uint32_t before = 0, all = 0;
  for (uint32_t w = 0; w < kPruneThreads / 32; ++w) {
    uint32_t s = warp_sums[w];
    before += w < warp ? s : 0;
    all += s;
  }
  *total = all;
  return before + incl - value;
}

__global__ void __launch_bounds__(kPruneThreads) prune_tile_counts(
    const int32_t *sample, uint64_t count, const double *kmin, const double *kmax,
    const uint8_t *valid, uint64_t vertex_count, double threshold, uint32_t *scratch) {
  uint32_t bits =
      thread_flags(sample, count, kmin, kmax, valid, vertex_count, threshold, scratch, true);
  uint32_t total;
  block_exclusive(__popc(bits), &total);
  if (threadIdx.x == 0) scratch[blockIdx.x] = total;
}

// One block: exclusive scan of counts[0..tiles) in place; *pruned_count =
// the total, or UINT64_MAX when a sample index was out of range.
__global__ void __launch_bounds__(kScanThreads) prune_tile_offsets(uint32_t tiles,
                                                                   uint32_t *scratch,
                                                                   uint64_t *pruned_count) {
  __shared__ uint32_t warp_sums[kScanThreads / 32];
  const uint32_t per = kPruneMaxTiles / kScanThreads;  // 16 counters per thread
  const uint32_t t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const uint32_t first = t * per;
  uint32_t local = 0;
  for (uint32_t j = 0; j < per; ++j)
    if (first + j < tiles) local += scratch[first + j];
  uint32_t incl = local;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t n = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= uint32_t(o)) incl += n;
  }
  if (lane == 31) warp_sums[warp] = incl;
  __syncthreads();
  uint32_t before = 0, all = 0;
  for (uint32_t w = 0; w < kScanThreads / 32; ++w) {
    uint32_t s = warp_sums[w];
    before += w < warp ? s : 0;
    all += s;
  }
  uint32_t run = before + incl - local;
  for (uint32_t j = 0; j < per; ++j)
    if (first + j < tiles) {
      uint32_t c = scratch[first + j];
      scratch[first + j] = run;
      run += c;
    }
  if (t == 0) *pruned_count = scratch[kStatusWord] ? ~uint64_t(0) : uint64_t(all);
}

__global__ void __launch_bounds__(kPruneThreads) prune_scatter(
    const int32_t *sample, uint64_t count, const double *kmin, const double *kmax,
    const uint8_t *valid, uint64_t vertex_count, double threshold, uint32_t *scratch,
    int32_t *pruned) {
  uint32_t bits =
      thread_flags(sample, count, kmin, kmax, valid, vertex_count, threshold, scratch, false);
  uint32_t total;
  uint32_t rank = block_exclusive(__popc(bits), &total);
  uint64_t out = uint64_t(scratch[blockIdx.x]) + rank;
  uint64_t base = uint64_t(blockIdx.x) * kPruneTile + uint64_t(threadIdx.x) * kPrunePerThread;
  for (uint32_t j = 0; j < kPrunePerThread; ++j)
    if (bits >> j & 1u) pruned[out++] = sample[base + j];
}

// Device address of g_prune_scratch per device, filled by the setup.
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
uint32_t *g_scratch_ptr[kMaxDevices] = {};

sym_status fail_with(sym_status status, const char *message) {
  sym_error_text = message;
  return status;
}

sym_status cuda_fail(cudaError_t e, const char *what) {
  sym_error_text = std::string(what) + ": " + cudaGetErrorString(e);
  return SYM_CUDA_ERROR;
}

// Scratch address on the current device.  The first use on a device looks
// it up; `refresh` looks it up again (after cudaDeviceReset the device's
// context, and with it the array's address, is new).
sym_status scratch_for_current_device(uint32_t **out, bool refresh) {
  int device = -1;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (device < 0 || device >= kMaxDevices)
    return fail_with(SYM_RUNTIME_ERROR, "device ordinal beyond the static scratch table");
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (refresh || !g_scratch_ptr[device]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_prune_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_prune_scratch)");
    g_scratch_ptr[device] = static_cast<uint32_t *>(p);
  }
  *out = g_scratch_ptr[device];
  return SYM_OK;
}

}  // namespace

extern "C" {

uint64_t sym_prune_static_max_samples(void) { return kPruneMaxSamples; }

sym_status sym_prune_static_setup(void) {
  uint32_t *p = nullptr;
  return scratch_for_current_device(&p, true);
}

sym_status sym_prune_static(const int32_t *sample, uint64_t count, const double *kmin,
                            const double *kmax, const uint8_t *valid, uint64_t vertex_count,
                            double prune, int32_t *pruned, uint64_t *pruned_count,
                            void *stream) {
  if (!pruned_count || (count && (!sample || !kmin || !kmax || !valid || !pruned)))
    return fail_with(SYM_INVALID_ARGUMENT, "null argument");
  if (count > kPruneMaxSamples)
    return fail_with(SYM_INVALID_ARGUMENT,
                     "sym_prune_static: sample count exceeds the static scratch limit of "
                     "16,777,216 samples; use sym_select");
  if (!(prune > 0 && prune < 1))
    return fail_with(SYM_INVALID_ARGUMENT, "prune must lie in (0, 1)");
  uint32_t *scratch = nullptr;
  sym_status s = scratch_for_current_device(&scratch, false);
  if (s != SYM_OK) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(scratch + kStatusWord, 0, sizeof(uint32_t), st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(status)");
  const uint32_t tiles = uint32_t((count + kPruneTile - 1) / kPruneTile);
  const double threshold = 1 - prune;
  if (tiles)
    prune_tile_counts<<<tiles, kPruneThreads, 0, st>>>(sample, count, kmin, kmax, valid,
                                                       vertex_count, threshold, scratch);
  prune_tile_offsets<<<1, kScanThreads, 0, st>>>(tiles, scratch, pruned_count);
  if (tiles)
    prune_scatter<<<tiles, kPruneThreads, 0, st>>>(sample, count, kmin, kmax, valid,
                                                   vertex_count, threshold, scratch, pruned);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "prune kernels");
  return SYM_OK;
}

}  // extern "C"
