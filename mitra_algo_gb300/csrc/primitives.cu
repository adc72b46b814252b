// SPDX-License-Identifier: MPL-2.0
#include "primitives.cuh"

namespace sym {
namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

// Block-wide exclusive scan of one value per thread; returns the block total.
__device__ uint64_t block_exclusive(uint64_t v, uint64_t &total) {
  __shared__ uint64_t warp_sums[32];
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint64_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    uint64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  int warps = blockDim.x >> 5;
  if (warp == 0) {
    uint64_t s = lane < warps ? warp_sums[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      uint64_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < warps) warp_sums[lane] = s;
  }
  __syncthreads();
  uint64_t before = warp ? warp_sums[warp - 1] : 0;
  total = warp_sums[warps - 1];
  __syncthreads();
  return before + x - v;
}

__global__ void tile_sums(const uint64_t *in, uint64_t n, uint64_t *partial) {
  uint64_t base = uint64_t(blockIdx.x) * kScanTile + threadIdx.x * kScanItems;
  uint64_t s = 0;
  for (int k = 0; k < kScanItems; ++k)
    if (base + k < n) s += in[base + k];
  uint64_t total;
  block_exclusive(s, total);
  if (threadIdx.x == 0) partial[blockIdx.x] = total;
}

// One block scans `count` partial sums in place (exclusive) sequentially in
// chunks of blockDim.
__global__ void scan_partials(uint64_t *partial, uint64_t count) {
  __shared__ uint64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (uint64_t at = 0; at < count; at += blockDim.x) {
    uint64_t i = at + threadIdx.x;
    uint64_t v = i < count ? partial[i] : 0, total;
    uint64_t ex = block_exclusive(v, total);
    if (i < count) partial[i] = carry + ex;
    __syncthreads();
    if (threadIdx.x == 0) carry += total;
    __syncthreads();
  }
}

__global__ void tile_scan(const uint64_t *in, uint64_t n, const uint64_t *partial,
                          uint64_t *out) {
  uint64_t base = uint64_t(blockIdx.x) * kScanTile + threadIdx.x * kScanItems;
  uint64_t v[kScanItems], s = 0;
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = base + k < n ? in[base + k] : 0;
    s += v[k];
  }
  uint64_t total;
  uint64_t run = block_exclusive(s, total) + partial[blockIdx.x];
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < n) out[base + k] = run;
    run += v[k];
  }
  if (base < n && base + kScanItems >= n) out[n] = run;  // thread holding the last item
}

// ---------------------------------------------------------------- radix sort
constexpr int kSortWarps = 8;
constexpr int kSortRounds = 8;                       // 32-key rounds per warp
constexpr int kSortTile = kSortWarps * kSortRounds * 32;  // 2048 keys per block

__global__ void radix_histogram(const uint64_t *keys, uint64_t n, int shift, uint64_t *hist,
                                unsigned blocks) {
  __shared__ unsigned counts[256];
  for (int d = threadIdx.x; d < 256; d += blockDim.x) counts[d] = 0;
  __syncthreads();
  uint64_t base = uint64_t(blockIdx.x) * kSortTile;
  for (int i = threadIdx.x; i < kSortTile; i += blockDim.x)
    if (base + i < n) atomicAdd(&counts[(keys[base + i] >> shift) & 0xff], 1u);
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += blockDim.x)
    hist[uint64_t(d) * blocks + blockIdx.x] = counts[d];
}

// Stable scatter: warp w ranks its 256 keys round by round (in input order),
// warps are then ordered by their index, blocks by the scanned histogram.
// The block's keys are first placed in digit order in shared memory, so the
// global writes of each digit are one consecutive run.
__global__ void __launch_bounds__(kSortWarps * 32) radix_scatter(
    const uint64_t *keys, const int32_t *vals, uint64_t n, int shift, const uint64_t *offsets,
    unsigned blocks, uint64_t *keys_out, int32_t *vals_out) {
  __shared__ unsigned warp_count[kSortWarps][256];
  __shared__ unsigned digit_start[256];
  __shared__ uint64_t skey[kSortTile];
  __shared__ int32_t sval[kSortTile];
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int d = threadIdx.x; d < kSortWarps * 256; d += blockDim.x)
    (&warp_count[0][0])[d] = 0;
  __syncthreads();
  uint64_t base = uint64_t(blockIdx.x) * kSortTile + uint64_t(warp) * kSortRounds * 32;
  uint64_t key[kSortRounds];
  int32_t val[kSortRounds];
  unsigned rank[kSortRounds];
  unsigned lt = (1u << lane) - 1;
  for (int r = 0; r < kSortRounds; ++r) {
    uint64_t i = base + r * 32 + lane;
    bool live = i < n;
    key[r] = live ? keys[i] : 0;
    val[r] = live ? vals[i] : 0;
    unsigned digit = live ? unsigned((key[r] >> shift) & 0xff) : 256u;
    unsigned peers = __match_any_sync(0xffffffffu, digit);
    unsigned before = digit < 256 ? warp_count[warp][digit] : 0;
    rank[r] = before + __popc(peers & lt);
    __syncwarp();
    if (live && (peers & lt) == 0) warp_count[warp][digit] = before + __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // per digit: each warp's start among the block's keys of that digit, and
  // the digit's count; then the digits' starts in the block
  unsigned digit_total = 0;
  if (threadIdx.x < 256) {
    const int d = threadIdx.x;
    for (int w = 0; w < kSortWarps; ++w) {
      unsigned c = warp_count[w][d];
      warp_count[w][d] = digit_total;
      digit_total += c;
    }
  }
  uint64_t all;
  const uint64_t start = block_exclusive(digit_total, all);  // blockDim.x == 256
  if (threadIdx.x < 256) digit_start[threadIdx.x] = unsigned(start);
  __syncthreads();
  for (int r = 0; r < kSortRounds; ++r) {
    uint64_t i = base + r * 32 + lane;
    if (i >= n) continue;
    unsigned digit = unsigned((key[r] >> shift) & 0xff);
    unsigned pos = digit_start[digit] + warp_count[warp][digit] + rank[r];
    skey[pos] = key[r];
    sval[pos] = val[r];
  }
  __syncthreads();
  const uint64_t block_base = uint64_t(blockIdx.x) * kSortTile;
  const unsigned count = unsigned(n - block_base < uint64_t(kSortTile) ? n - block_base : kSortTile);
  for (unsigned j = threadIdx.x; j < count; j += blockDim.x) {
    const uint64_t k = skey[j];
    const unsigned digit = unsigned((k >> shift) & 0xff);
    const uint64_t dst = offsets[uint64_t(digit) * blocks + blockIdx.x] + (j - digit_start[digit]);
    keys_out[dst] = k;
    vals_out[dst] = sval[j];
  }
}

__global__ void flags_to_counts(const uint8_t *flags, uint64_t n, uint64_t *counts) {
  uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) counts[i] = flags[i] != 0;
}

__global__ void scatter_flagged(const uint8_t *flags, const int32_t *values, uint64_t n,
                                const uint64_t *pos, int32_t *out, uint64_t *count) {
  uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n && flags[i]) out[pos[i]] = values ? values[i] : int32_t(i);
  if (i == 0) *count = pos[n];
}

}  // namespace

void exclusive_scan(Call &call, const uint64_t *in, uint64_t *out, uint64_t n) {
  if (n == 0) {
    SYM_CUDA(cudaMemsetAsync(out, 0, sizeof(uint64_t), call.stream()));
    return;
  }
  unsigned tiles = static_cast<unsigned>((n + kScanTile - 1) / kScanTile);
  uint64_t *partial = call.alloc<uint64_t>(tiles);
  tile_sums<<<tiles, kScanThreads, 0, call.stream()>>>(in, n, partial);
  check_launch();
  scan_partials<<<1, 1024, 0, call.stream()>>>(partial, tiles);
  check_launch();
  tile_scan<<<tiles, kScanThreads, 0, call.stream()>>>(in, n, partial, out);
  check_launch();
  call.launched(3);
}

void radix_sort_pairs(Call &call, const uint64_t *keys, const int32_t *values,
                      uint64_t *keys_out, int32_t *values_out, uint64_t n, int key_bits) {
  if (n == 0) return;
  unsigned blocks = static_cast<unsigned>((n + kSortTile - 1) / kSortTile);
  uint64_t hist_n = uint64_t(blocks) * 256;
  uint64_t *hist = call.alloc<uint64_t>(hist_n);
  uint64_t *offsets = call.alloc<uint64_t>(hist_n + 1);
  uint64_t *kbuf = call.alloc<uint64_t>(n);
  int32_t *vbuf = call.alloc<int32_t>(n);
  int passes = (key_bits + 7) / 8;
  // ping-pong so that the last pass writes keys_out/values_out
  const uint64_t *ksrc = keys;
  const int32_t *vsrc = values;
  for (int p = 0; p < passes; ++p) {
    bool last_to_out = ((passes - 1 - p) % 2) == 0;
    uint64_t *kdst = last_to_out ? keys_out : kbuf;
    int32_t *vdst = last_to_out ? values_out : vbuf;
    int shift = 8 * p;
    radix_histogram<<<blocks, 256, 0, call.stream()>>>(ksrc, n, shift, hist, blocks);
    check_launch();
    exclusive_scan(call, hist, offsets, hist_n);
    radix_scatter<<<blocks, kSortWarps * 32, 0, call.stream()>>>(ksrc, vsrc, n, shift, offsets,
                                                                 blocks, kdst, vdst);
    check_launch();
    call.launched(2);
    ksrc = kdst;
    vsrc = vdst;
  }
}

void compact_values(Call &call, const uint8_t *flags, const int32_t *values, uint64_t n,
                    int32_t *out, uint64_t *count) {
  if (n == 0) {
    SYM_CUDA(cudaMemsetAsync(count, 0, sizeof(uint64_t), call.stream()));
    return;
  }
  uint64_t *counts = call.alloc<uint64_t>(n);
  uint64_t *pos = call.alloc<uint64_t>(n + 1);
  flags_to_counts<<<blocks_for(n), kThreads, 0, call.stream()>>>(flags, n, counts);
  check_launch();
  exclusive_scan(call, counts, pos, n);
  scatter_flagged<<<blocks_for(n), kThreads, 0, call.stream()>>>(flags, values, n, pos, out, count);
  check_launch();
  call.launched(2);
}

void compact_indices(Call &call, const uint8_t *flags, uint64_t n, int32_t *out,
                     uint64_t *count) {
  compact_values(call, flags, nullptr, n, out, count);
}

}  // namespace sym
