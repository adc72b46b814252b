// SPDX-License-Identifier: MPL-2.0
// Area-weighted vertex sampling on the device, bit-exact with the reference's
// sample_vertices (src/core/sampling.cpp:5-24, called from
// src/cpu/selection.cpp:20 and src/cuda/backend.cu:379):
//
//   for each vertex i with w[i] > 0, in vertex order: one draw d of the
//   std::mt19937_64 engine, u = ((d >> 11) + 0.5) / 2^53, key -log(u) / w[i];
//   sort the (key, i) pairs; keep the first ceil(n * ratio); sort the ids.
//
// Device plan:
//  1. rank[i] = number of positive weights before i (exclusive scan), so
//     vertex i takes draw rank[i];
//  2. one block runs the engine from the caller's state (MT19937-64, the
//     generator of Matsumoto and Nishimura as the C++ standard specifies
//     std::mt19937_64): 312 words per regeneration, each output tempered,
//     the state handed back exactly as the host engine leaves it;
//  3. the keys, a stable 64-bit radix sort of (key, id) -- equal keys keep
//     ascending ids, the reference's pair order;
//  4. the boundary.  The device log and the host's std::log may differ in
//     the last bits, so the device keys are trusted only away from the
//     target-th key T: every key below T (1 - delta) is kept, every key above
//     T (1 + delta) dropped (delta = 2^-32, far above the few-ulp difference
//     of two faithfully rounded logs), and the keys inside that band are
//     recomputed on the host with std::log and ordered there.  The band
//     normally holds one key (T itself), in which case nothing is recomputed;
//  5. the kept ids are flagged and compacted in vertex order.
#include "primitives.cuh"
#include "sampling.cuh"

#include <algorithm>
#include <cmath>
#include <utility>

namespace sym {
namespace {

// MT19937-64 parameters (word size 64, degree 312, middle word 156,
// separation 31 bits, twist matrix a, tempering u d s b t c l).
constexpr int kWords = 312, kMiddle = 156;
constexpr uint64_t kTwist = 0xB5026F5AA96619E9ull;
constexpr uint64_t kLowerMask = (1ull << 31) - 1, kUpperMask = ~kLowerMask;

__device__ __forceinline__ uint64_t mt_next_word(uint64_t cur, uint64_t nxt, uint64_t far) {
  const uint64_t y = (cur & kUpperMask) | (nxt & kLowerMask);
  return far ^ (y >> 1) ^ ((y & 1) ? kTwist : 0ull);
}

__device__ __forceinline__ uint64_t mt_temper(uint64_t z) {
  z ^= (z >> 29) & 0x5555555555555555ull;
  z ^= (z << 17) & 0x71D67FFFEDA60000ull;
  z ^= (z << 37) & 0xFFF7EEE000000000ull;
  return z ^ (z >> 43);
}

__global__ void positive_flags(const double *w, uint64_t n, uint64_t *flags) {
  const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) flags[i] = w[i] > 0 ? 1 : 0;
}

// One block of kWords threads.  `state` holds the 312 words and the position
// (the layout of sym_rng); *count draws go to draws[0 .. count) and the
// final state back to `state`.  Regeneration follows the sequential in-place
// recurrence: words 0..155 from old words only, words 156..310 from the new
// word 156 places back, word 311 from new words 0 and 155; each thread keeps
// its own old words in registers across the two phases.
__global__ void __launch_bounds__(kWords) mt_draws(uint64_t *state, const uint64_t *count,
                                                   uint64_t *draws) {
  __shared__ uint64_t x[kWords];
  const int t = threadIdx.x;
  x[t] = state[t];
  uint64_t p = state[kWords];
  const uint64_t n = *count;
  __syncthreads();
  for (uint64_t j = 0;;) {
    const uint64_t left = p < kWords ? kWords - p : 0;
    const uint64_t take = left < n - j ? left : n - j;
    if (uint64_t(t) < take) draws[j + t] = mt_temper(x[p + t]);
    j += take;
    p += take;
    if (j >= n) break;
    const uint64_t cur = x[t], nxt = t + 1 < kWords ? x[t + 1] : 0;
    __syncthreads();
    if (t < kWords - kMiddle) x[t] = mt_next_word(cur, nxt, x[t + kMiddle]);
    __syncthreads();
    if (t >= kWords - kMiddle && t < kWords - 1) x[t] = mt_next_word(cur, nxt, x[t - (kWords - kMiddle)]);
    if (t == kWords - 1) x[t] = mt_next_word(cur, x[0], x[kMiddle - 1]);
    __syncthreads();
    p = 0;
  }
  state[t] = x[t];
  if (t == 0) state[kWords] = p;
}

__global__ void sample_keys(const double *w, uint64_t n, const uint64_t *rank,
                            const uint64_t *draws, uint64_t *keys, int32_t *ids) {
  const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double wi = w[i];
  uint64_t key = ~0ull;  // no draw: after every positive weight
  if (wi > 0) {
    const double u = (double(draws[rank[i]] >> 11) + 0.5) / 9007199254740992.0;
    key = orderable_key(-log(u) / wi);
  }
  keys[i] = key;
  ids[i] = int32_t(i);
}

struct Band {
  uint64_t target, positive, lo, hi;
};

__device__ __forceinline__ double key_value(uint64_t k) {  // inverse of orderable_key, k >= 0
  const uint64_t b = k & 0x7FFFFFFFFFFFFFFFull;
  double v;
  memcpy(&v, &b, 8);
  return v;
}

// One thread: the target count and the band [lo, hi) of sorted positions
// whose device keys lie within a factor 1 -+ delta of the target-th key.
__global__ void sample_band(const uint64_t *sorted, const uint64_t *positive, uint64_t n,
                            double ratio, Band *out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const uint64_t np = *positive;
  const double want = ceil(double(n) * ratio);
  const uint64_t target = want < double(np) ? uint64_t(want) : np;
  Band b{target, np, 0, 0};
  if (target) {
    const double delta = 2.3283064365386963e-10;  // 2^-32
    const double key = key_value(sorted[target - 1]);
    double lo_v = key * (1 - delta), hi_v = key * (1 + delta);
    if (key < 1e-289) {  // tiny keys: relative bounds do not hold, recompute all below
      lo_v = 0;
      hi_v = hi_v > 1e-270 ? hi_v : 1e-270;
    }
    const uint64_t klo = orderable_key(lo_v), khi = orderable_key(hi_v);
    uint64_t a = 0, z = target - 1;  // first position in [0, target - 1] with key >= klo
    while (a < z) {
      const uint64_t m = (a + z) / 2;
      if (sorted[m] < klo) a = m + 1; else z = m;
    }
    b.lo = a;
    a = target, z = np;  // first position in [target, np] with key > khi
    while (a < z) {
      const uint64_t m = (a + z) / 2;
      if (sorted[m] <= khi) a = m + 1; else z = m;
    }
    b.hi = a;
  }
  *out = b;
}

__global__ void band_inputs(const int32_t *ids, uint64_t lo, uint64_t count, const double *w,
                            const uint64_t *rank, const uint64_t *draws, int32_t *out_id,
                            uint64_t *out_draw, double *out_w) {
  const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const int32_t v = ids[lo + i];
  out_id[i] = v;
  out_draw[i] = draws[rank[v]];
  out_w[i] = w[v];
}

__global__ void flag_ids(const int32_t *ids, uint64_t count, uint8_t *flags) {
  const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < count) flags[ids[i]] = 1;
}

}  // namespace

uint64_t sample_device(Call &call, const double *w, uint64_t n, double ratio, sym_rng &rng,
                       int32_t *out) {
  static_assert(sizeof(sym_rng) == (kWords + 1) * sizeof(uint64_t), "sym_rng layout");
  if (n > uint64_t(INT32_MAX)) fail(SYM_INVALID_ARGUMENT, "too many vertices for int32 sample ids");
  if (!(ratio >= 0)) fail(SYM_INVALID_ARGUMENT, "sample ratio must be a non-negative number");
  cudaStream_t st = call.stream();
  uint64_t *flags = call.alloc<uint64_t>(n), *rank = call.alloc<uint64_t>(n + 1);
  uint64_t *draws = call.alloc<uint64_t>(n), *state = call.alloc<uint64_t>(kWords + 1);
  uint64_t *keys = call.alloc<uint64_t>(n), *skeys = call.alloc<uint64_t>(n);
  int32_t *ids = call.alloc<int32_t>(n), *sids = call.alloc<int32_t>(n);
  Band *band = call.alloc<Band>(1);
  call.h2d(state, &rng, sizeof(sym_rng));
  if (n) {
    positive_flags<<<blocks_for(n), kThreads, 0, st>>>(w, n, flags);
    check_launch();
    call.launched();
  }
  exclusive_scan(call, flags, rank, n);
  mt_draws<<<1, kWords, 0, st>>>(state, rank + n, draws);
  check_launch();
  call.launched();
  if (n) {
    sample_keys<<<blocks_for(n), kThreads, 0, st>>>(w, n, rank, draws, keys, ids);
    check_launch();
    call.launched();
    radix_sort_pairs(call, keys, ids, skeys, sids, n, 64);
  }
  sample_band<<<1, 32, 0, st>>>(skeys, rank + n, n, ratio, band);
  check_launch();
  call.launched();
  Band b{};
  call.d2h(&b, band, sizeof(Band));
  call.d2h(&rng, state, sizeof(sym_rng));
  call.sync();
  if (!b.target) return 0;
  uint8_t *keep = call.alloc<uint8_t>(n);
  SYM_CUDA(cudaMemsetAsync(keep, 0, n, st));
  if (b.lo) {
    flag_ids<<<blocks_for(b.lo), kThreads, 0, st>>>(sids, b.lo, keep);
    check_launch();
    call.launched();
  }
  const uint64_t m = b.hi - b.lo, need = b.target - b.lo;
  if (m == 1) {  // the target-th key alone in its band: the device order is exact
    flag_ids<<<1, 32, 0, st>>>(sids + b.lo, 1, keep);
    check_launch();
    call.launched();
  } else {  // order the band with the host's std::log, ties by vertex id
    int32_t *bid = call.alloc<int32_t>(m);
    uint64_t *bdraw = call.alloc<uint64_t>(m);
    double *bw = call.alloc<double>(m);
    band_inputs<<<blocks_for(m), kThreads, 0, st>>>(sids, b.lo, m, w, rank, draws, bid, bdraw, bw);
    check_launch();
    call.launched();
    std::vector<int32_t> hid(m);
    std::vector<uint64_t> hdraw(m);
    std::vector<double> hw(m);
    call.d2h(hid.data(), bid, m * sizeof(int32_t));
    call.d2h(hdraw.data(), bdraw, m * sizeof(uint64_t));
    call.d2h(hw.data(), bw, m * sizeof(double));
    call.sync();
    std::vector<std::pair<double, int>> exact(m);
    for (uint64_t i = 0; i < m; ++i) {
      const double u = (static_cast<double>(hdraw[i] >> 11) + 0.5) / 9007199254740992.0;
      exact[i] = {-std::log(u) / hw[i], hid[i]};
    }
    std::sort(exact.begin(), exact.end());
    std::vector<int32_t> chosen(need);
    for (uint64_t i = 0; i < need; ++i) chosen[i] = exact[i].second;
    int32_t *dchosen = call.upload(chosen.data(), need);
    flag_ids<<<blocks_for(need), kThreads, 0, st>>>(dchosen, need, keep);
    check_launch();
    call.launched();
  }
  uint64_t *count = call.alloc<uint64_t>(1);
  compact_indices(call, keep, n, out, count);
  return b.target;
}

}  // namespace sym
