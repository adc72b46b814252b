// SPDX-License-Identifier: MPL-2.0
// Stage (b), first half: the area-weighted sample (on the device,
// sampling.cu), its anisotropy prune, and curvature pair voting candidates.
//
// Reference: src/cpu/selection.cpp:15-29, src/cpu/pairing.cpp:14-35 (CPU);
// src/cuda/backend.cu:21-31,128-339 (existing GPU path).
//
// Pairing on GB300:
//  1. gather the pruned samples (ordinal order) and radix-sort ordinals by
//     their kmin key;
//  2. rebuild the sample SoA in key order, so every source's candidate window
//     is one contiguous, coalesced range;
//  3. bound each source's window with a conservative kmin radius derived
//     from the acceptance test (|dk| <= t M implies M_b <= M_a / (1 - t'));
//  4. count accepted targets per source (one CTA per source), scan, check
//     the budget, then fill: a shared-memory bitmask over target ordinals
//     turns the key-ordered window back into the reference's nested-loop
//     order (source ordinal, then target ordinal) with no segmented sort.
// The acceptance test is the reference's FP64 expression, evaluated in the
// same order without FMA contraction, so the pair set is bit-exact.  An FP32
// form of the test runs first and decides every candidate whose values clear
// the thresholds by more than the FP32 rounding of its inputs can move them;
// the others take the FP64 test.
#include "common.cuh"
#include "primitives.cuh"
#include "sampling.cuh"

#include <algorithm>
#include <cmath>
#include <limits>

namespace sym {
namespace {

__global__ void prune_kernel(const int32_t *sample, uint64_t count, const double *kmin,
                             const double *kmax, const uint8_t *valid, double threshold,
                             uint8_t *flags) {
  uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= count) return;
  int32_t v = sample[i];
  double a = kmin[v], b = kmax[v];
  double maximum = fabs(a) < fabs(b) ? fabs(b) : fabs(a);
  flags[i] = valid[v] && maximum > 1e-10 && fabs(a - b) / maximum > threshold;
}

// Samples in ordinal order + validation + sort keys.
__global__ void gather_samples(const int32_t *selected, uint64_t s, const double *xyz,
                               uint64_t nv, const double *kmin, const double *kmax,
                               uint64_t *keys, int32_t *ordinals, int *status) {
  uint64_t a = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (a >= s) return;
  int32_t v = selected[a];
  ordinals[a] = int32_t(a);
  if (v < 0 || uint64_t(v) >= nv) {
    atomicExch(status, DS_INDEX_RANGE);
    keys[a] = 0;
    return;
  }
  double k0 = kmin[v], k1 = kmax[v];
  if (!isfinite(k0) || !isfinite(k1) || !isfinite(xyz[v]) || !isfinite(xyz[nv + v]) ||
      !isfinite(xyz[2 * nv + v]))
    atomicExch(status, DS_NONFINITE);
  keys[a] = orderable_key(k0);
}

struct SortedSamples {  // SoA in kmin-key order (FP64, and its FP32 rounding)
  int32_t *ordinal;
  double *kmin, *kmax, *x, *y, *z;
  float *kmin32, *kmax32, *x32, *y32, *z32;
};

__global__ void build_sorted(const int32_t *sorted_ord, const int32_t *selected, uint64_t s,
                             const double *xyz, uint64_t nv, const double *kmin,
                             const double *kmax, SortedSamples out) {
  uint64_t k = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= s) return;
  int32_t a = sorted_ord[k];
  int32_t v = selected[a];
  out.ordinal[k] = a;
  out.kmin[k] = kmin[v];
  out.kmax[k] = kmax[v];
  out.x[k] = xyz[v];
  out.y[k] = xyz[nv + v];
  out.z[k] = xyz[2 * nv + v];
  out.kmin32[k] = float(kmin[v]);
  out.kmax32[k] = float(kmax[v]);
  out.x32[k] = float(xyz[v]);
  out.y32[k] = float(xyz[nv + v]);
  out.z32[k] = float(xyz[2 * nv + v]);
}

__device__ uint64_t lower_bound_key(const uint64_t *keys, uint64_t n, uint64_t key, bool upper) {
  uint64_t first = 0;
  while (n) {
    uint64_t half = n / 2, mid = first + half;
    if (keys[mid] < key || (upper && keys[mid] == key)) {
      first = mid + 1;
      n -= half + 1;
    } else {
      n = half;
    }
  }
  return first;
}

// Per ordinal: the kmin-order window [lo, hi) holding every possible
// partner, and the kmax window as truncated keys [klo, khi] (orderable key
// >> 16, rounded outward): a partner b passes |kmin_a - kmin_b| <= t M and
// |kmax_a - kmax_b| <= t M with M <= m_a / (1 - t), m_a = max(|kmin_a|,
// |kmax_a|), so both differences are at most r = t m_a / (1 - t).
__global__ void windows(const int32_t *selected, uint64_t s, const double *kmin,
                        const double *kmax, const uint64_t *sorted_keys, double t,
                        uint64_t *lo, uint64_t *hi, uint64_t *klo, uint64_t *khi) {
  uint64_t a = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (a >= s) return;
  int32_t v = selected[a];
  double k0 = kmin[v], k1 = kmax[v];
  const double u = 1.1102230246251565e-16;  // 2^-53
  double ts = t * (1 + 8 * u) + 4 * u;       // t(1+u)/(1-u) rounded up, with slack
  uint64_t l = 0, h = s, kl = 0, kh = (uint64_t(1) << 48) - 1;
  if (ts < 1) {
    double m = fmax(fmax(fabs(k0), fabs(k1)), 1e-10);
    double r = ts * m / (1 - ts);
    r = r * (1 + 16 * u);
    double pad = 64 * u * (fabs(k0) + r);
    double low = k0 - r - pad, high = k0 + r + pad;
    l = lower_bound_key(sorted_keys, s, orderable_key(low), false);
    h = lower_bound_key(sorted_keys, s, orderable_key(high), true);
    const double pad1 = 64 * u * (fabs(k1) + r);
    kl = orderable_key(k1 - r - pad1) >> 16;
    kh = orderable_key(k1 + r + pad1) >> 16;
  }
  lo[a] = l;
  hi[a] = h;
  klo[a] = kl;
  khi[a] = kh;
}

// The kmin-sorted samples cut into `cells` runs of equal size (position p
// in cell p * cells / s), each run re-sorted by kmax: a source's partners
// lie in the cells its kmin window touches, and in each cell in the run of
// members whose kmax lies in its kmax window.  ckeys: (cell << 48) | the
// member's kmax key >> 16, in that order.
struct PairCells {
  const uint64_t *ckeys;
  uint64_t s, cells;
  __device__ uint64_t cell_of(uint64_t p) const { return p * cells / s; }
  __device__ uint64_t start(uint64_t c) const { return (c * s + cells - 1) / cells; }
};

__global__ void cell_keys(SortedSamples srt, uint64_t s, uint64_t cells, uint64_t *keys,
                          int32_t *pos) {
  const uint64_t p = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (p >= s) return;
  keys[p] = (p * cells / s) << 48 | orderable_key(srt.kmax[p]) >> 16;
  pos[p] = int32_t(p);
}

// out[k] = in[pos[k]] for every array of the sorted samples.
__global__ void gather_sorted(SortedSamples in, const int32_t *pos, uint64_t s, SortedSamples out) {
  const uint64_t k = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= s) return;
  const uint64_t p = uint64_t(pos[k]);
  out.ordinal[k] = in.ordinal[p];
  out.kmin[k] = in.kmin[p], out.kmax[k] = in.kmax[p];
  out.x[k] = in.x[p], out.y[k] = in.y[p], out.z[k] = in.z[p];
  out.kmin32[k] = in.kmin32[p], out.kmax32[k] = in.kmax32[p];
  out.x32[k] = in.x32[p], out.y32[k] = in.y32[p], out.z32[k] = in.z32[p];
}

// The first position in [b, e) whose key is >= target (upper: > target),
// or e; keys ascending.  The whole warp searches: 32 probes per step, so a
// run of n keys takes about log_33 n dependent loads.
__device__ uint64_t warp_bound(const uint64_t *keys, uint64_t b, uint64_t e, uint64_t target,
                               bool upper) {
  const unsigned lane = threadIdx.x & 31;
  auto before = [&](uint64_t p) { return upper ? keys[p] <= target : keys[p] < target; };
  while (e - b > 32) {  // the bound lies in [b, e]
    const uint64_t span = e - b;
    const unsigned m = __ballot_sync(0xffffffffu, before(b + (uint64_t(lane) + 1) * span / 33));
    const uint64_t n = __popc(m);  // probes before the bound: a prefix of the lanes
    const uint64_t nb = n ? b + n * span / 33 + 1 : b;
    const uint64_t ne = n < 32 ? b + (n + 1) * span / 33 : e;
    b = nb, e = ne;
  }
  const uint64_t p = b + lane;
  return b + __popc(__ballot_sync(0xffffffffu, p < e && before(p)));
}

constexpr int kMaxCells = 64;
constexpr uint64_t kCellSamples = 65536;  // samples from which the cells pay off

// The candidate runs of source a (in cell order): one per cell its kmin
// window touches, the members whose kmax key lies in [klo, khi]; without
// cells (pc.ckeys null: the samples stay in kmin order) the window itself.
// Every warp of the block searches cells in turn; rb/re are shared arrays
// of kMaxCells entries.  Returns the number of runs (the same in every
// thread).
__device__ int source_runs(const PairCells &pc, uint64_t lo, uint64_t hi, uint64_t klo,
                           uint64_t khi, uint64_t *rb, uint64_t *re) {
  if (hi <= lo) return 0;
  if (!pc.ckeys) {
    if (threadIdx.x == 0) rb[0] = lo, re[0] = hi;
    __syncthreads();
    return 1;
  }
  const uint64_t c0 = pc.cell_of(lo), c1 = pc.cell_of(hi - 1);
  const int n = int(c1 - c0 + 1);
  const int warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
  for (int i = warp; i < n; i += warps) {
    const uint64_t c = c0 + uint64_t(i), b = pc.start(c), e = pc.start(c + 1);
    const uint64_t from = warp_bound(pc.ckeys, b, e, c << 48 | klo, false);
    const uint64_t to = warp_bound(pc.ckeys, from, e, c << 48 | khi, true);
    if ((threadIdx.x & 31) == 0) rb[i] = from, re[i] = to;
  }
  __syncthreads();
  return n;
}

// The reference's acceptance test (pairing.cpp:22-28) for ordinals a < b.
__device__ __forceinline__ bool accept(double pa0, double pa1, D3 pp, double qb0, double qb1,
                                       D3 qp, double t, double min_dist) {
  double m = fmax(fmax(fmax(fmax(fabs(pa0), fabs(pa1)), fabs(qb0)), fabs(qb1)), 1e-10);
  double tol = t * m;
  if (fabs(pa0 - qb0) > tol || fabs(pa1 - qb1) > tol) return false;
  return !(norm(pp - qp) < min_dist);
}

// A source's values for the test, in FP64 and rounded to FP32.
struct Source {
  int32_t v;
  double k0, k1;
  D3 p;
  float k0f, k1f, xf, yf, zf;
};
__device__ __forceinline__ Source load_source(const int32_t *selected, uint64_t a, const double *xyz,
                                              uint64_t nv, const double *kmin, const double *kmax) {
  Source o;
  o.v = selected[a];
  o.k0 = kmin[o.v], o.k1 = kmax[o.v];
  o.p = {xyz[o.v], xyz[nv + o.v], xyz[2 * nv + o.v]};
  o.k0f = float(o.k0), o.k1f = float(o.k1);
  o.xf = float(o.p.x), o.yf = float(o.p.y), o.zf = float(o.p.z);
  return o;
}

// accept() for source src and the k-th sorted sample.  Rounding the inputs
// to FP32 moves each curvature by at most 2^-24 of itself, so |dk| and t M
// move by less than 5e-7 M with M >= max |k|; each coordinate moves by at
// most 2^-24 of the largest coordinate magnitude S of the two points, so the
// distance moves by at most 2.1e-7 S.  Outside those bands (widened further
// for the FP32 arithmetic) the FP32 decision is the FP64 one.
__device__ __forceinline__ bool accept_filtered(const Source &src, const SortedSamples &srt,
                                                uint64_t k, float tf, float min_dist_f, double t,
                                                double min_dist) {
  const float b0 = srt.kmin32[k], b1 = srt.kmax32[k];
  const float bx = srt.x32[k], by = srt.y32[k], bz = srt.z32[k];
  const float m = fmaxf(fmaxf(fmaxf(fmaxf(fabsf(src.k0f), fabsf(src.k1f)), fabsf(b0)), fabsf(b1)),
                        1e-10f);
  const float tol = tf * m, slack = 2e-6f * m;
  const float e0 = fabsf(src.k0f - b0), e1 = fabsf(src.k1f - b1);
  const float dx = src.xf - bx, dy = src.yf - by, dz = src.zf - bz;
  const float d = sqrtf(dx * dx + dy * dy + dz * dz);
  const float S = fmaxf(fmaxf(fmaxf(fabsf(src.xf), fabsf(src.yf)), fmaxf(fabsf(src.zf), fabsf(bx))),
                        fmaxf(fabsf(by), fabsf(bz)));
  const float dslack = 1e-6f * S + 1e-5f * min_dist_f;
  if (e0 > tol + slack || e1 > tol + slack || d < min_dist_f - dslack) return false;
  if (e0 < tol - slack && e1 < tol - slack && d > min_dist_f + dslack) return true;
  return accept(src.k0, src.k1, src.p, srt.kmin[k], srt.kmax[k], {srt.x[k], srt.y[k], srt.z[k]}, t,
                min_dist);
}

__device__ unsigned block_sum(unsigned v) {
  __shared__ unsigned warp_sum[32];
  for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = v;
  __syncthreads();
  unsigned total = 0;
  if (threadIdx.x < 32) {
    total = threadIdx.x < (blockDim.x >> 5) ? warp_sum[threadIdx.x] : 0;
    for (int o = 16; o; o >>= 1) total += __shfl_down_sync(0xffffffffu, total, o);
  }
  return total;  // valid in thread 0
}

// The pair kernels take one source per block and test its candidate runs
// (source_runs) in srt: the samples in cell order, or in kmin order when
// there are no cells.
struct Windows {
  const uint64_t *lo, *hi, *klo, *khi;
};

__global__ void count_pairs(const int32_t *selected, uint64_t s, const double *xyz, uint64_t nv,
                            const double *kmin, const double *kmax, SortedSamples srt,
                            PairCells pc, Windows win, double t, double min_dist,
                            uint64_t *counts) {
  __shared__ uint64_t rb[kMaxCells], re[kMaxCells];
  uint64_t a = blockIdx.x;
  const Source src = load_source(selected, a, xyz, nv, kmin, kmax);
  const float tf = float(t), mdf = float(min_dist);
  const int runs = source_runs(pc, win.lo[a], win.hi[a], win.klo[a], win.khi[a], rb, re);
  unsigned c = 0;
  for (int i = 0; i < runs; ++i)
    for (uint64_t k = rb[i] + threadIdx.x; k < re[i]; k += blockDim.x) {
      int32_t b = srt.ordinal[k];
      if (uint64_t(b) <= a) continue;
      c += accept_filtered(src, srt, k, tf, mdf, t, min_dist);
    }
  unsigned total = block_sum(c);
  if (threadIdx.x == 0) counts[a] = total;
}

constexpr int kFillThreads = 256;
constexpr int kChunkWords = 8192;  // 262,144 target ordinals per pass (32 KiB)

__global__ void fill_pairs(const int32_t *selected, uint64_t s, const double *xyz, uint64_t nv,
                           const double *kmin, const double *kmax, SortedSamples srt,
                           PairCells pc, Windows win, const uint64_t *offsets,
                           double t, double min_dist, int32_t *out_a, int32_t *out_b) {
  __shared__ unsigned bits[kChunkWords];
  __shared__ unsigned warp_tot[kFillThreads / 32];
  __shared__ uint64_t rb[kMaxCells], re[kMaxCells];
  uint64_t a = blockIdx.x;
  const Source src = load_source(selected, a, xyz, nv, kmin, kmax);
  const int32_t v = src.v;
  const float tf = float(t), mdf = float(min_dist);
  uint64_t out = offsets[a];
  const uint64_t end_out = offsets[a + 1];
  if (out == end_out) return;
  const int runs = source_runs(pc, win.lo[a], win.hi[a], win.klo[a], win.khi[a], rb, re);
  const uint64_t base = (a + 1) & ~uint64_t(31);
  const uint64_t chunk_bits = uint64_t(kChunkWords) * 32;
  for (uint64_t cb = base; cb < s; cb += chunk_bits) {
    uint64_t ce = min(s, cb + chunk_bits);
    unsigned words = unsigned((ce - cb + 31) / 32);
    for (unsigned w = threadIdx.x; w < words; w += blockDim.x) bits[w] = 0;
    __syncthreads();
    for (int i = 0; i < runs; ++i)
      for (uint64_t k = rb[i] + threadIdx.x; k < re[i]; k += blockDim.x) {
        int32_t b = srt.ordinal[k];
        if (uint64_t(b) <= a || uint64_t(b) < cb || uint64_t(b) >= ce) continue;
        if (accept_filtered(src, srt, k, tf, mdf, t, min_dist)) {
          uint64_t bit = uint64_t(b) - cb;
          atomicOr(&bits[bit >> 5], 1u << (bit & 31));
        }
      }
    __syncthreads();
    // Each thread owns a contiguous run of words; prefix of popcounts.
    unsigned per = (words + blockDim.x - 1) / blockDim.x;
    unsigned w0 = threadIdx.x * per, w1 = min(words, w0 + per);
    unsigned mine = 0;
    for (unsigned w = w0; w < w1; ++w) mine += __popc(bits[w]);
    unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned incl = mine;
    for (int o = 1; o < 32; o <<= 1) {
      unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= unsigned(o)) incl += y;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    unsigned before = 0, total = 0;
    for (unsigned w = 0; w < blockDim.x / 32; ++w) {
      if (w < warp) before += warp_tot[w];
      total += warp_tot[w];
    }
    uint64_t pos = out + before + incl - mine;
    for (unsigned w = w0; w < w1; ++w) {
      unsigned m = bits[w];
      while (m) {
        unsigned bit = __ffs(m) - 1;
        m &= m - 1;
        uint64_t b = cb + uint64_t(w) * 32 + bit;
        if (pos < end_out) {
          out_a[pos] = v;
          out_b[pos] = selected[b];
        }
        ++pos;
      }
    }
    out += total;
    __syncthreads();
  }
}

// Single-evaluation form, used while the accept bitmaps of all sources fit
// the kBitmapBudget: mark_pairs evaluates the acceptance test once per
// candidate, counts the accepted partners b > a of source a and stores the
// bitmap over b in [(a + 1) & ~31, s) at bitmap[a * stride ..]; fill_from_bits
// then writes the pairs in ascending b from those words, so the (FP64) test
// is not evaluated a second time.  Same pairs, same order as fill_pairs.
constexpr uint64_t kBitmapBudget = 256ull << 20;  // bytes

__global__ void mark_pairs(const int32_t *selected, uint64_t s, const double *xyz, uint64_t nv,
                           const double *kmin, const double *kmax, SortedSamples srt,
                           PairCells pc, Windows win, double t, double min_dist,
                           uint64_t stride, uint64_t *counts, unsigned *bitmap) {
  __shared__ unsigned bits[kChunkWords];
  __shared__ uint64_t rb[kMaxCells], re[kMaxCells];
  const uint64_t a = blockIdx.x;
  const Source src = load_source(selected, a, xyz, nv, kmin, kmax);
  const float tf = float(t), mdf = float(min_dist);
  const uint64_t base = (a + 1) & ~uint64_t(31);
  const unsigned words = unsigned((s - base + 31) / 32);  // <= stride <= kChunkWords
  for (unsigned w = threadIdx.x; w < words; w += blockDim.x) bits[w] = 0;
  const int runs = source_runs(pc, win.lo[a], win.hi[a], win.klo[a], win.khi[a], rb, re);
  for (int i = 0; i < runs; ++i)
    for (uint64_t k = rb[i] + threadIdx.x; k < re[i]; k += blockDim.x) {
      const int32_t b = srt.ordinal[k];
      if (uint64_t(b) <= a) continue;
      if (accept_filtered(src, srt, k, tf, mdf, t, min_dist)) {
        const uint64_t bit = uint64_t(b) - base;
        atomicOr(&bits[bit >> 5], 1u << (bit & 31));
      }
    }
  __syncthreads();
  unsigned c = 0;
  for (unsigned w = threadIdx.x; w < words; w += blockDim.x) {
    const unsigned m = bits[w];
    c += __popc(m);
    bitmap[a * stride + w] = m;
  }
  const unsigned total = block_sum(c);
  if (threadIdx.x == 0) counts[a] = total;
}

__global__ void fill_from_bits(const int32_t *selected, uint64_t s, const unsigned *bitmap,
                               uint64_t stride, const uint64_t *offsets, int32_t *out_a,
                               int32_t *out_b) {
  __shared__ unsigned warp_tot[kFillThreads / 32];
  const uint64_t a = blockIdx.x;
  const uint64_t out = offsets[a], end_out = offsets[a + 1];
  if (out == end_out) return;
  const int32_t v = selected[a];
  const uint64_t base = (a + 1) & ~uint64_t(31);
  const unsigned words = unsigned((s - base + 31) / 32);
  const unsigned *bits = bitmap + a * stride;
  // Each thread owns a contiguous run of words; prefix of popcounts.
  const unsigned per = (words + blockDim.x - 1) / blockDim.x;
  const unsigned w0 = min(words, threadIdx.x * per), w1 = min(words, w0 + per);
  unsigned mine = 0;
  for (unsigned w = w0; w < w1; ++w) mine += __popc(bits[w]);
  const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned incl = mine;
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= unsigned(o)) incl += y;
  }
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  unsigned before = 0;
  for (unsigned w = 0; w < warp; ++w) before += warp_tot[w];
  uint64_t pos = out + before + incl - mine;
  for (unsigned w = w0; w < w1; ++w) {
    unsigned m = bits[w];
    while (m) {
      const unsigned bit = __ffs(m) - 1;
      m &= m - 1;
      const uint64_t b = base + uint64_t(w) * 32 + bit;
      if (pos < end_out) {
        out_a[pos] = v;
        out_b[pos] = selected[b];
      }
      ++pos;
    }
  }
}

}  // namespace

void prune_device(Call &call, const int32_t *sample, uint64_t count, const double *kmin,
                  const double *kmax, const uint8_t *valid, double prune, int32_t *pruned,
                  uint64_t *pruned_count) {
  uint8_t *flags = call.alloc<uint8_t>(count);
  if (count) {
    prune_kernel<<<blocks_for(count), kThreads, 0, call.stream()>>>(sample, count, kmin, kmax,
                                                                     valid, 1 - prune, flags);
    check_launch();
    call.launched();
  }
  compact_values(call, flags, sample, count, pruned, pruned_count);
}

void select_device(Call &call, const sym_mesh_view &m, const sym_features_view &f,
                   const double *weights, uint64_t weight_count, const sym_options &o,
                   sym_rng *rng, std::vector<int32_t> &sample, std::vector<int32_t> &pruned) {
  if (weight_count != m.vertices.count || f.count != weight_count)
    fail(SYM_INVALID_ARGUMENT, "SoA component lengths differ");
  const uint64_t n = weight_count;
  double *w = call.upload(weights, n);
  int32_t *dsample = call.alloc<int32_t>(n);
  const uint64_t count = sample_device(call, w, n, o.sample_ratio, *rng, dsample);
  sample.resize(count);
  pruned.clear();
  if (!count) return;
  double *kmin = call.upload(f.kmin, n);
  double *kmax = call.upload(f.kmax, n);
  uint8_t *valid = call.upload(f.valid, n);
  int32_t *dpruned = call.alloc<int32_t>(count);
  uint64_t *dcount = call.alloc<uint64_t>(1);
  prune_device(call, dsample, count, kmin, kmax, valid, o.prune, dpruned, dcount);
  uint64_t kept = 0;
  call.d2h(sample.data(), dsample, count * 4);
  call.d2h(&kept, dcount, 8);
  call.sync();
  pruned.resize(kept);
  call.d2h(pruned.data(), dpruned, kept * 4);
  call.sync();
}

// Device-resident pairing.  `selected` (s ordinals), `xyz` (3 x nv),
// kmin/kmax (nv) are device pointers.  Returns the pair count; out_a/out_b
// are allocated from the workspace.
uint64_t pairing_device(Call &call, const int32_t *selected, uint64_t s, const double *xyz,
                        uint64_t nv, const double *kmin, const double *kmax, double t,
                        double box, uint64_t max_pairs, int32_t **out_a, int32_t **out_b) {
  cudaStream_t st = call.stream();
  *out_a = *out_b = nullptr;
  if (s < 2) return 0;
  uint64_t *keys = call.alloc<uint64_t>(s), *sorted_keys = call.alloc<uint64_t>(s);
  int32_t *ord = call.alloc<int32_t>(s), *sorted_ord = call.alloc<int32_t>(s);
  gather_samples<<<blocks_for(s), kThreads, 0, st>>>(selected, s, xyz, nv, kmin, kmax, keys, ord,
                                                     call.status());
  check_launch();
  call.check_status("pairing");
  radix_sort_pairs(call, keys, ord, sorted_keys, sorted_ord, s, 64);
  SortedSamples srt{call.alloc<int32_t>(s), call.alloc<double>(s), call.alloc<double>(s),
                    call.alloc<double>(s), call.alloc<double>(s), call.alloc<double>(s),
                    call.alloc<float>(s),  call.alloc<float>(s),  call.alloc<float>(s),
                    call.alloc<float>(s),  call.alloc<float>(s)};
  build_sorted<<<blocks_for(s), kThreads, 0, st>>>(sorted_ord, selected, s, xyz, nv, kmin, kmax, srt);
  check_launch();
  uint64_t *lo = call.alloc<uint64_t>(s), *hi = call.alloc<uint64_t>(s);
  uint64_t *klo = call.alloc<uint64_t>(s), *khi = call.alloc<uint64_t>(s);
  windows<<<blocks_for(s), kThreads, 0, st>>>(selected, s, kmin, kmax, sorted_keys, t, lo, hi, klo,
                                               khi);
  check_launch();
  // Large samples: the kmin order cut into kMaxCells cells, each re-sorted
  // by kmax (stable: a cell's members keep their kmin order among equal
  // keys), so a source tests only the members of its cells within its kmax
  // window.  Measured on a 200,000-sample torus (mean kmin window 9,800
  // samples, 4% of them within the kmax window): pairing 20.1 -> 6.2 ms;
  // on 20,000 samples the extra sort and searches cost more than they save
  // (0.7 -> 1.1 ms), so smaller samples keep the kmin windows alone.
  SortedSamples cs = srt;
  PairCells pc{nullptr, s, 1};
  if (s >= kCellSamples) {
    const uint64_t cells = kMaxCells;
    uint64_t *ckeys = call.alloc<uint64_t>(s), *sorted_ckeys = call.alloc<uint64_t>(s);
    int32_t *cpos = call.alloc<int32_t>(s), *sorted_cpos = call.alloc<int32_t>(s);
    cell_keys<<<blocks_for(s), kThreads, 0, st>>>(srt, s, cells, ckeys, cpos);
    check_launch();
    radix_sort_pairs(call, ckeys, cpos, sorted_ckeys, sorted_cpos, s, 64);
    cs = SortedSamples{call.alloc<int32_t>(s), call.alloc<double>(s), call.alloc<double>(s),
                       call.alloc<double>(s), call.alloc<double>(s), call.alloc<double>(s),
                       call.alloc<float>(s),  call.alloc<float>(s),  call.alloc<float>(s),
                       call.alloc<float>(s),  call.alloc<float>(s)};
    gather_sorted<<<blocks_for(s), kThreads, 0, st>>>(srt, sorted_cpos, s, cs);
    check_launch();
    call.launched(2);
    pc = PairCells{sorted_ckeys, s, cells};
  }
  const Windows win{lo, hi, klo, khi};
  uint64_t *counts = call.alloc<uint64_t>(s), *offsets = call.alloc<uint64_t>(s + 1);
  double min_dist = 0.03 * box;
  const uint64_t stride = (s + 31) / 32 + 1;  // words of one source's bitmap, at most
  const bool single = stride <= uint64_t(kChunkWords) && s * stride * 4 <= kBitmapBudget;
  unsigned *bitmap = single ? call.alloc<unsigned>(s * stride) : nullptr;
  if (single)
    mark_pairs<<<unsigned(s), kFillThreads, 0, st>>>(selected, s, xyz, nv, kmin, kmax, cs, pc, win,
                                                     t, min_dist, stride, counts, bitmap);
  else
    count_pairs<<<unsigned(s), kFillThreads, 0, st>>>(selected, s, xyz, nv, kmin, kmax, cs, pc,
                                                      win, t, min_dist, counts);
  check_launch();
  exclusive_scan(call, counts, offsets, s);
  call.launched(4);
  uint64_t total = 0;
  call.d2h(&total, offsets + s, 8);
  call.sync();
  if (total > max_pairs || total > uint64_t(std::numeric_limits<int32_t>::max()))
    fail(SYM_RUNTIME_ERROR, "Pair budget exceeded; lower --sample-ratio or tighten --pair-threshold");
  if (!total) return 0;
  *out_a = call.alloc<int32_t>(total);
  *out_b = call.alloc<int32_t>(total);
  if (single)
    fill_from_bits<<<unsigned(s), kFillThreads, 0, st>>>(selected, s, bitmap, stride, offsets,
                                                         *out_a, *out_b);
  else
    fill_pairs<<<unsigned(s), kFillThreads, 0, st>>>(selected, s, xyz, nv, kmin, kmax, cs, pc, win,
                                                     offsets, t, min_dist, *out_a, *out_b);
  check_launch();
  call.launched();
  return total;
}

void pairing_host(Call &call, const sym_mesh_view &m, const sym_features_view &f,
                  const int32_t *selected, uint64_t s, const sym_model_context &ctx,
                  const sym_options &o, std::vector<int32_t> &a, std::vector<int32_t> &b) {
  a.clear();
  b.clear();
  if (s < 2) return;
  if (f.count != m.vertices.count) fail(SYM_INVALID_ARGUMENT, "SoA component lengths differ");
  if (s > uint64_t(std::numeric_limits<int32_t>::max()))
    fail(SYM_OVERFLOW, "selected ordinals exceed int32 range");
  if (!(ctx.box_size > 0) || !std::isfinite(ctx.box_size) ||
      !(o.pair_threshold > 0 && o.pair_threshold <= 1))
    fail(SYM_INVALID_ARGUMENT,
         "pairing requires positive finite box size and threshold in (0,1]");
  uint64_t nv = m.vertices.count;
  double *xyz = upload_points(call, m.vertices);
  double *kmin = call.upload(f.kmin, nv);
  double *kmax = call.upload(f.kmax, nv);
  int32_t *sel = call.upload(selected, s);
  int32_t *da, *db;
  uint64_t total = pairing_device(call, sel, s, xyz, nv, kmin, kmax, o.pair_threshold,
                                  ctx.box_size, o.max_pairs, &da, &db);
  a.resize(total);
  b.resize(total);
  if (total) {
    call.d2h(a.data(), da, total * 4);
    call.d2h(b.data(), db, total * 4);
  }
  call.check_status("pairing");
}

}  // namespace sym
