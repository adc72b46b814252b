// SPDX-License-Identifier: MPL-2.0
// SIMT mean-shift (FP32 and FP64) over a Morton-chunked 6-D vote set.
#include "meanshift_fast.cuh"
#include "primitives.cuh"

#include <algorithm>
#include <cmath>

namespace sym {
namespace {

// ------------------------------------------------------------ vote sort
__global__ void box_partials(const float *desc, uint64_t q, float *partial) {
  __shared__ float lo[6][256], hi[6][256];
  float l[6], h[6];
  for (int k = 0; k < 6; ++k) l[k] = INFINITY, h[k] = -INFINITY;
  for (uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; v < q;
       v += uint64_t(gridDim.x) * blockDim.x)
    for (int k = 0; k < 6; ++k) {
      float x = desc[v * 8 + k];
      l[k] = fminf(l[k], x), h[k] = fmaxf(h[k], x);
    }
  for (int k = 0; k < 6; ++k) lo[k][threadIdx.x] = l[k], hi[k][threadIdx.x] = h[k];
  __syncthreads();
  for (int s = 128; s; s >>= 1) {
    if (threadIdx.x < s)
      for (int k = 0; k < 6; ++k) {
        lo[k][threadIdx.x] = fminf(lo[k][threadIdx.x], lo[k][threadIdx.x + s]);
        hi[k][threadIdx.x] = fmaxf(hi[k][threadIdx.x], hi[k][threadIdx.x + s]);
      }
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < 6; ++k)
      partial[blockIdx.x * 12 + k] = lo[k][0], partial[blockIdx.x * 12 + 6 + k] = hi[k][0];
}

__global__ void box_final(const float *partial, int n, float *box) {
  int k = threadIdx.x;
  if (k >= 12) return;
  float v = k < 6 ? INFINITY : -INFINITY;
  for (int i = 0; i < n; ++i) v = k < 6 ? fminf(v, partial[i * 12 + k]) : fmaxf(v, partial[i * 12 + k]);
  box[k] = v;
}

// Morton key of a 6-D point over `bits` bits per coordinate (cells of
// 1/2^bits of the box; at most 10).
__device__ __forceinline__ uint64_t morton6(const float *x, const float *box, int bits = 10) {
  uint64_t key = 0;
  const int cells = 1 << bits;
  for (int k = 0; k < 6; ++k) {
    float lo = box[k], span = box[6 + k] - lo;
    float t = span > 0 ? (x[k] - lo) / span : 0.f;
    uint64_t cell = uint64_t(min(cells - 1, max(0, int(t * float(cells)))));
    for (int b = 0; b < bits; ++b) key |= ((cell >> b) & 1ull) << (6 * b + k);
  }
  return key;
}

// Votes are ordered by `bits` bits per coordinate (8 by default: a cell of
// the vote space is then ~1/256 of its extent, well under the bandwidth on
// the benchmark workloads, and the 48-bit key sorts in six radix passes).
__global__ void morton_keys(const float *desc, uint64_t q, const float *box, int bits,
                            uint64_t *keys, int32_t *idx) {
  uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (v >= q) return;
  keys[v] = morton6(desc + v * 8, box, bits);
  idx[v] = int32_t(v);
}

// dst row v = src row order[v]; rows of 8 values (32 or 64 bytes, and the
// buffers 16-byte aligned), moved as 16-byte words.
template <typename T>
__global__ void permute(const T *src, const int32_t *order, uint64_t q, T *dst) {
  uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (v >= q) return;
  uint64_t from = uint64_t(uint32_t(order[v]));
  constexpr int kWords = 8 * sizeof(T) / 16;
  const uint4 *s = reinterpret_cast<const uint4 *>(src + from * 8);
  uint4 w[kWords];
  for (int k = 0; k < kWords; ++k) w[k] = s[k];
  uint4 *d = reinterpret_cast<uint4 *>(dst + v * 8);
  for (int k = 0; k < kWords; ++k) d[k] = w[k];
}

__global__ void invert(const int32_t *order, uint64_t q, int32_t *rank) {
  uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (v < q) rank[order[v]] = int32_t(v);
}

// One warp per chunk: the chunk's box [lo0..lo5, hi0..hi5] and the boxes
// of its runs of kSubVotes votes (a run past q gets an empty box, lo = +inf
// and hi = -inf).  Lane l holds vote 32 r + l in round r, so a run is a
// group of consecutive lanes of one round.
__global__ void chunk_boxes(const float *desc, uint64_t q, uint64_t nchunks, float *cbox,
                            float *sbox) {
  uint64_t c = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (c >= nchunks) return;
  float l[6], h[6];
  for (int k = 0; k < 6; ++k) l[k] = INFINITY, h[k] = -INFINITY;
  for (int r = 0; r < kChunk / 32; ++r) {
    const int j = 32 * r + lane;
    const uint64_t v = c * kChunk + j;
    const bool in = v < q;
    float a[6], b[6];
    for (int k = 0; k < 6; ++k) {
      const float x = in ? desc[v * 8 + k] : 0.f;
      a[k] = in ? x : INFINITY, b[k] = in ? x : -INFINITY;
    }
    for (int o = kSubVotes / 2; o; o >>= 1)
      for (int k = 0; k < 6; ++k) {
        a[k] = fminf(a[k], __shfl_xor_sync(0xffffffffu, a[k], o));
        b[k] = fmaxf(b[k], __shfl_xor_sync(0xffffffffu, b[k], o));
      }
    if (lane % kSubVotes == 0) {
      float *s = sbox + (c * kSubs + j / kSubVotes) * 12;
      for (int k = 0; k < 6; ++k) s[k] = a[k], s[6 + k] = b[k];
    }
    for (int k = 0; k < 6; ++k) l[k] = fminf(l[k], a[k]), h[k] = fmaxf(h[k], b[k]);
  }
  for (int o = 16; o >= kSubVotes; o >>= 1)
    for (int k = 0; k < 6; ++k) {
      l[k] = fminf(l[k], __shfl_xor_sync(0xffffffffu, l[k], o));
      h[k] = fmaxf(h[k], __shfl_xor_sync(0xffffffffu, h[k], o));
    }
  if (lane == 0)
    for (int k = 0; k < 6; ++k) cbox[c * 12 + k] = l[k], cbox[c * 12 + 6 + k] = h[k];
}

// One block per run of kBlockChunks chunks: the union of their boxes.
__global__ void __launch_bounds__(kBlockChunks) block_boxes(const float *cbox, uint64_t nchunks,
                                                            float *bbox) {
  __shared__ float part[kBlockChunks / 32][12];
  const uint64_t c = uint64_t(blockIdx.x) * kBlockChunks + threadIdx.x;
  const bool live = c < nchunks;
  float v[12];
  for (int k = 0; k < 12; ++k) v[k] = live ? cbox[c * 12 + k] : (k < 6 ? INFINITY : -INFINITY);
  for (int o = 16; o; o >>= 1)
    for (int k = 0; k < 12; ++k) {
      const float w = __shfl_xor_sync(0xffffffffu, v[k], o);
      v[k] = k < 6 ? fminf(v[k], w) : fmaxf(v[k], w);
    }
  if ((threadIdx.x & 31) == 0)
    for (int k = 0; k < 12; ++k) part[threadIdx.x >> 5][k] = v[k];
  __syncthreads();
  if (threadIdx.x < 12) {
    const int k = threadIdx.x;
    float r = part[0][k];
    for (int w = 1; w < kBlockChunks / 32; ++w) r = k < 6 ? fminf(r, part[w][k]) : fmaxf(r, part[w][k]);
    bbox[uint64_t(blockIdx.x) * 12 + k] = r;
  }
}

// ------------------------------------------------------------ mean shift
__device__ __forceinline__ float box_gap2(const float *a_lo, const float *a_hi, const float *b) {
  float g = 0;
  for (int k = 0; k < 6; ++k) {
    float d = fmaxf(fmaxf(b[k] - a_hi[k], a_lo[k] - b[6 + k]), 0.f);
    g += d * d;
  }
  return g;
}

// One block = one tile of up to kChunk active seeds (ids[tile*kChunk + t])
// x one split of the chunk range.  Each thread accumulates, for its seed,
// sum w x and sum w over the votes of the chunks its tile cannot skip, and
// for a kNear seed also the unweighted in-window sums of d = v - x and
// d d^T (the Jacobian of the Newton step).
// COUNT: count the votes within the bandwidth instead.
// NEWTON: some seed of the launch is kNear (the plain instance keeps its
// register footprint small).  The FP32 instances are held to 64 registers,
// eight CTAs per SM (measured: the polish 0.4 ms faster on the benchmark).
template <typename T, bool COUNT, bool NEWTON>
__global__ void __launch_bounds__(kChunk, sizeof(T) == 4 ? 8 : 1)
    ms_tile(const T *desc, const float *cbox, const float *bbox, const float *sbox,
            uint64_t nchunks, uint64_t q, const T *means, const uint8_t *state,
            const int32_t *ids, uint64_t nactive, T h2, T gk, float skip_gap2,
            uint64_t chunks_per_split, T *partial, unsigned long long *evals) {
  constexpr int stride = COUNT ? 8 : kPartial;
  constexpr bool kFine = NEWTON || COUNT;  // sub-box tests
  __shared__ T xs[kChunk * 8];
  __shared__ float sb[kFine ? kSubs * 12 : 1];
  __shared__ float tlo[6][4], thi[6][4];
  // NEWTON: the 27 unweighted in-window sums of each thread's seed, in
  // shared memory (in-window votes are rare; registers stay free)
  __shared__ T nsum[NEWTON ? 27 * kChunk : 1];
  uint64_t slot = uint64_t(blockIdx.x) * kChunk + threadIdx.x, split = blockIdx.y;
  uint64_t slots = uint64_t(gridDim.x) * kChunk;
  bool live = slot < nactive;
  int32_t seed = live ? ids[slot] : 0;
  const bool newton = NEWTON && !COUNT && live && is_near(state[seed]);
  T m[6];
  for (int d = 0; d < 6; ++d) m[d] = live ? means[uint64_t(seed) * 8 + d] : T(0);
  float lo[6], hi[6];
  for (int d = 0; d < 6; ++d) {
    lo[d] = live ? float(m[d]) : INFINITY;
    hi[d] = live ? float(m[d]) : -INFINITY;
  }
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int o = 16; o; o >>= 1)
    for (int d = 0; d < 6; ++d) {
      lo[d] = fminf(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
      hi[d] = fmaxf(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
    }
  if (lane == 0)
    for (int d = 0; d < 6; ++d) tlo[d][warp] = lo[d], thi[d][warp] = hi[d];
  __syncthreads();
  for (int d = 0; d < 6; ++d) {
    lo[d] = fminf(fminf(tlo[d][0], tlo[d][1]), fminf(tlo[d][2], tlo[d][3]));
    hi[d] = fmaxf(fmaxf(thi[d][0], thi[d][1]), fmaxf(thi[d][2], thi[d][3]));
  }
  T acc[7] = {0, 0, 0, 0, 0, 0, 0};
  if (NEWTON)
    for (int j = 0; j < 27; ++j) nsum[j * kChunk + threadIdx.x] = T(0);
  uint64_t c0 = split * chunks_per_split;
  uint64_t c1 = c0 + chunks_per_split < nchunks ? c0 + chunks_per_split : nchunks;
  unsigned long long done = 0;
  for (uint64_t c = c0; c < c1; ++c) {
    if (c == c0 || c % kBlockChunks == 0) {  // the block's box first (one test for the CTA)
      const uint64_t blk = c / kBlockChunks;
      if (box_gap2(lo, hi, bbox + blk * 12) > skip_gap2) {
        c = (blk + 1) * kBlockChunks - 1;
        continue;
      }
    }
    if (box_gap2(lo, hi, cbox + c * 12) > skip_gap2) continue;
    // skip the chunk unless some seed of the block lies within the bandwidth
    // of its box (exact for Epanechnikov weights)
    const float *cb = cbox + c * 12;
    float g = 0;
    for (int d = 0; d < 6; ++d) {
      const float x = float(m[d]);
      const float e = fmaxf(fmaxf(cb[d] - x, x - cb[6 + d]), 0.f);
      g += e * e;
    }
    if (!__syncthreads_or(live && g <= skip_gap2)) continue;
    uint64_t v = c * kChunk + threadIdx.x;
    for (int d = 0; d < 8; ++d) xs[threadIdx.x * 8 + d] = v < q ? desc[v * 8 + d] : T(1e30);
    if (kFine)
      for (int i = threadIdx.x; i < kSubs * 12; i += kChunk) sb[i] = sbox[c * kSubs * 12 + i];
    __syncthreads();
    uint64_t rest = q - c * kChunk;
    int n = rest < uint64_t(kChunk) ? int(rest) : kChunk;
    done += n;
    auto eval = [&](int j) {
      T e[6], d2 = 0;
#pragma unroll
      for (int d = 0; d < 6; ++d) {
        e[d] = xs[j * 8 + d] - m[d];
        d2 += e[d] * e[d];
      }
      if (d2 < h2) {
        if (COUNT) {
          acc[6] += T(1);
        } else {
          const T floor_w = gk > T(0) ? exp2(-gk) : T(0);
          const T w = gk > T(0) ? exp2(-gk * (d2 / h2)) - floor_w : T(1) - d2 / h2;
          // sums of w (v - x), not of w v: the step m - x comes out without
          // the cancellation of a mean of large coordinates (votes moved
          // to their own cell of vote space lie up to 14 from the origin)
#pragma unroll
          for (int d = 0; d < 6; ++d) acc[d] += w * e[d];
          acc[6] += w;
          if (newton) {  // Epanechnikov: unweighted sums; Gaussian: by 2^(-k d^2/h^2)
            const T wn = gk > T(0) ? w + floor_w : T(1);
            T *ns = nsum + threadIdx.x;
            int at = 6;
#pragma unroll
            for (int d = 0; d < 6; ++d) {
              const T we = wn * e[d];
              ns[d * kChunk] += we;
#pragma unroll
              for (int l = d; l < 6; ++l, ++at) ns[at * kChunk] += we * e[l];
            }
          }
        }
      }
    };
    if (kFine) {
      // the polish (NEWTON) and the support count (COUNT) also skip per
      // warp, by runs of kSubVotes votes: a run none of the warp's 32 seeds
      // lies within the bandwidth of would only add zeros.  The approach
      // instance keeps the tile granularity of the tensor kernel (one
      // 128-seed tile per chunk), so the two forms of the approach make the
      // same seed-vote evaluations.
      if (!__any_sync(0xffffffffu, live && g <= skip_gap2)) continue;
#pragma unroll 1
      for (int r = 0; r < kSubs && r * kSubVotes < n; ++r) {
        const float *b = sb + r * 12;
        float gr = 0;
        for (int d = 0; d < 6; ++d) {
          const float x = float(m[d]);
          const float e = fmaxf(fmaxf(b[d] - x, x - b[6 + d]), 0.f);
          gr += e * e;
        }
        if (!__any_sync(0xffffffffu, live && gr <= skip_gap2)) continue;
        const int j1 = min(n, (r + 1) * kSubVotes);
        for (int j = r * kSubVotes; j < j1; ++j) eval(j);
      }
    } else {
      for (int j = 0; j < n; ++j) eval(j);
    }
  }
  // split-major layout: value d of slot s of split p at (p * stride + d) *
  // slots + s, so the reduction reads consecutive seeds contiguously
  T *out = partial + split * stride * slots + slot;
  for (int d = 0; d < 7; ++d) out[d * slots] = acc[d];
  if (newton)
    for (int j = 0; j < 27; ++j) out[(8 + j) * slots] = nsum[j * kChunk + threadIdx.x];
  if (threadIdx.x == 0 && done && evals) atomicAdd(evals, done * (unsigned long long)kChunk);
}

// b <- M^-1 b by Gaussian elimination with partial pivoting; false when a
// pivot is below `tiny` (singular system).
template <typename T>
__device__ bool solve6(T (&M)[6][6], T (&b)[6], T tiny) {
  for (int c = 0; c < 6; ++c) {
    int piv = c;
    T best = fabs(M[c][c]);
    for (int r = c + 1; r < 6; ++r)
      if (fabs(M[r][c]) > best) best = fabs(M[r][c]), piv = r;
    if (!(best > tiny)) return false;
    if (piv != c) {
      for (int j = 0; j < 6; ++j) {
        T t = M[c][j];
        M[c][j] = M[piv][j], M[piv][j] = t;
      }
      T t = b[c];
      b[c] = b[piv], b[piv] = t;
    }
    for (int r = c + 1; r < 6; ++r) {
      T f = M[r][c] / M[c][c];
      for (int j = c; j < 6; ++j) M[r][j] -= f * M[c][j];
      b[r] -= f * b[c];
    }
  }
  for (int c = 5; c >= 0; --c) {
    T s = b[c];
    for (int j = c + 1; j < 6; ++j) s -= M[c][j] * b[j];
    b[c] = s / M[c][c];
  }
  return true;
}

// One step of a seed from its summed values (ms_reduce): the
// mean-shift step m - x for a kMoving seed, the safeguarded Newton step
// (I - J)^-1 (m - x) for a kNear seed, where for Epanechnikov weights
//   J = dm/dx = 2 / (h^2 sum w) * (sum d d^T - (m - x) (sum d)^T),
// d = v - x over the votes within the bandwidth, and for the shifted
// Gaussian w = g - 2^-k, g = 2^(-k d^2 / h^2) (dw/dx = 2 k ln2 g d / h^2)
//   J = 2 k ln2 / (h^2 sum w) * (sum g d d^T - (m - x) (sum g d)^T).  Stopping rules: exhausted
// when the weight is <= 1e-14 (reference, src/cpu/clustering.cpp:169-181),
// converged when a Newton step^2 < kNewtonStop2 h^2, settled (plain step
// taken) when the Newton step is rejected, or when an accepted Newton step
// is still too long at polish iteration kNewtonCap (polish_it, -1 in the
// approach phase).

// Sum of the splits of one value of a tile's seeds: block (tile, j, g) adds
// value d = j (j < 7) or j + 1 (the Newton sums) over split group g (splits
// g, g + kGroups, ...), one thread per seed slot, so each split's row of 128
// values is read contiguously.  red[(g * kPartial + d) * slots + slot] = the
// group's sum; ms_update adds the groups in order.
constexpr int kGroups = 8;
template <typename T>
__global__ void __launch_bounds__(kChunk) ms_reduce(const T *partial, uint64_t splits, uint64_t slots,
                                                    uint64_t nactive, T *red) {
  const uint64_t slot = uint64_t(blockIdx.x) * kChunk + threadIdx.x;
  if (slot >= nactive) return;
  const int d = blockIdx.y < 7 ? int(blockIdx.y) : int(blockIdx.y) + 1;
  const uint64_t g = blockIdx.z;
  const T *in = partial + uint64_t(d) * slots + slot;
  const uint64_t step = uint64_t(kPartial) * slots;
  T s0 = 0, s1 = 0;  // two interleaved sums, added in a fixed order
  uint64_t p = g;
  for (; p + kGroups < splits; p += 2 * kGroups) s0 += in[p * step], s1 += in[(p + kGroups) * step];
  if (p < splits) s0 += in[p * step];
  red[(g * kPartial + d) * slots + slot] = s0 + s1;
}

// One thread per seed: the step from the summed values (ms_reduce).
template <typename T>
__global__ void __launch_bounds__(kChunk) ms_update(T *means, const T *red, uint64_t slots,
                                                    const int32_t *ids, uint64_t nactive, T h2,
                                                    T gk, int polish_it, uint8_t *state) {
  const uint64_t slot = uint64_t(blockIdx.x) * kChunk + threadIdx.x;
  if (slot >= nactive) return;
  const int32_t s = ids[slot];
  const uint8_t st_s = state[s];
  const bool near = is_near(st_s);
  T acc[7] = {0, 0, 0, 0, 0, 0, 0}, ns[27];
  for (int g = 0; g < kGroups; ++g)
    for (int d = 0; d < 7; ++d) acc[d] += red[(uint64_t(g) * kPartial + d) * slots + slot];
  if (near)
    for (int j = 0; j < 27; ++j) {
      ns[j] = 0;
      for (int g = 0; g < kGroups; ++g) ns[j] += red[(uint64_t(g) * kPartial + 8 + j) * slots + slot];
    }
  if (acc[6] <= T(1e-14)) {
    state[s] = kExhausted;
    return;
  }
  T x[6], delta[6], move = 0;
  for (int d = 0; d < 6; ++d) {
    x[d] = means[uint64_t(s) * 8 + d];
    delta[d] = acc[d] / acc[6];  // m - x from the sums of w (v - x)
    move += delta[d] * delta[d];
  }
  if (!near) {
    for (int d = 0; d < 6; ++d) means[uint64_t(s) * 8 + d] = x[d] + delta[d];
    if (move < T(kSwitch2) * h2) state[s] = kNear;
    return;
  }
  const T *sd = ns, *sdd = ns + 6;
  T M[6][6], step[6];
  const T g = (gk > T(0) ? T(2) * gk * T(0.69314718055994531) : T(2)) / (h2 * acc[6]);
  for (int d = 0, at = 0; d < 6; ++d)
    for (int l = d; l < 6; ++l, ++at) M[d][l] = M[l][d] = sdd[at];
  for (int d = 0; d < 6; ++d) {
    for (int l = 0; l < 6; ++l) M[d][l] = (d == l ? T(1) : T(0)) - g * (M[d][l] - delta[d] * sd[l]);
    step[d] = delta[d];
  }
  bool ok = solve6(M, step, T(sizeof(T) == 4 ? 1e-6 : 1e-12));
  T len = 0, along = 0;
  for (int d = 0; d < 6; ++d) len += step[d] * step[d], along += step[d] * delta[d];
  ok = ok && isfinite(len) && len <= T(kTrust * kTrust) * h2 &&
       (along > T(0) || len < T(kNewtonStop2) * h2);
  if (ok) {
    for (int d = 0; d < 6; ++d) means[uint64_t(s) * 8 + d] = x[d] + step[d];
    if (len < T(kNewtonStop2) * h2) state[s] = kConverged;
    else if (polish_it >= kNewtonCap) state[s] = kSettled;
  } else {  // rejected: the plain step, and Newton once more (settled at the second rejection)
    for (int d = 0; d < 6; ++d) means[uint64_t(s) * 8 + d] = x[d] + delta[d];
    state[s] = polish_it < kNewtonCap && st_s == kNear ? kNearRetry1 : kSettled;
  }
}

constexpr int kRetile = 2048;  // seeds sorted in one block (static shared memory)

__device__ __forceinline__ bool pair_less(unsigned long long ka, int32_t va, unsigned long long kb,
                                          int32_t vb) {
  return ka < kb || (ka == kb && va < vb);
}

// Sorts the n (<= kRetile) pairs keys[0..n), vals[0..n) of shared memory by
// (key, value) and writes the values in that order to out[0..n); one block
// of kRetile / 2 threads.  A bitonic network over the next power of two (at
// least 64; padding pairs (~0, INT32_MAX) sort last): thread t holds
// elements 2t and 2t + 1 in registers, so the stride-1 steps stay in the
// thread, strides 2-32 are shuffles within a warp, and only the strides of
// 64 and more go through the shared arrays.  The pairs are distinct (the
// values are seed ids), so the order is the sorted order whatever the
// network.
__device__ void sort_pairs(unsigned long long *keys, int32_t *vals, unsigned n, int32_t *out) {
  unsigned p2 = 64;
  while (p2 < n) p2 <<= 1;
  const unsigned t = threadIdx.x;
  const bool on = t < p2 / 2;  // whole warps: p2 / 2 is a multiple of 32
  unsigned long long k[2];
  int32_t v[2];
  for (int j = 0; j < 2; ++j) {
    const unsigned i = 2 * t + j;
    k[j] = on && i < n ? keys[i] : ~0ull;
    v[j] = on && i < n ? vals[i] : 0x7fffffff;
  }
  __syncthreads();  // every pair read before the shared steps write
  // element i keeps the smaller of (i, i ^ s) when it is the lower index of
  // an ascending pair or the upper index of a descending one
  auto step = [&](int j, unsigned size, unsigned s, unsigned long long pk, int32_t pv) {
    const unsigned i = 2 * t + j;
    const bool keep_min = ((i & s) == 0) == ((i & size) == 0);
    if (pair_less(pk, pv, k[j], v[j]) == keep_min) k[j] = pk, v[j] = pv;
  };
  for (unsigned size = 2; size <= p2; size <<= 1)
    for (unsigned s = size >> 1; s; s >>= 1) {
      if (s >= 64) {
        if (on)
          for (int j = 0; j < 2; ++j) keys[2 * t + j] = k[j], vals[2 * t + j] = v[j];
        __syncthreads();
        if (on)
          for (int j = 0; j < 2; ++j) {
            const unsigned p = (2 * t + j) ^ s;
            step(j, size, s, keys[p], vals[p]);
          }
        __syncthreads();
      } else if (on && s == 1) {
        const bool up = ((2 * t) & size) == 0;
        if (pair_less(k[1], v[1], k[0], v[0]) == up) {
          const unsigned long long tk = k[0];
          const int32_t tv = v[0];
          k[0] = k[1], v[0] = v[1], k[1] = tk, v[1] = tv;
        }
      } else if (on) {  // partner thread t ^ (s / 2), in the same warp
        for (int j = 0; j < 2; ++j) {
          const unsigned long long pk = __shfl_xor_sync(0xffffffffu, k[j], s >> 1);
          const int32_t pv = __shfl_xor_sync(0xffffffffu, v[j], s >> 1);
          step(j, size, s, pk, pv);
        }
      }
    }
  if (on)
    for (int j = 0; j < 2; ++j)
      if (2 * t + j < n) out[2 * t + j] = v[j];
}

// Active seeds (kMoving, and kNear when include_near) in seed order, then
// sorted by the Morton key of
// their current mean (ties by seed id) when k <= kRetile.  nactive[0] = the
// number of active seeds, nactive[1] = how many of them are kNear.  With
// `iter`, an iteration that finds active seeds records their number in
// trace[*iter] (while *iter < trace_cap) and counts itself in *iter.
template <typename T>
__global__ void __launch_bounds__(1024) retile(const T *means, const uint8_t *state, uint64_t k,
                                               const float *box, bool include_near, int32_t *ids,
                                               unsigned *nactive, unsigned *iter = nullptr,
                                               uint32_t *trace = nullptr, unsigned trace_cap = 0) {
  __shared__ unsigned long long keys[kRetile];
  __shared__ int32_t vals[kRetile];
  __shared__ unsigned warp_tot[32];
  __shared__ unsigned base_s, near_s;
  if (threadIdx.x == 0) base_s = 0, near_s = 0;
  __syncthreads();
  bool sort = k <= kRetile;
  for (uint64_t at = 0; at < k; at += blockDim.x) {
    uint64_t s = at + threadIdx.x;
    bool act = s < k && (state[s] == kMoving || (include_near && is_near(state[s])));
    unsigned bal = __ballot_sync(0xffffffffu, act);
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) warp_tot[warp] = __popc(bal);
    __syncthreads();
    unsigned before = 0, total = 0;
    for (int w = 0; w < int(blockDim.x >> 5); ++w) {
      if (w < warp) before += warp_tot[w];
      total += warp_tot[w];
    }
    unsigned pos = base_s + before + __popc(bal & ((1u << lane) - 1));
    if (act && is_near(state[s])) atomicAdd(&near_s, 1u);
    if (act) {
      if (sort) {
        float x[6];
        for (int d = 0; d < 6; ++d) x[d] = float(means[s * 8 + d]);
        keys[pos] = morton6(x, box);
        vals[pos] = int32_t(s);
      } else {
        ids[pos] = int32_t(s);
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) base_s += total;
    __syncthreads();
  }
  unsigned n = base_s;
  if (sort) sort_pairs(keys, vals, n, ids);
  __syncthreads();
  if (threadIdx.x == 0) {
    nactive[0] = n, nactive[1] = near_s;
    if (iter && n) {
      if (*iter < trace_cap) trace[*iter] = n;
      ++*iter;
    }
  }
}

template <typename T>
__global__ void gather_seeds(const T *desc, const int64_t *pos, uint64_t k, T *means) {
  uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= k) return;
  for (int d = 0; d < 8; ++d) means[i * 8 + d] = desc[uint64_t(pos[i]) * 8 + d];
}

__global__ void sum_counts(const float *partial, uint64_t splits, uint64_t slots, const int32_t *ids,
                           uint64_t n, unsigned long long *counts) {
  uint64_t slot = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (slot >= n) return;
  unsigned long long c = 0;
  for (uint64_t p = 0; p < splits; ++p) c += (unsigned long long)partial[(p * 8 + 6) * slots + slot];
  counts[ids[slot]] = c;
}

struct Grid {
  uint64_t tiles, splits, cps, slots;
};

Grid grid_for(uint64_t nactive, uint64_t nchunks, int blocks_per_sm) {
  Grid g;
  g.tiles = (nactive + kChunk - 1) / kChunk;
  uint64_t want = (uint64_t(blocks_per_sm) * 152 + g.tiles - 1) / g.tiles;
  g.splits = std::max<uint64_t>(1, std::min<uint64_t>(nchunks, want));
  g.cps = (nchunks + g.splits - 1) / g.splits;
  g.splits = (nchunks + g.cps - 1) / g.cps;
  g.slots = g.tiles * kChunk;
  return g;
}

template <typename T>
int shift_impl(Call &call, const VoteSet &v, const T *desc, T *means, uint8_t *state, uint64_t k,
               double h2, int max_iter, bool polish, double *seed_iterations,
               unsigned long long *evals, uint32_t *trace = nullptr, int trace_len = 0) {
  cudaStream_t st = call.stream();
  int32_t *ids = call.alloc<int32_t>(k);
  unsigned *nact = call.alloc<unsigned>(2);
  // partial capacity: splits x slots is at most ~blocks*152*kChunk (+ one tile)
  const int bps = v.tuning.simt_blocks_per_sm;
  uint64_t cap = (uint64_t(bps) * 152 + 2) * uint64_t(kChunk) + std::max<uint64_t>(k, kChunk) * 2;
  T *partial = call.alloc<T>(cap * kPartial);
  T *red = call.alloc<T>(uint64_t(kGroups) * kPartial * std::max<uint64_t>(k, kChunk) * 2);
  float gap = float(std::sqrt(h2)) + 1e-6f;
  int it = 0;
  for (; it < max_iter; ++it) {
    retile<T><<<1, 1024, 0, st>>>(means, state, k, v.gbox, polish, ids, nact);
    check_launch();
    unsigned counts[2] = {0, 0};
    SYM_CUDA(cudaMemcpyAsync(counts, nact, 2 * sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    call.sync();
    call.launched();
    const unsigned n = counts[0];
    if (!n) break;
    if (seed_iterations) *seed_iterations += n;
    if (trace && it < trace_len) trace[it] = n;
    Grid g = grid_for(n, v.nchunks, bps);
    if (g.splits * g.slots > cap) fail(SYM_RUNTIME_ERROR, "mean-shift partial buffer too small");
    const dim3 grid(unsigned(g.tiles), unsigned(g.splits));
    if (counts[1])
      ms_tile<T, false, true><<<grid, kChunk, 0, st>>>(desc, v.cbox, v.bbox, v.sbox, v.nchunks, v.q, means, state, ids,
                                                      n, T(h2), T(v.kernel_k), gap * gap, g.cps,
                                                      partial, evals);
    else
      ms_tile<T, false, false><<<grid, kChunk, 0, st>>>(desc, v.cbox, v.bbox, v.sbox, v.nchunks, v.q, means, state,
                                                       ids, n, T(h2), T(v.kernel_k), gap * gap,
                                                       g.cps, partial, evals);
    check_launch();
    ms_reduce<T><<<dim3(unsigned(g.tiles), counts[1] ? 34u : 7u, kGroups), kChunk, 0, st>>>(
        partial, g.splits, g.slots, n, red);
    check_launch();
    ms_update<T><<<unsigned(g.tiles), kChunk, 0, st>>>(means, red, g.slots, ids, n, T(h2),
                                                       T(v.kernel_k), polish ? it : -1, state);
    check_launch();
    call.launched(3);
  }
  return it;
}

}  // namespace

VoteSet build_vote_set(Call &call, const float *desc_raw, const double *desc64_raw, uint64_t q,
                       const Tuning &tuning) {
  cudaStream_t st = call.stream();
  if (tuning.vote_bits < 1 || tuning.vote_bits > 10 || tuning.simt_blocks_per_sm < 1 ||
      tuning.simt_blocks_per_sm > 256 || tuning.tc_ctas_per_sm < 1 || tuning.tc_ctas_per_sm > 8 ||
      tuning.check_interval < 1)
    fail(SYM_INVALID_ARGUMENT, "tuning parameter out of range");
  VoteSet v;
  v.tuning = tuning;
  v.q = q;
  v.nchunks = (q + kChunk - 1) / kChunk;
  const int kBoxBlocks = 256;
  float *bpart = call.alloc<float>(kBoxBlocks * 12);
  v.gbox = call.alloc<float>(12);
  box_partials<<<kBoxBlocks, 256, 0, st>>>(desc_raw, q, bpart);
  check_launch();
  box_final<<<1, 32, 0, st>>>(bpart, kBoxBlocks, v.gbox);
  check_launch();
  uint64_t *keys = call.alloc<uint64_t>(q), *skeys = call.alloc<uint64_t>(q);
  int32_t *idx = call.alloc<int32_t>(q);
  v.order = call.alloc<int32_t>(q);
  v.rank = call.alloc<int32_t>(q);
  morton_keys<<<blocks_for(q), kThreads, 0, st>>>(desc_raw, q, v.gbox, tuning.vote_bits, keys, idx);
  check_launch();
  radix_sort_pairs(call, keys, idx, skeys, v.order, q, 6 * tuning.vote_bits);
  invert<<<blocks_for(q), kThreads, 0, st>>>(v.order, q, v.rank);
  check_launch();
  v.desc = call.alloc<float>(q * 8);
  permute<float><<<blocks_for(q), kThreads, 0, st>>>(desc_raw, v.order, q, v.desc);
  check_launch();
  if (desc64_raw) {
    v.desc64 = call.alloc<double>(q * 8);
    permute<double><<<blocks_for(q), kThreads, 0, st>>>(desc64_raw, v.order, q, v.desc64);
    check_launch();
  }
  v.cbox = call.alloc<float>(v.nchunks * 12);
  v.sbox = call.alloc<float>(v.nchunks * kSubs * 12);
  chunk_boxes<<<blocks_for(v.nchunks * 32), kThreads, 0, st>>>(v.desc, q, v.nchunks, v.cbox,
                                                                v.sbox);
  check_launch();
  v.nblocks = (v.nchunks + kBlockChunks - 1) / kBlockChunks;
  v.bbox = call.alloc<float>(v.nblocks * 12);
  if (v.nblocks) {
    block_boxes<<<unsigned(v.nblocks), kBlockChunks, 0, st>>>(v.cbox, v.nchunks, v.bbox);
    check_launch();
  }
  call.launched(desc64_raw ? 9 : 8);
  return v;
}

void init_means(Call &call, const VoteSet &v, const int64_t *seed_rank, uint64_t k, float *means) {
  gather_seeds<float><<<blocks_for(k), kThreads, 0, call.stream()>>>(v.desc, seed_rank, k, means);
  check_launch();
  call.launched();
}

void init_means(Call &call, const VoteSet &v, const int64_t *seed_rank, uint64_t k, double *means) {
  gather_seeds<double><<<blocks_for(k), kThreads, 0, call.stream()>>>(v.desc64, seed_rank, k, means);
  check_launch();
  call.launched();
}

int shift(Call &call, const VoteSet &v, float *means, uint8_t *state, uint64_t k, double h2,
          int max_iter, bool polish, double *seed_iterations, unsigned long long *evals,
          uint32_t *trace, int trace_len) {
  return shift_impl<float>(call, v, v.desc, means, state, k, h2, max_iter, polish, seed_iterations,
                           evals, trace, trace_len);
}

int shift(Call &call, const VoteSet &v, double *means, uint8_t *state, uint64_t k, double h2,
          int max_iter, bool polish, double *seed_iterations, unsigned long long *evals) {
  return shift_impl<double>(call, v, v.desc64, means, state, k, h2, max_iter, polish,
                            seed_iterations, evals);
}

void active_seeds_async(Call &call, const VoteSet &v, const float *means, const uint8_t *state,
                        uint64_t k, int32_t *ids, unsigned *nact, unsigned *iter, uint32_t *trace,
                        unsigned trace_cap) {
  retile<float><<<1, 1024, 0, call.stream()>>>(means, state, k, v.gbox, false, ids, nact, iter,
                                               trace, trace_cap);
  check_launch();
  call.launched();
}

void count_within(Call &call, const VoteSet &v, const float *points, uint64_t nm, double h2,
                  unsigned long long *counts) {
  if (!nm) return;
  cudaStream_t st = call.stream();
  uint8_t *state = call.alloc<uint8_t>(nm);
  SYM_CUDA(cudaMemsetAsync(state, 0, nm, st));
  int32_t *ids = call.alloc<int32_t>(nm);
  unsigned *nact = call.alloc<unsigned>(2);
  retile<float><<<1, 1024, 0, st>>>(points, state, nm, v.gbox, false, ids, nact);
  check_launch();
  Grid g = grid_for(nm, v.nchunks, v.tuning.simt_blocks_per_sm);
  float *partial = call.alloc<float>(g.splits * g.slots * 8);
  float gap = float(std::sqrt(h2)) + 1e-6f;
  ms_tile<float, true, false><<<dim3(unsigned(g.tiles), unsigned(g.splits)), kChunk, 0, st>>>(
      v.desc, v.cbox, v.bbox, v.sbox, v.nchunks, v.q, points, nullptr, ids, nm, float(h2), 0.f, gap * gap, g.cps,
      partial, nullptr);
  check_launch();
  sum_counts<<<blocks_for(nm), kThreads, 0, st>>>(partial, g.splits, g.slots, ids, nm, counts);
  check_launch();
  call.launched(3);
}

}  // namespace sym
