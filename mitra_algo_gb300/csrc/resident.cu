// SPDX-License-Identifier: MPL-2.0
// Throughput pipeline on a device-resident mesh (no reference counterpart:
// the reference runs one mesh per detect() and re-uploads every stage).
//
// Stages, all on the context stream with device-resident intermediates:
//   curvature (exact kernels of curvature.cu) -> prune of the host sample
//   -> exact pairing (pairing.cu) -> 6-D rigid votes (FP32 transform, FP64
//   log map near pi) -> Morton sort of the votes into 128-vote chunks with
//   bounding boxes -> mean-shift from K seeds (block-sparse: a seed tile
//   skips every chunk whose box lies farther than the bandwidth from the
//   tile's box; Epanechnikov weights need nothing beyond it) -> greedy mode
//   merge (h^2/4 as the reference) and support counts -> verification of
//   the top modes (verification.cu).
// Precision: FP32 SIMT or BF16 tensor-core bulk (meanshift_tc.cu) polished
// in FP32; a subset of seeds re-runs in FP64 to measure the mode error.
#include "common.cuh"
#include "primitives.cuh"
#include "rng.hpp"

#include <algorithm>
#include <cmath>
#include <limits>
#include <vector>

namespace sym {
void curvature_device(Call &, const double *, uint64_t, const double *, uint64_t, const double *,
                      const uint64_t *, const int32_t *, uint64_t, const sym_edge *, uint64_t, int,
                      const sym_features_out &, const sym_edge *);
void prune_device(Call &, const int32_t *, uint64_t, const double *, const double *,
                  const uint8_t *, double, int32_t *, uint64_t *);
uint64_t pairing_device(Call &, const int32_t *, uint64_t, const double *, uint64_t, const double *,
                        const double *, double, double, uint64_t, int32_t **, int32_t **);
void verification_core(Call &, const sym_mesh_view &, const double *, const int32_t *,
                       const double *, const double *, const uint64_t *, const int32_t *,
                       const sym_cluster_record *, uint64_t, double,
                       std::vector<std::vector<int32_t>> &,
                       std::vector<std::vector<std::vector<int32_t>>> &, std::vector<double> &,
                       std::vector<double> &);
// BF16 tensor-core bulk iterations (meanshift_tc.cu); returns false when the
// tensor path cannot run this problem (the caller then stays in FP32).
bool meanshift_bf16_bulk(Call &call, const float *desc, const float *cbox, uint64_t nchunks,
                         uint64_t q, float *means, uint8_t *state, uint64_t k, float h2,
                         int max_iter, int *iterations, double *evaluations);
}  // namespace sym

struct sym_mesh_handle {
  sym_context *ctx = nullptr;
  sym_mesh_view host{};
  std::vector<sym_edge> host_edges;
  sym_model_context model{};
  uint64_t nv = 0, nf = 0, ne = 0, nbr_count = 0;
  char *block = nullptr;
  double *xyz = nullptr, *fn = nullptr, *vn = nullptr, *w = nullptr;
  int32_t *faces = nullptr, *nbr = nullptr;
  uint64_t *nbr_off = nullptr;
  sym_edge *edges = nullptr;
};

namespace sym {

constexpr int kChunk = 128;  // votes per chunk = seeds per tile

// --------------------------------------------------------------- 6-D votes
// Rotation log map: axis-angle w with |w| = theta in [0, pi].  Near pi the
// axis comes from the symmetric part in FP64.
template <typename T>
__device__ void log_map(const T r[9], T w[3]) {
  T c = (r[0] + r[4] + r[8] - T(1)) * T(0.5);
  c = c > T(1) ? T(1) : (c < T(-1) ? T(-1) : c);
  T sx = r[7] - r[5], sy = r[2] - r[6], sz = r[3] - r[1];  // 2 sin(theta) n
  if (c > T(0.9999)) {
    T theta2 = T(2) * (T(1) - c);  // theta^2 to leading order
    T f = T(0.5) * (T(1) + theta2 / T(6));
    w[0] = f * sx, w[1] = f * sy, w[2] = f * sz;
  } else if (c > T(-0.99)) {
    T theta = acos(c);
    T f = theta / (T(2) * sin(theta));
    w[0] = f * sx, w[1] = f * sy, w[2] = f * sz;
  } else {
    double rd[9];
    for (int i = 0; i < 9; ++i) rd[i] = double(r[i]);
    double cd = (rd[0] + rd[4] + rd[8] - 1) * 0.5;
    cd = cd > 1 ? 1 : (cd < -1 ? -1 : cd);
    double theta = acos(cd), one_c = 1 - cd;
    int k = 0;
    if (rd[4] > rd[k * 4]) k = 1;
    if (rd[8] > rd[k * 4]) k = 2;
    double n[3];
    n[k] = sqrt(fmax((rd[k * 4] - cd) / one_c, 0.0));
    for (int j = 0; j < 3; ++j)
      if (j != k) n[j] = (rd[k * 3 + j] + rd[j * 3 + k]) / (2 * one_c * n[k]);
    double s[3] = {rd[7] - rd[5], rd[2] - rd[6], rd[3] - rd[1]};
    if (n[0] * s[0] + n[1] * s[1] + n[2] * s[2] < 0) n[0] = -n[0], n[1] = -n[1], n[2] = -n[2];
    w[0] = T(theta * n[0]), w[1] = T(theta * n[1]), w[2] = T(theta * n[2]);
  }
}

// Two rigid votes per pair (b's frame with sign +1, then -1) as the
// reference's transformations.cpp:53-70, described in 6-D:
// [log(R) / 2, (R c + t - c) / box], then |d|^2, then padding.
template <typename T>
__global__ void votes6(const double *pos, const double *nrm, const double *dmn, const double *dmx,
                       uint64_t nv, const int32_t *pa, const int32_t *pb, uint64_t np, double box,
                       double cx, double cy, double cz, T *desc) {
  uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= np) return;
  int32_t a = pa[i], b = pb[i];
  auto ld = [&](const double *l, int32_t v, T out[3]) {
    out[0] = T(l[v]), out[1] = T(l[nv + v]), out[2] = T(l[2 * nv + v]);
  };
  T p[3], q[3], an[3], ad[3], ax[3], bn[3], bd[3], bx[3];
  ld(pos, a, p), ld(pos, b, q), ld(nrm, a, an), ld(dmn, a, ad), ld(dmx, a, ax);
  ld(nrm, b, bn), ld(dmn, b, bd), ld(dmx, b, bx);
  T c[3] = {T(cx), T(cy), T(cz)};
  T inv_box = T(1) / T(box);
  for (int sgn = 0; sgn < 2; ++sgn) {
    T s = sgn ? T(-1) : T(1);
    T r[9];
    for (int x = 0; x < 3; ++x)
      for (int y = 0; y < 3; ++y)
        r[x * 3 + y] = s * bd[x] * ad[y] + s * bx[x] * ax[y] + bn[x] * an[y];
    T d[8];
    log_map<T>(r, d);
    for (int k = 0; k < 3; ++k) d[k] *= T(0.5);
    for (int x = 0; x < 3; ++x) {
      T rp = r[x * 3] * p[0] + r[x * 3 + 1] * p[1] + r[x * 3 + 2] * p[2];
      T rc = r[x * 3] * c[0] + r[x * 3 + 1] * c[1] + r[x * 3 + 2] * c[2];
      T t = q[x] - rp;
      d[3 + x] = (rc + t - c[x]) * inv_box;
    }
    T n2 = 0;
    for (int k = 0; k < 6; ++k) n2 += d[k] * d[k];
    d[6] = n2;
    d[7] = 0;
    uint64_t v = 2 * i + sgn;
    for (int k = 0; k < 8; ++k) desc[v * 8 + k] = d[k];
  }
}

// ------------------------------------------------------ sort into chunks
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
    for (int k = 0; k < 6; ++k) partial[blockIdx.x * 12 + k] = lo[k][0], partial[blockIdx.x * 12 + 6 + k] = hi[k][0];
}

__global__ void box_final(const float *partial, int n, float *box) {
  int k = threadIdx.x;
  if (k >= 12) return;
  float v = k < 6 ? INFINITY : -INFINITY;
  for (int i = 0; i < n; ++i) v = k < 6 ? fminf(v, partial[i * 12 + k]) : fmaxf(v, partial[i * 12 + k]);
  box[k] = v;
}

__device__ __forceinline__ uint64_t spread6(uint64_t x) {  // 10 bits -> every 6th bit
  uint64_t r = 0;
  for (int b = 0; b < 10; ++b) r |= ((x >> b) & 1ull) << (6 * b);
  return r;
}

__global__ void morton_keys(const float *desc, uint64_t q, const float *box, uint64_t *keys,
                            int32_t *idx) {
  uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (v >= q) return;
  uint64_t key = 0;
  for (int k = 0; k < 6; ++k) {
    float lo = box[k], span = box[6 + k] - lo;
    float t = span > 0 ? (desc[v * 8 + k] - lo) / span : 0.f;
    int cell = min(1023, max(0, int(t * 1024.f)));
    key |= spread6(uint64_t(cell)) << k;
  }
  keys[v] = key;
  idx[v] = int32_t(v);
}

template <typename T>
__global__ void permute(const T *src, const int32_t *order, uint64_t q, T *dst) {
  uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (v >= q) return;
  uint64_t from = uint64_t(uint32_t(order[v]));
  for (int k = 0; k < 8; ++k) dst[v * 8 + k] = src[from * 8 + k];
}

// One warp per chunk: [lo0..lo5, hi0..hi5].
__global__ void chunk_boxes(const float *desc, uint64_t q, uint64_t nchunks, float *cbox) {
  uint64_t c = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (c >= nchunks) return;
  float l[6], h[6];
  for (int k = 0; k < 6; ++k) l[k] = INFINITY, h[k] = -INFINITY;
  for (int j = lane; j < kChunk; j += 32) {
    uint64_t v = c * kChunk + j;
    if (v >= q) break;
    for (int k = 0; k < 6; ++k) {
      float x = desc[v * 8 + k];
      l[k] = fminf(l[k], x), h[k] = fmaxf(h[k], x);
    }
  }
  for (int o = 16; o; o >>= 1)
    for (int k = 0; k < 6; ++k) {
      l[k] = fminf(l[k], __shfl_xor_sync(0xffffffffu, l[k], o));
      h[k] = fmaxf(h[k], __shfl_xor_sync(0xffffffffu, h[k], o));
    }
  if (lane == 0)
    for (int k = 0; k < 6; ++k) cbox[c * 12 + k] = l[k], cbox[c * 12 + 6 + k] = h[k];
}

// --------------------------------------------------------------- mean shift
// Squared gap between two boxes, widened by `slack` per side.
__device__ __forceinline__ float box_gap2(const float *a_lo, const float *a_hi, const float *b) {
  float g = 0;
  for (int k = 0; k < 6; ++k) {
    float d = fmaxf(fmaxf(b[k] - a_hi[k], a_lo[k] - b[6 + k]), 0.f);
    g += d * d;
  }
  return g;
}

// One block = one tile of 128 seeds x one split of the chunk range.  The
// tile's box (over its active seeds) skips chunks that cannot contribute.
template <typename T>
__global__ void __launch_bounds__(kChunk) ms_tile(const T *desc, const float *cbox, uint64_t nchunks,
                                                  uint64_t q, const T *means, const uint8_t *state,
                                                  const uint8_t *tile_active, uint64_t k, T h2,
                                                  float skip_gap2, uint64_t chunks_per_split,
                                                  T *partial, unsigned long long *evals) {
  __shared__ T xs[kChunk * 8];
  __shared__ float tlo[6][4], thi[6][4];
  uint64_t tile = blockIdx.x, split = blockIdx.y;
  if (!tile_active[tile]) return;
  uint64_t seed = tile * kChunk + threadIdx.x;
  bool live = seed < k && state[seed] == 0;
  T m[6];
  for (int d = 0; d < 6; ++d) m[d] = seed < k ? means[seed * 8 + d] : T(0);
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
  uint64_t c0 = split * chunks_per_split, c1 = min(nchunks, c0 + chunks_per_split);
  unsigned long long done = 0;
  for (uint64_t c = c0; c < c1; ++c) {
    if (box_gap2(lo, hi, cbox + c * 12) > skip_gap2) continue;
    __syncthreads();
    uint64_t v = c * kChunk + threadIdx.x;
    for (int d = 0; d < 8; ++d) xs[threadIdx.x * 8 + d] = v < q ? desc[v * 8 + d] : T(1e30);
    __syncthreads();
    uint64_t rest = q - c * kChunk;
    int n = rest < uint64_t(kChunk) ? int(rest) : kChunk;
    done += n;
    for (int j = 0; j < n; ++j) {
      T d2 = 0;
#pragma unroll
      for (int d = 0; d < 6; ++d) {
        T e = m[d] - xs[j * 8 + d];
        d2 += e * e;
      }
      if (d2 < h2) {
        T w = T(1) - d2 / h2;
#pragma unroll
        for (int d = 0; d < 6; ++d) acc[d] += w * xs[j * 8 + d];
        acc[6] += w;
      }
    }
  }
  if (seed < k)
    for (int d = 0; d < 7; ++d) partial[(split * k + seed) * 8 + d] = acc[d];
  if (threadIdx.x == 0 && done) atomicAdd(evals, done * kChunk);
}

// Sum the splits (fixed order), move the seed, test convergence like the
// reference (movement < 1e-6 h^2, exhausted when the weight is <= 1e-14).
template <typename T>
__global__ void ms_update(T *means, const T *partial, uint64_t splits, uint64_t k, T h2,
                          uint8_t *state, const uint8_t *tile_active, uint8_t *tile_next,
                          unsigned *active) {
  uint64_t s = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (s >= k || state[s] || !tile_active[s / kChunk]) return;
  T acc[7] = {0, 0, 0, 0, 0, 0, 0};
  for (uint64_t p = 0; p < splits; ++p)
    for (int d = 0; d < 7; ++d) acc[d] += partial[(p * k + s) * 8 + d];
  if (acc[6] <= T(1e-14)) {
    state[s] = 2;
    return;
  }
  T move = 0;
  for (int d = 0; d < 6; ++d) {
    T nx = acc[d] / acc[6];
    T e = means[s * 8 + d] - nx;
    move += e * e;
    means[s * 8 + d] = nx;
  }
  if (move < T(1e-6) * h2) {
    state[s] = 1;
    return;
  }
  tile_next[s / kChunk] = 1;
  atomicAdd(active, 1u);
}

// Votes within the bandwidth of each mode (one block per chunk).
__global__ void mode_support(const float *desc, const float *cbox, uint64_t nchunks, uint64_t q,
                             const float *modes, uint64_t nm, float h2, float skip_gap2,
                             unsigned long long *support) {
  uint64_t c = blockIdx.x;
  uint64_t v = c * kChunk + threadIdx.x;
  float x[6];
  for (int d = 0; d < 6; ++d) x[d] = v < q ? desc[v * 8 + d] : 1e30f;
  const float *b = cbox + c * 12;
  for (uint64_t m = 0; m < nm; ++m) {
    const float *mm = modes + m * 8;
    if (box_gap2(mm, mm, b) > skip_gap2) continue;
    float d2 = 0;
    for (int d = 0; d < 6; ++d) {
      float e = mm[d] - x[d];
      d2 += e * e;
    }
    unsigned hit = __ballot_sync(0xffffffffu, v < q && d2 < h2);
    if ((threadIdx.x & 31) == 0 && hit) atomicAdd(&support[m], (unsigned long long)__popc(hit));
  }
}

template <typename T>
struct Shift {
  T *means;
  uint8_t *state, *tile_active, *tile_next;
  T *partial;
  unsigned *active;
};

// Runs FP32/FP64 iterations until every seed stops or `max_iter` is hit.
template <typename T>
int run_shift(Call &call, const T *desc, const float *cbox, uint64_t nchunks, uint64_t q,
              Shift<T> &s, uint64_t k, double h2, int max_iter, unsigned long long *evals,
              double *seed_iterations = nullptr) {
  cudaStream_t st = call.stream();
  uint64_t tiles = (k + kChunk - 1) / kChunk;
  uint64_t splits = std::max<uint64_t>(1, std::min<uint64_t>(nchunks, (64 * 152 + tiles - 1) / tiles));
  uint64_t cps = (nchunks + splits - 1) / splits;
  splits = (nchunks + cps - 1) / cps;
  float gap = float(std::sqrt(h2)) + 1e-6f;
  int it = 0;
  unsigned live = unsigned(k);
  for (; it < max_iter; ++it) {
    if (seed_iterations) *seed_iterations += live;
    ms_tile<T><<<dim3(unsigned(tiles), unsigned(splits)), kChunk, 0, st>>>(
        desc, cbox, nchunks, q, s.means, s.state, s.tile_active, k, T(h2), gap * gap, cps,
        s.partial, evals);
    check_launch();
    SYM_CUDA(cudaMemsetAsync(s.tile_next, 0, tiles, st));
    SYM_CUDA(cudaMemsetAsync(s.active, 0, sizeof(unsigned), st));
    ms_update<T><<<blocks_for(k), kThreads, 0, st>>>(s.means, s.partial, splits, k, T(h2), s.state,
                                                     s.tile_active, s.tile_next, s.active);
    check_launch();
    call.launched(2);
    SYM_CUDA(cudaMemcpyAsync(s.tile_active, s.tile_next, tiles, cudaMemcpyDeviceToDevice, st));
    unsigned active = 0;
    SYM_CUDA(cudaMemcpyAsync(&active, s.active, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    call.sync();
    live = active;
    if (!active) {
      ++it;
      break;
    }
  }
  return it;
}

template <typename T>
__global__ void gather_seeds(const T *desc, const int64_t *pos, uint64_t k, T *means) {
  uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= k) return;
  for (int d = 0; d < 8; ++d) means[i * 8 + d] = desc[uint64_t(pos[i]) * 8 + d];
}

template <typename T>
Shift<T> make_shift(Call &call, uint64_t k, uint64_t nchunks, const T *desc,
                    const std::vector<int64_t> &seed_pos) {
  Shift<T> s;
  uint64_t tiles = (k + kChunk - 1) / kChunk;
  uint64_t splits_max = std::max<uint64_t>(1, std::min<uint64_t>(nchunks, (64 * 152 + tiles - 1) / tiles)) + 1;
  s.means = call.alloc<T>(k * 8);
  s.state = call.alloc<uint8_t>(k);
  s.tile_active = call.alloc<uint8_t>(tiles);
  s.tile_next = call.alloc<uint8_t>(tiles);
  s.partial = call.alloc<T>(splits_max * k * 8);
  s.active = call.alloc<unsigned>(1);
  SYM_CUDA(cudaMemsetAsync(s.state, 0, k, call.stream()));
  SYM_CUDA(cudaMemsetAsync(s.tile_active, 1, tiles, call.stream()));
  int64_t *pos = call.upload(seed_pos.data(), k);
  gather_seeds<T><<<blocks_for(k), kThreads, 0, call.stream()>>>(desc, pos, k, s.means);
  check_launch();
  call.launched();
  return s;
}

// Rodrigues: R = exp([w]x).
void exp_map(const double w[3], double r[9]) {
  double th = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
  double a, b;
  if (th < 1e-8) {
    a = 1 - th * th / 6, b = 0.5 - th * th / 24;
  } else {
    a = std::sin(th) / th, b = (1 - std::cos(th)) / (th * th);
  }
  double K[9] = {0, -w[2], w[1], w[2], 0, -w[0], -w[1], w[0], 0};
  double K2[9] = {};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      for (int l = 0; l < 3; ++l) K2[i * 3 + j] += K[i * 3 + l] * K[l * 3 + j];
  for (int i = 0; i < 9; ++i) r[i] = (i % 4 == 0 ? 1.0 : 0.0) + a * K[i] + b * K2[i];
}

class StageClock {
public:
  explicit StageClock(cudaStream_t s) : s_(s) {
    for (auto &e : ev_) cudaEventCreate(&e);
  }
  ~StageClock() {
    for (auto &e : ev_) cudaEventDestroy(e);
  }
  void mark(int i) { cudaEventRecord(ev_[i], s_); }
  double ms(int a, int b) {
    float t = 0;
    cudaEventElapsedTime(&t, ev_[a], ev_[b]);
    return t;
  }

private:
  cudaStream_t s_;
  cudaEvent_t ev_[10];
};

void detect_fast(Call &call, sym_mesh_handle &h, const int32_t *sample, uint64_t ns,
                 const sym_options &o, const sym_fast_options &fo, sym_fast_result &r) {
  r = sym_fast_result{};
  cudaStream_t st = call.stream();
  StageClock clock(st);
  const uint64_t nv = h.nv;
  clock.mark(0);
  // ---- (a) curvature
  double *lanes = call.alloc<double>(11 * nv);
  uint8_t *valid = call.alloc<uint8_t>(nv);
  sym_features_out f{};
  double **cols[11] = {&f.normal_x, &f.normal_y, &f.normal_z, &f.dmin_x, &f.dmin_y, &f.dmin_z,
                       &f.dmax_x,   &f.dmax_y,   &f.dmax_z,   &f.kmin,   &f.kmax};
  for (int k = 0; k < 11; ++k) *cols[k] = lanes + k * nv;
  f.valid = valid;
  f.count = nv;
  curvature_device(call, h.xyz, nv, h.fn, h.nf, h.vn, h.nbr_off, h.nbr, h.nbr_count, h.edges, h.ne,
                   o.smoothing, f, h.host_edges.data());
  clock.mark(1);
  // ---- prune of the host sample
  int32_t *dsample = call.upload(sample, ns);
  int32_t *pruned = call.alloc<int32_t>(ns);
  uint64_t *pcount = call.alloc<uint64_t>(1);
  prune_device(call, dsample, ns, f.kmin, f.kmax, valid, o.prune, pruned, pcount);
  uint64_t s = 0;
  call.d2h(&s, pcount, 8);
  call.sync();
  r.pruned = s;
  clock.mark(2);
  // ---- (b) pairing + 6-D votes
  int32_t *pa = nullptr, *pb = nullptr;
  uint64_t np = pairing_device(call, pruned, s, h.xyz, nv, f.kmin, f.kmax, o.pair_threshold,
                               h.model.box_size, o.max_pairs, &pa, &pb);
  r.pairs = np;
  clock.mark(3);
  uint64_t q = 2 * np;
  if (q > o.max_votes || q > uint64_t(std::numeric_limits<int32_t>::max()))
    fail(SYM_RUNTIME_ERROR, "Vote budget exceeded; lower --sample-ratio or tighten --pair-threshold");
  r.votes = q;
  if (!q) {
    clock.mark(4);
    return;
  }
  const bool want64 = fo.reference_seeds > 0;
  float *desc_raw = call.alloc<float>(q * 8);
  double *desc64_raw = want64 ? call.alloc<double>(q * 8) : nullptr;
  const double *c = h.model.center;
  votes6<float><<<blocks_for(np), kThreads, 0, st>>>(h.xyz, f.normal_x, f.dmin_x, f.dmax_x, nv, pa,
                                                     pb, np, h.model.box_size, c[0], c[1], c[2],
                                                     desc_raw);
  check_launch();
  if (want64) {
    votes6<double><<<blocks_for(np), kThreads, 0, st>>>(h.xyz, f.normal_x, f.dmin_x, f.dmax_x, nv,
                                                        pa, pb, np, h.model.box_size, c[0], c[1],
                                                        c[2], desc64_raw);
    check_launch();
  }
  call.launched(want64 ? 2 : 1);
  clock.mark(4);
  // ---- Morton sort into chunks
  const int kBoxBlocks = 256;
  float *bpart = call.alloc<float>(kBoxBlocks * 12), *gbox = call.alloc<float>(12);
  box_partials<<<kBoxBlocks, 256, 0, st>>>(desc_raw, q, bpart);
  check_launch();
  box_final<<<1, 32, 0, st>>>(bpart, kBoxBlocks, gbox);
  check_launch();
  uint64_t *keys = call.alloc<uint64_t>(q), *skeys = call.alloc<uint64_t>(q);
  int32_t *idx = call.alloc<int32_t>(q), *order = call.alloc<int32_t>(q);
  morton_keys<<<blocks_for(q), kThreads, 0, st>>>(desc_raw, q, gbox, keys, idx);
  check_launch();
  radix_sort_pairs(call, keys, idx, skeys, order, q, 60);
  float *desc = call.alloc<float>(q * 8);
  permute<float><<<blocks_for(q), kThreads, 0, st>>>(desc_raw, order, q, desc);
  check_launch();
  double *desc64 = nullptr;
  if (want64) {
    desc64 = call.alloc<double>(q * 8);
    permute<double><<<blocks_for(q), kThreads, 0, st>>>(desc64_raw, order, q, desc64);
    check_launch();
  }
  uint64_t nchunks = (q + kChunk - 1) / kChunk;
  float *cbox = call.alloc<float>(nchunks * 12);
  chunk_boxes<<<blocks_for(nchunks * 32), kThreads, 0, st>>>(desc, q, nchunks, cbox);
  check_launch();
  call.launched(want64 ? 6 : 5);
  clock.mark(5);
  // ---- (c) mean shift from K seeds (uniform draw, in sorted vote order)
  uint64_t k = std::min<uint64_t>(uint64_t(std::max(fo.seeds, 1)), q);
  std::mt19937_64 rng(fo.seed_rng);
  std::vector<int64_t> seed_pos;
  {
    std::vector<int64_t> pool;  // Floyd's sampling of k distinct positions
    std::vector<char> taken;
    if (q <= (1u << 26)) taken.assign(q, 0);
    for (uint64_t j = q - k; j < q; ++j) {
      uint64_t t = rng() % (j + 1);
      bool dup = taken.empty() ? std::find(pool.begin(), pool.end(), int64_t(t)) != pool.end() : taken[t];
      uint64_t pick = dup ? j : t;
      pool.push_back(int64_t(pick));
      if (!taken.empty()) taken[pick] = 1;
    }
    std::sort(pool.begin(), pool.end());
    seed_pos = pool;
  }
  const double h2 = o.bandwidth * o.bandwidth;
  unsigned long long *evals = call.alloc<unsigned long long>(1);
  SYM_CUDA(cudaMemsetAsync(evals, 0, 8, st));
  Shift<float> s32 = make_shift<float>(call, k, nchunks, desc, seed_pos);
  int bulk = 0, polish = 0;
  double bf16_evals = 0;
  if (fo.precision == SYM_MS_BF16_REFINED) {
    if (meanshift_bf16_bulk(call, desc, cbox, nchunks, q, s32.means, s32.state, k, float(h2),
                            fo.max_iterations, &bulk, &bf16_evals)) {
      // polish: every seed restarts in FP32 from its BF16 mode
      SYM_CUDA(cudaMemsetAsync(s32.state, 0, k, st));
      SYM_CUDA(cudaMemsetAsync(s32.tile_active, 1, (k + kChunk - 1) / kChunk, st));
      polish = run_shift<float>(call, desc, cbox, nchunks, q, s32, k, h2, fo.polish_iterations, evals,
                                &r.seed_iterations);
    } else {
      bulk = run_shift<float>(call, desc, cbox, nchunks, q, s32, k, h2, fo.max_iterations, evals,
                              &r.seed_iterations);
    }
  } else {
    bulk = run_shift<float>(call, desc, cbox, nchunks, q, s32, k, h2, fo.max_iterations, evals,
                            &r.seed_iterations);
  }
  r.iterations = bulk;
  r.polish_iterations = polish;
  unsigned long long ev = 0;
  call.d2h(&ev, evals, 8);
  std::vector<float> means(k * 8);
  std::vector<uint8_t> state(k);
  call.d2h(means.data(), s32.means, k * 8 * 4);
  call.d2h(state.data(), s32.state, k);
  call.sync();
  r.mean_shift_pairs = double(ev) + bf16_evals;
  r.h2d_bytes = call.ctx->metrics.current.h2d_bytes;
  r.d2h_bytes = call.ctx->metrics.current.d2h_bytes;
  clock.mark(6);
  // ---- FP64 reference on the first seeds (mode error)
  if (want64) {
    uint64_t k64 = std::min<uint64_t>(k, uint64_t(fo.reference_seeds));
    std::vector<int64_t> sp(seed_pos.begin(), seed_pos.begin() + k64);
    Shift<double> s64 = make_shift<double>(call, k64, nchunks, desc64, sp);
    unsigned long long *ev64 = call.alloc<unsigned long long>(1);
    run_shift<double>(call, desc64, cbox, nchunks, q, s64, k64, h2, 1000, ev64);
    std::vector<double> m64(k64 * 8);
    std::vector<uint8_t> st64(k64);
    call.d2h(m64.data(), s64.means, k64 * 8 * 8);
    call.d2h(st64.data(), s64.state, k64);
    call.sync();
    double emax = 0, esum = 0;
    uint64_t n = 0;
    for (uint64_t i = 0; i < k64; ++i) {
      double num = 0, den = 0;
      for (int d = 0; d < 6; ++d) {
        double e = double(means[i * 8 + d]) - m64[i * 8 + d];
        num += e * e, den += m64[i * 8 + d] * m64[i * 8 + d];
      }
      double rel = std::sqrt(num) / std::max(std::sqrt(den), 1e-300);
      emax = std::max(emax, rel), esum += rel, ++n;
    }
    r.mode_error_max = emax;
    r.mode_error_mean = n ? esum / n : 0;
  }
  clock.mark(7);
  // ---- modes: greedy merge (h^2/4, first mode wins) + support
  std::vector<double> mode_pos;
  std::vector<uint64_t> mode_seeds;
  for (uint64_t i = 0; i < k; ++i) {
    if (state[i] == 2) continue;  // exhausted
    int hit = -1;
    for (size_t m = 0; m < mode_seeds.size(); ++m) {
      double d2 = 0;
      for (int d = 0; d < 6; ++d) {
        double e = double(means[i * 8 + d]) - mode_pos[m * 6 + d];
        d2 += e * e;
      }
      if (d2 < h2 / 4) {
        hit = int(m);
        break;
      }
    }
    if (hit < 0) {
      for (int d = 0; d < 6; ++d) mode_pos.push_back(means[i * 8 + d]);
      mode_seeds.push_back(1);
    } else {
      double n = double(mode_seeds[hit]);
      for (int d = 0; d < 6; ++d)
        mode_pos[hit * 6 + d] = (n * mode_pos[hit * 6 + d] + means[i * 8 + d]) / (n + 1);
      ++mode_seeds[hit];
    }
  }
  uint64_t nm = mode_seeds.size();
  r.modes = nm;
  std::vector<uint64_t> support(nm, 0);
  if (nm) {
    std::vector<float> mp(nm * 8, 0.f);
    for (uint64_t m = 0; m < nm; ++m)
      for (int d = 0; d < 6; ++d) mp[m * 8 + d] = float(mode_pos[m * 6 + d]);
    float *dmodes = call.upload(mp.data(), mp.size());
    unsigned long long *dsup = call.alloc<unsigned long long>(nm);
    SYM_CUDA(cudaMemsetAsync(dsup, 0, nm * 8, st));
    float gap = float(o.bandwidth) + 1e-6f;
    mode_support<<<unsigned(nchunks), kChunk, 0, st>>>(desc, cbox, nchunks, q, dmodes, nm, float(h2),
                                                     gap * gap, dsup);
    check_launch();
    call.launched();
    call.d2h(support.data(), dsup, nm * 8);
    call.sync();
  }
  std::vector<uint64_t> rank(nm);
  for (uint64_t m = 0; m < nm; ++m) rank[m] = m;
  std::stable_sort(rank.begin(), rank.end(), [&](uint64_t a, uint64_t b) { return support[a] > support[b]; });
  uint64_t nc = std::min<uint64_t>({nm, uint64_t(std::max(o.max_clusters, 0)), SYM_FAST_MAX_CLUSTERS});
  r.clusters = nc;
  for (uint64_t i = 0; i < nc; ++i) {
    const double *d = &mode_pos[rank[i] * 6];
    double w[3] = {2 * d[0], 2 * d[1], 2 * d[2]}, R[9];
    exp_map(w, R);
    sym_cluster_record &rec = r.records[i];
    rec = sym_cluster_record{};
    for (int j = 0; j < 9; ++j) rec.rotation[j] = R[j];
    for (int x = 0; x < 3; ++x) {
      double rc = R[x * 3] * c[0] + R[x * 3 + 1] * c[1] + R[x * 3 + 2] * c[2];
      rec.translation[x] = d[3 + x] * h.model.box_size + c[x] - rc;
    }
    r.support[i] = support[rank[i]];
  }
  clock.mark(8);
  // ---- (d) verification of the top modes
  if (fo.verify && nc) {
    std::vector<std::vector<int32_t>> side;
    std::vector<std::vector<std::vector<int32_t>>> patches;
    std::vector<double> coverage, rms;
    verification_core(call, h.host, h.xyz, h.faces, h.vn, h.w, h.nbr_off, h.nbr, r.records, nc,
                      o.verify_threshold * h.model.box_size, side, patches, coverage, rms);
    for (uint64_t i = 0; i < nc; ++i) r.coverage[i] = coverage[i], r.rms[i] = rms[i];
  }
  clock.mark(9);
  call.sync();
  // stage order: curvature, prune, pairing, votes, sort, mean shift (+fp64 ref excluded), modes, verification
  r.stage_ms[0] = clock.ms(0, 1);
  r.stage_ms[1] = clock.ms(1, 2);
  r.stage_ms[2] = clock.ms(2, 3);
  r.stage_ms[3] = clock.ms(3, 4);
  r.stage_ms[4] = clock.ms(4, 5);
  r.stage_ms[5] = clock.ms(5, 6);
  r.stage_ms[6] = clock.ms(7, 8);
  r.stage_ms[7] = clock.ms(8, 9);
}

}  // namespace sym

extern "C" {

void sym_fast_options_default(sym_fast_options *o) {
  *o = sym_fast_options{SYM_MS_BF16_REFINED, 2048, 7, 100, 100, 0, 1};
}

sym_status sym_mesh_load(sym_context *ctx, const sym_mesh_view *mesh, const sym_topology_view *g,
                         const sym_model_context *model, sym_mesh_handle **out) {
  if (!ctx || !mesh || !g || !model || !out) return SYM_INVALID_ARGUMENT;
  *out = nullptr;
  try {
    SYM_CUDA(cudaSetDevice(ctx->device));
    const uint64_t nv = mesh->vertices.count, nf = mesh->faces.count, ne = g->edge_count;
    if (g->normals.count != nv || g->weight_count != nv || g->face_normals.count != nf)
      sym::fail(SYM_INVALID_ARGUMENT, "SoA component lengths differ");
    sym::validate_csr(g->neighbors, nv, nv, "neighbors");
    for (uint64_t f = 0; f < nf; ++f)
      if (mesh->faces.v0[f] < 0 || mesh->faces.v1[f] < 0 || mesh->faces.v2[f] < 0 ||
          uint64_t(mesh->faces.v0[f]) >= nv || uint64_t(mesh->faces.v1[f]) >= nv ||
          uint64_t(mesh->faces.v2[f]) >= nv)
        sym::fail(SYM_INVALID_ARGUMENT, "Face index out of range");
    auto h = new sym_mesh_handle();
    h->ctx = ctx;
    h->host = *mesh;
    h->model = *model;
    h->nv = nv, h->nf = nf, h->ne = ne;
    h->nbr_count = g->neighbors.offsets[nv];
    h->host_edges.assign(g->edges, g->edges + ne);
    auto pad = [](uint64_t b) { return (b + 255) & ~uint64_t(255); };
    uint64_t sizes[9] = {pad(24 * nv), pad(24 * nf), pad(24 * nv), pad(8 * nv), pad(12 * nf),
                         pad(8 * (nv + 1)), pad(4 * h->nbr_count), pad(24 * ne), 0};
    uint64_t total = 0;
    for (auto b : sizes) total += b;
    if (cudaMalloc(&h->block, total ? total : 256) != cudaSuccess) {
      delete h;
      sym::fail(SYM_CUDA_ERROR, "CUDA: mesh allocation failed");
    }
    char *p = h->block;
    h->xyz = reinterpret_cast<double *>(p), p += sizes[0];
    h->fn = reinterpret_cast<double *>(p), p += sizes[1];
    h->vn = reinterpret_cast<double *>(p), p += sizes[2];
    h->w = reinterpret_cast<double *>(p), p += sizes[3];
    h->faces = reinterpret_cast<int32_t *>(p), p += sizes[4];
    h->nbr_off = reinterpret_cast<uint64_t *>(p), p += sizes[5];
    h->nbr = reinterpret_cast<int32_t *>(p), p += sizes[6];
    h->edges = reinterpret_cast<sym_edge *>(p);
    cudaStream_t st = ctx->stream;
    auto put = [&](void *dst, const void *src, uint64_t bytes) {
      if (bytes) SYM_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
    };
    const sym_points_view *pts[3] = {&mesh->vertices, &g->face_normals, &g->normals};
    double *dst[3] = {h->xyz, h->fn, h->vn};
    for (int i = 0; i < 3; ++i) {
      uint64_t n = pts[i]->count;
      put(dst[i], pts[i]->x, 8 * n), put(dst[i] + n, pts[i]->y, 8 * n), put(dst[i] + 2 * n, pts[i]->z, 8 * n);
    }
    put(h->w, g->weights, 8 * nv);
    put(h->faces, mesh->faces.v0, 4 * nf), put(h->faces + nf, mesh->faces.v1, 4 * nf);
    put(h->faces + 2 * nf, mesh->faces.v2, 4 * nf);
    put(h->nbr_off, g->neighbors.offsets, 8 * (nv + 1));
    put(h->nbr, g->neighbors.indices, 4 * h->nbr_count);
    put(h->edges, g->edges, 24 * ne);
    SYM_CUDA(cudaStreamSynchronize(st));
    *out = h;
    return SYM_OK;
  } catch (const sym::Error &e) {
    sym_error_text = e.what();
    return e.status;
  }
}

void sym_mesh_free(sym_mesh_handle *h) {
  if (!h) return;
  cudaSetDevice(h->ctx->device);
  cudaStreamSynchronize(h->ctx->stream);
  cudaFree(h->block);
  delete h;
}

sym_status sym_detect_fast(sym_context *ctx, sym_mesh_handle *mesh, const int32_t *sample,
                           uint64_t sample_count, const sym_options *options,
                           const sym_fast_options *fast, sym_fast_result *out) {
  if (!ctx || !mesh || !options || !fast || !out || (sample_count && !sample)) return SYM_INVALID_ARGUMENT;
  try {
    sym::Call call(ctx, "detect_fast");
    for (uint64_t i = 0; i < sample_count; ++i)
      if (sample[i] < 0 || uint64_t(sample[i]) >= mesh->nv)
        sym::fail(SYM_INVALID_ARGUMENT, "sample vertex index out of range");
    sym::detect_fast(call, *mesh, sample, sample_count, *options, *fast, *out);
    out->launches = ctx->metrics.current.custom_launches;
    return SYM_OK;
  } catch (const sym::Error &e) {
    sym_error_text = e.what();
    return e.status;
  } catch (const std::exception &e) {
    sym_error_text = e.what();
    return SYM_RUNTIME_ERROR;
  }
}

}  // extern "C"
