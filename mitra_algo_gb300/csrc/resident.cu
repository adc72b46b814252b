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
// in FP32 (the seeds near a mode finish with Newton steps, see
// meanshift_fast.cuh); a subset of seeds re-runs in FP64 to measure the mode
// error.
#include "common.cuh"
#include "primitives.cuh"
#include "meanshift_fast.cuh"
#include "rng.hpp"
#include "sampling.cuh"
#include "verification.cuh"
#include "prepare.cuh"

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <limits>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace sym {
void curvature_device(Call &, const double *, uint64_t, const double *, uint64_t, const double *,
                      const uint64_t *, const int32_t *, uint64_t, const sym_edge *, uint64_t, int,
                      const sym_features_out &, const sym_edge *);
void prune_device(Call &, const int32_t *, uint64_t, const double *, const double *,
                  const uint8_t *, double, int32_t *, uint64_t *);
uint64_t pairing_device(Call &, const int32_t *, uint64_t, const double *, uint64_t, const double *,
                        const double *, double, double, uint64_t, int32_t **, int32_t **);
// BF16 tensor-core bulk iterations (meanshift_tc.cu); returns false when the
// tensor path cannot run this problem (the caller then stays in FP32).
// seed_iterations (optional) receives the sum over iterations of the
// active seeds.
bool meanshift_bf16_bulk(Call &call, const VoteSet &v, float *means, uint8_t *state, uint64_t k,
                         double h2, int max_iter, int *iterations, double *evaluations,
                         uint32_t *trace = nullptr, int trace_len = 0, double *kernel_ms = nullptr,
                         uint64_t *kernel_launches = nullptr, double *seed_iterations = nullptr);
void tc_selftest_host(Call &call, const uint16_t *a1, const uint16_t *b1, const uint16_t *a2,
                      const uint16_t *b2, float *d_out, float *acc_out);
}  // namespace sym

struct sym_mesh_handle {
  int device = 0;  // the device holding its memory (not tied to the loading context)
  sym_mesh_view host{};
  std::vector<sym_edge> host_edges;  // sym_mesh_load only (an edge table in any order)
  sym_model_context model{};
  uint64_t nv = 0, nf = 0, ne = 0, nbr_count = 0;
  char *block = nullptr;
  double *xyz = nullptr, *fn = nullptr, *vn = nullptr, *w = nullptr;
  int32_t *faces = nullptr, *nbr = nullptr;
  uint64_t *nbr_off = nullptr;
  sym_edge *edges = nullptr;
  sym::Lbvh lbvh;  // FP32 linear BVH of the faces (verification of the fast path)
  // the reference-order BVH (verification ties), built on a host thread
  // from the load on
  sym::RefBvhSource ref;
  sym::ResidentSurface surface() {
    return {&lbvh, xyz, vn, w, faces, nbr_off, nbr, nv, nf, &ref};
  }
  void release() {  // the device memory (after the context's stream is idle)
    sym::lbvh_free(lbvh);
    ref.release();
    if (block) cudaFree(block);
    block = nullptr;
  }
};

namespace sym {

// --------------------------------------------------------------- 6-D votes
// Rotation log map: the axis-angle vector w of R (|w| = theta in [0, pi]).
// theta = atan2(|s| / 2, c) from c = (tr R - 1) / 2 and the antisymmetric
// part s = (R21 - R12, R02 - R20, R10 - R01) = 2 sin(theta) n, which is well
// conditioned at every angle (acos(c) amplifies the rounding of c by
// 1 / sin(theta) near 0 and pi).  Away from pi the axis is s / |s|.  For
// c <= -0.99 (theta within about 8 degrees of pi, where s vanishes) the axis
// comes, in FP64, from the symmetric part (R + R^T) / 2 = c I + (1 - c) n n^T
// through its largest diagonal entry, normalised, with the sign of s.
template <typename T>
__device__ void log_map(const T r[9], T w[3]) {
  const T c = (r[0] + r[4] + r[8] - T(1)) * T(0.5);
  const T sx = r[7] - r[5], sy = r[2] - r[6], sz = r[3] - r[1];  // 2 sin(theta) n
  if (c > T(-0.99)) {
    const T sn = sqrt(sx * sx + sy * sy + sz * sz);
    const T f = sn > T(0) ? atan2(T(0.5) * sn, c) / sn : T(0.5);
    w[0] = f * sx, w[1] = f * sy, w[2] = f * sz;
    return;
  }
  double rd[9];
  for (int i = 0; i < 9; ++i) rd[i] = double(r[i]);
  const double cd = (rd[0] + rd[4] + rd[8] - 1) * 0.5;
  const double s[3] = {rd[7] - rd[5], rd[2] - rd[6], rd[3] - rd[1]};
  const double theta = atan2(0.5 * sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]), cd);
  const double one_c = 1 - cd;
  int k = 0;
  if (rd[4] > rd[k * 4]) k = 1;
  if (rd[8] > rd[k * 4]) k = 2;
  double n[3];
  n[k] = sqrt(fmax((rd[k * 4] - cd) / one_c, 0.0));
  for (int j = 0; j < 3; ++j)
    if (j != k) n[j] = (rd[k * 3 + j] + rd[j * 3 + k]) / (2 * one_c * n[k]);
  const double len = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
  const double sign = n[0] * s[0] + n[1] * s[1] + n[2] * s[2] < 0 ? -1.0 : 1.0;
  const double g = sign * theta / len;
  w[0] = T(g * n[0]), w[1] = T(g * n[1]), w[2] = T(g * n[2]);
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

// The FP32 form of votes6 in two passes.  frames_f32 converts each
// vertex's position, normal and principal directions once into a 48-byte
// record (three float4), so a pair gathers two records instead of 24
// scattered doubles.  votes6_f32 writes every vote whose rotation is not
// near pi (the FP32 log map) and lists the others; votes6_near_pi then
// takes the listed votes through the FP64 branch of log_map in full warps
// (near pi the FP64 branch would otherwise run in almost every warp).  Each
// vote follows the formulas of votes6<float>; the compiler may contract
// them into FMAs differently, so votes can differ from votes6<float> in the
// last bit.
__global__ void frames_f32(const double *pos, const double *nrm, const double *dmn,
                           const double *dmx, uint64_t nv, float4 *frames) {
  const uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  auto f = [&](const double *l, int d) { return float(l[uint64_t(d) * nv + v]); };
  frames[3 * v] = make_float4(f(pos, 0), f(pos, 1), f(pos, 2), f(nrm, 0));
  frames[3 * v + 1] = make_float4(f(nrm, 1), f(nrm, 2), f(dmn, 0), f(dmn, 1));
  frames[3 * v + 2] = make_float4(f(dmn, 2), f(dmx, 0), f(dmx, 1), f(dmx, 2));
}

struct Frame32 {
  float p[3], n[3], dn[3], dx[3];
};
__device__ __forceinline__ Frame32 load_frame(const float4 *frames, int32_t v) {
  const float4 a = frames[3 * uint64_t(v)], b = frames[3 * uint64_t(v) + 1],
               c = frames[3 * uint64_t(v) + 2];
  return {{a.x, a.y, a.z}, {a.w, b.x, b.y}, {b.z, b.w, c.x}, {c.y, c.z, c.w}};
}

// Rotation of vote sgn of the pair (a's frame to b's), as votes6.
__device__ __forceinline__ void pair_rotation(const Frame32 &fa, const Frame32 &fb, int sgn,
                                              float r[9]) {
  const float s = sgn ? -1.f : 1.f;
  for (int x = 0; x < 3; ++x)
    for (int y = 0; y < 3; ++y)
      r[x * 3 + y] = s * fb.dn[x] * fa.dn[y] + s * fb.dx[x] * fa.dx[y] + fb.n[x] * fa.n[y];
}

__device__ __forceinline__ void finish_vote(const float r[9], float d[8], const Frame32 &fa,
                                            const Frame32 &fb, const float c[3], float inv_box) {
  for (int k = 0; k < 3; ++k) d[k] *= 0.5f;
  for (int x = 0; x < 3; ++x) {
    float rp = r[x * 3] * fa.p[0] + r[x * 3 + 1] * fa.p[1] + r[x * 3 + 2] * fa.p[2];
    float rc = r[x * 3] * c[0] + r[x * 3 + 1] * c[1] + r[x * 3 + 2] * c[2];
    float t = fb.p[x] - rp;
    d[3 + x] = (rc + t - c[x]) * inv_box;
  }
  float n2 = 0;
  for (int k = 0; k < 6; ++k) n2 += d[k] * d[k];
  d[6] = n2;
  d[7] = 0;
}

__device__ __forceinline__ bool near_pi(const float r[9]) {
  const float c = (r[0] + r[4] + r[8] - 1.f) * 0.5f;
  return !(c > -0.99f);  // log_map's FP64 branch
}

__global__ void votes6_f32(const float4 *frames, const int32_t *pa, const int32_t *pb, uint64_t np,
                           double box, double cx, double cy, double cz, float *desc,
                           unsigned long long *near_list, unsigned long long *near_count) {
  const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const Frame32 fa = load_frame(frames, pa[i]), fb = load_frame(frames, pb[i]);
  const float c[3] = {float(cx), float(cy), float(cz)};
  const float inv_box = 1.f / float(box);
  for (int sgn = 0; sgn < 2; ++sgn) {
    float r[9], d[8];
    pair_rotation(fa, fb, sgn, r);
    const uint64_t v = 2 * i + sgn;
    if (near_pi(r)) {
      near_list[atomicAdd(near_count, 1ull)] = v;
      continue;
    }
    log_map<float>(r, d);
    finish_vote(r, d, fa, fb, c, inv_box);
    float4 *o = reinterpret_cast<float4 *>(desc + v * 8);
    o[0] = make_float4(d[0], d[1], d[2], d[3]);
    o[1] = make_float4(d[4], d[5], d[6], d[7]);
  }
}

__global__ void votes6_near_pi(const float4 *frames, const int32_t *pa, const int32_t *pb,
                               double box, double cx, double cy, double cz, float *desc,
                               const unsigned long long *near_list,
                               const unsigned long long *near_count) {
  const float c[3] = {float(cx), float(cy), float(cz)};
  const float inv_box = 1.f / float(box);
  const unsigned long long n = *near_count;
  for (unsigned long long j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < n;
       j += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t v = near_list[j], i = v / 2;
    const Frame32 fa = load_frame(frames, pa[i]), fb = load_frame(frames, pb[i]);
    float r[9], d[8];
    pair_rotation(fa, fb, int(v & 1), r);
    log_map<float>(r, d);
    finish_vote(r, d, fa, fb, c, inv_box);
    float4 *o = reinterpret_cast<float4 *>(desc + v * 8);
    o[0] = make_float4(d[0], d[1], d[2], d[3]);
    o[1] = make_float4(d[4], d[5], d[6], d[7]);
  }
}

// Reflection mode.  The plane of a pair is the perpendicular bisector of
// its two points, n = unit(q - p) with its dominant component made positive
// and d = -n.(p + q)/2; the pair votes for it when the mirrored frames agree
// (the reference's test, transformations.cpp:17-73: the mirrored normal of a
// within 0.75 of b's, the mirrored first direction within 0.75 of +-b's).
// The test is made in FP64 once, so the FP32 and FP64 vote sets are the
// same pairs; the descriptors [n, (d + n.c)/box] (zero-padded to 6-D) are
// then written in each precision.
__device__ __forceinline__ D3 plane_of(D3 p, D3 q, double &d) {
  D3 n = unit(q - p);
  int dom = 0;
  for (int k = 1; k < 3; ++k)
    if (fabs(comp(n, k)) > fabs(comp(n, dom))) dom = k;
  if (comp(n, dom) < 0) n = n * -1;
  d = -dot(n, div(p + q, 2));
  return n;
}

__global__ void plane_flags(const double *pos, const double *nrm, const double *dmn, uint64_t nv,
                            const int32_t *pa, const int32_t *pb, uint64_t np, uint8_t *flags) {
  const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const int32_t a = pa[i], b = pb[i];
  auto ld = [&](const double *l, int32_t v) { return D3{l[v], l[nv + v], l[2 * nv + v]}; };
  double d;
  const D3 n = plane_of(ld(pos, a), ld(pos, b), d);
  const M3 refl = mirror(n);
  flags[i] = dot(mul(refl, ld(nrm, a)), ld(nrm, b)) > 0.75 &&
             fabs(dot(mul(refl, ld(dmn, a)), ld(dmn, b))) > 0.75;
}

template <typename T>
__global__ void plane_votes(const double *pos, uint64_t nv, const int32_t *pa, const int32_t *pb,
                            const int32_t *list, uint64_t q, double box, double cx, double cy,
                            double cz, T *desc) {
  const uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (v >= q) return;
  const int32_t i = list[v], a = pa[i], b = pb[i];
  T p[3] = {T(pos[a]), T(pos[nv + a]), T(pos[2 * nv + a])};
  T r[3] = {T(pos[b]), T(pos[nv + b]), T(pos[2 * nv + b])};
  T n[3], len = 0;
  for (int k = 0; k < 3; ++k) n[k] = r[k] - p[k], len += n[k] * n[k];
  len = sqrt(len);
  int dom = 0;
  for (int k = 0; k < 3; ++k) {
    n[k] /= len;
    if (fabs(n[k]) > fabs(n[dom])) dom = k;
  }
  if (n[dom] < T(0))
    for (int k = 0; k < 3; ++k) n[k] = -n[k];
  T d = 0;
  for (int k = 0; k < 3; ++k) d -= n[k] * ((p[k] + r[k]) / T(2));
  T out[8] = {n[0], n[1], n[2], (d + n[0] * T(cx) + n[1] * T(cy) + n[2] * T(cz)) / T(box), 0, 0, 0, 0};
  out[6] = out[0] * out[0] + out[1] * out[1] + out[2] * out[2] + out[3] * out[3];
  for (int k = 0; k < 8; ++k) desc[v * 8 + k] = out[k];
}

// The FP32 rigid votes of np pairs into desc (2 np records of 8 floats):
// frames_f32, votes6_f32, then votes6_near_pi for the votes near pi.
void rigid_votes_f32(Call &call, const double *xyz, const double *nrm, const double *dmn,
                     const double *dmx, uint64_t nv, const int32_t *pa, const int32_t *pb,
                     uint64_t np, const sym_model_context &model, float *desc) {
  if (!np) return;
  cudaStream_t st = call.stream();
  const double *c = model.center;
  float4 *frames = call.alloc<float4>(3 * nv);
  unsigned long long *near_list = call.alloc<unsigned long long>(2 * np);
  unsigned long long *near_count = call.alloc<unsigned long long>(1);
  SYM_CUDA(cudaMemsetAsync(near_count, 0, 8, st));
  frames_f32<<<blocks_for(nv), kThreads, 0, st>>>(xyz, nrm, dmn, dmx, nv, frames);
  check_launch();
  votes6_f32<<<blocks_for(np), kThreads, 0, st>>>(frames, pa, pb, np, model.box_size, c[0], c[1],
                                                   c[2], desc, near_list, near_count);
  check_launch();
  votes6_near_pi<<<152 * 8, kThreads, 0, st>>>(frames, pa, pb, model.box_size, c[0], c[1], c[2],
                                               desc, near_list, near_count);
  check_launch();
  call.launched(3);
}

// Reflection mode: the indices of the np pairs whose mirrored frames agree
// (plane_flags, in FP64), in pair order, into list; returns their number.
uint64_t plane_vote_pairs(Call &call, const double *xyz, const double *nrm, const double *dmn,
                          uint64_t nv, const int32_t *pa, const int32_t *pb, uint64_t np,
                          int32_t *list) {
  cudaStream_t st = call.stream();
  uint8_t *flags = call.alloc<uint8_t>(std::max<uint64_t>(np, 1));
  uint64_t *count = call.alloc<uint64_t>(1);
  if (np) {
    plane_flags<<<blocks_for(np), kThreads, 0, st>>>(xyz, nrm, dmn, nv, pa, pb, np, flags);
    check_launch();
    call.launched();
  }
  compact_indices(call, flags, np, list, count);
  uint64_t q = 0;
  call.d2h(&q, count, 8);
  call.sync();
  return q;
}

// keep[i]: item i of n enters the subsample (probability p, from a hash of
// i and the seed: the same items for every precision and every run).
__global__ void subsample_flags(uint64_t n, double p, uint64_t seed, uint8_t *keep) {
  const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t z = i + seed * 0x9E3779B97F4A7C15ull + 0x9E3779B97F4A7C15ull;  // splitmix64
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  keep[i] = double(z >> 11) * (1.0 / 9007199254740992.0) < p;
}

// K distinct vote indices drawn uniformly (Floyd's algorithm), ascending.
std::vector<int64_t> draw_seeds(uint64_t q, uint64_t k, uint64_t seed) {
  std::mt19937_64 rng(seed);
  std::vector<int64_t> pool;
  std::vector<char> taken(q, 0);
  for (uint64_t j = q - k; j < q; ++j) {
    uint64_t t = rng() % (j + 1);
    uint64_t pick = taken[t] ? j : t;
    pool.push_back(int64_t(pick));
    taken[pick] = 1;
  }
  std::sort(pool.begin(), pool.end());
  return pool;
}

__global__ void ranks_of(const int32_t *rank, const int64_t *seeds, uint64_t k, int64_t *out) {
  uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < k) out[i] = rank[seeds[i]];
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

// `sample` (ns host ids) is the area-weighted sample; with sample_rng set it
// is drawn here instead, on the device from the mesh's weights (sampling.cu).
// The motion of a mode position d (6-D): for a reflection vote the
// reference's decode of a plane cluster (clustering.cpp:117-124), for a
// rigid one the rotation exp(2 d[0..2]) and the translation that maps the
// model centre as the centred translation d[3..5] says.
void decode_mode(const double *d, bool reflection, const sym_model_context &model,
                 sym_cluster_record &rec) {
  const double *c = model.center;
  rec = sym_cluster_record{};
  if (reflection) {  // the reference's decode, clustering.cpp:117-124
    const D3 nr{d[0], d[1], d[2]};
    const double len = norm(nr);
    const D3 n = unit(nr);
    const double off = d[3] * model.box_size / len - dot(n, D3{c[0], c[1], c[2]});
    const M3 R = mirror(n);
    rec.reflection = 1;
    rec.plane_normal[0] = n.x, rec.plane_normal[1] = n.y, rec.plane_normal[2] = n.z;
    rec.plane_offset = off;
    for (int j = 0; j < 9; ++j) rec.rotation[j] = R.m[j];
    rec.translation[0] = -2 * off * n.x, rec.translation[1] = -2 * off * n.y;
    rec.translation[2] = -2 * off * n.z;
  } else {
    double w[3] = {2 * d[0], 2 * d[1], 2 * d[2]}, R[9];
    exp_map(w, R);
    for (int j = 0; j < 9; ++j) rec.rotation[j] = R[j];
    for (int x = 0; x < 3; ++x) {
      double rc = R[x * 3] * c[0] + R[x * 3 + 1] * c[1] + R[x * 3 + 2] * c[2];
      rec.translation[x] = d[3 + x] * model.box_size + c[x] - rc;
    }
  }
}

// Modes of one mesh from the final seed positions (host, k x 8; any
// offset of a fused run removed): greedy merge, support counts over the
// vote set (positions shifted by `offset` when not null), ranking by
// support, and the top records.  Fills r.modes, r.clusters, r.records,
// r.support and r.precise; returns the merged positions and the ranking.
void mode_phase(Call &call, const sym_mesh_handle &h, const VoteSet &vs,
                const std::vector<float> &means, const std::vector<uint8_t> &state, uint64_t k,
                double h2, bool reflection, const float *offset, const sym_options &o,
                sym_fast_result &r, std::vector<double> &mode_pos, std::vector<uint64_t> &rank) {
  // ---- modes: greedy merge (h^2/4, first mode wins) + support
  // Greedy merge in seed order: a seed joins the earliest-created mode within
  // h/2 (squared distance < h^2/4).  Candidates come from a window of the
  // modes sorted by their first coordinate.  Newton-converged seeds (a mode
  // with a well-defined position) go first and average into their mode;
  // the other seeds then join a mode within h/2 without moving it, or start
  // a mode of their own (averaged only with seeds of the same kind).
  mode_pos.clear();
  std::vector<uint64_t> mode_seeds;
  std::vector<uint8_t> mode_precise;
  std::multimap<double, uint64_t> by_x;
  const double half = 0.5 * std::sqrt(h2) * (1 + 1e-12);
  for (int pass = 0; pass < 2; ++pass)
    for (uint64_t i = 0; i < k; ++i) {
      if (state[i] == kExhausted || (state[i] == kConverged) != (pass == 0)) continue;
      bool finite = true;
      for (int d = 0; d < 6; ++d) finite = finite && std::isfinite(means[i * 8 + d]);
      if (!finite) continue;  // no mode (and no NaN key in the ordered index)
      double x0 = means[i * 8];
      int64_t hit = -1;
      for (auto it = by_x.lower_bound(x0 - half); it != by_x.end() && it->first <= x0 + half; ++it) {
        uint64_t m = it->second;
        if (hit >= 0 && int64_t(m) > hit) continue;
        double d2 = 0;
        for (int d = 0; d < 6; ++d) {
          double e = double(means[i * 8 + d]) - mode_pos[m * 6 + d];
          d2 += e * e;
        }
        if (d2 < h2 / 4) hit = int64_t(m);
      }
      if (hit < 0) {
        for (int d = 0; d < 6; ++d) mode_pos.push_back(means[i * 8 + d]);
        mode_seeds.push_back(1);
        mode_precise.push_back(pass == 0);
        by_x.emplace(mode_pos[(mode_seeds.size() - 1) * 6], mode_seeds.size() - 1);
      } else if (bool(mode_precise[hit]) != (pass == 0)) {
        ++mode_seeds[hit];  // a settled seed in a precise mode: counted, not averaged
      } else {
        double n = double(mode_seeds[hit]);
        double old_x = mode_pos[hit * 6];
        for (int d = 0; d < 6; ++d)
          mode_pos[hit * 6 + d] = (n * mode_pos[hit * 6 + d] + means[i * 8 + d]) / (n + 1);
        ++mode_seeds[hit];
        auto range = by_x.equal_range(old_x);
        for (auto it = range.first; it != range.second; ++it)
          if (it->second == uint64_t(hit)) {
            by_x.erase(it);
            break;
          }
        by_x.emplace(mode_pos[hit * 6], uint64_t(hit));
      }
    }
  uint64_t nm = mode_seeds.size();
  r.modes = nm;
  std::vector<uint64_t> support(nm, 0);
  if (nm) {
    std::vector<float> mp(nm * 8, 0.f);
    for (uint64_t m = 0; m < nm; ++m)
      for (int d = 0; d < 6; ++d) mp[m * 8 + d] = float(mode_pos[m * 6 + d] + (offset ? offset[d] : 0.f));
    float *dmodes = call.upload(mp.data(), mp.size());
    unsigned long long *dsup = call.alloc<unsigned long long>(nm);
    count_within(call, vs, dmodes, nm, h2, dsup);
    call.d2h(support.data(), dsup, nm * 8);
    call.sync();
  }
  rank.assign(nm, 0);
  for (uint64_t m = 0; m < nm; ++m) rank[m] = m;
  std::stable_sort(rank.begin(), rank.end(), [&](uint64_t a, uint64_t b) { return support[a] > support[b]; });
  uint64_t nc = std::min<uint64_t>({nm, uint64_t(std::max(o.max_clusters, 0)), SYM_FAST_MAX_CLUSTERS});
  r.clusters = nc;
  for (uint64_t i = 0; i < nc; ++i) {
    decode_mode(&mode_pos[rank[i] * 6], reflection, h.model, r.records[i]);
    r.support[i] = support[rank[i]];
    r.precise[i] = mode_precise[rank[i]];
  }
}

// The stages before the mean shift on one resident mesh: curvature, the
// area-weighted sample (the caller's, or drawn on the device with
// sample_rng) and its prune, exact pairing, and the votes as 8-float records
// (*desc_out; *desc64_out in FP64 as well when want64).  Fills the counts of
// `r` and marks the clock at 1-4; returns the number of votes.
uint64_t vote_phase(Call &call, sym_mesh_handle &h, const int32_t *sample, uint64_t ns,
                    const sym_options &o, const sym_fast_options &fo, sym_fast_result &r,
                    sym_rng *sample_rng, bool want64, StageClock &clock, float **desc_out,
                    double **desc64_out) {
  cudaStream_t st = call.stream();
  const uint64_t nv = h.nv;
  *desc_out = nullptr;
  *desc64_out = nullptr;
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
                   o.smoothing, f, h.host_edges.empty() ? nullptr : h.host_edges.data());
  clock.mark(1);
  // ---- area-weighted sample and its prune
  int32_t *dsample = nullptr;
  if (sample_rng) {
    dsample = call.alloc<int32_t>(nv);
    ns = sample_device(call, h.w, nv, o.sample_ratio, *sample_rng, dsample);
  } else {
    dsample = call.upload(sample, ns);
  }
  int32_t *pruned = call.alloc<int32_t>(ns);
  uint64_t *pcount = call.alloc<uint64_t>(1);
  prune_device(call, dsample, ns, f.kmin, f.kmax, valid, o.prune, pruned, pcount);
  uint64_t s = 0;
  call.d2h(&s, pcount, 8);
  call.sync();
  r.sampled = ns;
  r.pruned = s;
  clock.mark(2);
  // ---- (b) pairing + 6-D votes
  int32_t *pa = nullptr, *pb = nullptr;
  uint64_t np = pairing_device(call, pruned, s, h.xyz, nv, f.kmin, f.kmax, o.pair_threshold,
                               h.model.box_size, o.max_pairs, &pa, &pb);
  r.pairs = np;
  clock.mark(3);
  const bool reflection = fo.mode == SYM_REFLECTION;
  if (fo.mode != SYM_RIGID && !reflection) fail(SYM_INVALID_ARGUMENT, "unknown detection mode");
  // uniform subsample of n items (the parallel arrays a and, when not null,
  // b) to about vote_cap votes, order preserved; returns the kept count
  auto subsample = [&](uint64_t n, uint64_t votes_per_item, int32_t *&a, int32_t *&b) -> uint64_t {
    if (!fo.vote_cap || n * votes_per_item <= fo.vote_cap) return n;
    const double p = double(fo.vote_cap) / double(n * votes_per_item);
    uint8_t *keep = call.alloc<uint8_t>(n);
    subsample_flags<<<blocks_for(n), kThreads, 0, st>>>(n, p, fo.seed_rng, keep);
    check_launch();
    call.launched();
    int32_t *na = call.alloc<int32_t>(n), *nb = b ? call.alloc<int32_t>(n) : nullptr;
    uint64_t *cnt = call.alloc<uint64_t>(2);
    compact_values(call, keep, a, n, na, cnt);
    if (b) compact_values(call, keep, b, n, nb, cnt + 1);
    uint64_t kept = 0;
    call.d2h(&kept, cnt, 8);
    call.sync();
    a = na, b = nb;
    return kept;
  };
  if (!reflection) np = subsample(np, 2, pa, pb);
  int32_t *plane_list = nullptr;
  uint64_t q = 2 * np;
  if (reflection) {  // one vote per pair whose mirrored frames agree
    plane_list = call.alloc<int32_t>(std::max<uint64_t>(np, 1));
    q = plane_vote_pairs(call, h.xyz, f.normal_x, f.dmin_x, nv, pa, pb, np, plane_list);
    int32_t *none = nullptr;
    q = subsample(q, 1, plane_list, none);
  }
  if (q > o.max_votes || q > uint64_t(std::numeric_limits<int32_t>::max()))
    fail(SYM_RUNTIME_ERROR, "Vote budget exceeded; lower --sample-ratio or tighten --pair-threshold");
  r.votes = q;
  if (!q) {
    clock.mark(4);
    return 0;
  }
  float *desc_raw = *desc_out = call.alloc<float>(q * 8);
  double *desc64_raw = *desc64_out = want64 ? call.alloc<double>(q * 8) : nullptr;
  const double *c = h.model.center;
  if (reflection) {
    plane_votes<float><<<blocks_for(q), kThreads, 0, st>>>(h.xyz, nv, pa, pb, plane_list, q,
                                                           h.model.box_size, c[0], c[1], c[2],
                                                           desc_raw);
    check_launch();
    if (want64) {
      plane_votes<double><<<blocks_for(q), kThreads, 0, st>>>(h.xyz, nv, pa, pb, plane_list, q,
                                                              h.model.box_size, c[0], c[1], c[2],
                                                              desc64_raw);
      check_launch();
    }
    call.launched(want64 ? 2 : 1);
  } else {
    rigid_votes_f32(call, h.xyz, f.normal_x, f.dmin_x, f.dmax_x, nv, pa, pb, np, h.model, desc_raw);
    if (want64) {
      votes6<double><<<blocks_for(np), kThreads, 0, st>>>(h.xyz, f.normal_x, f.dmin_x, f.dmax_x,
                                                          nv, pa, pb, np, h.model.box_size, c[0],
                                                          c[1], c[2], desc64_raw);
      check_launch();
      call.launched();
    }
  }
  clock.mark(4);
  return q;
}

void detect_fast(Call &call, sym_mesh_handle &h, const int32_t *sample, uint64_t ns,
                 const sym_options &o, const sym_fast_options &fo, sym_fast_result &r,
                 sym_rng *sample_rng = nullptr) {
  r = sym_fast_result{};
  cudaStream_t st = call.stream();
  StageClock clock(st);
  clock.mark(0);
  const bool reflection = fo.mode == SYM_REFLECTION;
  const bool want64 = fo.reference_seeds > 0;
  float *desc_raw = nullptr;
  double *desc64_raw = nullptr;
  const uint64_t q = vote_phase(call, h, sample, ns, o, fo, r, sample_rng, want64, clock,
                                &desc_raw, &desc64_raw);
  if (!q) return;
  // ---- Morton sort into chunks
  Tuning tuning;
  if (fo.vote_bits) tuning.vote_bits = fo.vote_bits;
  if (fo.simt_blocks_per_sm) tuning.simt_blocks_per_sm = fo.simt_blocks_per_sm;
  if (fo.tc_ctas_per_sm) tuning.tc_ctas_per_sm = fo.tc_ctas_per_sm;
  if (fo.check_interval) tuning.check_interval = fo.check_interval;
  VoteSet vs = build_vote_set(call, desc_raw, desc64_raw, q, tuning);
  if (fo.kernel != SYM_KERNEL_EPANECHNIKOV && fo.kernel != SYM_KERNEL_GAUSSIAN)
    fail(SYM_INVALID_ARGUMENT, "unknown mean-shift kernel");
  vs.kernel_k = fo.kernel == SYM_KERNEL_GAUSSIAN ? kGauss2 : 0.0;
  clock.mark(5);
  // ---- (c) mean shift from K seeds (uniform draw of distinct votes)
  uint64_t k = std::min<uint64_t>(uint64_t(std::max(fo.seeds, 1)), q);
  std::vector<int64_t> seeds = draw_seeds(q, k, fo.seed_rng);
  int64_t *dseeds = call.upload(seeds.data(), k);
  int64_t *seed_rank = call.alloc<int64_t>(k);
  ranks_of<<<blocks_for(k), kThreads, 0, st>>>(vs.rank, dseeds, k, seed_rank);
  check_launch();
  const double h2 = o.bandwidth * o.bandwidth;
  unsigned long long *evals = call.alloc<unsigned long long>(1);
  SYM_CUDA(cudaMemsetAsync(evals, 0, 8, st));
  float *m32 = call.alloc<float>(k * 8);
  uint8_t *st32 = call.alloc<uint8_t>(k);
  SYM_CUDA(cudaMemsetAsync(st32, 0, k, st));
  init_means(call, vs, seed_rank, k, m32);
  int bulk = 0, polish = 0;
  double tc_evals = 0;
  cudaEvent_t ph[3];
  for (auto &e : ph) cudaEventCreate(&e);
  cudaEventRecord(ph[0], st);
  // approach phase (BF16 tensor cores or FP32 SIMT), then the same FP32
  // polish for both forms: kNear seeds take Newton steps, kMoving ones keep
  // approaching
  bool tensor = fo.precision == SYM_MS_BF16_REFINED &&
                meanshift_bf16_bulk(call, vs, m32, st32, k, h2, fo.max_iterations, &bulk, &tc_evals,
                                    r.bulk_trace, 320, &r.tc_kernel_ms, &r.tc_launches,
                                    &r.seed_iterations);
  r.tc_evaluations = tc_evals;
  if (!tensor)
    bulk = shift(call, vs, m32, st32, k, h2, fo.max_iterations, false, &r.seed_iterations, evals,
                 r.bulk_trace, 320);
  cudaEventRecord(ph[1], st);
  polish = shift(call, vs, m32, st32, k, h2, fo.polish_iterations, true, &r.seed_iterations, evals,
                 r.polish_trace, 320);
  cudaEventRecord(ph[2], st);
  cudaEventSynchronize(ph[2]);
  {
    float a = 0, b = 0;
    cudaEventElapsedTime(&a, ph[0], ph[1]);
    cudaEventElapsedTime(&b, ph[1], ph[2]);
    r.bulk_ms = a;
    r.polish_ms = b;
  }
  for (auto &e : ph) cudaEventDestroy(e);
  r.iterations = bulk;
  r.polish_iterations = polish;
  unsigned long long ev = 0;
  call.d2h(&ev, evals, 8);
  std::vector<float> means(k * 8);
  std::vector<uint8_t> state(k);
  call.d2h(means.data(), m32, k * 8 * 4);
  call.d2h(state.data(), st32, k);
  call.sync();
  r.mean_shift_pairs = double(ev) + tc_evals;
  r.h2d_bytes = call.ctx->metrics.current.h2d_bytes;
  r.d2h_bytes = call.ctx->metrics.current.d2h_bytes;
  clock.mark(6);
  // ---- FP64 reference on the first seeds (mode error)
  if (want64) {
    uint64_t k64 = std::min<uint64_t>(k, uint64_t(fo.reference_seeds));
    double *m64 = call.alloc<double>(k64 * 8);
    uint8_t *st64 = call.alloc<uint8_t>(k64);
    SYM_CUDA(cudaMemsetAsync(st64, 0, k64, st));
    init_means(call, vs, seed_rank, k64, m64);
    shift(call, vs, m64, st64, k64, h2, fo.max_iterations, false, nullptr, nullptr);
    shift(call, vs, m64, st64, k64, h2, fo.polish_iterations, true, nullptr, nullptr);
    std::vector<double> hm(k64 * 8);
    std::vector<uint8_t> hs64(k64);
    call.d2h(hm.data(), m64, k64 * 8 * 8);
    call.d2h(hs64.data(), st64, k64);
    call.sync();
    // every reference seed is compared; the pair of final states puts it
    // in one of three groups: Newton-converged in both runs (a mode with a
    // well-defined position), settled on a ridge in either run, or still
    // unconverged (or without weight) in either
    double emax = 0, esum = 0, all_max = 0, all_sum = 0, settled_max = 0, open_max = 0;
    uint64_t compared = 0, within = 0, within_all = 0, settled = 0, open = 0;
    for (uint64_t i = 0; i < k64; ++i) {
      double num = 0, den = 0;
      for (int d = 0; d < 6; ++d) {
        double e = double(means[i * 8 + d]) - hm[i * 8 + d];
        num += e * e, den += hm[i * 8 + d] * hm[i * 8 + d];
      }
      double rel = std::sqrt(num) / std::max(std::sqrt(den), 1e-300);
      if (!std::isfinite(rel)) rel = std::numeric_limits<double>::infinity();
      all_max = std::max(all_max, rel), all_sum += rel, within_all += rel <= 1e-4;
      const bool both = hs64[i] == kConverged && state[i] == kConverged;
      const bool ridge = !both && (hs64[i] == kConverged || hs64[i] == kSettled) &&
                         (state[i] == kConverged || state[i] == kSettled);
      if (both) {
        emax = std::max(emax, rel), esum += rel, ++compared;
        within += rel <= 1e-4;
      } else if (ridge) {
        settled_max = std::max(settled_max, rel), ++settled;
      } else {
        open_max = std::max(open_max, rel), ++open;
      }
    }
    r.mode_error_max = emax;
    r.mode_error_mean = compared ? esum / compared : 0;
    r.modes_compared = compared;
    r.modes_within = within;
    r.seeds_compared = k64;
    r.seeds_within = within_all;
    r.seeds_settled = settled;
    r.seeds_unconverged = open;
    r.mode_error_all_max = all_max;
    r.mode_error_all_mean = k64 ? all_sum / k64 : 0;
    r.mode_error_settled_max = settled_max;
    r.mode_error_unconverged_max = open_max;
  }
  clock.mark(7);
  std::vector<double> mode_pos;
  std::vector<uint64_t> rank;
  mode_phase(call, h, vs, means, state, k, h2, reflection, nullptr, o, r, mode_pos, rank);
  const uint64_t nc = r.clusters;
  auto decode = [&](const double *d, sym_cluster_record &rec) {
    decode_mode(d, reflection, h.model, rec);
  };
  // each reported motion against FP64: the FP64 mean shift restarted from
  // the mode's position (approach and polish as above) reaches the FP64 mode
  // the GPU's approximates; the relative error of the motion [R, t / box]
  sym_cluster_record rec64[SYM_FAST_MAX_CLUSTERS];
  auto motion_error = [&](const sym_cluster_record &a, const sym_cluster_record &b) {
    double num = 0, den = 0;
    for (int j = 0; j < 12; ++j) {
      const double x = j < 9 ? a.rotation[j] : a.translation[j - 9] / h.model.box_size;
      const double y = j < 9 ? b.rotation[j] : b.translation[j - 9] / h.model.box_size;
      num += (x - y) * (x - y), den += y * y;
    }
    return std::sqrt(num) / std::max(std::sqrt(den), 1e-300);
  };
  if (want64 && nc) {
    std::vector<double> start(nc * 8, 0.0);
    for (uint64_t i = 0; i < nc; ++i) {
      double n2 = 0;
      for (int d = 0; d < 6; ++d) {
        start[i * 8 + d] = mode_pos[rank[i] * 6 + d];
        n2 += start[i * 8 + d] * start[i * 8 + d];
      }
      start[i * 8 + 6] = n2;
    }
    double *m64 = call.upload(start.data(), nc * 8);
    uint8_t *st64 = call.alloc<uint8_t>(nc);
    SYM_CUDA(cudaMemsetAsync(st64, 0, nc, st));
    shift(call, vs, m64, st64, nc, h2, fo.max_iterations, false, nullptr, nullptr);
    shift(call, vs, m64, st64, nc, h2, fo.polish_iterations, true, nullptr, nullptr);
    call.d2h(start.data(), m64, nc * 64);
    call.sync();
    for (uint64_t i = 0; i < nc; ++i) {
      double d6[6];
      for (int d = 0; d < 6; ++d) d6[d] = start[i * 8 + d];
      decode(d6, rec64[i]);
      r.transform_error[i] = motion_error(r.records[i], rec64[i]);
      r.transform_error_max = std::max(r.transform_error_max, r.transform_error[i]);
    }
  }
  clock.mark(8);
  // ---- (d) verification of the top modes
  if (fo.verify && nc) {
    verification_fast(call, h.surface(), r.records, nc, o.verify_threshold * h.model.box_size,
                      fo.refine, h.model.center, r.coverage, r.rms, r.patches,
                      &r.verify_undecided, &r.verify_fp64_rows);
    if (want64 && fo.refine > 0) {  // the same refinement of the FP64 motions
      double cov[SYM_FAST_MAX_CLUSTERS], rms[SYM_FAST_MAX_CLUSTERS];
      uint32_t patches[2 * SYM_FAST_MAX_CLUSTERS];
      verification_fast(call, h.surface(), rec64, nc, o.verify_threshold * h.model.box_size,
                        fo.refine, h.model.center, cov, rms, patches, nullptr, nullptr);
      for (uint64_t i = 0; i < nc; ++i) {
        r.transform_error_refined[i] = motion_error(r.records[i], rec64[i]);
        r.transform_error_refined_max =
            std::max(r.transform_error_refined_max, r.transform_error_refined[i]);
      }
    }
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

// The vote records of the throughput path for given pairs (sym_fast_votes).
uint64_t fast_votes_host(Call &call, const sym_points_view &pos, const sym_features_view &fv,
                         const sym_pairs_view &pr, const sym_model_context &model, int mode,
                         float *out, int32_t *pair_of) {
  const uint64_t nv = pos.count, np = pr.count;
  if (fv.count != nv || fv.normal.count != nv || fv.dmin.count != nv || fv.dmax.count != nv)
    fail(SYM_INVALID_ARGUMENT, "SoA component lengths differ");
  if (mode != SYM_RIGID && mode != SYM_REFLECTION) fail(SYM_INVALID_ARGUMENT, "unknown detection mode");
  for (uint64_t i = 0; i < np; ++i)
    if (pr.a[i] < 0 || pr.b[i] < 0 || uint64_t(pr.a[i]) >= nv || uint64_t(pr.b[i]) >= nv)
      fail(SYM_INVALID_ARGUMENT, "pair vertex index out of range");
  if (!np) return 0;
  const double *xyz = upload_points(call, pos), *nrm = upload_points(call, fv.normal),
               *dmn = upload_points(call, fv.dmin), *dmx = upload_points(call, fv.dmax);
  const int32_t *pa = call.upload(pr.a, np), *pb = call.upload(pr.b, np);
  uint64_t q = 0;
  if (mode == SYM_RIGID) {
    q = 2 * np;
    float *desc = call.alloc<float>(q * 8);
    rigid_votes_f32(call, xyz, nrm, dmn, dmx, nv, pa, pb, np, model, desc);
    call.d2h(out, desc, q * 32);
    for (uint64_t v = 0; v < q; ++v) pair_of[v] = int32_t(v / 2);
  } else {
    int32_t *list = call.alloc<int32_t>(np);
    q = plane_vote_pairs(call, xyz, nrm, dmn, nv, pa, pb, np, list);
    if (q) {
      float *desc = call.alloc<float>(q * 8);
      const double *c = model.center;
      plane_votes<float><<<blocks_for(q), kThreads, 0, call.stream()>>>(
          xyz, nv, pa, pb, list, q, model.box_size, c[0], c[1], c[2], desc);
      check_launch();
      call.launched();
      call.d2h(out, desc, q * 32);
      call.d2h(pair_of, list, q * 4);
    }
  }
  call.check_status("fast_votes");
  return q;
}

// ------------------------------------------------- many meshes, one mean shift
// Vote-space tiling: every mesh's votes (each component within [-2, 2]: a
// rotation part of at most pi/2, a centred translation of at most 2 boxes,
// a unit normal and an offset of at most one box) are moved by their own
// offset on a grid of pitch 8 -- one of {-12, -4, 4, 12} per coordinate,
// 4,096 cells -- so votes of different meshes lie at least 4 apart, beyond
// any bandwidth below 2: their weights are exactly zero and the chunk tests
// never pair a seed with another mesh's chunk.  One mean-shift run then
// serves every mesh's seeds, one launch per kernel and iteration.
constexpr uint64_t kFusedMax = 4096;

void fused_offset(uint64_t i, float off[6]) {
  static const float steps[4] = {-12.f, -4.f, 4.f, 12.f};
  for (int d = 0; d < 6; ++d) off[d] = steps[(i >> (2 * d)) & 3];
}

__global__ void place_votes(const float *desc, uint64_t q, float o0, float o1, float o2, float o3,
                            float o4, float o5, float *out) {
  const uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (v >= q) return;
  const float off[6] = {o0, o1, o2, o3, o4, o5};
  float x[8], n2 = 0;
  for (int d = 0; d < 6; ++d) x[d] = desc[v * 8 + d] + off[d], n2 += x[d] * x[d];
  x[6] = n2, x[7] = 0;
  float4 *o = reinterpret_cast<float4 *>(out + v * 8);
  o[0] = make_float4(x[0], x[1], x[2], x[3]);
  o[1] = make_float4(x[4], x[5], x[6], x[7]);
}

// The first n helper contexts of ctx, created on first use.
const std::vector<sym_context *> &helper_contexts(sym_context *ctx, int n) {
  while (int(ctx->helpers.size()) < n) {
    sym_context *h = nullptr;
    const sym_status st = sym_context_create(ctx->device, &h);
    if (st != SYM_OK) fail(st, "helper context: " + sym_error_text);
    ctx->helpers.push_back(h);
  }
  return ctx->helpers;
}

constexpr int kFusedWorkers = 8;  // host threads (helper contexts) for the per-mesh finish

void detect_fast_fused(Call &call, sym_batch_item *items, uint64_t count, sym_fused_stats &stats) {
  stats = sym_fused_stats{};
  if (!count) return;
  if (count > kFusedMax) fail(SYM_INVALID_ARGUMENT, "fused detection takes at most 4,096 meshes");
  const sym_fast_options &f0 = *items[0].fast;
  const double h = items[0].options->bandwidth, h2 = h * h;
  for (uint64_t i = 0; i < count; ++i) {
    const sym_fast_options &f = *items[i].fast;
    if (!items[i].mesh || !items[i].options || !items[i].out)
      fail(SYM_INVALID_ARGUMENT, "batch item without mesh, options or result");
    if (f.precision != f0.precision || f.kernel != f0.kernel ||
        f.max_iterations != f0.max_iterations || f.polish_iterations != f0.polish_iterations ||
        f.vote_bits != f0.vote_bits || f.simt_blocks_per_sm != f0.simt_blocks_per_sm ||
        f.tc_ctas_per_sm != f0.tc_ctas_per_sm || f.check_interval != f0.check_interval ||
        items[i].options->bandwidth != h)
      fail(SYM_INVALID_ARGUMENT, "fused detection needs one precision, kernel, iteration counts, "
                                 "launch shape and bandwidth for every mesh");
    if (f.reference_seeds) fail(SYM_INVALID_ARGUMENT, "fused detection runs no FP64 reference seeds");
    if (f.kernel != SYM_KERNEL_EPANECHNIKOV && f.kernel != SYM_KERNEL_GAUSSIAN)
      fail(SYM_INVALID_ARGUMENT, "unknown mean-shift kernel");
  }
  if (!(h > 0 && h < 2)) fail(SYM_INVALID_ARGUMENT, "fused detection needs a bandwidth below 2");
  cudaStream_t st = call.stream();
  cudaEvent_t ev[5];
  for (auto &e : ev) SYM_CUDA(cudaEventCreate(&e));
  SYM_CUDA(cudaEventRecord(ev[0], st));
  // ---- the stages before the mean shift, mesh by mesh on helper contexts:
  // one Call per helper thread for the whole phase, so each mesh's votes
  // stay in its helper's workspace (an arena is reset only when the next
  // Call on that context begins, after the shared mean shift) until the
  // main stream has gathered them; offsets follow the meshes' order
  struct Part {
    float *desc = nullptr;
    uint64_t q = 0, base = 0, k = 0, seed_base = 0;
    bool ok = false, done = false;
  };
  std::vector<Part> parts(count);
  const int workers = int(std::min<uint64_t>(count, kFusedWorkers));
  const std::vector<sym_context *> &helpers = helper_contexts(call.ctx, workers);
  {
    std::atomic<uint64_t> next{0};
    std::string failure;
    std::mutex failure_lock;
    auto prepare_votes = [&](sym_context *hctx) {
      try {
        Call hcall(hctx, "detect_fast_fused");
        StageClock hclock(hcall.stream());
        for (uint64_t i = next++; i < count; i = next++) {
          sym_batch_item &it = items[i];
          sym_fast_result &r = *it.out;
          r = sym_fast_result{};
          it.status = SYM_OK;
          it.message[0] = 0;
          parts[i].done = true;
          try {
            sym_rng rng;
            const bool on_device = !it.sample && it.sample_count == SYM_SAMPLE_ON_DEVICE;
            if (on_device) {
              validate_prepare_options(*it.options);
              sym_rng_seed(&rng, it.options->seed);
            } else {
              for (uint64_t j = 0; j < it.sample_count; ++j)
                if (it.sample[j] < 0 || uint64_t(it.sample[j]) >= it.mesh->nv)
                  fail(SYM_INVALID_ARGUMENT, "sample vertex index out of range");
            }
            double *unused = nullptr;
            parts[i].q = vote_phase(hcall, *it.mesh, on_device ? nullptr : it.sample,
                                    on_device ? 0 : it.sample_count, *it.options, *it.fast, r,
                                    on_device ? &rng : nullptr, false, hclock, &parts[i].desc,
                                    &unused);
            parts[i].ok = true;
          } catch (const Error &e) {
            it.status = e.status;
            std::snprintf(it.message, sizeof(it.message), "%s", e.what());
          } catch (const std::exception &e) {  // nothing may leave a worker thread
            it.status = SYM_RUNTIME_ERROR;
            std::snprintf(it.message, sizeof(it.message), "%s", e.what());
          }
        }
        hcall.sync();  // this helper's votes are complete
      } catch (const std::exception &e) {
        std::lock_guard<std::mutex> g(failure_lock);
        failure = e.what();
      }
    };
    std::vector<std::thread> pool;
    for (int w = 1; w < workers; ++w) pool.emplace_back(prepare_votes, helpers[w]);
    prepare_votes(helpers[0]);
    for (auto &t : pool) t.join();
    for (uint64_t i = 0; i < count; ++i)
      if (!parts[i].done) {  // a helper that could not start left it
        items[i].status = SYM_RUNTIME_ERROR;
        *items[i].out = sym_fast_result{};
        std::snprintf(items[i].message, sizeof(items[i].message), "%s",
                      failure.empty() ? "not processed" : failure.c_str());
      }
  }
  uint64_t total = 0;
  for (uint64_t i = 0; i < count; ++i)
    if (parts[i].ok) parts[i].base = total, total += parts[i].q;
  if (total > uint64_t(std::numeric_limits<int32_t>::max()))
    fail(SYM_RUNTIME_ERROR, "Vote budget exceeded; lower --sample-ratio or tighten --pair-threshold");
  SYM_CUDA(cudaEventRecord(ev[1], st));
  // ---- one vote set, one seed set
  std::vector<int64_t> seeds;
  if (total) {
    float *all = call.alloc<float>(total * 8);
    for (uint64_t i = 0; i < count; ++i) {
      Part &pt = parts[i];
      if (!pt.q) continue;
      float off[6];
      fused_offset(i, off);
      place_votes<<<blocks_for(pt.q), kThreads, 0, st>>>(pt.desc, pt.q, off[0], off[1], off[2],
                                                         off[3], off[4], off[5],
                                                         all + pt.base * 8);
      check_launch();
      call.launched();
      pt.k = std::min<uint64_t>(uint64_t(std::max(items[i].fast->seeds, 1)), pt.q);
      pt.seed_base = seeds.size();
      for (int64_t v : draw_seeds(pt.q, pt.k, items[i].fast->seed_rng))
        seeds.push_back(int64_t(pt.base) + v);
    }
    Tuning tuning;
    if (f0.vote_bits) tuning.vote_bits = f0.vote_bits;
    if (f0.simt_blocks_per_sm) tuning.simt_blocks_per_sm = f0.simt_blocks_per_sm;
    if (f0.tc_ctas_per_sm) tuning.tc_ctas_per_sm = f0.tc_ctas_per_sm;
    if (f0.check_interval) tuning.check_interval = f0.check_interval;
    VoteSet vs = build_vote_set(call, all, nullptr, total, tuning);
    vs.kernel_k = f0.kernel == SYM_KERNEL_GAUSSIAN ? kGauss2 : 0.0;
    const uint64_t k = seeds.size();
    int64_t *dseeds = call.upload(seeds.data(), k);
    int64_t *seed_rank = call.alloc<int64_t>(k);
    ranks_of<<<blocks_for(k), kThreads, 0, st>>>(vs.rank, dseeds, k, seed_rank);
    check_launch();
    float *m32 = call.alloc<float>(k * 8);
    uint8_t *st32 = call.alloc<uint8_t>(k);
    SYM_CUDA(cudaMemsetAsync(st32, 0, k, st));
    init_means(call, vs, seed_rank, k, m32);
    unsigned long long *evals = call.alloc<unsigned long long>(1);
    SYM_CUDA(cudaMemsetAsync(evals, 0, 8, st));
    SYM_CUDA(cudaEventRecord(ev[2], st));
    int bulk = 0, polish = 0;
    double tc_evals = 0, seed_iterations = 0;
    const bool tensor =
        f0.precision == SYM_MS_BF16_REFINED &&
        meanshift_bf16_bulk(call, vs, m32, st32, k, h2, f0.max_iterations, &bulk, &tc_evals,
                            nullptr, 0, &stats.tc_kernel_ms, &stats.tc_launches, &seed_iterations);
    if (!tensor)
      bulk = shift(call, vs, m32, st32, k, h2, f0.max_iterations, false, &seed_iterations, evals);
    SYM_CUDA(cudaEventRecord(ev[3], st));
    polish = shift(call, vs, m32, st32, k, h2, f0.polish_iterations, true, &seed_iterations, evals);
    std::vector<float> means(k * 8);
    std::vector<uint8_t> state(k);
    call.d2h(means.data(), m32, k * 32);
    call.d2h(state.data(), st32, k);
    SYM_CUDA(cudaEventRecord(ev[4], st));
    call.sync();
    stats.iterations = bulk;
    stats.polish_iterations = polish;
    stats.tc_evaluations = tc_evals;
    stats.seed_iterations = seed_iterations;
    stats.votes = total;
    stats.seeds = k;
    // ---- modes and verification, mesh by mesh on helper contexts: the
    // meshes are independent and the vote set is complete (the stream was
    // synchronised above), so a few host threads overlap their launches and
    // host round trips, each mesh in its own workspace
    std::atomic<uint64_t> next{0};
    auto finish = [&](sym_context *hctx) {
     for (uint64_t i = next++; i < count; i = next++) {
      Part &pt = parts[i];
      sym_batch_item &it = items[i];
      if (!pt.q) continue;
      sym_fast_result &r = *it.out;
      try {
        Call hcall(hctx, "detect_fast_fused");
        float off[6];
        fused_offset(i, off);
        std::vector<float> mi(pt.k * 8);
        std::vector<uint8_t> si(state.begin() + pt.seed_base, state.begin() + pt.seed_base + pt.k);
        for (uint64_t j = 0; j < pt.k; ++j)
          for (int d = 0; d < 8; ++d)
            mi[j * 8 + d] = means[(pt.seed_base + j) * 8 + d] - (d < 6 ? off[d] : 0.f);
        r.iterations = bulk;
        r.polish_iterations = polish;
        std::vector<double> mode_pos;
        std::vector<uint64_t> rank;
        mode_phase(hcall, *it.mesh, vs, mi, si, pt.k, h2, it.fast->mode == SYM_REFLECTION, off,
                   *it.options, r, mode_pos, rank);
        if (it.fast->verify && r.clusters)
          verification_fast(hcall, it.mesh->surface(), r.records, r.clusters,
                            it.options->verify_threshold * it.mesh->model.box_size,
                            it.fast->refine, it.mesh->model.center, r.coverage, r.rms, r.patches,
                            &r.verify_undecided, &r.verify_fp64_rows);
      } catch (const Error &e) {
        it.status = e.status;
        std::snprintf(it.message, sizeof(it.message), "%s", e.what());
      } catch (const std::exception &e) {  // nothing may leave a worker thread
        it.status = SYM_RUNTIME_ERROR;
        std::snprintf(it.message, sizeof(it.message), "%s", e.what());
      }
     }
    };
    std::vector<std::thread> pool;
    for (int w = 1; w < workers; ++w) pool.emplace_back(finish, helpers[w]);
    finish(helpers[0]);
    for (auto &t : pool) t.join();
  } else {
    for (int j = 2; j < 5; ++j) SYM_CUDA(cudaEventRecord(ev[j], st));
  }
  cudaEvent_t done;
  SYM_CUDA(cudaEventCreate(&done));
  SYM_CUDA(cudaEventRecord(done, st));
  SYM_CUDA(cudaEventSynchronize(done));
  float t[4] = {0, 0, 0, 0};
  cudaEventElapsedTime(&t[0], ev[0], ev[1]);
  cudaEventElapsedTime(&t[1], ev[1], ev[2]);
  cudaEventElapsedTime(&t[2], ev[2], ev[3]);
  cudaEventElapsedTime(&t[3], ev[3], ev[4]);
  // ev[4] -> done spans the per-mesh finish: the main stream is idle while
  // the helper contexts run it, so its events mark the phase's wall time
  float t_rest = 0;
  cudaEventElapsedTime(&t_rest, ev[4], done);
  stats.meshes = count;
  stats.votes_ms = t[0];
  stats.vote_set_ms = t[1];
  stats.bulk_ms = t[2];
  stats.polish_ms = t[3];
  stats.modes_verification_ms = t_rest;
  for (auto &e : ev) cudaEventDestroy(e);
  cudaEventDestroy(done);
}

}  // namespace sym

extern "C" {

void sym_fast_options_default(sym_fast_options *o) {
  *o = sym_fast_options{SYM_MS_BF16_REFINED, 2048, 7, 100, 100, 0, 1, SYM_RIGID, 0, 0, 0, 0, 0, 0,
                        SYM_KERNEL_EPANECHNIKOV};
}

sym_status sym_refine_transforms(sym_context *ctx, sym_mesh_handle *mesh,
                                 const sym_options *options, sym_cluster_record *records,
                                 uint64_t count, int32_t iterations, double *coverage,
                                 double *rms, uint32_t *patches) {
  if (!ctx || !mesh || !options || (count && (!records || !coverage || !rms || !patches)))
    return SYM_INVALID_ARGUMENT;
  try {
    sym::Call call(ctx, "refine_transforms");
    if (iterations < 0) sym::fail(SYM_INVALID_ARGUMENT, "negative refinement iterations");
    sym::verification_fast(call, mesh->surface(), records, count,
                           options->verify_threshold * mesh->model.box_size, iterations,
                           mesh->model.center, coverage, rms, patches, nullptr, nullptr);
    return SYM_OK;
  } catch (const sym::Error &e) {
    sym_error_text = e.what();
    return e.status;
  } catch (const std::exception &e) {
    sym_error_text = e.what();
    return SYM_RUNTIME_ERROR;
  }
}

sym_status sym_verification_resident(sym_context *ctx, sym_mesh_handle *mesh,
                                     const sym_clusters_view *clusters, const sym_options *options,
                                     sym_verification_result *out, uint64_t *undecided) {
  if (!ctx || !mesh || !clusters || !options || !out || (clusters->count && !clusters->records))
    return SYM_INVALID_ARGUMENT;
  *out = sym_verification_result{};
  try {
    sym::Call call(ctx, "verification");
    const uint64_t nc = clusters->count;
    if (nc && (!mesh->nv || !mesh->nf))
      sym::fail(SYM_INVALID_ARGUMENT, "verification requires a nonempty surface");
    std::vector<std::vector<int32_t>> side;
    std::vector<std::vector<std::vector<int32_t>>> patches;
    std::vector<double> coverage, rms;
    uint64_t n = 0;
    sym::verification_resident(call, mesh->surface(), clusters->records, nc,
                               options->verify_threshold * mesh->model.box_size, side, patches,
                               coverage, rms, &n);
    if (undecided) *undecided = n;
    sym::fill_verification_result(nc, side, patches, coverage, rms, *out, std::malloc);
    return SYM_OK;
  } catch (const sym::Error &e) {
    sym_error_text = e.what();
    return e.status;
  } catch (const std::exception &e) {
    sym_error_text = e.what();
    return SYM_RUNTIME_ERROR;
  }
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
    h->device = ctx->device;
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
    try {
      if (nf >= (uint64_t(1) << 30)) sym::fail(SYM_INVALID_ARGUMENT, "too many faces for the LBVH");
      sym::Call call(ctx, "mesh_load");
      h->lbvh = sym::lbvh_build(call, h->xyz, h->vn, nv, h->faces, nf);
      call.check_status("mesh_load");
      std::vector<double> hx(3 * nv);
      std::vector<int32_t> hf(3 * nf);
      std::copy(mesh->vertices.x, mesh->vertices.x + nv, hx.begin());
      std::copy(mesh->vertices.y, mesh->vertices.y + nv, hx.begin() + nv);
      std::copy(mesh->vertices.z, mesh->vertices.z + nv, hx.begin() + 2 * nv);
      std::copy(mesh->faces.v0, mesh->faces.v0 + nf, hf.begin());
      std::copy(mesh->faces.v1, mesh->faces.v1 + nf, hf.begin() + nf);
      std::copy(mesh->faces.v2, mesh->faces.v2 + nf, hf.begin() + 2 * nf);
      h->ref.start(std::move(hx), std::move(hf), nv, nf);
    } catch (...) {
      h->release();
      delete h;
      throw;
    }
    *out = h;
    return SYM_OK;
  } catch (const sym::Error &e) {
    sym_error_text = e.what();
    return e.status;
  }
}

sym_status sym_mesh_load_raw(sym_context *ctx, const sym_mesh_view *mesh,
                             const sym_options *options, sym_mesh_handle **out) {
  if (!ctx || !mesh || !options || !out) return SYM_INVALID_ARGUMENT;
  *out = nullptr;
  sym_mesh_handle *h = nullptr;
  try {
    sym::Call call(ctx, "mesh_load_raw");
    const sym::PreparedDevice p = sym::prepare_device(call, *mesh, *options);
    h = new sym_mesh_handle();
    h->device = ctx->device;
    h->host = sym_mesh_view{};  // the vertices and faces live on the device only
    h->model = p.context;
    h->nv = p.nv, h->nf = p.nf, h->ne = p.ne, h->nbr_count = p.nbr_count;
    // no host copy of the edge table: the GPU prepare emits it sorted by
    // (lo, hi), so the curvature never needs the host-side reordering
    const uint64_t nv = p.nv, nf = p.nf, ne = p.ne;
    auto pad = [](uint64_t b) { return (b + 255) & ~uint64_t(255); };
    uint64_t sizes[8] = {pad(24 * nv), pad(24 * nf), pad(24 * nv), pad(8 * nv), pad(12 * nf),
                         pad(8 * (nv + 1)), pad(4 * h->nbr_count), pad(24 * ne)};
    uint64_t total = 0;
    for (auto b : sizes) total += b;
    if (cudaMalloc(&h->block, total ? total : 256) != cudaSuccess)
      sym::fail(SYM_CUDA_ERROR, "CUDA: mesh allocation failed");
    char *q = h->block;
    h->xyz = reinterpret_cast<double *>(q), q += sizes[0];
    h->fn = reinterpret_cast<double *>(q), q += sizes[1];
    h->vn = reinterpret_cast<double *>(q), q += sizes[2];
    h->w = reinterpret_cast<double *>(q), q += sizes[3];
    h->faces = reinterpret_cast<int32_t *>(q), q += sizes[4];
    h->nbr_off = reinterpret_cast<uint64_t *>(q), q += sizes[5];
    h->nbr = reinterpret_cast<int32_t *>(q), q += sizes[6];
    h->edges = reinterpret_cast<sym_edge *>(q);
    cudaStream_t st = ctx->stream;
    auto d2d = [&](void *dst, const void *src, uint64_t bytes) {
      if (bytes) SYM_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st));
    };
    d2d(h->xyz, p.xyz, 24 * nv);
    d2d(h->fn, p.fn, 24 * nf);
    d2d(h->vn, p.vn, 24 * nv);
    d2d(h->w, p.w, 8 * nv);
    d2d(h->faces, p.faces, 12 * nf);
    d2d(h->nbr_off, p.nbr_off, 8 * (nv + 1));
    d2d(h->nbr, p.nbr, 4 * h->nbr_count);
    d2d(h->edges, p.edges, 24 * ne);
    if (nf >= (uint64_t(1) << 30)) sym::fail(SYM_INVALID_ARGUMENT, "too many faces for the LBVH");
    h->lbvh = sym::lbvh_build(call, h->xyz, h->vn, nv, h->faces, nf);
    call.check_status("mesh_load_raw");
    {  // the prepared vertices and faces to the host thread that builds the
       // reference-order BVH while the GPU works
      std::vector<double> hx(3 * nv);
      std::vector<int32_t> hf(3 * nf);
      call.d2h(hx.data(), h->xyz, 24 * nv);
      call.d2h(hf.data(), h->faces, 12 * nf);
      call.sync();
      h->ref.start(std::move(hx), std::move(hf), nv, nf);
    }
    *out = h;
    return SYM_OK;
  } catch (const sym::Error &e) {
    if (h) {
      cudaStreamSynchronize(ctx->stream);
      h->release();
      delete h;
    }
    sym_error_text = e.what();
    return e.status;
  } catch (const std::exception &e) {
    if (h) {
      cudaStreamSynchronize(ctx->stream);
      h->release();
      delete h;
    }
    sym_error_text = e.what();
    return SYM_RUNTIME_ERROR;
  }
}

void sym_mesh_free(sym_mesh_handle *h) {
  if (!h) return;
  // every stream of the device may still read the mesh (any context can
  // use it); the loading context may already be gone
  cudaSetDevice(h->device);
  cudaDeviceSynchronize();
  h->release();
  delete h;
}

namespace {
// 6-D votes given as q x 6 doubles -> the 8-wide FP32 / FP64 layout.
__global__ void pack_votes(const double *in, uint64_t q, float *d32, double *d64) {
  uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (v >= q) return;
  double n2 = 0;
  float n2f = 0;
  for (int d = 0; d < 6; ++d) {
    double x = in[v * 6 + d];
    d64[v * 8 + d] = x, d32[v * 8 + d] = float(x);
    n2 += x * x, n2f += float(x) * float(x);
  }
  d64[v * 8 + 6] = n2, d64[v * 8 + 7] = 0;
  d32[v * 8 + 6] = n2f, d32[v * 8 + 7] = 0;
}
}  // namespace

sym_status sym_meanshift6(sym_context *ctx, const double *votes, uint64_t q, const int64_t *seeds,
                          uint64_t k, double bandwidth, int32_t precision, int32_t max_iterations,
                          int32_t polish_iterations, int32_t kernel, double *means_out,
                          uint8_t *state_out, int32_t *iterations_out) {
  if (!ctx || (q && !votes) || (k && (!seeds || !means_out || !state_out)) || !iterations_out)
    return SYM_INVALID_ARGUMENT;
  try {
    sym::Call call(ctx, "mean_shift6");
    if (!(bandwidth > 0) || max_iterations < 1 || polish_iterations < 0)
      sym::fail(SYM_INVALID_ARGUMENT, "Invalid parameter range; see --help");
    if (kernel != SYM_KERNEL_EPANECHNIKOV && kernel != SYM_KERNEL_GAUSSIAN)
      sym::fail(SYM_INVALID_ARGUMENT, "unknown mean-shift kernel");
    if (q > uint64_t(std::numeric_limits<int32_t>::max()))
      sym::fail(SYM_OVERFLOW, "vote ids exceed int32 range");
    for (uint64_t i = 0; i < k; ++i)
      if (seeds[i] < 0 || uint64_t(seeds[i]) >= q)
        sym::fail(SYM_INVALID_ARGUMENT, "seed vote index out of range");
    iterations_out[0] = iterations_out[1] = 0;
    if (!k) return SYM_OK;
    cudaStream_t st = call.stream();
    double *raw = call.upload(votes, q * 6);
    float *d32 = call.alloc<float>(q * 8);
    double *d64 = call.alloc<double>(q * 8);
    pack_votes<<<sym::blocks_for(q), sym::kThreads, 0, st>>>(raw, q, d32, d64);
    sym::check_launch();
    sym::VoteSet vs = sym::build_vote_set(call, d32, d64, q);
    vs.kernel_k = kernel == SYM_KERNEL_GAUSSIAN ? sym::kGauss2 : 0.0;
    int64_t *dseeds = call.upload(seeds, k);
    int64_t *rank = call.alloc<int64_t>(k);
    sym::ranks_of<<<sym::blocks_for(k), sym::kThreads, 0, st>>>(vs.rank, dseeds, k, rank);
    sym::check_launch();
    uint8_t *state = call.alloc<uint8_t>(k);
    SYM_CUDA(cudaMemsetAsync(state, 0, k, st));
    double h2 = bandwidth * bandwidth;
    std::vector<double> out(k * 8);
    if (precision == SYM_MS_FP64) {
      double *m = call.alloc<double>(k * 8);
      sym::init_means(call, vs, rank, k, m);
      iterations_out[0] =
          sym::shift(call, vs, m, state, k, h2, max_iterations, false, nullptr, nullptr);
      iterations_out[1] =
          sym::shift(call, vs, m, state, k, h2, polish_iterations, true, nullptr, nullptr);
      call.d2h(out.data(), m, k * 8 * 8);
    } else {
      float *m = call.alloc<float>(k * 8);
      sym::init_means(call, vs, rank, k, m);
      int bulk = 0;
      double ev = 0;
      if (!(precision == SYM_MS_BF16_REFINED &&
            sym::meanshift_bf16_bulk(call, vs, m, state, k, h2, max_iterations, &bulk, &ev)))
        bulk = sym::shift(call, vs, m, state, k, h2, max_iterations, false, nullptr, nullptr);
      iterations_out[0] = bulk;
      iterations_out[1] =
          sym::shift(call, vs, m, state, k, h2, polish_iterations, true, nullptr, nullptr);
      std::vector<float> mf(k * 8);
      call.d2h(mf.data(), m, k * 8 * 4);
      call.sync();
      for (uint64_t i = 0; i < k * 8; ++i) out[i] = mf[i];
    }
    call.d2h(state_out, state, k);
    call.check_status("mean_shift6");
    for (uint64_t i = 0; i < k; ++i)  // a seed between Newton retries is near a mode
      if (sym::is_near(state_out[i])) state_out[i] = sym::kNear;
    for (uint64_t i = 0; i < k; ++i)
      for (int d = 0; d < 6; ++d) means_out[i * 6 + d] = out[i * 8 + d];
    return SYM_OK;
  } catch (const sym::Error &e) {
    sym_error_text = e.what();
    return e.status;
  } catch (const std::exception &e) {
    sym_error_text = e.what();
    return SYM_RUNTIME_ERROR;
  }
}

sym_status sym_tc_selftest(sym_context *ctx, const uint16_t *a1, const uint16_t *b1,
                           const uint16_t *a2, const uint16_t *b2, float *d_out, float *acc_out) {
  if (!ctx || !a1 || !b1 || !a2 || !b2 || !d_out || !acc_out) return SYM_INVALID_ARGUMENT;
  try {
    sym::Call call(ctx, "tc_selftest");
    sym::tc_selftest_host(call, a1, b1, a2, b2, d_out, acc_out);
    return SYM_OK;
  } catch (const sym::Error &e) {
    sym_error_text = e.what();
    return e.status;
  }
}

sym_status sym_fast_votes(sym_context *ctx, const sym_points_view *positions,
                          const sym_features_view *features, const sym_pairs_view *pairs,
                          const sym_model_context *model, int32_t mode, float *out,
                          int32_t *pair_of, uint64_t *count) {
  if (!ctx || !positions || !features || !pairs || !model || !count ||
      (pairs->count && (!out || !pair_of)))
    return SYM_INVALID_ARGUMENT;
  try {
    sym::Call call(ctx, "fast_votes");
    *count = sym::fast_votes_host(call, *positions, *features, *pairs, *model, mode, out, pair_of);
    return SYM_OK;
  } catch (const sym::Error &e) {
    sym_error_text = e.what();
    return e.status;
  } catch (const std::exception &e) {
    sym_error_text = e.what();
    return SYM_RUNTIME_ERROR;
  }
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

sym_status sym_detect_fast_sampled(sym_context *ctx, sym_mesh_handle *mesh,
                                   const sym_options *options, const sym_fast_options *fast,
                                   sym_fast_result *out) {
  if (!ctx || !mesh || !options || !fast || !out) return SYM_INVALID_ARGUMENT;
  try {
    sym::Call call(ctx, "detect_fast");
    sym::validate_prepare_options(*options);
    sym_rng rng;
    sym_rng_seed(&rng, options->seed);  // the engine detect() seeds (pipeline.cpp:25)
    sym::detect_fast(call, *mesh, nullptr, 0, *options, *fast, *out, &rng);
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

sym_status sym_detect_fast_fused(sym_context *ctx, sym_batch_item *items, uint64_t count,
                                 sym_fused_stats *stats) {
  if (!ctx || (count && !items) || !stats) return SYM_INVALID_ARGUMENT;
  try {
    sym::Call call(ctx, "detect_fast_fused");
    sym::detect_fast_fused(call, items, count, *stats);
    stats->launches = ctx->metrics.current.custom_launches;
    for (uint64_t i = 0; i < count; ++i)
      if (items[i].status != SYM_OK) {
        sym_error_text = items[i].message;
        return items[i].status;
      }
    return SYM_OK;
  } catch (const sym::Error &e) {
    sym_error_text = e.what();
    return e.status;
  } catch (const std::exception &e) {
    sym_error_text = e.what();
    return SYM_RUNTIME_ERROR;
  }
}

sym_status sym_detect_fast_batch(sym_context *const *workers, int32_t worker_count,
                                 sym_batch_item *items, uint64_t count) {
  if (!workers || worker_count <= 0 || (count && !items)) return SYM_INVALID_ARGUMENT;
  for (int32_t w = 0; w < worker_count; ++w)
    for (int32_t x = 0; x < w; ++x)
      if (!workers[w] || workers[w] == workers[x]) {
        sym_error_text = "batch workers must be distinct contexts";
        return SYM_INVALID_ARGUMENT;
      }
  for (uint64_t i = 0; i < count; ++i) items[i].status = SYM_OK, items[i].message[0] = 0;
  std::atomic<uint64_t> next{0};
  auto run = [&](sym_context *ctx) {
    for (uint64_t i = next++; i < count; i = next++) {
      sym_batch_item &it = items[i];
      it.status = it.sample_count == SYM_SAMPLE_ON_DEVICE && !it.sample
                      ? sym_detect_fast_sampled(ctx, it.mesh, it.options, it.fast, it.out)
                      : sym_detect_fast(ctx, it.mesh, it.sample, it.sample_count, it.options,
                                        it.fast, it.out);
      if (it.status != SYM_OK) {
        std::snprintf(it.message, sizeof(it.message), "%s", sym_error_text.c_str());
        if (!it.message[0]) std::snprintf(it.message, sizeof(it.message), "invalid argument");
      }
    }
  };
  const int32_t used = int32_t(std::min<uint64_t>(uint64_t(worker_count), count));
  std::vector<std::thread> pool;
  for (int32_t w = 1; w < used; ++w) pool.emplace_back(run, workers[w]);
  if (used > 0) run(workers[0]);
  for (auto &t : pool) t.join();
  for (uint64_t i = 0; i < count; ++i)
    if (items[i].status != SYM_OK) {
      sym_error_text = items[i].message;
      return items[i].status;
    }
  return SYM_OK;
}

}  // extern "C"
