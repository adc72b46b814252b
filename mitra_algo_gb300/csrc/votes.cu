// SPDX-License-Identifier: MPL-2.0
// Stage (b), second half: the transform of every surviving pair.
//
// Reference: src/cpu/transformations.cpp:17-73 (CPU),
// src/cuda/backend.cu:32-125,410-489 (existing GPU path).
// Per pair: a reflection vote when the mirrored frames agree, then two rigid
// votes (b's frame with sign +1 and -1).  Votes are emitted in pair order, so
// each pair's first vote index comes from a scan of its vote count (2 or 3).
// The output is the reference's 28-lane SoA (rotation 9, translation 3,
// plane normal 3, offset, descriptor 12) plus pair id and kind, in FP64 with
// the reference's operation order (no FMA contraction): bit-exact.
#include "common.cuh"
#include "primitives.cuh"

#include <cmath>
#include <limits>

namespace sym {
namespace {

struct PairFrames {
  D3 p, q, an, ad, ax, bn, bd, bx, n;
  double d;
  M3 refl;
  bool reflection;
};

// xyzf: 12 lanes of nv rows: position, normal, dmin, dmax.
__device__ PairFrames pair_frames(const double *xyzf, uint64_t nv, int32_t a, int32_t b) {
  auto lane3 = [&](int lane, int32_t i) {
    return D3{xyzf[lane * nv + i], xyzf[(lane + 1) * nv + i], xyzf[(lane + 2) * nv + i]};
  };
  PairFrames g;
  g.p = lane3(0, a), g.q = lane3(0, b);
  g.an = lane3(3, a), g.ad = lane3(6, a), g.ax = lane3(9, a);
  g.bn = lane3(3, b), g.bd = lane3(6, b), g.bx = lane3(9, b);
  D3 n = unit(g.q - g.p);
  int dom = 0;
  for (int k = 1; k < 3; ++k)
    if (fabs(comp(n, k)) > fabs(comp(n, dom))) dom = k;
  if (comp(n, dom) < 0) n = n * -1;
  g.n = n;
  g.d = -dot(n, div(g.p + g.q, 2));
  g.refl = mirror(n);
  g.reflection = dot(mul(g.refl, g.an), g.bn) > 0.75 && fabs(dot(mul(g.refl, g.ad), g.bd)) > 0.75;
  return g;
}

__global__ void vote_counts(const double *xyzf, uint64_t nv, const int32_t *pa, const int32_t *pb,
                            uint64_t np, uint64_t *counts, uint8_t *refl, int *status) {
  uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= np) return;
  int32_t a = pa[i], b = pb[i];
  if (a < 0 || b < 0 || uint64_t(a) >= nv || uint64_t(b) >= nv) {
    atomicExch(status, DS_INDEX_RANGE);
    counts[i] = 0;
    refl[i] = 0;
    return;
  }
  bool r = pair_frames(xyzf, nv, a, b).reflection;
  refl[i] = r;
  counts[i] = r ? 3 : 2;
}

struct VoteLanes {  // 28 lanes of `total` rows + ids + kinds
  double *lanes;
  int32_t *pair;
  uint8_t *kind;
  uint64_t total;
};

__device__ void write_vote(const VoteLanes &o, uint64_t row, int32_t pair, bool reflection,
                           const M3 &r, D3 t, D3 n, double d, const double *desc) {
  o.pair[row] = pair;
  o.kind[row] = reflection ? SYM_REFLECTION : SYM_RIGID;
  double *L = o.lanes;
  uint64_t T = o.total;
  for (int k = 0; k < 9; ++k) L[k * T + row] = r.m[k];
  L[9 * T + row] = t.x, L[10 * T + row] = t.y, L[11 * T + row] = t.z;
  L[12 * T + row] = n.x, L[13 * T + row] = n.y, L[14 * T + row] = n.z;
  L[15 * T + row] = d;
  for (int k = 0; k < 12; ++k) L[(16 + k) * T + row] = desc[k];
}

__global__ void vote_fill(const double *xyzf, uint64_t nv, const int32_t *pa, const int32_t *pb,
                          uint64_t np, const uint64_t *offsets, double box, D3 center,
                          VoteLanes out) {
  uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= np) return;
  int32_t a = pa[i], b = pb[i];
  if (a < 0 || b < 0 || uint64_t(a) >= nv || uint64_t(b) >= nv) return;
  PairFrames g = pair_frames(xyzf, nv, a, b);
  uint64_t row = offsets[i];
  if (g.reflection) {
    double desc[12] = {g.n.x, g.n.y, g.n.z, (g.d + dot(g.n, center)) / box, 0, 0, 0, 0, 0, 0, 0, 0};
    write_vote(out, row++, int32_t(i), true, g.refl, g.n * (-2 * g.d), g.n, g.d, desc);
  }
  M3 fa = columns(g.ad, g.ax, g.an);
  M3 fat = transpose(fa);
  for (int sgn = 0; sgn < 2; ++sgn) {
    double s = sgn ? -1.0 : 1.0;
    M3 fb = columns(g.bd * s, g.bx * s, g.bn);
    M3 r = matmul(fb, fat);
    D3 t = g.q - mul(r, g.p);
    D3 centered = div(mul(r, center) + t - center, box);
    double desc[12];
    for (int k = 0; k < 9; ++k) desc[k] = r.m[k] / 2;
    desc[9] = centered.x, desc[10] = centered.y, desc[11] = centered.z;
    write_vote(out, row++, int32_t(i), false, r, t, D3{0, 0, 0}, 0, desc);
  }
}

}  // namespace

// Device-resident transforms: returns the vote count; lanes allocated from
// the workspace (28 x total doubles, lane-major) plus pair ids and kinds.
uint64_t transformations_device(Call &call, const double *xyzf, uint64_t nv, const int32_t *pa,
                                const int32_t *pb, uint64_t np, double box, const double center[3],
                                uint64_t max_votes, double **lanes, int32_t **pair,
                                uint8_t **kind) {
  cudaStream_t st = call.stream();
  uint64_t *counts = call.alloc<uint64_t>(np), *offsets = call.alloc<uint64_t>(np + 1);
  uint8_t *refl = call.alloc<uint8_t>(np);
  vote_counts<<<blocks_for(np), kThreads, 0, st>>>(xyzf, nv, pa, pb, np, counts, refl,
                                                   call.status());
  check_launch();
  exclusive_scan(call, counts, offsets, np);
  call.launched();
  uint64_t total = 0;
  call.d2h(&total, offsets + np, 8);
  call.check_status("transformations");
  if (total > max_votes || total > uint64_t(std::numeric_limits<int32_t>::max()))
    fail(SYM_RUNTIME_ERROR, "Vote budget exceeded; lower --sample-ratio or tighten --pair-threshold");
  VoteLanes out{call.alloc<double>(28 * total), call.alloc<int32_t>(total),
                call.alloc<uint8_t>(total), total};
  vote_fill<<<blocks_for(np), kThreads, 0, st>>>(xyzf, nv, pa, pb, np, offsets, box,
                                                 D3{center[0], center[1], center[2]}, out);
  check_launch();
  call.launched();
  *lanes = out.lanes;
  *pair = out.pair;
  *kind = out.kind;
  return total;
}

void transformations_host(Call &call, const sym_mesh_view &m, const sym_features_view &f,
                          const sym_pairs_view &p, const sym_model_context &ctx,
                          const sym_options &o, sym_votes &out, void *(*allocate)(size_t)) {
  uint64_t np = p.count, nv = m.vertices.count;
  out = sym_votes{};
  if (np) {
    if (f.count != nv) fail(SYM_INVALID_ARGUMENT, "SoA component lengths differ");
    if (!(ctx.box_size > 0) || !std::isfinite(ctx.box_size) || !std::isfinite(ctx.center[0]) ||
        !std::isfinite(ctx.center[1]) || !std::isfinite(ctx.center[2]))
      fail(SYM_INVALID_ARGUMENT,
           "transformations require a positive finite box size and finite center");
    if (np > uint64_t(std::numeric_limits<int32_t>::max()))
      fail(SYM_OVERFLOW, "pair ids exceed int32 range");
  }
  double *lanes = nullptr;
  int32_t *pair = nullptr;
  uint8_t *kind = nullptr;
  uint64_t total = 0;
  if (np) {
    double *xyzf = call.alloc<double>(12 * nv);
    const sym_points_view *pts[4] = {&m.vertices, &f.normal, &f.dmin, &f.dmax};
    for (int k = 0; k < 4; ++k) {
      call.h2d(xyzf + (3 * k) * nv, pts[k]->x, nv * 8);
      call.h2d(xyzf + (3 * k + 1) * nv, pts[k]->y, nv * 8);
      call.h2d(xyzf + (3 * k + 2) * nv, pts[k]->z, nv * 8);
    }
    int32_t *pa = call.upload(p.a, np), *pb = call.upload(p.b, np);
    total = transformations_device(call, xyzf, nv, pa, pb, np, ctx.box_size, ctx.center,
                                   o.max_votes, &lanes, &pair, &kind);
  }
  // One host block: pair ids, kinds, 28 lanes.
  size_t bytes = total * (4 + 1 + 28 * 8) + 64 * 3;
  char *block = static_cast<char *>(allocate(bytes ? bytes : 64));
  if (!block) fail(SYM_RUNTIME_ERROR, "host allocation failed");
  out.storage = block;
  out.count = total;
  double *hl = reinterpret_cast<double *>(block);
  out.pair = reinterpret_cast<int32_t *>(block + total * 28 * 8);
  out.kind = reinterpret_cast<uint8_t *>(block + total * 28 * 8 + total * 4);
  for (int k = 0; k < 9; ++k) out.rotation[k] = hl + k * total;
  for (int k = 0; k < 3; ++k) out.translation[k] = hl + (9 + k) * total;
  for (int k = 0; k < 3; ++k) out.plane_normal[k] = hl + (12 + k) * total;
  out.plane_offset = hl + 15 * total;
  for (int k = 0; k < 12; ++k) out.descriptor[k] = hl + (16 + k) * total;
  if (total) {
    call.d2h(hl, lanes, total * 28 * 8);
    call.d2h(out.pair, pair, total * 4);
    call.d2h(out.kind, kind, total);
  }
  call.check_status("transformations");
}

}  // namespace sym
