// SPDX-License-Identifier: MPL-2.0
// Mesh preparation on the GPU: the reference's prepare() without subdivision
// (src/core/prepare.cpp:102-149) and its topology() (prepare.cpp:13-58).
//
//  1. bounding-box diagonal (min/max per coordinate, exact in any order) and
//     the non-finite check;
//  2. degenerate faces (|cross| <= 1e-14 box^2) removed by an ordered
//     compaction, so the kept faces keep their order;
//  3. face normals and areas, one thread per face;
//  4. incident faces: the 3F corners stably radix-sorted by vertex, so each
//     vertex lists its faces in face order, and the vertex normals and
//     weights are the sequential sums over that list - the order in which
//     the reference accumulates them corner by corner;
//  5. the neighbour ring: both directions of every corner edge as 64-bit
//     (source, target) keys, sorted, duplicates dropped;
//  6. the edge table: the corner edges stably sorted by (lo, hi), one edge per
//     run of equal keys with its first two corners - the order and content of
//     the reference's std::map, plus its non-manifold / winding checks;
//  7. the vertex centroid as one sequential sum.
// FP64 without FMA contraction in the reference's operation order, so every
// output is bit-exact with the CPU path.
#include "common.cuh"
#include "prepare.cuh"
#include "primitives.cuh"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <limits>

namespace sym {
namespace {

constexpr int kBoxBlocks = 256;

__global__ void box_partials64(const double *xyz, uint64_t nv, double *part, int *nonfinite) {
  __shared__ double lo_s[3][kThreads], hi_s[3][kThreads];
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  bool bad = false;
  for (uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; v < nv;
       v += uint64_t(gridDim.x) * blockDim.x)
    for (int k = 0; k < 3; ++k) {
      const double x = xyz[k * nv + v];
      bad |= !isfinite(x);
      lo[k] = fmin(lo[k], x), hi[k] = fmax(hi[k], x);
    }
  if (bad) atomicExch(nonfinite, 1);
  for (int k = 0; k < 3; ++k) lo_s[k][threadIdx.x] = lo[k], hi_s[k][threadIdx.x] = hi[k];
  __syncthreads();
  for (int s = blockDim.x / 2; s; s >>= 1) {
    if (int(threadIdx.x) < s)
      for (int k = 0; k < 3; ++k) {
        lo_s[k][threadIdx.x] = fmin(lo_s[k][threadIdx.x], lo_s[k][threadIdx.x + s]);
        hi_s[k][threadIdx.x] = fmax(hi_s[k][threadIdx.x], hi_s[k][threadIdx.x + s]);
      }
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < 3; ++k) part[blockIdx.x * 6 + k] = lo_s[k][0], part[blockIdx.x * 6 + 3 + k] = hi_s[k][0];
}

__device__ __forceinline__ D3 point(const double *xyz, uint64_t nv, int32_t v) {
  return {xyz[v], xyz[nv + v], xyz[2 * nv + v]};
}

// keep[f]: the face's indices are in range and it is not degenerate.
__global__ void face_flags(const double *xyz, uint64_t nv, const int32_t *faces, uint64_t nf,
                           double limit, uint8_t *keep, int *bad_index) {
  const uint64_t f = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const int32_t a = faces[f], b = faces[nf + f], c = faces[2 * nf + f];
  if (a < 0 || b < 0 || c < 0 || uint64_t(a) >= nv || uint64_t(b) >= nv || uint64_t(c) >= nv) {
    atomicExch(bad_index, 1);
    keep[f] = 0;
    return;
  }
  const D3 p0 = point(xyz, nv, a);
  keep[f] = !(norm(cross(point(xyz, nv, b) - p0, point(xyz, nv, c) - p0)) <= limit);
}

// Face normal (unit) and area of every kept face.
__global__ void face_geometry(const double *xyz, uint64_t nv, const int32_t *faces, uint64_t nf,
                              double *fn, double *area) {
  const uint64_t f = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const D3 p0 = point(xyz, nv, faces[f]);
  const D3 n = cross(point(xyz, nv, faces[nf + f]) - p0, point(xyz, nv, faces[2 * nf + f]) - p0);
  area[f] = norm(n) / 2;
  const D3 u = unit(n);
  fn[f] = u.x, fn[nf + f] = u.y, fn[2 * nf + f] = u.z;
}

// Corner c = 3 f + k: vertex faces[k][f]; keys for the incident sort, the
// ring (both directions of the corner edge a -> b = f[k] -> f[k+1]) and the
// edge table (lo * nv + hi).
__global__ void corner_keys(const int32_t *faces, uint64_t nf, uint64_t nv, uint64_t *vkey,
                            int32_t *corner, uint64_t *ring_key, uint64_t *edge_key) {
  const uint64_t c = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (c >= 3 * nf) return;
  const uint64_t f = c / 3;
  const int k = int(c % 3);
  const uint64_t a = uint64_t(faces[k * nf + f]), b = uint64_t(faces[((k + 1) % 3) * nf + f]);
  vkey[c] = a;
  corner[c] = int32_t(c);
  ring_key[2 * c] = a * nv + b;
  ring_key[2 * c + 1] = b * nv + a;
  edge_key[c] = (a < b ? a : b) * nv + (a < b ? b : a);
}

// Incident faces, normals and weights of every vertex from its corners in
// face order (sorted_corner[off[v] .. off[v+1])).
__global__ void vertex_sums(const int32_t *sorted_corner, const uint64_t *off, uint64_t nv,
                            uint64_t nf, const double *fn, const double *area, int32_t *incident,
                            double *vn, double *w) {
  const uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  D3 n{0, 0, 0};
  double weight = 0;
  for (uint64_t j = off[v]; j < off[v + 1]; ++j) {
    const uint64_t f = uint64_t(sorted_corner[j]) / 3;
    incident[j] = int32_t(f);
    n = n + D3{fn[f], fn[nf + f], fn[2 * nf + f]};
    weight += area[f] / 3;
  }
  const D3 u = unit(n);
  vn[v] = u.x, vn[nv + v] = u.y, vn[2 * nv + v] = u.z;
  w[v] = weight;
}

// off[v] = first index of vertex v in the sorted keys (key / div = v).
__global__ void row_starts(const uint64_t *sorted, uint64_t n, uint64_t div, uint64_t rows,
                           uint64_t *off) {
  const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i > n) return;
  const uint64_t cur = i < n ? sorted[i] / div : rows;
  const uint64_t prev = i == 0 ? 0 : sorted[i - 1] / div + 1;
  for (uint64_t r = prev; r <= cur && r <= rows; ++r) off[r] = i;
}

__global__ void first_of_run(const uint64_t *sorted, uint64_t n, uint8_t *first) {
  const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) first[i] = i == 0 || sorted[i] != sorted[i - 1];
}

// uring[i] = sorted[pos[i]] (the unique keys), nbr[i] = their target.
__global__ void ring_unique(const uint64_t *sorted, const int32_t *pos, uint64_t n, uint64_t nv,
                            uint64_t *uring, int32_t *nbr) {
  const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t key = sorted[pos[i]];
  uring[i] = key;
  nbr[i] = int32_t(key % nv);
}

// One edge per run of equal (lo, hi) keys: runs start at starts[e]
// (positions into the stably sorted corners), the next run at starts[e+1].
__global__ void edge_records(const int32_t *faces, uint64_t nf, const uint64_t *sorted_key,
                             const int32_t *sorted_corner, const int32_t *starts, uint64_t ne,
                             uint64_t total, uint64_t nv, sym_edge *edges,
                             unsigned long long *nonmanifold, unsigned long long *conflicts) {
  const uint64_t e = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const uint64_t s = uint64_t(starts[e]), t = e + 1 < ne ? uint64_t(starts[e + 1]) : total;
  auto ends = [&](uint64_t j, int32_t &a, int32_t &b, int32_t &f) {
    const uint64_t c = uint64_t(sorted_corner[j]);
    const uint64_t ff = c / 3;
    const int k = int(c % 3);
    f = int32_t(ff), a = faces[k * nf + ff], b = faces[((k + 1) % 3) * nf + ff];
  };
  int32_t a0, b0, f0, a1 = 0, b1 = 0, f1 = -1;
  ends(s, a0, b0, f0);
  if (t - s >= 2) ends(s + 1, a1, b1, f1);
  if (t - s > 2) atomicAdd(nonmanifold, 1ull);
  if (t - s == 2 && a0 != b1) atomicAdd(conflicts, 1ull);
  const uint64_t key = sorted_key[s];
  edges[e] = sym_edge{int32_t(key / nv), int32_t(key % nv), a0, b0, f0, t - s == 2 ? f1 : -1};
}

__global__ void centroid(const double *xyz, uint64_t nv, double *out) {
  if (blockIdx.x || threadIdx.x > 2) return;
  const int k = threadIdx.x;
  double s = 0;
  for (uint64_t v = 0; v < nv; ++v) s += xyz[k * nv + v];  // the reference's order
  out[k] = s;
}

int key_bits(uint64_t max_key) {
  int b = 8;
  while (b < 64 && (max_key >> b)) b += 8;
  return b;
}

}  // namespace

void validate_prepare_options(const sym_options &o) {
  const uint64_t imax = uint64_t(std::numeric_limits<int32_t>::max());
  if (o.max_pairs > imax || o.max_votes > imax)
    fail(SYM_INVALID_ARGUMENT, "Pair/vote budgets exceed 32-bit ID capacity");
  if (!(o.sample_ratio > 0 && o.sample_ratio <= 1) || !(o.prune > 0 && o.prune < 1) ||
      !(o.pair_threshold > 0 && o.pair_threshold <= 1) ||
      !(o.bandwidth > 0 && o.bandwidth <= 2) ||
      !(o.verify_threshold > 0 && o.verify_threshold < 0.5) || o.smoothing < 0 ||
      o.smoothing > 1000 || o.subdivide < 0 || o.subdivide > 3 || o.max_iterations < 1 ||
      o.max_iterations > 10000 || o.max_clusters < 1 || o.max_clusters > 1000 ||
      o.max_pairs < 1 || o.max_votes < 1)
    fail(SYM_RUNTIME_ERROR, "Invalid parameter range; see --help");
}

PreparedDevice prepare_device(Call &call, const sym_mesh_view &m, const sym_options &o) {
  validate_prepare_options(o);
  if (o.subdivide != 0)
    fail(SYM_INVALID_ARGUMENT, "subdivision is not part of the GPU prepare (use subdivide = 0)");
  const uint64_t nv = m.vertices.count, nf_in = m.faces.count;
  if (!nv || !nf_in) fail(SYM_RUNTIME_ERROR, "Mesh is empty");
  const uint64_t imax = uint64_t(std::numeric_limits<int32_t>::max());
  if (nv > imax || nf_in > imax) fail(SYM_RUNTIME_ERROR, "Mesh exceeds 32-bit index capacity");
  if (3 * nf_in > imax) fail(SYM_RUNTIME_ERROR, "Mesh exceeds 32-bit index capacity");
  cudaStream_t st = call.stream();
  PreparedDevice p;
  p.nv = nv;
  p.xyz = call.alloc<double>(3 * nv);
  call.h2d(p.xyz, m.vertices.x, 8 * nv);
  call.h2d(p.xyz + nv, m.vertices.y, 8 * nv);
  call.h2d(p.xyz + 2 * nv, m.vertices.z, 8 * nv);
  int32_t *faces_in = call.alloc<int32_t>(3 * nf_in);
  call.h2d(faces_in, m.faces.v0, 4 * nf_in);
  call.h2d(faces_in + nf_in, m.faces.v1, 4 * nf_in);
  call.h2d(faces_in + 2 * nf_in, m.faces.v2, 4 * nf_in);
  // 1. box
  double *part = call.alloc<double>(kBoxBlocks * 6);
  int *flags2 = call.alloc<int>(2);  // non-finite, bad face index
  SYM_CUDA(cudaMemsetAsync(flags2, 0, 2 * sizeof(int), st));
  box_partials64<<<kBoxBlocks, kThreads, 0, st>>>(p.xyz, nv, part, flags2);
  check_launch();
  std::vector<double> hp(kBoxBlocks * 6);
  int hflags[2];
  call.d2h(hp.data(), part, hp.size() * 8);
  call.d2h(hflags, flags2, sizeof(hflags));
  call.sync();
  if (hflags[0]) fail(SYM_RUNTIME_ERROR, "Non-finite coordinate");
  D3 lo{hp[0], hp[1], hp[2]}, hi{hp[3], hp[4], hp[5]};
  for (int b = 1; b < kBoxBlocks; ++b) {
    lo = D3{std::fmin(lo.x, hp[b * 6]), std::fmin(lo.y, hp[b * 6 + 1]), std::fmin(lo.z, hp[b * 6 + 2])};
    hi = D3{std::fmax(hi.x, hp[b * 6 + 3]), std::fmax(hi.y, hp[b * 6 + 4]), std::fmax(hi.z, hp[b * 6 + 5])};
  }
  const double box = norm(hi - lo);
  if (box < 1e-14) fail(SYM_RUNTIME_ERROR, "Mesh has zero extent");
  // 2. degenerate faces
  uint8_t *keep = call.alloc<uint8_t>(nf_in);
  face_flags<<<blocks_for(nf_in), kThreads, 0, st>>>(p.xyz, nv, faces_in, nf_in, 1e-14 * box * box,
                                                      keep, flags2 + 1);
  check_launch();
  uint64_t *kept = call.alloc<uint64_t>(3);
  p.faces = call.alloc<int32_t>(3 * nf_in);
  for (int k = 0; k < 3; ++k)
    compact_values(call, keep, faces_in + k * nf_in, nf_in, p.faces + k * nf_in, kept + k);
  uint64_t nf = 0;
  call.d2h(&nf, kept, 8);
  call.d2h(hflags + 1, flags2 + 1, sizeof(int));
  call.sync();
  if (hflags[1]) fail(SYM_RUNTIME_ERROR, "Face index out of range");
  if (!nf) fail(SYM_RUNTIME_ERROR, "No nondegenerate triangles");
  p.rejected = nf_in - nf;
  // kept faces as three contiguous columns of nf rows
  if (nf != nf_in) {
    int32_t *packed = call.alloc<int32_t>(3 * nf);
    for (int k = 0; k < 3; ++k)
      SYM_CUDA(cudaMemcpyAsync(packed + k * nf, p.faces + k * nf_in, 4 * nf,
                               cudaMemcpyDeviceToDevice, st));
    p.faces = packed;
  }
  p.nf = nf;
  // 3. face geometry
  p.fn = call.alloc<double>(3 * nf);
  double *area = call.alloc<double>(nf);
  face_geometry<<<blocks_for(nf), kThreads, 0, st>>>(p.xyz, nv, p.faces, nf, p.fn, area);
  check_launch();
  // 4-6. corner keys and sorts
  const uint64_t nc = 3 * nf;
  uint64_t *vkey = call.alloc<uint64_t>(nc), *svkey = call.alloc<uint64_t>(nc);
  int32_t *corner = call.alloc<int32_t>(nc), *scorner = call.alloc<int32_t>(nc);
  uint64_t *ring = call.alloc<uint64_t>(2 * nc), *sring = call.alloc<uint64_t>(2 * nc);
  int32_t *ring_val = call.alloc<int32_t>(2 * nc), *sring_val = call.alloc<int32_t>(2 * nc);
  uint64_t *ekey = call.alloc<uint64_t>(nc), *sekey = call.alloc<uint64_t>(nc);
  int32_t *secorner = call.alloc<int32_t>(nc);
  corner_keys<<<blocks_for(nc), kThreads, 0, st>>>(p.faces, nf, nv, vkey, corner, ring, ekey);
  check_launch();
  SYM_CUDA(cudaMemsetAsync(ring_val, 0, 8 * nc, st));
  const int vbits = key_bits(nv), pbits = key_bits(nv * nv);
  radix_sort_pairs(call, vkey, corner, svkey, scorner, nc, vbits);
  radix_sort_pairs(call, ring, ring_val, sring, sring_val, 2 * nc, pbits);
  radix_sort_pairs(call, ekey, corner, sekey, secorner, nc, pbits);
  // incident faces, vertex normals and weights
  p.inc_off = call.alloc<uint64_t>(nv + 1);
  row_starts<<<blocks_for(nc + 1), kThreads, 0, st>>>(svkey, nc, 1, nv, p.inc_off);
  check_launch();
  p.inc = call.alloc<int32_t>(nc);
  p.vn = call.alloc<double>(3 * nv);
  p.w = call.alloc<double>(nv);
  vertex_sums<<<blocks_for(nv), kThreads, 0, st>>>(scorner, p.inc_off, nv, nf, p.fn, area, p.inc,
                                                   p.vn, p.w);
  check_launch();
  // neighbour ring: unique (source, target) keys
  uint8_t *first = call.alloc<uint8_t>(2 * nc);
  first_of_run<<<blocks_for(2 * nc), kThreads, 0, st>>>(sring, 2 * nc, first);
  check_launch();
  uint64_t *uring = call.alloc<uint64_t>(2 * nc);
  int32_t *pos = call.alloc<int32_t>(2 * nc);
  uint64_t *count = call.alloc<uint64_t>(2);
  compact_indices(call, first, 2 * nc, pos, count);
  uint64_t nr = 0;
  call.d2h(&nr, count, 8);
  call.sync();
  p.nbr_count = nr;
  p.nbr = call.alloc<int32_t>(std::max<uint64_t>(nr, 1));
  p.nbr_off = call.alloc<uint64_t>(nv + 1);
  ring_unique<<<blocks_for(nr), kThreads, 0, st>>>(sring, pos, nr, nv, uring, p.nbr);
  check_launch();
  row_starts<<<blocks_for(nr + 1), kThreads, 0, st>>>(uring, nr, nv, nv, p.nbr_off);
  check_launch();
  // edge table
  first_of_run<<<blocks_for(nc), kThreads, 0, st>>>(sekey, nc, first);
  check_launch();
  compact_indices(call, first, nc, pos, count + 1);
  uint64_t ne = 0;
  call.d2h(&ne, count + 1, 8);
  call.sync();
  p.ne = ne;
  p.edges = call.alloc<sym_edge>(std::max<uint64_t>(ne, 1));
  unsigned long long *diag = call.alloc<unsigned long long>(2);
  SYM_CUDA(cudaMemsetAsync(diag, 0, 16, st));
  edge_records<<<blocks_for(ne), kThreads, 0, st>>>(p.faces, nf, sekey, secorner, pos, ne, nc, nv,
                                                    p.edges, diag, diag + 1);
  check_launch();
  // 7. centroid
  double *csum = call.alloc<double>(3);
  centroid<<<1, 32, 0, st>>>(p.xyz, nv, csum);
  check_launch();
  unsigned long long hd[2];
  double hc[3];
  call.d2h(hd, diag, 16);
  call.d2h(hc, csum, 24);
  call.sync();
  call.launched(12);  // own kernels; the primitives count theirs
  p.nonmanifold = hd[0], p.conflicts = hd[1];
  if (hd[0] || hd[1])
    fail(SYM_RUNTIME_ERROR,
         "Mesh must have manifold edges and consistent face winding; repair input mesh first");
  const D3 c = D3{hc[0], hc[1], hc[2]} * (1 / double(nv));
  p.context.box_size = box;
  p.context.center[0] = c.x, p.context.center[1] = c.y, p.context.center[2] = c.z;
  return p;
}

}  // namespace sym

extern "C" {

sym_status sym_prepare(sym_context *ctx, const sym_mesh_view *mesh, const sym_options *options,
                       sym_prepared *out) {
  if (!ctx || !mesh || !options || !out) return SYM_INVALID_ARGUMENT;
  *out = sym_prepared{};
  try {
    sym::Call call(ctx, "prepare");
    const sym::PreparedDevice p = sym::prepare_device(call, *mesh, *options);
    const uint64_t nv = p.nv, nf = p.nf, ne = p.ne, nr = p.nbr_count, nc = 3 * nf;
    const uint64_t bytes = 8 * (3 * nv + 3 * nf + nv + 2 * (nv + 1)) + 4 * (3 * nf + nr + nc) +
                           sizeof(sym_edge) * ne + 64;
    char *block = static_cast<char *>(std::malloc(bytes));
    if (!block) sym::fail(SYM_RUNTIME_ERROR, "host allocation failed");
    char *at = block;
    auto take = [&](uint64_t b) {
      char *r = at;
      at += (b + 7) & ~uint64_t(7);
      return r;
    };
    out->storage = block;
    out->context = p.context;
    out->vertex_count = nv, out->face_count = nf, out->edge_count = ne;
    out->rejected_faces = p.rejected;
    for (int k = 0; k < 3; ++k) {
      out->faces[k] = reinterpret_cast<int32_t *>(take(4 * nf));
      out->normals[k] = reinterpret_cast<double *>(take(8 * nv));
      out->face_normals[k] = reinterpret_cast<double *>(take(8 * nf));
      call.d2h(out->faces[k], p.faces + k * nf, 4 * nf);
      call.d2h(out->normals[k], p.vn + k * nv, 8 * nv);
      call.d2h(out->face_normals[k], p.fn + k * nf, 8 * nf);
    }
    out->weights = reinterpret_cast<double *>(take(8 * nv));
    out->neighbor_offsets = reinterpret_cast<uint64_t *>(take(8 * (nv + 1)));
    out->neighbor_indices = reinterpret_cast<int32_t *>(take(4 * nr));
    out->incident_offsets = reinterpret_cast<uint64_t *>(take(8 * (nv + 1)));
    out->incident_indices = reinterpret_cast<int32_t *>(take(4 * nc));
    out->edges = reinterpret_cast<sym_edge *>(take(sizeof(sym_edge) * ne));
    call.d2h(out->weights, p.w, 8 * nv);
    call.d2h(out->neighbor_offsets, p.nbr_off, 8 * (nv + 1));
    call.d2h(out->neighbor_indices, p.nbr, 4 * nr);
    call.d2h(out->incident_offsets, p.inc_off, 8 * (nv + 1));
    call.d2h(out->incident_indices, p.inc, 4 * nc);
    call.d2h(out->edges, p.edges, sizeof(sym_edge) * ne);
    call.sync();
    return SYM_OK;
  } catch (const sym::Error &e) {
    sym_prepared_release(out);
    sym_error_text = e.what();
    return e.status;
  } catch (const std::exception &e) {
    sym_prepared_release(out);
    sym_error_text = e.what();
    return SYM_RUNTIME_ERROR;
  }
}

void sym_prepared_release(sym_prepared *p) {
  if (!p) return;
  std::free(p->storage);
  *p = sym_prepared{};
}

}  // extern "C"
