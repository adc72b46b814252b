// SPDX-License-Identifier: MPL-2.0
// Stage (a): per-vertex curvature tensors and principal frames.
//
// Reference: src/cpu/curvature.cpp:14-79 (CPU), src/cuda/curvature.cu (the
// existing GPU path).  Design on GB300:
//  * no per-edge tensor buffer and no float atomics: every vertex gathers its
//    incident interior edges itself, in edge-table order, and recomputes the
//    edge's dihedral angle, so sums are added in the reference's order and the
//    result is deterministic;
//  * the edge of each neighbour slot is found through the (lo, hi)-sorted
//    edge table (prepare() emits it sorted): neighbours of v in ascending
//    order are exactly v's edges in edge-table order;
//  * smoothing ping-pongs a V x 9 tensor buffer; the principal-frame solve is
//    fused into the last pass.
// FP64 throughout; the translation unit is compiled without FMA contraction.
#include "common.cuh"

#include <algorithm>
#include <cmath>

namespace sym {
namespace {

struct Edge6 {
  int32_t lo, hi, a, b, face0, face1;
};

// first[u] = first edge with lo >= u, for u in [0, V]; flags unsorted tables.
__global__ void lo_starts(const Edge6 *edges, uint64_t ne, uint64_t nv, int64_t *first,
                          int *unsorted, int *status) {
  uint64_t e = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e > ne) return;
  int64_t lo = e < ne ? edges[e].lo : int64_t(nv);
  int64_t prev = e ? edges[e - 1].lo : -1;
  if (e < ne) {
    const Edge6 &x = edges[e];
    if (x.lo < 0 || x.hi < 0 || uint64_t(x.lo) >= nv || uint64_t(x.hi) >= nv || x.a < 0 ||
        x.b < 0 || uint64_t(x.a) >= nv || uint64_t(x.b) >= nv)
      atomicExch(status, DS_INDEX_RANGE);
    if (e) {
      const Edge6 &p = edges[e - 1];
      if (p.lo > x.lo || (p.lo == x.lo && p.hi >= x.hi)) atomicExch(unsorted, 1);
    }
  }
  if (lo < 0 || lo > int64_t(nv) || prev > lo) return;
  for (int64_t u = prev + 1; u <= lo; ++u) first[u] = int64_t(e);
}

// edge_of_slot[k] = edge joining v and its k-th neighbour.
__global__ void slot_edges(const uint64_t *nbr_off, const int32_t *nbr, uint64_t nv,
                           const Edge6 *edges, const int64_t *first, int32_t *edge_of_slot,
                           int *status) {
  uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  for (uint64_t k = nbr_off[v]; k < nbr_off[v + 1]; ++k) {
    int32_t u = nbr[k];
    if (u < 0 || uint64_t(u) >= nv) {
      atomicExch(status, DS_INDEX_RANGE);
      edge_of_slot[k] = -1;
      continue;
    }
    int32_t lo = min(int32_t(v), u), hi = max(int32_t(v), u);
    int32_t found = -1;
    for (int64_t e = first[lo]; e < first[lo + 1]; ++e)
      if (edges[e].hi == hi) {
        found = int32_t(e);
        break;
      }
    if (found < 0) atomicExch(status, DS_EDGE_LOOKUP);
    edge_of_slot[k] = found;
  }
}

// Fixed-order sum of edge lengths: block partials, then one block.
__global__ void edge_length_partials(const double *xyz, uint64_t nv, const Edge6 *edges,
                                     uint64_t ne, double *partial) {
  __shared__ double s[256];
  double acc = 0;
  uint64_t chunk = (ne + gridDim.x - 1) / gridDim.x;
  uint64_t begin = blockIdx.x * chunk, end = min(ne, begin + chunk);
  for (uint64_t e = begin + threadIdx.x; e < end; e += blockDim.x) {
    D3 hi = load3(xyz, xyz + nv, xyz + 2 * nv, edges[e].hi);
    D3 lo = load3(xyz, xyz + nv, xyz + 2 * nv, edges[e].lo);
    acc += norm(hi - lo);
  }
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = s[0];
}

__global__ void mean_length(const double *partial, int count, uint64_t ne, double *mean) {
  if (threadIdx.x == 0) {
    double t = 0;
    for (int i = 0; i < count; ++i) t += partial[i];
    *mean = t / double(ne);
  }
}

// Per-vertex tensor: sum over incident interior edges in edge order of
// d d^T * beta * |e| / mean, divided by the edge count.
__global__ void vertex_tensors(const double *xyz, uint64_t nv, const double *fn, uint64_t nf,
                               const Edge6 *edges, const uint64_t *slot_off,
                               const int32_t *slot_edge, const double *mean, double *tensor,
                               int *status) {
  uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  double t[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  int count = 0;
  double m = *mean;
  for (uint64_t k = slot_off[v]; k < slot_off[v + 1]; ++k) {
    int32_t e = slot_edge[k];
    if (e < 0) continue;
    Edge6 ed = edges[e];
    if (ed.face1 < 0) continue;
    if (ed.face0 < 0 || uint64_t(ed.face0) >= nf || uint64_t(ed.face1) >= nf) {
      atomicExch(status, DS_INDEX_RANGE);
      continue;
    }
    D3 dir = load3(xyz, xyz + nv, xyz + 2 * nv, ed.b) - load3(xyz, xyz + nv, xyz + 2 * nv, ed.a);
    double len = norm(dir);
    dir = unit(dir);
    D3 n1 = load3(fn, fn + nf, fn + 2 * nf, ed.face0), n2 = load3(fn, fn + nf, fn + 2 * nf, ed.face1);
    double c = dot(n1, n2);
    c = c < -1.0 ? -1.0 : (1.0 < c ? 1.0 : c);
    double beta = atan2(dot(cross(n1, n2), dir), c);
    double d[3] = {dir.x, dir.y, dir.z};
    ++count;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) t[i * 3 + j] += d[i] * d[j] * beta * len / m;
  }
  double div_by = double(count > 1 ? count : 1);
  for (int k = 0; k < 9; ++k) tensor[v * 9 + k] = t[k] / div_by;
}

__device__ void principal_frame(uint64_t v, const double *t, const double *vn, uint64_t nv,
                                uint64_t degree, sym_features_out out) {
  D3 n = load3(vn, vn + nv, vn + 2 * nv, v);
  D3 dmin = {0, 0, 0}, dmax = {0, 0, 0};
  double kmin = 0, kmax = 0;
  bool valid = false;
  if (!(norm(n) < 0.5 || degree < 3)) {
    D3 axis = fabs(n.x) < 0.8 ? D3{1, 0, 0} : D3{0, 1, 0};
    D3 u = unit(cross(n, axis)), w = cross(n, u);
    M3 T;
    for (int k = 0; k < 9; ++k) T.m[k] = t[k];
    double a = dot(u, mul(T, u)), b = dot(u, mul(T, w)), c = dot(w, mul(T, w));
    double angle = 0.5 * atan2(2 * b, a - c);
    D3 high = u * cos(angle) + w * sin(angle);
    D3 low = unit(cross(high, n));
    double delta = hypot(a - c, 2 * b);
    kmin = (a + c - delta) / 2;
    kmax = (a + c + delta) / 2;
    dmin = low;
    dmax = unit(cross(n, low));
    valid = isfinite(kmin) && isfinite(kmax) && delta > 1e-10;
  } else {
    n = {0, 0, 0};
  }
  out.normal_x[v] = n.x, out.normal_y[v] = n.y, out.normal_z[v] = n.z;
  out.dmin_x[v] = dmin.x, out.dmin_y[v] = dmin.y, out.dmin_z[v] = dmin.z;
  out.dmax_x[v] = dmax.x, out.dmax_y[v] = dmax.y, out.dmax_z[v] = dmax.z;
  out.kmin[v] = kmin, out.kmax[v] = kmax, out.valid[v] = valid;
}

// One smoothing pass (self + neighbours in CSR order) / (degree + 1); the
// last pass also solves the principal frame.
__global__ void smooth(const double *src, double *dst, const uint64_t *nbr_off,
                       const int32_t *nbr, uint64_t nv, bool last, const double *vn,
                       sym_features_out out) {
  uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  double t[9];
  for (int k = 0; k < 9; ++k) t[k] = src[v * 9 + k];
  uint64_t b = nbr_off[v], e = nbr_off[v + 1];
  for (uint64_t s = b; s < e; ++s) {
    int32_t u = nbr[s];
    for (int k = 0; k < 9; ++k) t[k] += src[uint64_t(u) * 9 + k];
  }
  double div_by = double(e - b + 1);
  for (int k = 0; k < 9; ++k) t[k] /= div_by;
  if (last)
    principal_frame(v, t, vn, nv, e - b, out);
  else
    for (int k = 0; k < 9; ++k) dst[v * 9 + k] = t[k];
}

__global__ void frames(const double *tensor, const uint64_t *nbr_off, uint64_t nv,
                       const double *vn, sym_features_out out) {
  uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  principal_frame(v, tensor + v * 9, vn, nv, nbr_off[v + 1] - nbr_off[v], out);
}

}  // namespace

// Device-resident curvature.  All pointers are device pointers; `out` lanes
// are device buffers of nv rows.
void curvature_device(Call &call, const double *xyz, uint64_t nv, const double *face_normals,
                      uint64_t nf, const double *vertex_normals, const uint64_t *nbr_off,
                      const int32_t *nbr, uint64_t nbr_count, const sym_edge *edges_in,
                      uint64_t ne, int smoothing, const sym_features_out &out,
                      const sym_edge *host_edges) {
  cudaStream_t s = call.stream();
  const Edge6 *edges = reinterpret_cast<const Edge6 *>(edges_in);
  int64_t *first = call.alloc<int64_t>(nv + 2);
  int *unsorted = call.alloc<int>(1);
  SYM_CUDA(cudaMemsetAsync(unsorted, 0, sizeof(int), s));
  SYM_CUDA(cudaMemsetAsync(first, 0, (nv + 2) * sizeof(int64_t), s));
  lo_starts<<<blocks_for(ne + 1), kThreads, 0, s>>>(edges, ne, nv, first, unsorted, call.status());
  check_launch();
  int host_unsorted = 0;
  SYM_CUDA(cudaMemcpyAsync(&host_unsorted, unsorted, sizeof(int), cudaMemcpyDeviceToHost, s));
  call.check_status("curvature");
  const uint64_t *slot_off = nbr_off;
  int32_t *slot_edge = nullptr;
  if (!host_unsorted) {
    slot_edge = call.alloc<int32_t>(nbr_count);
    slot_edges<<<blocks_for(nv), kThreads, 0, s>>>(nbr_off, nbr, nv, edges, first, slot_edge,
                                                   call.status());
    check_launch();
    call.launched(2);
    call.check_status("curvature");
  } else {
    // Edge table not (lo, hi)-sorted: list each vertex's interior edges in
    // edge-table order on the host (the reference CUDA backend always does
    // this, src/cuda/curvature.cu:157-167).
    if (!host_edges) fail(SYM_INVALID_ARGUMENT, "curvature: edge table must be sorted by (lo, hi)");
    std::vector<uint64_t> off(nv + 1, 0);
    for (uint64_t e = 0; e < ne; ++e)
      if (host_edges[e].face1 >= 0) ++off[host_edges[e].a + 1], ++off[host_edges[e].b + 1];
    for (uint64_t v = 0; v < nv; ++v) off[v + 1] += off[v];
    std::vector<int32_t> ids(off[nv]);
    std::vector<uint64_t> at(off.begin(), off.end() - 1);
    for (uint64_t e = 0; e < ne; ++e)
      if (host_edges[e].face1 >= 0) ids[at[host_edges[e].a]++] = int32_t(e), ids[at[host_edges[e].b]++] = int32_t(e);
    slot_off = call.upload(off.data(), off.size());
    slot_edge = call.upload(ids.data(), ids.size());
    call.launched(1);
  }
  const int kPartials = 64;
  double *partial = call.alloc<double>(kPartials);
  double *mean = call.alloc<double>(1);
  edge_length_partials<<<kPartials, 256, 0, s>>>(xyz, nv, edges, ne, partial);
  check_launch();
  mean_length<<<1, 32, 0, s>>>(partial, kPartials, ne, mean);
  check_launch();
  double *t0 = call.alloc<double>(9 * nv), *t1 = call.alloc<double>(9 * nv);
  vertex_tensors<<<blocks_for(nv), kThreads, 0, s>>>(xyz, nv, face_normals, nf, edges, slot_off,
                                                     slot_edge, mean, t0, call.status());
  check_launch();
  call.launched(3);
  if (smoothing == 0) {
    frames<<<blocks_for(nv), kThreads, 0, s>>>(t0, nbr_off, nv, vertex_normals, out);
    check_launch();
    call.launched();
  }
  for (int it = 0; it < smoothing; ++it) {
    smooth<<<blocks_for(nv), kThreads, 0, s>>>(t0, t1, nbr_off, nbr, nv, it + 1 == smoothing,
                                               vertex_normals, out);
    check_launch();
    call.launched();
    std::swap(t0, t1);
  }
}

void curvature_host(Call &call, const sym_mesh_view &m, const sym_topology_view &g,
                    const sym_options &o, const sym_features_out &out) {
  const uint64_t nv = m.vertices.count, nf = m.faces.count, ne = g.edge_count;
  if (out.count != nv || g.normals.count != nv || g.neighbors.rows != nv)
    fail(SYM_INVALID_ARGUMENT, "SoA component lengths differ");
  if (nv == 0) return;
  if (o.smoothing < 0) fail(SYM_INVALID_ARGUMENT, "Invalid parameter range; see --help");
  validate_csr(g.neighbors, nv, nv, "neighbors");
  uint64_t nbr_count = g.neighbors.offsets[nv];
  double *xyz = upload_points(call, m.vertices);
  double *fn = upload_points(call, g.face_normals);
  double *vn = upload_points(call, g.normals);
  uint64_t *nbr_off = call.upload(g.neighbors.offsets, nv + 1);
  int32_t *nbr = call.upload(g.neighbors.indices, nbr_count);
  sym_edge *edges = call.upload(g.edges, ne);
  sym_features_out dev{};
  double *lanes = call.alloc<double>(11 * nv);
  uint8_t *valid = call.alloc<uint8_t>(nv);
  double **cols[11] = {&dev.normal_x, &dev.normal_y, &dev.normal_z, &dev.dmin_x, &dev.dmin_y,
                       &dev.dmin_z,   &dev.dmax_x,   &dev.dmax_y,   &dev.dmax_z, &dev.kmin,
                       &dev.kmax};
  for (int k = 0; k < 11; ++k) *cols[k] = lanes + k * nv;
  dev.valid = valid;
  dev.count = nv;
  (void)nf;
  curvature_device(call, xyz, nv, fn, g.face_normals.count, vn, nbr_off, nbr, nbr_count, edges, ne,
                   o.smoothing, dev, g.edges);
  double *host_cols[11] = {out.normal_x, out.normal_y, out.normal_z, out.dmin_x, out.dmin_y,
                           out.dmin_z,   out.dmax_x,   out.dmax_y,   out.dmax_z, out.kmin,
                           out.kmax};
  for (int k = 0; k < 11; ++k) call.d2h(host_cols[k], lanes + k * nv, nv * 8);
  call.d2h(out.valid, valid, nv);
  call.check_status("curvature");
}

}  // namespace sym
