// SPDX-License-Identifier: MPL-2.0
// Stage (d): verification of every cluster by closest-point tests and
// region growing.
//
// Reference: src/cpu/verification.cpp:22-110, src/cpu/surface.h:12-96,
// src/core/math.cpp:72-112 (CPU); src/cuda/verification.cu (existing GPU
// path: one launch per cluster and a host-driven label propagation loop).
//
// GB300 design:
//  * the median-split BVH is built exactly as the reference builds it
//    (std::nth_element on face centroids, leaves of <= 8 faces), so the
//    near-first, strict-< traversal returns the same face on distance ties
//    and the normal test agrees; the traversal itself runs on the GPU;
//  * ONE launch covers every cluster, both directions and every vertex;
//  * rms / coverage use the reference's serial summation order (one thread
//    per cluster), so coverage is bit-exact;
//  * patches are connected components grown on the GPU with lock-free
//    union-find that always links the larger root under the smaller one, so
//    a component's root is its smallest vertex; a stable sort by (cluster,
//    side, root) then yields the reference's breadth-first patch order
//    (patches by smallest vertex, members ascending).
#include "common.cuh"
#include "primitives.cuh"
#include "verification.cuh"

#include <algorithm>
#include <cmath>
#include <limits>
#include <numeric>
#include <vector>

namespace sym {

__host__ __device__ inline double segment_d2(D3 p, D3 a, D3 b) {
  D3 d = b - a;
  double l = dot(d, d);
  double t = 0;
  if (l > 1e-14) {
    t = dot(p - a, d) / l;
    t = t < 0.0 ? 0.0 : (1.0 < t ? 1.0 : t);
  }
  D3 e = p - (a + d * t);
  return dot(e, e);
}

// Ericson, "Real-Time Collision Detection" 5.1.5 region test; degenerate
// triangles use the nearest of their three segments (reference math.cpp).
__host__ __device__ inline double triangle_d2(D3 p, D3 a, D3 b, D3 c) {
  D3 ab = b - a, ac = c - a, ap = p - a;
  D3 n = cross(ab, ac);
  if (dot(n, n) < 1e-14 * 1e-14) {
    double s0 = segment_d2(p, a, b), s1 = segment_d2(p, a, c), s2 = segment_d2(p, b, c);
    double m = s1 < s0 ? s1 : s0;
    return s2 < m ? s2 : m;
  }
  double d1 = dot(ab, ap), d2 = dot(ac, ap);
  if (d1 <= 0 && d2 <= 0) return dot(ap, ap);
  D3 bp = p - b;
  double d3 = dot(ab, bp), d4 = dot(ac, bp);
  if (d3 >= 0 && d4 <= d3) return dot(bp, bp);
  double vc = d1 * d4 - d3 * d2;
  if (vc <= 0 && d1 >= 0 && d3 <= 0) {
    D3 e = p - (a + ab * (d1 / (d1 - d3)));
    return dot(e, e);
  }
  D3 cp = p - c;
  double d5 = dot(ab, cp), d6 = dot(ac, cp);
  if (d6 >= 0 && d5 <= d6) return dot(cp, cp);
  double vb = d5 * d2 - d1 * d6;
  if (vb <= 0 && d2 >= 0 && d6 <= 0) {
    D3 e = p - (a + ac * (d2 / (d2 - d6)));
    return dot(e, e);
  }
  double va = d3 * d6 - d5 * d4;
  if (va <= 0 && (d4 - d3) >= 0 && (d5 - d6) >= 0) {
    D3 e = p - (b + (c - b) * ((d4 - d3) / ((d4 - d3) + (d5 - d6))));
    return dot(e, e);
  }
  D3 e = p - (a + ab * (vb / (va + vb + vc)) + ac * (vc / (va + vb + vc)));
  double r = dot(e, e);
  return r > 0.0 ? r : 0.0;
}

namespace {

struct Node {
  double lo[3], hi[3];
  int32_t left, right, begin, end;
};

// Host BVH with the reference's construction order.
class HostBvh {
public:
  std::vector<Node> nodes;
  std::vector<int32_t> ids;
  HostBvh(const sym_mesh_view &m) : m_(m) {
    ids.resize(m.faces.count);
    std::iota(ids.begin(), ids.end(), 0);
    if (!ids.empty()) build(0, int(ids.size()), 0);
  }
  int depth = 0;

private:
  const sym_mesh_view &m_;
  double coord(int f, int corner, int axis) const {
    const int32_t *col = corner == 0 ? m_.faces.v0 : (corner == 1 ? m_.faces.v1 : m_.faces.v2);
    int32_t v = col[f];
    const double *c = axis == 0 ? m_.vertices.x : (axis == 1 ? m_.vertices.y : m_.vertices.z);
    return c[v];
  }
  int build(int begin, int end, int level) {
    depth = std::max(depth, level);
    Node n;
    for (int k = 0; k < 3; ++k) n.lo[k] = 1e300, n.hi[k] = -1e300;
    for (int i = begin; i < end; ++i)
      for (int corner = 0; corner < 3; ++corner)
        for (int k = 0; k < 3; ++k) {
          double x = coord(ids[i], corner, k);
          n.lo[k] = std::min(n.lo[k], x);
          n.hi[k] = std::max(n.hi[k], x);
        }
    n.begin = begin, n.end = end, n.left = -1, n.right = -1;
    int index = int(nodes.size());
    nodes.push_back(n);
    if (end - begin > 8) {
      double ext[3] = {n.hi[0] - n.lo[0], n.hi[1] - n.lo[1], n.hi[2] - n.lo[2]};
      int axis = ext[1] > ext[0] ? 1 : 0;
      if (ext[2] > ext[axis]) axis = 2;
      int mid = (begin + end) / 2;
      auto centroid = [&](int f) {
        return (coord(f, 0, axis) + coord(f, 1, axis) + coord(f, 2, axis)) / 3;
      };
      std::nth_element(ids.begin() + begin, ids.begin() + mid, ids.begin() + end,
                       [&](int a, int b) { return centroid(a) < centroid(b); });
      int l = build(begin, mid, level + 1), r = build(mid, end, level + 1);
      nodes[index].left = l;
      nodes[index].right = r;
    }
    return index;
  }
};

__device__ double box_d2(D3 p, const Node &n) {
  double s = 0, a[3] = {p.x, p.y, p.z};
  for (int k = 0; k < 3; ++k) {
    double d = fmax(fmax(n.lo[k] - a[k], 0.0), a[k] - n.hi[k]);
    s += d * d;
  }
  return s;
}

struct Surface {
  const double *xyz;
  uint64_t nv;
  const int32_t *faces;  // 3 x nf
  uint64_t nf;
  const Node *nodes;
  const int32_t *ids;
};

__device__ D3 vertex(const Surface &s, int32_t v) { return {s.xyz[v], s.xyz[s.nv + v], s.xyz[2 * s.nv + v]}; }
__device__ D3 corner(const Surface &s, int32_t f, int k) { return vertex(s, s.faces[uint64_t(k) * s.nf + f]); }

constexpr int kStack = 96;

// Near-first search identical to the reference's recursion: a node is
// skipped when its box is farther than the best so far, the nearer child
// is searched first, faces win only with a strictly smaller distance.
// The search starts from `limit` (the next double above tau^2) instead of
// infinity: the caller rejects every distance above tau^2, nodes farther
// than the limit can hold no face the reference would accept, and the
// visiting order of the nodes that remain is unchanged, so an accepted
// query finds the reference's face and distance.  Rejected queries report
// no face.
__device__ double nearest_face(const Surface &s, D3 p, double limit, int32_t &face, int *status) {
  double best = limit;
  face = -1;
  int stack[kStack], top = 0;
  stack[top++] = 0;
  while (top) {
    const Node &n = s.nodes[stack[--top]];
    if (box_d2(p, n) > best) continue;
    if (n.left < 0) {
      for (int i = n.begin; i < n.end; ++i) {
        int32_t f = s.ids[i];
        double d = triangle_d2(p, corner(s, f, 0), corner(s, f, 1), corner(s, f, 2));
        if (d < best) best = d, face = f;
      }
    } else {
      int first = n.left, second = n.right;
      if (box_d2(p, s.nodes[first]) > box_d2(p, s.nodes[second])) {
        int t = first;
        first = second;
        second = t;
      }
      if (top + 2 > kStack) {
        atomicExch(status, DS_CAPACITY);
        return best;
      }
      stack[top++] = second;
      stack[top++] = first;
    }
  }
  return best;
}

struct ClusterMotion {
  double r[9], t[3], n[3], offset;
  int32_t reflection;
};

// flags[(c * 2 + dir) * nv + i], err[c * nv + i] (forward direction).
__global__ void verify_vertices(Surface s, const double *vn, const ClusterMotion *clusters,
                                uint64_t nc, double tau, double limit, uint8_t *flags, double *err,
                                int *status) {
  uint64_t row = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  uint64_t nv = s.nv;
  if (row >= nc * 2 * nv) return;
  uint64_t c = row / (2 * nv), rem = row % (2 * nv);
  bool inverse = rem >= nv;
  uint64_t i = rem % nv;
  flags[row] = 0;
  if (!inverse) err[c * nv + i] = 0;
  const ClusterMotion &m = clusters[c];
  M3 r;
  for (int k = 0; k < 9; ++k) r.m[k] = m.r[k];
  if (inverse) r = transpose(r);
  D3 t{m.t[0], m.t[1], m.t[2]}, pn{m.n[0], m.n[1], m.n[2]};
  D3 p = vertex(s, int32_t(i));
  D3 q = inverse ? mul(r, p - t) : mul(r, p) + t;
  if (norm(q - p) < tau * 2) return;
  if (m.reflection) {
    double side = dot(pn, p) + m.offset;
    if (inverse ? side <= tau : side >= -tau) return;
  }
  int32_t face;
  double d = nearest_face(s, q, limit, face, status);
  if (d > tau * tau || face < 0) return;
  D3 a = corner(s, face, 0), b = corner(s, face, 1), cc = corner(s, face, 2);
  D3 fnorm = unit(cross(b - a, cc - a));
  D3 ni{vn[i], vn[nv + i], vn[2 * nv + i]};
  if (dot(mul(r, ni), fnorm) < 0.5) return;
  flags[row] = 1;
  if (!inverse) err[c * nv + i] = d;
}

// Serial sums in the reference's order: thread c < nc handles cluster c,
// thread nc the total weight.
__global__ void ordered_sums(const uint8_t *flags, const double *err, const double *w, uint64_t nv,
                             uint64_t nc, double *error, double *area, uint64_t *side_a_size,
                             double *total) {
  uint64_t c = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (c > nc) return;
  if (c == nc) {
    double t = 0;
    for (uint64_t i = 0; i < nv; ++i) t += w[i];
    *total = t;
    return;
  }
  double e = 0, a = 0;
  uint64_t na = 0;
  const uint8_t *fa = flags + c * 2 * nv, *fb = fa + nv;
  for (uint64_t i = 0; i < nv; ++i)
    if (fa[i]) e += err[c * nv + i], a += w[i], ++na;
  for (uint64_t i = 0; i < nv; ++i)
    if (fb[i]) a += w[i];
  error[c] = e;
  area[c] = a;
  side_a_size[c] = na;
}

}  // namespace

// Union-find over (set, vertex) rows (find_root: verification.cuh).
// parent index space: (c * 2 + dir) * nv + i ; -1 marks excluded vertices.
__global__ void init_parents(const uint8_t *flags, uint64_t n, int32_t *parent, uint64_t nv) {
  uint64_t k = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < n) parent[k] = flags[k] ? int32_t(k % nv) : -1;
}

__global__ void unite_edges(const uint64_t *nbr_off, const int32_t *nbr, uint64_t nv, uint64_t sets,
                            int32_t *parent_all, int *status) {
  uint64_t k = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= sets * nv) return;
  uint64_t set = k / nv;
  int32_t i = int32_t(k % nv);
  int32_t *parent = parent_all + set * nv;
  if (parent[i] < 0) return;
  for (uint64_t e = nbr_off[i]; e < nbr_off[i + 1]; ++e) {
    int32_t u = nbr[e];
    if (u <= i || parent[u] < 0) continue;  // each edge once, allowed ends only
    for (int guard = 0;; ++guard) {
      if (guard > (1 << 20)) {
        atomicExch(status, DS_SPIN_LIMIT);
        return;
      }
      int32_t a = find_root(parent, i), b = find_root(parent, u);
      if (a < 0 || b < 0) {
        atomicExch(status, DS_SPIN_LIMIT);
        return;
      }
      if (a == b) break;
      if (a > b) {
        int32_t t = a;
        a = b;
        b = t;
      }
      if (atomicCAS(&parent[b], b, a) == b) break;
    }
  }
}

namespace {

// keys for the grouping sort: (set << 32) | root, values: vertex.
__global__ void root_keys(int32_t *parent_all, uint64_t nv, uint64_t sets, uint64_t *keys,
                          int32_t *vals, uint8_t *allowed) {
  uint64_t k = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= sets * nv) return;
  uint64_t set = k / nv;
  int32_t *parent = parent_all + set * nv;
  int32_t i = int32_t(k % nv);
  allowed[k] = parent[i] >= 0;
  int32_t r = parent[i] >= 0 ? find_root(parent, i) : 0;
  keys[k] = (set << 32) | uint64_t(uint32_t(r));
  vals[k] = i;
}

__global__ void gather_kept(const int32_t *pos, uint64_t n, const uint64_t *keys, uint64_t nv,
                            uint64_t *out_keys, int32_t *out_vals) {
  uint64_t k = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= n) return;
  uint64_t at = uint64_t(uint32_t(pos[k]));
  out_keys[k] = keys[at];
  out_vals[k] = int32_t(at % nv);
}

__global__ void triangle_query(const double *q, uint64_t n, double *out) {
  uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double *r = q + i * 12;
  out[i] = triangle_d2({r[0], r[1], r[2]}, {r[3], r[4], r[5]}, {r[6], r[7], r[8]}, {r[9], r[10], r[11]});
}

}  // namespace

void triangle_distances_host(Call &call, const double *queries, uint64_t count, double *out) {
  if (!count) return;
  double *q = call.upload(queries, count * 12);
  double *d = call.alloc<double>(count);
  triangle_query<<<blocks_for(count), kThreads, 0, call.stream()>>>(q, count, d);
  check_launch();
  call.launched();
  call.d2h(out, d, count * 8);
  call.sync();
}

// Device core shared by the ABI entry point and the resident pipeline.
// Mesh arrays are device pointers; `m` is the host mesh (the BVH is built on
// the host with the reference's construction order).  Fills per (cluster,
// side) vertex lists, patches, rms and coverage.
void verification_core(Call &call, const sym_mesh_view &m, const double *xyz, const int32_t *faces,
                       const double *vn, const double *w, const uint64_t *nbr_off,
                       const int32_t *nbr, const sym_cluster_record *records, uint64_t nc,
                       double tau, std::vector<std::vector<int32_t>> &side,
                       std::vector<std::vector<std::vector<int32_t>>> &patches,
                       std::vector<double> &coverage, std::vector<double> &rms) {
  const uint64_t nv = m.vertices.count, nf = m.faces.count;
  cudaStream_t st = call.stream();
  side.assign(2 * nc, {});
  patches.assign(2 * nc, {});
  coverage.assign(nc, 0);
  rms.assign(nc, 0);
  if (!nc) return;
  HostBvh bvh(m);
  if (2 * bvh.depth + 4 > kStack) fail(SYM_RUNTIME_ERROR, "verification: BVH too deep");
  Surface s;
  s.xyz = xyz;
  s.nv = nv;
  s.faces = faces;
  s.nf = nf;
  s.nodes = call.upload(bvh.nodes.data(), bvh.nodes.size());
  s.ids = call.upload(bvh.ids.data(), bvh.ids.size());
  std::vector<ClusterMotion> motions(nc);
  for (uint64_t c = 0; c < nc; ++c) {
    const sym_cluster_record &r = records[c];
    for (int k = 0; k < 9; ++k) motions[c].r[k] = r.rotation[k];
    for (int k = 0; k < 3; ++k) motions[c].t[k] = r.translation[k], motions[c].n[k] = r.plane_normal[k];
    motions[c].offset = r.plane_offset;
    motions[c].reflection = r.reflection != 0;
  }
  ClusterMotion *dm = call.upload(motions.data(), nc);
  uint64_t rows = nc * 2 * nv;
  uint8_t *flags = call.alloc<uint8_t>(rows);
  double *err = call.alloc<double>(nc * nv);
  double limit = std::nextafter(tau * tau, std::numeric_limits<double>::infinity());
  verify_vertices<<<blocks_for(rows), kThreads, 0, st>>>(s, vn, dm, nc, tau, limit, flags, err,
                                                         call.status());
  check_launch();
  double *error = call.alloc<double>(nc), *area = call.alloc<double>(nc), *total = call.alloc<double>(1);
  uint64_t *na = call.alloc<uint64_t>(nc);
  ordered_sums<<<blocks_for(nc + 1, 64), 64, 0, st>>>(flags, err, w, nv, nc, error, area, na, total);
  check_launch();
  int32_t *parent = call.alloc<int32_t>(rows);
  init_parents<<<blocks_for(rows), kThreads, 0, st>>>(flags, rows, parent, nv);
  check_launch();
  unite_edges<<<blocks_for(rows), kThreads, 0, st>>>(nbr_off, nbr, nv, 2 * nc, parent, call.status());
  check_launch();
  uint64_t *keys = call.alloc<uint64_t>(rows), *skeys = call.alloc<uint64_t>(rows);
  int32_t *vals = call.alloc<int32_t>(rows), *svals = call.alloc<int32_t>(rows);
  uint8_t *allowed = call.alloc<uint8_t>(rows);
  root_keys<<<blocks_for(rows), kThreads, 0, st>>>(parent, nv, 2 * nc, keys, vals, allowed);
  check_launch();
  uint64_t *kept = call.alloc<uint64_t>(1);
  int32_t *pos = call.alloc<int32_t>(rows);
  compact_indices(call, allowed, rows, pos, kept);
  uint64_t nkept = 0;
  call.d2h(&nkept, kept, 8);
  call.sync();
  call.launched(5);
  std::vector<uint64_t> hkeys(nkept);
  std::vector<int32_t> hvals(nkept);
  if (nkept) {
    uint64_t *dk = call.alloc<uint64_t>(nkept);
    int32_t *dv = call.alloc<int32_t>(nkept);
    gather_kept<<<blocks_for(nkept), kThreads, 0, st>>>(pos, nkept, keys, nv, dk, dv);
    check_launch();
    int bits = 32;
    while ((uint64_t(1) << (bits - 32)) < 2 * nc) ++bits;
    radix_sort_pairs(call, dk, dv, skeys, svals, nkept, bits);
    call.d2h(hkeys.data(), skeys, nkept * 8);
    call.d2h(hvals.data(), svals, nkept * 4);
  }
  std::vector<double> herr(nc), harea(nc);
  std::vector<uint64_t> hna(nc);
  double htotal = 0;
  call.d2h(herr.data(), error, nc * 8);
  call.d2h(harea.data(), area, nc * 8);
  call.d2h(hna.data(), na, nc * 8);
  call.d2h(&htotal, total, 8);
  call.check_status("verification");
  for (uint64_t k = 0; k < nkept; ++k) {
    uint64_t set = hkeys[k] >> 32;
    side[set].push_back(hvals[k]);
    if (k == 0 || hkeys[k] != hkeys[k - 1]) patches[set].emplace_back();
    patches[set].back().push_back(hvals[k]);
  }
  for (auto &sv : side) std::sort(sv.begin(), sv.end());
  for (uint64_t c = 0; c < nc; ++c) {
    rms[c] = hna[c] ? std::sqrt(herr[c] / double(hna[c])) : 0;
    coverage[c] = htotal > 0 ? std::min(1.0, harea[c] / htotal) : 0;
  }
}

void verification_host(Call &call, const sym_mesh_view &m, const sym_topology_view &g,
                       const sym_clusters_view &cl, const sym_model_context &ctx,
                       const sym_options &o, sym_verification_result &out,
                       void *(*allocate)(size_t)) {
  const uint64_t nv = m.vertices.count, nf = m.faces.count, nc = cl.count;
  std::vector<std::vector<int32_t>> side;
  std::vector<std::vector<std::vector<int32_t>>> patches;
  std::vector<double> coverage, rms;
  if (nc) {
    if (!nv || !nf) fail(SYM_INVALID_ARGUMENT, "verification requires a nonempty surface");
    if (g.normals.count != nv || g.weight_count != nv || g.neighbors.rows != nv)
      fail(SYM_INVALID_ARGUMENT, "SoA component lengths differ");
    validate_csr(g.neighbors, nv, nv, "neighbors");
    for (uint64_t f = 0; f < nf; ++f)
      if (m.faces.v0[f] < 0 || m.faces.v1[f] < 0 || m.faces.v2[f] < 0 ||
          uint64_t(m.faces.v0[f]) >= nv || uint64_t(m.faces.v1[f]) >= nv ||
          uint64_t(m.faces.v2[f]) >= nv)
        fail(SYM_INVALID_ARGUMENT, "Face index out of range");
    double *xyz = upload_points(call, m.vertices);
    int32_t *faces = upload_faces(call, m.faces);
    double *vn = upload_points(call, g.normals);
    double *w = call.upload(g.weights, nv);
    uint64_t nbr_count = g.neighbors.offsets[nv];
    uint64_t *nbr_off = call.upload(g.neighbors.offsets, nv + 1);
    int32_t *nbr = call.upload(g.neighbors.indices, nbr_count);
    verification_core(call, m, xyz, faces, vn, w, nbr_off, nbr, cl.records, nc,
                      o.verify_threshold * ctx.box_size, side, patches, coverage, rms);
  } else {
    side.assign(0, {});
    patches.assign(0, {});
  }
  uint64_t na = 0, nb = 0, ra = 0, rb = 0;
  for (uint64_t c = 0; c < nc; ++c) {
    na += side[2 * c].size(), nb += side[2 * c + 1].size();
    ra += patches[2 * c].size(), rb += patches[2 * c + 1].size();
  }
  size_t bytes = (2 * (nc + 1) + 2 * (nc + 1) + (ra + 1) + (rb + 1)) * 8 + 2 * (na + nb) * 4 +
                 2 * nc * 8 + 256;
  char *block = static_cast<char *>(allocate(bytes));
  if (!block) fail(SYM_RUNTIME_ERROR, "host allocation failed");
  out.storage = block;
  out.cluster_count = nc;
  uint64_t *u = reinterpret_cast<uint64_t *>(block);
  out.side_a_offsets = u, u += nc + 1;
  out.side_b_offsets = u, u += nc + 1;
  out.patches_a.groups = u, u += nc + 1;
  out.patches_b.groups = u, u += nc + 1;
  out.patches_a.offsets = u, u += ra + 1;
  out.patches_b.offsets = u, u += rb + 1;
  double *dd = reinterpret_cast<double *>(u);
  out.coverage = dd, dd += nc;
  out.rms = dd, dd += nc;
  int32_t *ii = reinterpret_cast<int32_t *>(dd);
  out.side_a = ii, ii += na;
  out.side_b = ii, ii += nb;
  out.patches_a.indices = ii, ii += na;
  out.patches_b.indices = ii, ii += nb;
  auto fill = [&](int dir, uint64_t *off, int32_t *idx, sym_grouped_csr &pg) {
    off[0] = 0;
    pg.groups[0] = 0;
    pg.offsets[0] = 0;
    uint64_t row = 0, at = 0;
    for (uint64_t c = 0; c < nc; ++c) {
      auto &sv = side[2 * c + dir];
      std::copy(sv.begin(), sv.end(), idx + off[c]);
      off[c + 1] = off[c] + sv.size();
      for (auto &p : patches[2 * c + dir]) {
        std::copy(p.begin(), p.end(), pg.indices + at);
        at += p.size();
        pg.offsets[++row] = at;
      }
      pg.groups[c + 1] = row;
    }
    pg.rows = row;
  };
  fill(0, out.side_a_offsets, out.side_a, out.patches_a);
  fill(1, out.side_b_offsets, out.side_b, out.patches_b);
  std::copy(coverage.begin(), coverage.end(), out.coverage);
  std::copy(rms.begin(), rms.end(), out.rms);
}

}  // namespace sym
