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

HostBvh::HostBvh(const sym_mesh_view &m) {
  ids.resize(m.faces.count);
  for (uint64_t i = 0; i < ids.size(); ++i) ids[i] = int32_t(i);
  auto coord = [&](int f, int corner, int axis) {
    const int32_t *col = corner == 0 ? m.faces.v0 : (corner == 1 ? m.faces.v1 : m.faces.v2);
    const double *c = axis == 0 ? m.vertices.x : (axis == 1 ? m.vertices.y : m.vertices.z);
    return c[col[f]];
  };
  struct Builder {
    HostBvh &t;
    decltype(coord) &co;
    int build(int begin, int end, int level) {
      t.depth = std::max(t.depth, level);
      BvhNode n;
      for (int k = 0; k < 3; ++k) n.lo[k] = 1e300, n.hi[k] = -1e300;
      for (int i = begin; i < end; ++i)
        for (int corner = 0; corner < 3; ++corner)
          for (int k = 0; k < 3; ++k) {
            double x = co(t.ids[i], corner, k);
            n.lo[k] = std::min(n.lo[k], x);
            n.hi[k] = std::max(n.hi[k], x);
          }
      n.begin = begin, n.end = end, n.left = -1, n.right = -1;
      int index = int(t.nodes.size());
      t.nodes.push_back(n);
      if (end - begin > 8) {
        double ext[3] = {n.hi[0] - n.lo[0], n.hi[1] - n.lo[1], n.hi[2] - n.lo[2]};
        int axis = ext[1] > ext[0] ? 1 : 0;
        if (ext[2] > ext[axis]) axis = 2;
        int mid = (begin + end) / 2;
        auto centroid = [&](int f) { return (co(f, 0, axis) + co(f, 1, axis) + co(f, 2, axis)) / 3; };
        std::nth_element(t.ids.begin() + begin, t.ids.begin() + mid, t.ids.begin() + end,
                         [&](int a, int b) { return centroid(a) < centroid(b); });
        int l = build(begin, mid, level + 1), r = build(mid, end, level + 1);
        t.nodes[index].left = l;
        t.nodes[index].right = r;
      }
      return index;
    }
  } builder{*this, coord};
  if (!ids.empty()) builder.build(0, int(ids.size()), 0);
  if (depth > 31) throw Error(SYM_RUNTIME_ERROR, "verification: BVH too deep");
  path.assign(nodes.size(), 0);
  leaf_slot.assign(nodes.size(), -1);
  face_leaf.assign(ids.size(), -1);
  face_pos.assign(ids.size(), -1);
  std::vector<int32_t> node_depth(nodes.size(), 0), parent(nodes.size(), -1);
  int32_t leaves = 0;
  for (size_t n = 0; n < nodes.size(); ++n) {  // parents precede their children
    const BvhNode &b = nodes[n];
    if (b.left >= 0) {
      const int d = node_depth[n];
      parent[b.left] = parent[b.right] = int32_t(n);
      node_depth[b.left] = node_depth[b.right] = d + 1;
      path[b.left] = path[n];
      path[b.right] = path[n] | (1u << (31 - d));
    } else {
      leaf_slot[n] = leaves++;
      for (int32_t i = b.begin; i < b.end; ++i) face_leaf[ids[i]] = int32_t(n), face_pos[ids[i]] = i;
    }
  }
  ancestors.assign(size_t(leaves) * 32, -1);
  for (size_t n = 0; n < nodes.size(); ++n)
    if (leaf_slot[n] >= 0)
      for (int32_t a = int32_t(n); a >= 0; a = parent[a])
        ancestors[size_t(leaf_slot[n]) * 32 + node_depth[a]] = a;
}

RefBvh ref_bvh_upload(const HostBvh &bvh, cudaStream_t stream) {
  RefBvh b;
  b.depth = bvh.depth;
  auto pad = [](size_t x) { return (x + 255) & ~size_t(255); };
  const size_t nn = bvh.nodes.size(), nf = bvh.ids.size(), na = bvh.ancestors.size();
  const size_t s_nodes = pad(nn * sizeof(BvhNode)), s_face = pad(nf * 4), s_node = pad(nn * 4),
               s_anc = pad(na * 4);
  SYM_CUDA(cudaMalloc(&b.block, s_nodes + 3 * s_face + 2 * s_node + s_anc + 256));
  char *at = b.block;
  auto put = [&](const void *src, size_t bytes, size_t room) {
    if (bytes) SYM_CUDA(cudaMemcpyAsync(at, src, bytes, cudaMemcpyHostToDevice, stream));
    char *here = at;
    at += room;
    return here;
  };
  b.nodes = reinterpret_cast<const BvhNode *>(put(bvh.nodes.data(), nn * sizeof(BvhNode), s_nodes));
  b.ids = reinterpret_cast<const int32_t *>(put(bvh.ids.data(), nf * 4, s_face));
  b.face_leaf = reinterpret_cast<const int32_t *>(put(bvh.face_leaf.data(), nf * 4, s_face));
  b.face_pos = reinterpret_cast<const int32_t *>(put(bvh.face_pos.data(), nf * 4, s_face));
  b.path = reinterpret_cast<const uint32_t *>(put(bvh.path.data(), nn * 4, s_node));
  b.leaf_slot = reinterpret_cast<const int32_t *>(put(bvh.leaf_slot.data(), nn * 4, s_node));
  b.ancestors = reinterpret_cast<const int32_t *>(put(bvh.ancestors.data(), na * 4, s_anc));
  SYM_CUDA(cudaStreamSynchronize(stream));
  return b;
}

void ref_bvh_free(RefBvh &b) {
  if (b.block) cudaFree(b.block);
  b = RefBvh{};
}

void RefBvhSource::start(std::vector<double> xyz, std::vector<int32_t> faces, uint64_t nv,
                         uint64_t nf) {
  pending = std::async(std::launch::async, [x = std::move(xyz), f = std::move(faces), nv, nf]() {
    const sym_mesh_view mv{{x.data(), x.data() + nv, x.data() + 2 * nv, nv},
                           {f.data(), f.data() + nf, f.data() + 2 * nf, nf}};
    return std::make_unique<HostBvh>(mv);
  });
}

void RefBvhSource::release() {
  if (pending.valid()) pending.wait();
  ref_bvh_free(dev);
}

namespace {

// flags[(c * 2 + dir) * nv + i], err[c * nv + i] (forward direction).
// Query (c, direction, j) takes vertex i = order[j], the vertices in Morton
// order of their position, so a warp walks neighbouring vertices through
// nearly the same BVH nodes; flags and errors stay per vertex (row).
__global__ void verify_vertices(Surface s, const double *vn, const int32_t *order,
                                const ClusterMotion *clusters, uint64_t nc, double tau,
                                double limit, uint8_t *flags, double *err, int *status) {
  const uint64_t qid = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const uint64_t nv = s.nv;
  if (qid >= nc * 2 * nv) return;
  const uint64_t c = qid / (2 * nv), rem = qid % (2 * nv);
  const bool inverse = rem >= nv;
  const uint64_t i = uint64_t(order[rem % nv]), row = qid - rem % nv + i;
  flags[row] = 0;
  if (!inverse) err[c * nv + i] = 0;
  double d = 0;
  if (!exact_query(s, vn, clusters[c], inverse, i, tau, limit, d, status)) return;
  flags[row] = 1;
  if (!inverse) err[c * nv + i] = d;
}

// One warp per cluster (block c < nc) or for the total weight (block nc):
// rows are staged 32 at a time in shared memory and lane 0 adds them in
// vertex order; a group of 32 rows with no flag set is skipped (adding
// nothing leaves the sums unchanged).
__global__ void __launch_bounds__(32) ordered_sums_warp(const uint8_t *flags, const double *err,
                                                         const double *w, uint64_t nv, uint64_t nc,
                                                         double *error, double *area,
                                                         uint64_t *count, double *total) {
  __shared__ double sv[32], sw[32];
  const uint64_t c = blockIdx.x;
  const unsigned lane = threadIdx.x;
  if (c == nc) {
    double t = 0;
    for (uint64_t base = 0; base < nv; base += 32) {
      const uint64_t i = base + lane;
      sw[lane] = i < nv ? w[i] : 0.0;
      __syncwarp();
      if (lane == 0) {
        const unsigned m = nv - base < 32 ? unsigned(nv - base) : 32u;
        for (unsigned j = 0; j < m; ++j) t += sw[j];
      }
      __syncwarp();
    }
    if (lane == 0) *total = t;
    return;
  }
  double e = 0, a = 0;
  unsigned long long n = 0;
  for (int dir = 0; dir < 2; ++dir) {
    const uint8_t *f = flags + (c * 2 + dir) * nv;
    for (uint64_t base = 0; base < nv; base += 32) {
      const uint64_t i = base + lane;
      const bool on = i < nv && f[i];
      const unsigned mask = __ballot_sync(0xffffffffu, on);
      if (!mask) continue;
      sw[lane] = on ? w[i] : 0.0;
      if (dir == 0) sv[lane] = on ? err[c * nv + i] : 0.0;
      __syncwarp();
      if (lane == 0)
        for (unsigned j = 0; j < 32; ++j)
          if (mask >> j & 1u) {
            if (dir == 0) e += sv[j], ++n;
            a += sw[j];
          }
      __syncwarp();
    }
  }
  if (lane == 0) error[c] = e, area[c] = a, count[c] = n;
}

}  // namespace

void ordered_verification_sums(Call &call, const uint8_t *flags, const double *err,
                               const double *w, uint64_t nv, uint64_t nc, double *error,
                               double *area, uint64_t *count, double *total) {
  ordered_sums_warp<<<unsigned(nc + 1), 32, 0, call.stream()>>>(flags, err, w, nv, nc, error, area,
                                                                 count, total);
  check_launch();
  call.launched();
}

// Union-find over (set, vertex) rows (find_root: verification.cuh).
// parent index space: (c * 2 + dir) * nv + i ; -1 marks excluded vertices.
__global__ void init_parents(const uint8_t *flags, uint64_t n, int32_t *parent, uint64_t nv) {
  uint64_t k = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < n) parent[k] = flags[k] ? int32_t(k % nv) : -1;
}

__global__ void unite_edges(const uint64_t *nbr_off, const int32_t *nbr, uint64_t nv, uint64_t sets,
                            int32_t *parent_all, int *status, int retry_limit) {
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
      if (guard >= retry_limit) {
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

// The union-find's bounded retry loop on a path of 64 vertices (every
// vertex supporting one set) with `retry_limit` retries: with 0 every union
// gives up at once and the call ends in the device-status error that a
// retry loop running out raises; with the regular limit the path becomes
// one component.  Returns the number of components.
uint64_t unite_selftest_host(Call &call, int retry_limit) {
  constexpr uint64_t n = 64;
  std::vector<uint64_t> off(n + 1);
  std::vector<int32_t> idx;
  for (uint64_t i = 0; i < n; ++i) {
    off[i] = idx.size();
    if (i > 0) idx.push_back(int32_t(i - 1));
    if (i + 1 < n) idx.push_back(int32_t(i + 1));
  }
  off[n] = idx.size();
  std::vector<uint8_t> flags(n, 1);
  cudaStream_t st = call.stream();
  const uint64_t *doff = call.upload(off.data(), n + 1);
  const int32_t *didx = call.upload(idx.data(), idx.size());
  const uint8_t *dflags = call.upload(flags.data(), n);
  int32_t *parent = call.alloc<int32_t>(n);
  init_parents<<<1, 64, 0, st>>>(dflags, n, parent, n);
  check_launch();
  unite_edges<<<1, 64, 0, st>>>(doff, didx, n, 1, parent, call.status(), retry_limit);
  check_launch();
  call.launched(2);
  std::vector<int32_t> h(n);
  call.d2h(h.data(), parent, n * 4);
  call.check_status("union-find self-test");
  uint64_t roots = 0;
  for (uint64_t i = 0; i < n; ++i) roots += h[i] == int32_t(i);
  return roots;
}

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

ClusterMotion cluster_motion(const sym_cluster_record &r) {
  ClusterMotion m{};
  for (int k = 0; k < 9; ++k) m.r[k] = r.rotation[k];
  for (int k = 0; k < 3; ++k) m.t[k] = r.translation[k], m.n[k] = r.plane_normal[k];
  m.offset = r.plane_offset;
  m.reflection = r.reflection != 0;
  return m;
}

void finish_verification(Call &call, const uint8_t *flags, const double *err, const double *w,
                         const uint64_t *nbr_off, const int32_t *nbr, uint64_t nv, uint64_t nc,
                         std::vector<std::vector<int32_t>> &side,
                         std::vector<std::vector<std::vector<int32_t>>> &patches,
                         std::vector<double> &coverage, std::vector<double> &rms) {
  cudaStream_t st = call.stream();
  side.assign(2 * nc, {});
  patches.assign(2 * nc, {});
  coverage.assign(nc, 0);
  rms.assign(nc, 0);
  if (!nc) return;
  const uint64_t rows = nc * 2 * nv;
  double *error = call.alloc<double>(nc), *area = call.alloc<double>(nc), *total = call.alloc<double>(1);
  uint64_t *na = call.alloc<uint64_t>(nc);
  ordered_verification_sums(call, flags, err, w, nv, nc, error, area, na, total);
  int32_t *parent = call.alloc<int32_t>(rows);
  init_parents<<<blocks_for(rows), kThreads, 0, st>>>(flags, rows, parent, nv);
  check_launch();
  unite_edges<<<blocks_for(rows), kThreads, 0, st>>>(nbr_off, nbr, nv, 2 * nc, parent, call.status(),
                                                      kUniteRetries);
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
  call.launched(3);
  std::vector<uint64_t> hkeys(nkept);
  std::vector<int32_t> hvals(nkept);
  if (nkept) {
    uint64_t *dk = call.alloc<uint64_t>(nkept);
    int32_t *dv = call.alloc<int32_t>(nkept);
    gather_kept<<<blocks_for(nkept), kThreads, 0, st>>>(pos, nkept, keys, nv, dk, dv);
    check_launch();
    call.launched();
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

// The vertices in Morton order of their position (10 bits per axis over
// the mesh's box, ties in index order): the query order of the
// verification kernels.
static std::vector<int32_t> morton_order(const sym_mesh_view &m) {
  const uint64_t nv = m.vertices.count;
  const double *x[3] = {m.vertices.x, m.vertices.y, m.vertices.z};
  double lo[3], ext = 0;
  for (int a = 0; a < 3; ++a) {
    lo[a] = nv ? *std::min_element(x[a], x[a] + nv) : 0.0;
    const double hi = nv ? *std::max_element(x[a], x[a] + nv) : 0.0;
    ext = std::max(ext, hi - lo[a]);
  }
  std::vector<uint64_t> key(nv);
  for (uint64_t v = 0; v < nv; ++v) {
    uint64_t code = 0;
    for (int a = 0; a < 3; ++a) {
      const double u = ext > 0 ? (x[a][v] - lo[a]) / ext * 1024.0 : 0.0;
      const uint64_t cell = uint64_t(std::min(1023.0, std::max(0.0, u)));
      for (int bit = 0; bit < 10; ++bit) code |= ((cell >> bit) & 1u) << (3 * bit + (2 - a));
    }
    key[v] = code << 32 | v;
  }
  std::sort(key.begin(), key.end());
  std::vector<int32_t> order(nv);
  for (uint64_t j = 0; j < nv; ++j) order[j] = int32_t(uint32_t(key[j]));
  return order;
}

// Device core of sym_verification.  Mesh arrays are device pointers; `m` is
// the host mesh (the BVH is built on the host with the reference's
// construction order).  Fills per (cluster, side) vertex lists, patches,
// rms and coverage.
void verification_core(Call &call, const sym_mesh_view &m, const double *xyz, const int32_t *faces,
                       const double *vn, const double *w, const uint64_t *nbr_off,
                       const int32_t *nbr, const sym_cluster_record *records, uint64_t nc,
                       double tau, std::vector<std::vector<int32_t>> &side,
                       std::vector<std::vector<std::vector<int32_t>>> &patches,
                       std::vector<double> &coverage, std::vector<double> &rms) {
  const uint64_t nv = m.vertices.count, nf = m.faces.count;
  cudaStream_t st = call.stream();
  if (!nc) {
    finish_verification(call, nullptr, nullptr, w, nbr_off, nbr, nv, 0, side, patches, coverage, rms);
    return;
  }
  HostBvh bvh(m);
  if (2 * bvh.depth + 4 > kRefStack) fail(SYM_RUNTIME_ERROR, "verification: BVH too deep");
  Surface s;
  s.xyz = xyz;
  s.nv = nv;
  s.faces = faces;
  s.nf = nf;
  s.nodes = call.upload(bvh.nodes.data(), bvh.nodes.size());
  s.ids = call.upload(bvh.ids.data(), bvh.ids.size());
  std::vector<ClusterMotion> motions(nc);
  for (uint64_t c = 0; c < nc; ++c) motions[c] = cluster_motion(records[c]);
  ClusterMotion *dm = call.upload(motions.data(), nc);
  uint64_t rows = nc * 2 * nv;
  uint8_t *flags = call.alloc<uint8_t>(rows);
  double *err = call.alloc<double>(nc * nv);
  double limit = std::nextafter(tau * tau, std::numeric_limits<double>::infinity());
  const std::vector<int32_t> order = morton_order(m);
  const int32_t *dorder = call.upload(order.data(), order.size());
  verify_vertices<<<blocks_for(rows), kThreads, 0, st>>>(s, vn, dorder, dm, nc, tau, limit, flags,
                                                         err, call.status());
  check_launch();
  call.launched();
  finish_verification(call, flags, err, w, nbr_off, nbr, nv, nc, side, patches, coverage, rms);
}

void fill_verification_result(uint64_t nc, const std::vector<std::vector<int32_t>> &side,
                              const std::vector<std::vector<std::vector<int32_t>>> &patches,
                              const std::vector<double> &coverage, const std::vector<double> &rms,
                              sym_verification_result &out, void *(*allocate)(size_t)) {
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
  }
  fill_verification_result(nc, side, patches, coverage, rms, out, allocate);
}

}  // namespace sym
