// SPDX-License-Identifier: MPL-2.0
// Pieces of the verification stage shared by the exact path
// (verification.cu) and the throughput path (verify_fast.cu).  Both units
// are compiled without FMA contraction, so the FP64 expressions below round
// exactly like the reference's (src/core/math.cpp:72-112,
// src/cpu/verification.cpp:50-110, src/cpu/surface.h:52-83).
#pragma once
#include "common.cuh"

#include <future>
#include <memory>
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

// Squared distance from p to triangle abc: Ericson, "Real-Time Collision
// Detection" 5.1.5 region tests; a triangle without area uses the nearest of
// its three segments (the reference's point_triangle_distance2).
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

// ------------------------------------------ the reference's median-split BVH
struct BvhNode {
  double lo[3], hi[3];
  int32_t left, right, begin, end;
};

__device__ inline double box_d2(D3 p, const BvhNode &n) {
  double s = 0, a[3] = {p.x, p.y, p.z};
  for (int k = 0; k < 3; ++k) {
    double d = fmax(fmax(n.lo[k] - a[k], 0.0), a[k] - n.hi[k]);
    s += d * d;
  }
  return s;
}

// Host build in the reference's construction order (surface.h:16-50:
// median split by std::nth_element on the longest axis, leaves of <= 8
// faces), so that a near-first strict-< traversal visits faces in the
// reference's order and resolves distance ties as it does.
struct HostBvh {
  std::vector<BvhNode> nodes;
  std::vector<int32_t> ids;
  // the visiting order's bookkeeping: each node's path from the root (bit
  // 31 - k = 1 when the step from depth k went to the right child), each
  // face's leaf and position in `ids`, and each leaf's ancestors by depth
  // (32 slots per leaf, leaf_slot[node] = the leaf's row, -1 inside)
  std::vector<uint32_t> path;
  std::vector<int32_t> leaf_slot, ancestors, face_leaf, face_pos;
  int depth = 0;
  explicit HostBvh(const sym_mesh_view &m);
};

// A copy of a HostBvh in device memory (cudaMalloc, owned).
struct RefBvh {
  const BvhNode *nodes = nullptr;
  const int32_t *ids = nullptr;
  const uint32_t *path = nullptr;
  const int32_t *leaf_slot = nullptr, *ancestors = nullptr, *face_leaf = nullptr,
                *face_pos = nullptr;
  char *block = nullptr;
  int depth = 0;
};
RefBvh ref_bvh_upload(const HostBvh &bvh, cudaStream_t stream);
void ref_bvh_free(RefBvh &b);

// Of two faces at exactly the same FP64 distance from q, the one the
// reference's search (surface.h:52-83) visits first: the lower position in
// a shared leaf, else the face under the child of their lowest common
// ancestor that the near-first rule searches first (the left child unless
// its box is strictly farther).  The search reaches both faces, since no
// node holding a face at the minimum distance is farther than it.
__device__ inline int32_t first_in_reference_order(const RefBvh &t, D3 q, int32_t a, int32_t b) {
  if (a == b) return a;
  const int32_t la = t.face_leaf[a], lb = t.face_leaf[b];
  if (la == lb) return t.face_pos[a] < t.face_pos[b] ? a : b;
  const uint32_t pa = t.path[la], pb = t.path[lb];
  const int depth = __clz(pa ^ pb);  // depth of the lowest common ancestor
  const BvhNode &lca = t.nodes[t.ancestors[t.leaf_slot[la] * 32 + depth]];
  const bool right_first = box_d2(q, t.nodes[lca.left]) > box_d2(q, t.nodes[lca.right]);
  const bool a_right = (pa >> (31 - depth)) & 1u;
  return a_right == right_first ? a : b;
}

constexpr int kRefStack = 96;

struct Surface {
  const double *xyz;
  uint64_t nv;
  const int32_t *faces;  // 3 x nf
  uint64_t nf;
  const BvhNode *nodes;
  const int32_t *ids;
};

__device__ inline D3 vertex(const Surface &s, int32_t v) {
  return {s.xyz[v], s.xyz[s.nv + v], s.xyz[2 * s.nv + v]};
}
__device__ inline D3 corner(const Surface &s, int32_t f, int k) {
  return vertex(s, s.faces[uint64_t(k) * s.nf + f]);
}

// Near-first search identical to the reference's recursion (surface.h:
// 52-83): a node is skipped when its box is farther than the best so far,
// the nearer child is searched first, faces win only with a strictly
// smaller distance.  The search starts from `limit` (the next double above
// tau^2) instead of infinity: the caller rejects every distance above tau^2,
// nodes farther than the limit can hold no face the reference would accept,
// and the visiting order of the nodes that remain is unchanged, so an
// accepted query finds the reference's face and distance.  Rejected queries
// report no face.
__device__ inline double nearest_face(const Surface &s, D3 p, double limit, int32_t &face,
                                      int *status) {
  double best = limit;
  face = -1;
  int stack[kRefStack], top = 0;
  stack[top++] = 0;
  while (top) {
    const BvhNode &n = s.nodes[stack[--top]];
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
      if (top + 2 > kRefStack) {
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

ClusterMotion cluster_motion(const sym_cluster_record &r);

// The motion of one query direction: R (R^T for the inverse direction).
__device__ inline M3 query_rotation(const ClusterMotion &m, bool inverse) {
  M3 r;
  for (int k = 0; k < 9; ++k) r.m[k] = m.r[k];
  return inverse ? transpose(r) : r;
}

// The reference's tests before the closest-point search
// (verification.cpp:63-67 and :81-85): the image q of vertex p, and whether
// the vertex is skipped (moves less than 2 tau, or lies on the wrong side of
// a reflection plane).
__device__ inline bool query_skipped(const ClusterMotion &m, const M3 &r, bool inverse, D3 p,
                                     double tau, D3 &q) {
  const D3 t{m.t[0], m.t[1], m.t[2]}, pn{m.n[0], m.n[1], m.n[2]};
  q = inverse ? mul(r, p - t) : mul(r, p) + t;
  if (norm(q - p) < tau * 2) return true;
  if (m.reflection) {
    const double side = dot(pn, p) + m.offset;
    if (inverse ? side <= tau : side >= -tau) return true;
  }
  return false;
}

// The reference's normal test against face f (verification.cpp:70-73):
// the vertex normal, turned by the query's rotation, within 60 degrees of
// the face normal.  A face without area gets the zero vector as its unit
// normal (unit(), math.cpp:18-21) and fails the test, as in the reference.
__device__ inline bool normal_agrees(const Surface &s, int32_t f, const M3 &r, D3 ni) {
  const D3 a = corner(s, f, 0), b = corner(s, f, 1), c = corner(s, f, 2);
  const D3 fnorm = unit(cross(b - a, c - a));
  return !(dot(mul(r, ni), fnorm) < 0.5);
}

// One (cluster, direction, vertex) query of the reference's verification
// through the reference-order BVH: returns whether the vertex supports the
// cluster in that direction, and its squared distance in `d2`.
__device__ inline bool exact_query(const Surface &s, const double *vn, const ClusterMotion &m,
                                   bool inverse, uint64_t i, double tau, double limit, double &d2,
                                   int *status) {
  const M3 r = query_rotation(m, inverse);
  const D3 p = vertex(s, int32_t(i));
  D3 q;
  if (query_skipped(m, r, inverse, p, tau, q)) return false;
  int32_t face;
  const double d = nearest_face(s, q, limit, face, status);
  if (d > tau * tau || face < 0) return false;
  const D3 ni{vn[i], vn[s.nv + i], vn[2 * s.nv + i]};
  if (!normal_agrees(s, face, r, ni)) return false;
  d2 = d;
  return true;
}

// Union-find over rows (set * nv + vertex): parent = own vertex for the
// rows whose flag is set, -1 for the others; unite_edges joins the allowed
// ends of every mesh edge within a set, always linking the larger root
// under the smaller, so a component's root is its smallest vertex.
__device__ __forceinline__ int32_t find_root(int32_t *parent, int32_t x) {
  for (int guard = 0; guard < (1 << 26); ++guard) {
    int32_t p = parent[x];
    if (p == x) return x;
    int32_t g = parent[p];
    if (g != p) parent[x] = g;  // path halving; parents only decrease
    x = p;
  }
  return -1;
}
__global__ void init_parents(const uint8_t *flags, uint64_t n, int32_t *parent, uint64_t nv);
// A union that keeps losing its compare-and-swap retries at most
// retry_limit times, then records DS_SPIN_LIMIT and stops (kUniteRetries in
// regular calls).
constexpr int kUniteRetries = 1 << 20;
__global__ void unite_edges(const uint64_t *nbr_off, const int32_t *nbr, uint64_t nv, uint64_t sets,
                            int32_t *parent_all, int *status, int retry_limit);

// Sums of the reference's verification in its serial order
// (verification.cpp:75-77, :93-96, :98-99): per cluster the forward
// squared distances and the supporting weight (forward vertices in vertex
// order, then inverse ones), the forward count, and the total weight.  One
// warp per cluster stages 32 rows at a time and adds them in order, so the
// results equal the reference's bit for bit.  flags[(c * 2 + dir) * nv + i],
// err[c * nv + i].
void ordered_verification_sums(Call &call, const uint8_t *flags, const double *err,
                               const double *w, uint64_t nv, uint64_t nc, double *error,
                               double *area, uint64_t *count, double *total);

// From the flags and forward errors of nc clusters: patches (connected
// components of the supporting vertices, in the reference's breadth-first
// order), side lists, coverage and rms, all as the reference computes them.
void finish_verification(Call &call, const uint8_t *flags, const double *err, const double *w,
                         const uint64_t *nbr_off, const int32_t *nbr, uint64_t nv, uint64_t nc,
                         std::vector<std::vector<int32_t>> &side,
                         std::vector<std::vector<std::vector<int32_t>>> &patches,
                         std::vector<double> &coverage, std::vector<double> &rms);

// Writes side lists, patches, coverage and rms into a library-owned
// sym_verification_result (one host block from `allocate`).
void fill_verification_result(uint64_t nc, const std::vector<std::vector<int32_t>> &side,
                              const std::vector<std::vector<std::vector<int32_t>>> &patches,
                              const std::vector<double> &coverage, const std::vector<double> &rms,
                              sym_verification_result &out, void *(*allocate)(size_t));

// Linear BVH over the faces of a resident mesh, FP32 (throughput path).
struct Lbvh {
  uint64_t nv = 0, nf = 0;
  const int32_t *faces = nullptr;  // 3 x nf (the mesh's)
  float *xyz = nullptr;            // 3 x nv, FP32 copy of the vertices
  int32_t *child = nullptr;        // (nf - 1) x 2: >= 0 internal node, < 0 leaf ~face
  float *box = nullptr;            // (nf - 1) x 12: the two children's lo[3], hi[3]
  float *vn = nullptr;             // 3 x nv, FP32 copy of the vertex normals
  float4 *fn = nullptr;            // nf: unit face normals from the FP64 corners, w = 1 (0: none)
  int32_t *order = nullptr;        // nv: the vertices in Morton order of their position
  double *fn64 = nullptr;          // nf x 3: unit(cross(b - a, c - a)) of each face, FP64
  char *block = nullptr;           // owns every array above (cudaMalloc)
  float scale = 0;                 // largest vertex coordinate magnitude
};

// The reference-order BVH of a resident mesh: built on a host thread from
// the moment the mesh is loaded (`pending`), uploaded when a verification
// first needs it (`dev`).
struct RefBvhSource {
  RefBvh dev;
  std::future<std::unique_ptr<HostBvh>> pending;
  // starts the host build from copies of the mesh's vertices and faces
  void start(std::vector<double> xyz, std::vector<int32_t> faces, uint64_t nv, uint64_t nf);
  void release();  // waits for a pending build, frees the device copy
};

// A resident mesh as the throughput verification sees it (device arrays).
struct ResidentSurface {
  const Lbvh *lbvh;
  const double *xyz, *vn, *w;  // 3 x nv, 3 x nv, nv
  const int32_t *faces;        // 3 x nf
  const uint64_t *nbr_off;     // nv + 1
  const int32_t *nbr;
  uint64_t nv, nf;
  RefBvhSource *ref;  // the reference-order BVH (owned by the mesh)
};

// Flags and forward errors of nc motions (`records`, and dm: the same on the
// device) with the reference's decisions: FP32 decisions outside the error
// bands of their tests, FP64 rechecks of the rows inside (their number in
// *fp64_rows), and the reference-order BVH for the queries those leave
// undecided (their number is returned).
uint64_t exact_flags(Call &call, const ResidentSurface &m, const ClusterMotion *dm,
                     const sym_cluster_record *records, uint64_t nc, double tau, uint8_t *flags,
                     double *err, uint64_t *fp64_rows);

// Coverage, rms and patch counts (forward, inverse) of nc motions after
// `refine` FP64 refinement passes (the refined motions are written back).
// Supporting vertices and patches are the reference's; coverage and rms
// come from fixed-order tree sums, within a few units of rounding of the
// reference's serial sums.
void verification_fast(Call &call, const ResidentSurface &m, sym_cluster_record *records,
                       uint64_t nc, double tau, int refine, const double origin[3],
                       double *coverage, double *rms, uint32_t *patches, uint64_t *undecided,
                       uint64_t *fp64_rows);

// The reference's full verification of nc records on a resident mesh.
void verification_resident(Call &call, const ResidentSurface &m, const sym_cluster_record *records,
                           uint64_t nc, double tau, std::vector<std::vector<int32_t>> &side,
                           std::vector<std::vector<std::vector<int32_t>>> &patches,
                           std::vector<double> &coverage, std::vector<double> &rms,
                           uint64_t *undecided);

// Builds the LBVH on the device (synchronises); release with lbvh_free.
Lbvh lbvh_build(Call &call, const double *xyz, const double *vn, uint64_t nv,
                const int32_t *faces, uint64_t nf);
void lbvh_free(Lbvh &b);

}  // namespace sym
