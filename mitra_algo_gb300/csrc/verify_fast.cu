// SPDX-License-Identifier: MPL-2.0
// Stage (d) on the throughput path: verification of resident meshes with a
// linear BVH built on the GPU, FP32 closest-point searches and FP64
// rechecks, with results identical to the reference's.
//
// The tests are the reference's (src/cpu/verification.cpp:22-110): a vertex
// supports a mode in one direction when its image under the mode's motion
// lies at least 2 tau from itself, on the correct side of a reflection
// plane, within tau of the surface, and its transformed normal is within
// 60 degrees of the nearest face's normal; coverage is the supporting
// vertices' weight over the total, rms the root mean square of the forward
// distances; patches are the connected components of the supporting
// vertices (region growing).
//
// How the decisions stay the reference's: the LBVH (Karras 2012: 30-bit
// Morton codes of the face centroids, radix sort, longest-common-prefix
// splits, boxes merged bottom-up, built once per resident mesh) is searched
// in FP32 for every face whose FP32 distance lies within a margin of the
// nearest one -- a margin several hundred times the FP32 error of a
// distance, so the face of smallest FP64 distance is always among them.
// Those candidates are re-evaluated with the reference's FP64 distance, and
// the FP64 nearest face takes the reference's FP64 distance and normal
// tests.  A query whose FP64 minimum is shared by faces that disagree on the
// normal test (the reference then keeps the face its BVH visits first), or
// whose candidates overflow the list, is re-run through the reference-order
// BVH (verification.cuh), built on the host once per resident mesh when the
// first such query appears.  Sums use the reference's serial order.
#include "primitives.cuh"
#include "verification.cuh"

#include <algorithm>
#include <cmath>
#include <limits>
#include <vector>

namespace sym {
namespace {

struct F3 {
  float x, y, z;
};
__device__ __forceinline__ F3 operator-(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ F3 operator+(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ F3 operator*(F3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ float dotf(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ F3 crossf(F3 a, F3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

__device__ float segment_d2f(F3 p, F3 a, F3 b) {
  F3 d = b - a;
  float l = dotf(d, d), t = 0;
  if (l > 1e-14f) t = fminf(fmaxf(dotf(p - a, d) / l, 0.f), 1.f);
  F3 e = p - (a + d * t);
  return dotf(e, e);
}

// The region test of triangle_d2 (verification.cu) in FP32.
__device__ float triangle_d2f(F3 p, F3 a, F3 b, F3 c) {
  F3 ab = b - a, ac = c - a, ap = p - a;
  F3 n = crossf(ab, ac);
  if (dotf(n, n) < 1e-28f)
    return fminf(fminf(segment_d2f(p, a, b), segment_d2f(p, a, c)), segment_d2f(p, b, c));
  float d1 = dotf(ab, ap), d2 = dotf(ac, ap);
  if (d1 <= 0 && d2 <= 0) return dotf(ap, ap);
  F3 bp = p - b;
  float d3 = dotf(ab, bp), d4 = dotf(ac, bp);
  if (d3 >= 0 && d4 <= d3) return dotf(bp, bp);
  float vc = d1 * d4 - d3 * d2;
  if (vc <= 0 && d1 >= 0 && d3 <= 0) {
    F3 e = p - (a + ab * (d1 / (d1 - d3)));
    return dotf(e, e);
  }
  F3 cp = p - c;
  float d5 = dotf(ab, cp), d6 = dotf(ac, cp);
  if (d6 >= 0 && d5 <= d6) return dotf(cp, cp);
  float vb = d5 * d2 - d1 * d6;
  if (vb <= 0 && d2 >= 0 && d6 <= 0) {
    F3 e = p - (a + ac * (d2 / (d2 - d6)));
    return dotf(e, e);
  }
  float va = d3 * d6 - d5 * d4;
  if (va <= 0 && (d4 - d3) >= 0 && (d5 - d6) >= 0) {
    F3 e = p - (b + (c - b) * ((d4 - d3) / ((d4 - d3) + (d5 - d6))));
    return dotf(e, e);
  }
  float den = va + vb + vc;
  F3 e = p - (a + ab * (vb / den) + ac * (vc / den));
  return fmaxf(dotf(e, e), 0.f);
}

// --------------------------------------------------------------- LBVH build
__device__ __forceinline__ uint32_t spread3(uint32_t v) {  // 10 bits -> every third of 30
  v &= 0x3ffu;
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

__global__ void lbvh_vertices(const double *xyz, uint64_t nv, float *xyz32) {
  uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < 3 * nv) xyz32[i] = float(xyz[i]);
}

// key = Morton code of the face centroid (30 bits) << 32 | face: unique.
__global__ void lbvh_keys(const float *xyz, uint64_t nv, const int32_t *faces, uint64_t nf,
                          float3 lo, float3 inv, uint64_t *keys, int32_t *ids) {
  uint64_t f = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  float c[3] = {0, 0, 0};
  for (int k = 0; k < 3; ++k) {
    int32_t v = faces[uint64_t(k) * nf + f];
    for (int a = 0; a < 3; ++a) c[a] += xyz[uint64_t(a) * nv + v];
  }
  float l[3] = {lo.x, lo.y, lo.z}, s[3] = {inv.x, inv.y, inv.z};
  uint32_t q[3];
  for (int a = 0; a < 3; ++a) {
    float u = (c[a] / 3.f - l[a]) * s[a];
    q[a] = uint32_t(fminf(fmaxf(u * 1024.f, 0.f), 1023.f));
  }
  uint32_t code = (spread3(q[0]) << 2) | (spread3(q[1]) << 1) | spread3(q[2]);
  keys[f] = (uint64_t(code) << 32) | uint64_t(uint32_t(f));
  ids[f] = int32_t(f);
}

// key = Morton code of vertex v (30 bits, the faces' quantisation) << 32 | v.
__global__ void lbvh_vertex_keys(const float *xyz, uint64_t nv, float3 lo, float3 inv,
                                 uint64_t *keys, int32_t *ids) {
  uint64_t v = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  float l[3] = {lo.x, lo.y, lo.z}, s[3] = {inv.x, inv.y, inv.z};
  uint32_t q[3];
  for (int a = 0; a < 3; ++a) {
    float u = (xyz[uint64_t(a) * nv + v] - l[a]) * s[a];
    q[a] = uint32_t(fminf(fmaxf(u * 1024.f, 0.f), 1023.f));
  }
  uint32_t code = (spread3(q[0]) << 2) | (spread3(q[1]) << 1) | spread3(q[2]);
  keys[v] = (uint64_t(code) << 32) | uint64_t(uint32_t(v));
  ids[v] = int32_t(v);
}

__device__ __forceinline__ int lcp(const uint64_t *keys, int64_t n, int64_t i, int64_t j) {
  if (j < 0 || j >= n) return -1;
  return __clzll(keys[i] ^ keys[j]);
}

// Internal node i of n - 1 (Karras 2012): its range, split and children;
// child < 0 encodes the leaf ~sorted position; parent_* = 2 * parent + slot.
__global__ void lbvh_internal(const uint64_t *keys, int64_t n, int32_t *child, int32_t *parent_in,
                              int32_t *parent_leaf) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const int d = lcp(keys, n, i, i + 1) > lcp(keys, n, i, i - 1) ? 1 : -1;
  const int dmin = lcp(keys, n, i, i - d);
  int64_t lmax = 2;
  while (lcp(keys, n, i, i + lmax * d) > dmin) lmax *= 2;
  int64_t l = 0;
  for (int64_t t = lmax / 2; t >= 1; t /= 2)
    if (lcp(keys, n, i, i + (l + t) * d) > dmin) l += t;
  const int64_t j = i + l * d;
  const int dnode = lcp(keys, n, i, j);
  int64_t s = 0, t = l;
  do {
    t = (t + 1) / 2;
    if (lcp(keys, n, i, i + (s + t) * d) > dnode) s += t;
  } while (t > 1);
  const int64_t gamma = i + s * d + (d < 0 ? d : 0);
  const int64_t lo = i < j ? i : j, hi = i < j ? j : i;
  int32_t left = lo == gamma ? ~int32_t(gamma) : int32_t(gamma);
  int32_t right = hi == gamma + 1 ? ~int32_t(gamma + 1) : int32_t(gamma + 1);
  child[2 * i] = left, child[2 * i + 1] = right;
  if (left < 0) parent_leaf[gamma] = int32_t(2 * i);
  else parent_in[gamma] = int32_t(2 * i);
  if (right < 0) parent_leaf[gamma + 1] = int32_t(2 * i + 1);
  else parent_in[gamma + 1] = int32_t(2 * i + 1);
}

// Boxes bottom-up: every leaf writes its box into its parent's slot; the
// second child to arrive at a node merges both slots into the node's box
// and carries it one level up.  Leaves are renamed from sorted positions to
// face ids on the way.
__global__ void lbvh_boxes(const float *xyz, uint64_t nv, const int32_t *faces, int64_t n,
                           const int32_t *sorted_ids, int32_t *child, const int32_t *parent_in,
                           const int32_t *parent_leaf, float *box, unsigned *arrivals) {
  int64_t leaf = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (leaf >= n) return;
  const int32_t f = sorted_ids[leaf];
  float b[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
  for (int k = 0; k < 3; ++k) {
    int32_t v = faces[uint64_t(k) * uint64_t(n) + f];
    for (int a = 0; a < 3; ++a) {
      float x = xyz[uint64_t(a) * nv + v];
      b[a] = fminf(b[a], x), b[3 + a] = fmaxf(b[3 + a], x);
    }
  }
  int32_t node = parent_leaf[leaf] >> 1;
  int slot = parent_leaf[leaf] & 1;
  child[2 * node + slot] = ~f;  // leaves now name faces
  for (int guard = 0; guard < 128; ++guard) {
    volatile float *dst = box + int64_t(node) * 12 + slot * 6;
    for (int k = 0; k < 6; ++k) dst[k] = b[k];
    __threadfence();
    if (atomicAdd(&arrivals[node], 1u) == 0) return;  // the sibling finishes the node
    __threadfence();
    volatile const float *src = box + int64_t(node) * 12;
    for (int a = 0; a < 3; ++a) {
      b[a] = fminf(src[a], src[6 + a]);
      b[3 + a] = fmaxf(src[3 + a], src[9 + a]);
    }
    if (node == 0) return;
    slot = parent_in[node] & 1;
    node = parent_in[node] >> 1;
  }
}

// ------------------------------------------------------------ verification
constexpr int kStackFast = 96;

__device__ __forceinline__ float box_d2f(F3 p, const float *b) {
  float dx = fmaxf(fmaxf(b[0] - p.x, p.x - b[3]), 0.f);
  float dy = fmaxf(fmaxf(b[1] - p.y, p.y - b[4]), 0.f);
  float dz = fmaxf(fmaxf(b[2] - p.z, p.z - b[5]), 0.f);
  return dx * dx + dy * dy + dz * dz;
}

struct BvhView {
  uint64_t nv, nf;
  const int32_t *faces;
  const float *xyz;
  const int32_t *child;
  const float *box;
  const float4 *fn;  // nf: unit face normal from the FP64 corners, w = 1 (0: none usable)
  const int32_t *order;  // nv: query order of the vertices (Morton order of their position)
  const double *fn64;    // nf x 3: the faces' FP64 unit normals of the normal test
};

__device__ __forceinline__ F3 vtx(const BvhView &b, int32_t v) {
  return {b.xyz[v], b.xyz[b.nv + v], b.xyz[2 * b.nv + v]};
}
__device__ __forceinline__ float face_d2(const BvhView &b, F3 p, int32_t f) {
  return triangle_d2f(p, vtx(b, b.faces[f]), vtx(b, b.faces[b.nf + f]), vtx(b, b.faces[2 * b.nf + f]));
}

// Nearest face within `best` (FP32), near-first; -1 when none.
__device__ int32_t nearest_face_fast(const BvhView &b, F3 p, float &best, int *status) {
  int32_t face = -1;
  if (b.nf == 1) {
    float d = face_d2(b, p, 0);
    if (d < best) best = d, face = 0;
    return face;
  }
  int32_t stack[kStackFast];
  float dist[kStackFast];
  int top = 0;
  stack[top] = 0, dist[top++] = 0.f;
  while (top) {
    --top;
    if (dist[top] >= best) continue;
    const int32_t node = stack[top];
    const float *bx = b.box + int64_t(node) * 12;
    const int32_t c0 = b.child[2 * node], c1 = b.child[2 * node + 1];
    float d0 = box_d2f(p, bx), d1 = box_d2f(p, bx + 6);
    if (c0 < 0 && d0 < best) {
      float d = face_d2(b, p, ~c0);
      if (d < best) best = d, face = ~c0;
    }
    if (c1 < 0 && d1 < best) {
      float d = face_d2(b, p, ~c1);
      if (d < best) best = d, face = ~c1;
    }
    const bool p0 = c0 >= 0 && d0 < best, p1 = c1 >= 0 && d1 < best;
    if (top + 2 > kStackFast) {
      atomicExch(status, DS_CAPACITY);
      return face;
    }
    if (p0 && p1) {  // the nearer child is popped first
      bool first0 = d0 <= d1;
      stack[top] = first0 ? c1 : c0, dist[top++] = first0 ? d1 : d0;
      stack[top] = first0 ? c0 : c1, dist[top++] = first0 ? d0 : d1;
    } else if (p0) {
      stack[top] = c0, dist[top++] = d0;
    } else if (p1) {
      stack[top] = c1, dist[top++] = d1;
    }
  }
  return face;
}

// The verification tests of one (mode, vertex, direction) query with the
// FP32 search (the refinement's correspondences): returns the nearest face
// when vertex i supports mode m in that direction (-1 otherwise), its FP32
// squared distance in `best` (entering as tau^2) and the image of the vertex
// in q.  The motion is applied in FP64.
__device__ __forceinline__ int32_t support_query(const BvhView &b, const double *xyz,
                                                 const double *vn, const ClusterMotion &m,
                                                 uint64_t i, bool inverse, double tau, float &best,
                                                 double q[3], int *status) {
  const uint64_t nv = b.nv;
  double r[9];
  for (int k = 0; k < 9; ++k) r[k] = inverse ? m.r[(k % 3) * 3 + k / 3] : m.r[k];
  const double p[3] = {xyz[i], xyz[nv + i], xyz[2 * nv + i]};
  double move2 = 0;
  for (int a = 0; a < 3; ++a) {
    double s = 0;
    for (int k = 0; k < 3; ++k) s += r[a * 3 + k] * (inverse ? p[k] - m.t[k] : p[k]);
    q[a] = inverse ? s : s + m.t[a];
    move2 += (q[a] - p[a]) * (q[a] - p[a]);
  }
  if (move2 < 4 * tau * tau) return -1;
  if (m.reflection) {
    double side = m.n[0] * p[0] + m.n[1] * p[1] + m.n[2] * p[2] + m.offset;
    if (inverse ? side <= tau : side >= -tau) return -1;
  }
  const F3 qf{float(q[0]), float(q[1]), float(q[2])};
  const int32_t face = nearest_face_fast(b, qf, best, status);
  if (face < 0) return -1;
  const F3 a = vtx(b, b.faces[face]), bb = vtx(b, b.faces[b.nf + face]),
           cc = vtx(b, b.faces[2 * b.nf + face]);
  F3 fn = crossf(bb - a, cc - a);
  float len = sqrtf(dotf(fn, fn));
  if (!(len > 0.f)) return -1;
  const double ni[3] = {vn[i], vn[nv + i], vn[2 * nv + i]};
  float rn[3];
  for (int k = 0; k < 3; ++k)
    rn[k] = float(r[k * 3] * ni[0] + r[k * 3 + 1] * ni[1] + r[k * 3 + 2] * ni[2]);
  if ((rn[0] * fn.x + rn[1] * fn.y + rn[2] * fn.z) / len < 0.5f) return -1;
  return face;
}

// ------------------------------------------- exact decisions, FP32 search
// Error bound of the FP32 search, in distance units: kErr (512 FP32 units u)
// times M, the largest coordinate magnitude of the vertex, its image, the
// translation and the mesh.  The FP32 corners and image are within a few
// u M of their FP64 values, and the distance is 1-Lipschitz in each; the
// face's unit normal comes from the FP64 corners (rounded once to FP32), so
// the plane distance n . (p - a) and the three edge functions
// (n x e) . (p - v) carry errors of a few u (M + |p - v|) whatever the
// face's shape, and the segment distances of a few u M as well -- far below
// kErr M.  A face decided by face_d2n therefore has its FP32 distance within
// kErr M of the reference's FP64 distance; a face without a usable normal
// (its FP64 normal not accurate to well below u: no area, or a corner angle
// with sin below 1e-6), or whose projection falls within the rounding band
// of an edge line, enters the candidates by a lower bound and leaves the
// decision to FP64.  The same bound serves as the band of the FP32 threshold
// tests (2 tau, the plane side, tau), and kNormalBand (on the cosine) as
// that of the normal test, whose FP32 error is a few u.
constexpr float kErr = 1.0f / 32768.0f;
constexpr float kNormalBand = 1.0f / 1024.0f;
constexpr int kCandidates = 16;

// FP32 squared distance from p to the face (a, b, c) with unit normal n;
// um = u M, the FP32 unit at the query's magnitude.  The plane distance
// when p projects inside all three edges by more than their rounding band
// (p then projects into the face), the nearest of the three edge segments
// when it projects outside one of them by more than its band (the nearest
// point then lies on the boundary).  Otherwise `d2` receives min(plane,
// segments), a lower bound of the distance, and the function returns
// false.  Band of an edge function E = (n x e) . (p - v): with |dn| <= u,
// corners within 1.8 u M and the image within 30 u M of their FP64 values,
// and the cross and dot products' rounding, |dE| <= u (11 |e| |p - v| +
// 3.6 M |p - v| + 32 M |e|) <= 42 u M (|p - v| + |e|) for |e| <= 3.5 M; the
// band is 64 u M (|p - v| + |e|).
__device__ bool face_d2n(F3 p, F3 a, F3 b, F3 c, F3 n, float um, float &d2) {
  const F3 ab = b - a, bc = c - b, ca = a - c, ap = p - a, bp = p - b, cp = p - c;
  const float k = 64.f * um;
  const float ba = k * (sqrtf(dotf(ap, ap)) + sqrtf(dotf(ab, ab)));
  const float bb = k * (sqrtf(dotf(bp, bp)) + sqrtf(dotf(bc, bc)));
  const float bcb = k * (sqrtf(dotf(cp, cp)) + sqrtf(dotf(ca, ca)));
  const float ea = dotf(crossf(n, ab), ap), eb = dotf(crossf(n, bc), bp), ec = dotf(crossf(n, ca), cp);
  const float seg = fminf(segment_d2f(p, a, b), fminf(segment_d2f(p, b, c), segment_d2f(p, c, a)));
  if (ea < -ba || eb < -bb || ec < -bcb) {
    d2 = seg;
    return true;
  }
  const float h = dotf(n, ap);
  if (ea > ba && eb > bb && ec > bcb) {
    d2 = h * h;
    return true;
  }
  d2 = fminf(h * h, seg);
  return false;
}

// Faces whose FP64 distance to the image can be the smallest: every face
// whose FP32 distance (or, for a face face_d2n leaves undecided or one
// without a usable normal, a lower bound: the face_d2n bound or the box
// distance) is within 2 error bounds of min(best FP32 distance, tau +
// bound) -- the face of smallest FP64 distance is at most 2 bounds farther
// in FP32 than the best FP32 face.  Nodes are pruned with a slightly larger
// radius, for the rounding of their boxes' distances.  Undecided faces are
// listed as ~face.  Returns the count (N + 1 on overflow: faces and keys
// hold N entries); `best` receives the smallest FP32 squared distance of a
// decided face (INFINITY when none lies within tau + 3 bounds).
template <int N = kCandidates>
__device__ int candidate_faces(const BvhView &b, F3 p, float tau_err, float err, int32_t *faces,
                               float *keys, float &best, int *status) {
  best = INFINITY;
  float radius = tau_err + 2.f * err;
  float lim = radius * radius, lim_box = (radius + err * 0.03125f) * (radius + err * 0.03125f);
  int n = 0;
  bool overflow = false;
  const float um = err * (1.f / 512.f);  // err = kErr M = 512 u M
  auto consider = [&](int32_t f, float box) {
    const float4 fn = b.fn[f];
    float key = box;
    int32_t id = ~f;
    if (fn.w != 0.f) {
      const F3 a = vtx(b, b.faces[f]), bb = vtx(b, b.faces[b.nf + f]), cc = vtx(b, b.faces[2 * b.nf + f]);
      if (face_d2n(p, a, bb, cc, F3{fn.x, fn.y, fn.z}, um, key)) id = f;
    }
    if (id >= 0) {
      if (key < best) {
        best = key;
        radius = fminf(tau_err, sqrtf(best)) + 2.f * err;
        lim = radius * radius;
        lim_box = (radius + err * 0.03125f) * (radius + err * 0.03125f);
      }
    }
    if (key > lim) return;
    if (n == N) {  // drop entries beyond the current limit
      int m = 0;
      for (int j = 0; j < n; ++j)
        if (keys[j] <= lim) faces[m] = faces[j], keys[m++] = keys[j];
      n = m;
    }
    if (n == N) {
      overflow = true;
      return;
    }
    faces[n] = id, keys[n++] = key;
  };
  if (b.nf == 1) {
    consider(0, 0.f);
  } else {
    int32_t stack[kStackFast];
    float dist[kStackFast];
    int top = 0;
    stack[top] = 0, dist[top++] = 0.f;
    while (top) {
      --top;
      if (dist[top] > lim_box) continue;
      const int32_t node = stack[top];
      const float *bx = b.box + int64_t(node) * 12;
      const int32_t c0 = b.child[2 * node], c1 = b.child[2 * node + 1];
      const float d0 = box_d2f(p, bx), d1 = box_d2f(p, bx + 6);
      if (c0 < 0 && d0 <= lim_box) consider(~c0, d0);
      if (c1 < 0 && d1 <= lim_box) consider(~c1, d1);
      const bool p0 = c0 >= 0 && d0 <= lim_box, p1 = c1 >= 0 && d1 <= lim_box;
      if (top + 2 > kStackFast) {
        atomicExch(status, DS_CAPACITY);
        return N + 1;
      }
      if (p0 && p1) {  // the nearer child is popped first
        const bool first0 = d0 <= d1;
        stack[top] = first0 ? c1 : c0, dist[top++] = first0 ? d1 : d0;
        stack[top] = first0 ? c0 : c1, dist[top++] = first0 ? d0 : d1;
      } else if (p0) {
        stack[top] = c0, dist[top++] = d0;
      } else if (p1) {
        stack[top] = c1, dist[top++] = d1;
      }
    }
  }
  if (overflow) return N + 1;
  int m = 0;
  for (int j = 0; j < n; ++j)
    if (keys[j] <= lim) faces[m] = faces[j], keys[m++] = keys[j];
  return m;
}

// A cluster's motion in FP32 (the FP32 decisions).
struct MotionF {
  float r[9], t[3], n[3], offset;
  int32_t reflection;
};

// Row lists between the verification kernels.
// A row (c, direction, vertex i) holds the flag and error of one query;
// the kernels take the queries qid = (c, direction, j) of vertex order[j],
// the vertices in Morton order of their position, so a warp serves
// neighbouring vertices of one motion and walks nearly the same BVH nodes
// (in the mesh's own vertex order the warps of the benchmark mesh spread
// over 3x more of it).  The FP64 and reference-order queries are marked
// per query and compacted in ascending order (compact_indices), so their
// warps keep that locality; appended in completion order they made every
// load of a warp 32 scattered ones.
constexpr uint32_t kNoSlot = 0xffffffffu;
constexpr uint32_t kWideSlot = 0xfffffffeu;  // overflowed the list: for verify_rows_wide
constexpr int32_t kNoFace = INT32_MIN;  // padding of a candidate list (~f marks an undecided face)

struct RowLists {
  uint32_t *forward;    // accepted forward rows whose FP64 distance is still needed
  int32_t *faces;       // kCandidates faces per forward row (-1 padded)
  uint8_t *mark;        // per query: 1 = left to the next kernel (FP64, then reference order)
  int32_t *fp64;        // queries decided in FP64, ascending
  int32_t *reference;   // queries left to the wide list, then to the reference-order BVH
  // the FP32 candidates of an FP64 query (kCandidates per slot, kNoFace
  // padded), so the FP64 decisions need no search of their own; slot_of[qid]
  // = kNoSlot for a query sent on before its candidates were known,
  // kWideSlot for one whose candidates overflowed the list
  uint32_t *slot_of;
  int32_t *cand;
  unsigned long long slots;    // capacity of cand, in slots
  unsigned long long *counts;  // [forward, slots used, unused, tie]
};

// Decisions in FP32 (verify_fp32).  The reference's tests are made with
// the FP32 image of the vertex; each threshold test that falls within its
// band of the threshold, a badly shaped face among the candidates,
// candidates that disagree on the normal test, or a candidate overflow send
// the row to the FP64 decisions.  An accepted forward row is listed with its
// candidates, the faces its FP64 distance is the smallest of.
__global__ void verify_fp32(BvhView b, const float *vn32, const MotionF *motions, uint64_t nc,
                            float tau, float scale, uint8_t *flags, double *err, RowLists lists,
                            int *status) {
  // query q = (c, direction, j) takes vertex i = order[j]: the warps walk
  // neighbouring vertices; flags and errors stay per vertex (row)
  const uint64_t qid = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const uint64_t nv = b.nv;
  if (qid >= nc * 2 * nv) return;
  const uint64_t c = qid / (2 * nv), rem = qid % (2 * nv);
  const bool inverse = rem >= nv;
  const uint64_t i = uint64_t(b.order[rem % nv]);
  const uint64_t row = qid - rem % nv + i;
  flags[row] = 0;
  lists.mark[qid] = 0;
  if (!inverse) err[c * nv + i] = 0.0;
  const MotionF &m = motions[c];
  float r[9];
  for (int k = 0; k < 9; ++k) r[k] = inverse ? m.r[(k % 3) * 3 + k / 3] : m.r[k];
  const F3 p = vtx(b, int32_t(i));
  const F3 u = inverse ? F3{p.x - m.t[0], p.y - m.t[1], p.z - m.t[2]} : p;
  F3 q{r[0] * u.x + r[1] * u.y + r[2] * u.z, r[3] * u.x + r[4] * u.y + r[5] * u.z,
       r[6] * u.x + r[7] * u.y + r[8] * u.z};
  if (!inverse) q = q + F3{m.t[0], m.t[1], m.t[2]};
  const float mag = fmaxf(scale, fmaxf(fabsf(q.x), fmaxf(fabsf(q.y), fabsf(q.z))));
  const float e = kErr * fmaxf(mag, fmaxf(fabsf(m.t[0]), fmaxf(fabsf(m.t[1]), fabsf(m.t[2]))));
  auto to_fp64 = [&]() {
    lists.mark[qid] = 1;
    lists.slot_of[qid] = kNoSlot;
  };
  // the image moves at least 2 tau (verification.cpp:64)
  const F3 dq = q - p;
  const float moved = sqrtf(dotf(dq, dq));
  if (fabsf(moved - 2.f * tau) <= 2.f * e) return to_fp64();
  if (moved < 2.f * tau) return;
  if (m.reflection) {  // the vertex lies on the plane's side (verification.cpp:66, :84)
    const float side = m.n[0] * p.x + m.n[1] * p.y + m.n[2] * p.z + m.offset;
    const float at = inverse ? tau : -tau;
    if (fabsf(side - at) <= e) return to_fp64();
    if (inverse ? side <= tau : side >= -tau) return;
  }
  int32_t faces[kCandidates];
  float keys[kCandidates];
  float best;
  const int n = candidate_faces(b, q, tau + e, e, faces, keys, best, status);
  if (n > kCandidates) {  // the same search would overflow again: straight to the wide list
    lists.mark[qid] = 1;
    lists.slot_of[qid] = kWideSlot;
    return;
  }
  // from here on an FP64 row keeps its candidates: they hold every face at
  // the FP64 minimum (the window covers the FP32 error of the FP64 image)
  auto to_fp64_listed = [&]() {
    lists.mark[qid] = 1;
    const unsigned long long k = atomicAdd(&lists.counts[1], 1ull);
    if (k >= lists.slots) {
      lists.slot_of[qid] = kNoSlot;
      return;
    }
    lists.slot_of[qid] = uint32_t(k);
    for (int j = 0; j < kCandidates; ++j) lists.cand[k * kCandidates + j] = j < n ? faces[j] : kNoFace;
  };
  for (int j = 0; j < n; ++j)
    if (faces[j] < 0) return to_fp64_listed();  // an undecided face
  if (!n) return;                        // no face within tau (all farther than tau + 3e)
  const float dbest = sqrtf(best);
  if (dbest - e > tau) return;           // every face farther than tau
  if (dbest + e >= tau) return to_fp64_listed();
  // the normal test of every candidate (verification.cpp:70-73)
  const F3 ni{vn32[i], vn32[nv + i], vn32[2 * nv + i]};
  const F3 rn{r[0] * ni.x + r[1] * ni.y + r[2] * ni.z, r[3] * ni.x + r[4] * ni.y + r[5] * ni.z,
              r[6] * ni.x + r[7] * ni.y + r[8] * ni.z};
  int agree = 0, disagree = 0;
  for (int j = 0; j < n; ++j) {
    // the face's unit normal from its FP64 corners (every candidate here
    // has one): the cosine is good to a few u
    const float4 fn = b.fn[faces[j]];
    const float v = dotf(rn, F3{fn.x, fn.y, fn.z});
    if (fabsf(v - 0.5f) <= kNormalBand) return to_fp64_listed();
    if (v >= 0.5f) ++agree;
    else ++disagree;
  }
  if (agree && disagree) return to_fp64_listed();
  if (!agree) return;
  flags[row] = 1;
  if (!inverse) {
    const unsigned long long k = atomicAdd(&lists.counts[0], 1ull);
    lists.forward[k] = uint32_t(row);
    for (int j = 0; j < kCandidates; ++j) lists.faces[k * kCandidates + j] = j < n ? faces[j] : -1;
  }
}

// The reference's FP64 squared distance of each listed forward row: the
// smallest over its candidate faces (the face it keeps is among them).
__global__ void forward_errors(Surface s, const ClusterMotion *motions, RowLists lists,
                               unsigned long long count, double *err) {
  const uint64_t k = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const uint64_t row = lists.forward[k], nv = s.nv;
  const uint64_t c = row / (2 * nv), i = row % (2 * nv);
  const ClusterMotion &m = motions[c];
  const M3 r = query_rotation(m, false);
  const D3 q = mul(r, vertex(s, int32_t(i))) + D3{m.t[0], m.t[1], m.t[2]};
  double dmin = INFINITY;
  for (int j = 0; j < kCandidates; ++j) {
    const int32_t f = lists.faces[k * kCandidates + j];
    if (f < 0) break;
    dmin = fmin(dmin, triangle_d2(q, corner(s, f, 0), corner(s, f, 1), corner(s, f, 2)));
  }
  err[c * nv + i] = dmin;
}

// The reference's normal test (verification.cpp:70-73, normal_agrees) with
// the face's unit normal from the per-mesh table: the same FP64 values.
__device__ __forceinline__ bool normal_agrees_t(const BvhView &b, int32_t f, const M3 &r, D3 ni) {
  const D3 fnorm{b.fn64[3 * uint64_t(f)], b.fn64[3 * uint64_t(f) + 1], b.fn64[3 * uint64_t(f) + 2]};
  return !(dot(mul(r, ni), fnorm) < 0.5);
}

// One query of the reference's verification, decided with the FP32
// candidates and FP64 rechecks.  Returns 1 (supports; `d2` = the reference's
// FP64 squared distance), 0 (does not), 3 (the faces at the minimum, listed
// in `tied`, N entries, -1 padded, disagree on the normal test; `d2` = the
// minimum) or 2 (more than N candidates; `d2` = the tau^2 search limit).
//
// The reference keeps the face of strictly smallest FP64 distance, the first
// its BVH visits among faces at exactly that distance (surface.h:52-83).
// The candidates hold every face that can be at the minimum, so their FP64
// minimum is the reference's distance; the normal test of the faces at
// exactly that minimum decides when they all give the same outcome; when
// they do not, the reference's visiting order decides (verify_listed_ref).
template <int N = kCandidates>
__device__ int hybrid_query(const BvhView &b, const Surface &s, const double *vn,
                            const ClusterMotion &m, bool inverse, uint64_t i, double tau,
                            float scale, double &d2, int32_t *tied, int *status) {
  const M3 r = query_rotation(m, inverse);
  const D3 p = vertex(s, int32_t(i));
  D3 q;
  if (query_skipped(m, r, inverse, p, tau, q)) return 0;
  const F3 qf{float(q.x), float(q.y), float(q.z)};
  const float mag = fmaxf(scale, fmaxf(fabsf(qf.x), fmaxf(fabsf(qf.y), fabsf(qf.z))));
  const float e = kErr * mag;
  int32_t faces[N];
  float keys[N];
  float best;
  const int n = candidate_faces<N>(b, qf, float(tau) + e, e, faces, keys, best, status);
  if (n > N) {
    d2 = nextafter(tau * tau, double(INFINITY));
    return 2;
  }
  double dmin = INFINITY;
  double dist[N];
  for (int j = 0; j < n; ++j) {
    faces[j] = faces[j] < 0 ? ~faces[j] : faces[j];
    dist[j] = triangle_d2(q, corner(s, faces[j], 0), corner(s, faces[j], 1), corner(s, faces[j], 2));
    dmin = fmin(dmin, dist[j]);
  }
  if (!(dmin <= tau * tau)) return 0;
  const D3 ni{vn[i], vn[s.nv + i], vn[2 * s.nv + i]};
  int agree = 0, disagree = 0, t = 0;
  for (int j = 0; j < n; ++j) {
    if (dist[j] != dmin) continue;
    tied[t++] = faces[j];
    if (normal_agrees_t(b, faces[j], r, ni)) ++agree;
    else ++disagree;
  }
  d2 = dmin;
  if (agree && disagree) {
    for (int j = t; j < N; ++j) tied[j] = -1;
    return 3;
  }
  return agree ? 1 : 0;
}

// The FP64 decisions of the rows verify_fp32 listed.  Where the faces at
// the minimum disagree on the normal test, the first of them the reference's
// search reaches takes the test (first_in_reference_order); rows whose
// candidates overflow the list are listed for verify_listed_ref.
__global__ void verify_rows_fp64(BvhView b, Surface s, RefBvh t, const double *vn,
                                 const ClusterMotion *motions, double tau, float scale,
                                 uint8_t *flags, double *err, RowLists lists,
                                 unsigned long long count, int *status) {
  constexpr int kGroup = 8;  // lanes per row: candidates j = sub and sub + 8
  const uint64_t gid = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const uint64_t k = gid / kGroup;
  const int sub = threadIdx.x % kGroup;
  const unsigned group_mask = 0xffu << (threadIdx.x & 31 & ~(kGroup - 1));
  if (k >= count) return;  // whole groups (count rows x 8 lanes)
  const uint64_t qid = uint64_t(lists.fp64[k]), nv = b.nv;  // a query, as verify_fp32's
  const uint64_t c = qid / (2 * nv), rem = qid % (2 * nv);
  const bool inverse = rem >= nv;
  const uint64_t i = uint64_t(b.order[rem % nv]);
  const uint64_t row = qid - rem % nv + i;
  const uint32_t slot = lists.slot_of[qid];
  if (slot == kWideSlot) return;  // left marked for verify_rows_wide
  if (slot == kNoSlot) {  // no candidates yet: the search, on one lane
    if (sub) return;
    double d = 0;
    int32_t tied[kCandidates];
    int v = hybrid_query(b, s, vn, motions[c], inverse, i, tau, scale, d, tied, status);
    if (v == 3) {
      atomicAdd(&lists.counts[3], 1ull);
      const M3 r = query_rotation(motions[c], inverse);
      D3 q;
      query_skipped(motions[c], r, inverse, vertex(s, int32_t(i)), tau, q);
      int32_t first = tied[0];
      for (int x = 1; x < kCandidates && tied[x] >= 0; ++x)
        first = first_in_reference_order(t, q, first, tied[x]);
      v = normal_agrees_t(b, first, r, D3{vn[i], vn[nv + i], vn[2 * nv + i]}) ? 1 : 0;
    }
    flags[row] = v == 1;
    if (!inverse) err[c * nv + i] = v == 1 ? d : 0.0;
    if (v != 2) lists.mark[qid] = 0;  // marked queries go on to the reference-order search
    return;
  }
  const ClusterMotion &m = motions[c];
  const M3 r = query_rotation(m, inverse);
  D3 q;
  const bool skipped = query_skipped(m, r, inverse, vertex(s, int32_t(i)), tau, q);
  int v = 0;
  double dmin = INFINITY;
  if (!skipped) {
    // the reference's FP64 distance of each candidate, and the minimum
    const int32_t *cl = lists.cand + uint64_t(slot) * kCandidates;
    int32_t f[2];
    double d[2];
    for (int h = 0; h < 2; ++h) {
      const int32_t x = cl[sub + kGroup * h];
      f[h] = x == kNoFace ? -1 : (x < 0 ? ~x : x);
      d[h] = f[h] < 0 ? INFINITY
                      : triangle_d2(q, corner(s, f[h], 0), corner(s, f[h], 1), corner(s, f[h], 2));
      dmin = fmin(dmin, d[h]);
    }
    for (int o = kGroup / 2; o; o >>= 1) dmin = fmin(dmin, __shfl_xor_sync(group_mask, dmin, o));
    if (dmin <= tau * tau) {
      // the normal test of the faces at exactly the minimum
      const D3 ni{vn[i], vn[nv + i], vn[2 * nv + i]};
      int agree = 0, disagree = 0;
      bool ok[2] = {false, false};
      int32_t first = -1;  // this lane's face at the minimum the reference visits first
      for (int h = 0; h < 2; ++h)
        if (f[h] >= 0 && d[h] == dmin) {
          ok[h] = normal_agrees_t(b, f[h], r, ni);
          if (ok[h]) ++agree;
          else ++disagree;
          first = first < 0 ? f[h] : first_in_reference_order(t, q, first, f[h]);
        }
      for (int o = kGroup / 2; o; o >>= 1) {
        agree += __shfl_xor_sync(group_mask, agree, o);
        disagree += __shfl_xor_sync(group_mask, disagree, o);
      }
      if (agree && disagree) {
        // faces at the minimum disagree: the one the reference visits first
        // (its visiting order is a total order on the faces for this
        // query, so the group reduces it like a minimum)
        for (int o = kGroup / 2; o; o >>= 1) {
          const int32_t other = __shfl_xor_sync(group_mask, first, o);
          if (other >= 0) first = first < 0 ? other : first_in_reference_order(t, q, first, other);
        }
        const bool mine_agrees = (f[0] == first && first >= 0 && ok[0]) || (f[1] == first && first >= 0 && ok[1]);
        v = (__ballot_sync(group_mask, mine_agrees) & group_mask) ? 1 : 0;
        if (sub == 0) {  // one count per converged set of groups
          const unsigned active = __activemask();
          const unsigned leaders = active & 0x01010101u;
          if ((threadIdx.x & 31) == __ffs(leaders) - 1) atomicAdd(&lists.counts[3], __popc(leaders));
        }
      } else {
        v = agree ? 1 : 0;
      }
    }
  }
  if (sub == 0) {
    flags[row] = v == 1;
    if (!inverse) err[c * nv + i] = v == 1 ? dmin : 0.0;
    lists.mark[qid] = 0;
  }
}

// Queries whose candidates overflowed the list of verify_fp32 and of
// verify_rows_fp64: the same FP32 search and FP64 decision with room for
// kWideCandidates faces (one thread per query; such queries are rare, and
// the reference-order search they would otherwise take walks the
// reference's BVH one FP64 node at a time).  A query that overflows this
// list as well stays marked for verify_listed_ref.
constexpr int kWideCandidates = 64;
__global__ void verify_rows_wide(BvhView b, Surface s, RefBvh t, const double *vn,
                                 const ClusterMotion *motions, double tau, float scale,
                                 uint8_t *flags, double *err, RowLists lists,
                                 unsigned long long count, int *status) {
  const uint64_t k = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const uint64_t qid = uint64_t(lists.reference[k]), nv = b.nv;  // a query, as verify_fp32's
  const uint64_t c = qid / (2 * nv), rem = qid % (2 * nv);
  const bool inverse = rem >= nv;
  const uint64_t i = uint64_t(b.order[rem % nv]);
  const uint64_t row = qid - rem % nv + i;
  double d = 0;
  int32_t tied[kWideCandidates];
  int v = hybrid_query<kWideCandidates>(b, s, vn, motions[c], inverse, i, tau, scale, d, tied,
                                        status);
  if (v == 2) return;  // still marked
  if (v == 3) {
    atomicAdd(&lists.counts[3], 1ull);
    const M3 r = query_rotation(motions[c], inverse);
    D3 q;
    query_skipped(motions[c], r, inverse, vertex(s, int32_t(i)), tau, q);
    int32_t first = tied[0];
    for (int x = 1; x < kWideCandidates && tied[x] >= 0; ++x)
      first = first_in_reference_order(t, q, first, tied[x]);
    v = normal_agrees_t(b, first, r, D3{vn[i], vn[nv + i], vn[2 * nv + i]}) ? 1 : 0;
  }
  flags[row] = v == 1;
  if (!inverse) err[c * nv + i] = v == 1 ? d : 0.0;
  lists.mark[qid] = 0;
}

// Queries whose candidates overflowed the wide list too: the reference's
// search itself (exact_query) with the search limit nextafter(tau^2, inf).
__global__ void verify_listed_ref(Surface s, const double *vn, const int32_t *order,
                                  const ClusterMotion *motions, double tau, RowLists lists,
                                  unsigned long long count, uint8_t *flags, double *err,
                                  int *status) {
  const uint64_t k = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const uint64_t qid = lists.reference[k], nv = s.nv;  // a query, as verify_fp32's
  const uint64_t c = qid / (2 * nv), rem = qid % (2 * nv);
  const bool inverse = rem >= nv;
  const uint64_t i = uint64_t(order[rem % nv]);
  const uint64_t row = qid - rem % nv + i;
  double d = 0;
  const bool ok = exact_query(s, vn, motions[c], inverse, i, tau,
                              nextafter(tau * tau, double(INFINITY)), d, status);
  flags[row] = ok;
  if (!inverse) err[c * nv + i] = ok ? d : 0.0;
}

// Block c < nc: sum of the forward errors, supporting weight (both
// directions) and forward count of cluster c; block nc: the total weight.
// Fixed-order strided partials and a fixed tree: reproducible, and within
// a few units of rounding of the reference's serial sums.
__global__ void __launch_bounds__(256) tree_sums(const uint8_t *flags, const double *err,
                                                 const double *w, uint64_t nv, uint64_t nc,
                                                 double *error, double *area, uint64_t *count,
                                                 double *total) {
  __shared__ double se[256], sa[256];
  __shared__ unsigned long long sn[256];
  const uint64_t c = blockIdx.x;
  double e = 0, a = 0;
  unsigned long long n = 0;
  if (c == nc) {
    for (uint64_t i = threadIdx.x; i < nv; i += 256) a += w[i];
  } else {
    const uint8_t *fa = flags + c * 2 * nv, *fb = fa + nv;
    for (uint64_t i = threadIdx.x; i < nv; i += 256) {
      if (fa[i]) e += err[c * nv + i], a += w[i], ++n;
      if (fb[i]) a += w[i];
    }
  }
  se[threadIdx.x] = e, sa[threadIdx.x] = a, sn[threadIdx.x] = n;
  __syncthreads();
  for (int h = 128; h; h >>= 1) {
    if (int(threadIdx.x) < h) {
      se[threadIdx.x] += se[threadIdx.x + h];
      sa[threadIdx.x] += sa[threadIdx.x + h];
      sn[threadIdx.x] += sn[threadIdx.x + h];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if (c == nc) {
      *total = sa[0];
    } else {
      error[c] = se[0], area[c] = sa[0], count[c] = sn[0];
    }
  }
}

// ------------------------------------------------ FP64 transform refinement
// Closest point of triangle abc to p in FP64: the region tests of Ericson,
// Real-Time Collision Detection, 2005, section 5.1.5, and for a triangle
// without area (|ab x ac|^2 < 1e-28) the nearest of its three segments, the
// rule of the verification's distance (the reference's
// point_triangle_distance2).
__device__ void closest_on_segment(const double p[3], const double a[3], const double b[3],
                                   double out[3]) {
  double d[3], l = 0, t = 0;
  for (int k = 0; k < 3; ++k) d[k] = b[k] - a[k], l += d[k] * d[k];
  if (l > 1e-14) {
    t = ((p[0] - a[0]) * d[0] + (p[1] - a[1]) * d[1] + (p[2] - a[2]) * d[2]) / l;
    t = t < 0.0 ? 0.0 : (1.0 < t ? 1.0 : t);
  }
  for (int k = 0; k < 3; ++k) out[k] = a[k] + d[k] * t;
}

__device__ void closest_point(const double p[3], const double a[3], const double b[3],
                              const double c[3], double out[3]) {
  double ab[3], ac[3], ap[3], bp[3], cp[3];
  for (int k = 0; k < 3; ++k)
    ab[k] = b[k] - a[k], ac[k] = c[k] - a[k], ap[k] = p[k] - a[k], bp[k] = p[k] - b[k],
    cp[k] = p[k] - c[k];
  auto dot3 = [](const double *x, const double *y) { return x[0] * y[0] + x[1] * y[1] + x[2] * y[2]; };
  const double n[3] = {ab[1] * ac[2] - ab[2] * ac[1], ab[2] * ac[0] - ab[0] * ac[2],
                       ab[0] * ac[1] - ab[1] * ac[0]};
  if (dot3(n, n) < 1e-14 * 1e-14) {  // no area: the nearest of the three segments
    double s[3][3], e[3];
    closest_on_segment(p, a, b, s[0]);
    closest_on_segment(p, a, c, s[1]);
    closest_on_segment(p, b, c, s[2]);
    for (int j = 0; j < 3; ++j) {
      const double r[3] = {p[0] - s[j][0], p[1] - s[j][1], p[2] - s[j][2]};
      e[j] = dot3(r, r);
    }
    const int m01 = e[1] < e[0] ? 1 : 0;
    const int pick = e[2] < e[m01] ? 2 : m01;
    for (int k = 0; k < 3; ++k) out[k] = s[pick][k];
    return;
  }
  auto set = [&](const double *base, const double *dir, double t) {
    for (int k = 0; k < 3; ++k) out[k] = base[k] + dir[k] * t;
  };
  const double d1 = dot3(ab, ap), d2 = dot3(ac, ap);
  if (d1 <= 0 && d2 <= 0) return set(a, ab, 0);
  const double d3 = dot3(ab, bp), d4 = dot3(ac, bp);
  if (d3 >= 0 && d4 <= d3) return set(b, ab, 0);
  const double vc = d1 * d4 - d3 * d2;
  if (vc <= 0 && d1 >= 0 && d3 <= 0) return set(a, ab, d1 / (d1 - d3));
  const double d5 = dot3(ab, cp), d6 = dot3(ac, cp);
  if (d6 >= 0 && d5 <= d6) return set(c, ab, 0);
  const double vb = d5 * d2 - d1 * d6;
  if (vb <= 0 && d2 >= 0 && d6 <= 0) return set(a, ac, d2 / (d2 - d6));
  const double va = d3 * d6 - d5 * d4;
  if (va <= 0 && (d4 - d3) >= 0 && (d5 - d6) >= 0) {
    const double bc[3] = {c[0] - b[0], c[1] - b[1], c[2] - b[2]};
    return set(b, bc, (d4 - d3) / ((d4 - d3) + (d5 - d6)));
  }
  const double den = va + vb + vc;
  for (int k = 0; k < 3; ++k) out[k] = a[k] + ab[k] * (vb / den) + ac[k] * (vc / den);
}

struct Origin {
  double x[3];
};

// Forward correspondences: for each vertex i that supports mode c forward
// (the verification's tests), the FP64 closest point of its nearest face to
// the vertex's image, relative to `o`; ok[c * nv + i] says which.
__global__ void refine_pairs(BvhView b, const double *xyz, const double *vn,
                             const ClusterMotion *motions, uint64_t nc, double tau, float tau2, Origin o,
                             double *target, uint8_t *ok, int *status) {
  // query (c, j) takes vertex i = order[j] (neighbouring vertices in a
  // warp); the pairs stay per vertex (row), so the sums keep their order
  const uint64_t qid = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const uint64_t nv = b.nv;
  if (qid >= nc * nv) return;
  const uint64_t c = qid / nv, i = uint64_t(b.order[qid % nv]), row = c * nv + i;
  ok[row] = 0;
  float best = tau2;
  double q[3];
  const int32_t face = support_query(b, xyz, vn, motions[c], i, false, tau, best, q, status);
  if (face < 0) return;
  double corner[3][3], out[3];
  for (int k = 0; k < 3; ++k) {
    const int32_t v = b.faces[uint64_t(k) * b.nf + face];
    for (int a = 0; a < 3; ++a) corner[k][a] = xyz[uint64_t(a) * nv + v];
  }
  closest_point(q, corner[0], corner[1], corner[2], out);
  for (int a = 0; a < 3; ++a) target[row * 3 + a] = out[a] - o.x[a];
  ok[row] = 1;
}

constexpr int kRefineSums = 28, kRefineThreads = 128;

// Block c: the weighted sums of mode c's correspondences (p the vertex, q its
// target, both relative to o; weights = vertex weights): W, W p, W q,
// W p q^T (row-major), W p p^T and W q q^T (upper triangles).  Fixed-order
// strided partials and a fixed tree.
__global__ void __launch_bounds__(kRefineThreads) refine_sums(const double *xyz, const double *w,
                                                              uint64_t nv, const uint8_t *ok,
                                                              const double *target, Origin o,
                                                              double *sums) {
  __shared__ double part[kRefineSums][kRefineThreads];
  const uint64_t c = blockIdx.x;
  double acc[kRefineSums];
  for (int k = 0; k < kRefineSums; ++k) acc[k] = 0;
  for (uint64_t i = threadIdx.x; i < nv; i += kRefineThreads) {
    if (!ok[c * nv + i]) continue;
    const double wi = w[i];
    double p[3], q[3];
    for (int a = 0; a < 3; ++a) p[a] = xyz[a * nv + i] - o.x[a], q[a] = target[(c * nv + i) * 3 + a];
    acc[0] += wi;
    for (int a = 0; a < 3; ++a) acc[1 + a] += wi * p[a], acc[4 + a] += wi * q[a];
    for (int a = 0; a < 3; ++a)
      for (int e = 0; e < 3; ++e) acc[7 + a * 3 + e] += wi * p[a] * q[e];
    for (int a = 0, at = 0; a < 3; ++a)
      for (int e = a; e < 3; ++e, ++at) acc[16 + at] += wi * p[a] * p[e], acc[22 + at] += wi * q[a] * q[e];
  }
  for (int k = 0; k < kRefineSums; ++k) part[k][threadIdx.x] = acc[k];
  __syncthreads();
  for (int s = kRefineThreads / 2; s; s >>= 1) {
    if (int(threadIdx.x) < s)
      for (int k = 0; k < kRefineSums; ++k) part[k][threadIdx.x] += part[k][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x < kRefineSums) sums[c * kRefineSums + threadIdx.x] = part[threadIdx.x][0];
}

// Eigen-decomposition of a symmetric 3x3 matrix (row-major) by cyclic
// Jacobi rotations: eigenvalues in `val`, eigenvectors in the columns of
// `vec`, sorted by decreasing eigenvalue.
__device__ void jacobi3(const double m[9], double val[3], double vec[9]) {
  double a[9];
  for (int k = 0; k < 9; ++k) a[k] = m[k], vec[k] = (k % 4 == 0) ? 1 : 0;
  for (int sweep = 0; sweep < 32; ++sweep) {
    const double off = a[1] * a[1] + a[2] * a[2] + a[5] * a[5];
    const double diag = a[0] * a[0] + a[4] * a[4] + a[8] * a[8];
    if (!(off > 1e-40 * diag)) break;
    for (int pi = 0; pi < 2; ++pi)
      for (int qi = pi + 1; qi < 3; ++qi) {
        const double apq = a[pi * 3 + qi];
        if (apq == 0) continue;
        // the rotation that zeroes a[p][q]: tan of its angle is the smaller
        // root of t^2 + 2 theta t - 1 = 0, theta = (a_qq - a_pp) / (2 a_pq)
        const double theta = (a[qi * 4] - a[pi * 4]) / (2 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1));
        const double cs = 1 / sqrt(t * t + 1), sn = t * cs;
        for (int k = 0; k < 3; ++k) {  // columns p, q of a
          const double akp = a[k * 3 + pi], akq = a[k * 3 + qi];
          a[k * 3 + pi] = cs * akp - sn * akq, a[k * 3 + qi] = sn * akp + cs * akq;
        }
        for (int k = 0; k < 3; ++k) {  // rows p, q
          const double apk = a[pi * 3 + k], aqk = a[qi * 3 + k];
          a[pi * 3 + k] = cs * apk - sn * aqk, a[qi * 3 + k] = sn * apk + cs * aqk;
        }
        for (int k = 0; k < 3; ++k) {
          const double vkp = vec[k * 3 + pi], vkq = vec[k * 3 + qi];
          vec[k * 3 + pi] = cs * vkp - sn * vkq, vec[k * 3 + qi] = sn * vkp + cs * vkq;
        }
      }
  }
  for (int k = 0; k < 3; ++k) val[k] = a[k * 4];
  for (int i = 0; i < 2; ++i)  // sort the columns, largest first
    for (int j = 0; j < 2 - i; ++j)
      if (val[j] < val[j + 1]) {
        double tv = val[j];
        val[j] = val[j + 1], val[j + 1] = tv;
        for (int k = 0; k < 3; ++k) {
          double tc = vec[k * 3 + j];
          vec[k * 3 + j] = vec[k * 3 + j + 1], vec[k * 3 + j + 1] = tc;
        }
      }
}

// One thread per mode: the least-squares motion of its correspondences.
// Rigid: the rotation R maximising tr(R H), H = sum w (p - pbar)(q - qbar)^T,
// from H's singular vectors (Kabsch: H = U S V^T, R = V diag(1, 1, d) U^T
// with d making det R = +1), t = qbar - R pbar.  Reflection: the plane
// normal is the top eigenvector of sum w (q - p)(q - p)^T (the displacements
// run along it), oriented like the previous one, and the plane passes
// through the weighted mean of the midpoints (p + q) / 2.  A mode with too
// few or degenerate correspondences keeps its motion.
__global__ void refine_solve(const double *sums, uint64_t nc, Origin o, ClusterMotion *motions) {
  const uint64_t c = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const double *s = sums + c * kRefineSums;
  const double W = s[0];
  if (!(W > 0)) return;
  double pb[3], qb[3];
  for (int a = 0; a < 3; ++a) pb[a] = s[1 + a] / W, qb[a] = s[4 + a] / W;
  ClusterMotion &m = motions[c];
  if (!m.reflection) {
    double H[9], HtH[9], S2[3], V[9];
    for (int a = 0; a < 3; ++a)
      for (int e = 0; e < 3; ++e) H[a * 3 + e] = s[7 + a * 3 + e] / W - pb[a] * qb[e];
    for (int a = 0; a < 3; ++a)
      for (int e = 0; e < 3; ++e)
        HtH[a * 3 + e] = H[a] * H[e] + H[3 + a] * H[3 + e] + H[6 + a] * H[6 + e];
    jacobi3(HtH, S2, V);
    const double s0 = sqrt(fmax(S2[0], 0.0)), s1 = sqrt(fmax(S2[1], 0.0));
    if (!(s1 > 1e-9 * s0)) return;  // collinear correspondences: rotation undetermined
    double U[9];  // U_k = H V_k / s_k for k = 0, 1; U_2 = U_0 x U_1
    for (int k = 0; k < 2; ++k)
      for (int a = 0; a < 3; ++a)
        U[a * 3 + k] = (H[a * 3] * V[k] + H[a * 3 + 1] * V[3 + k] + H[a * 3 + 2] * V[6 + k]) /
                       (k ? s1 : s0);
    U[2] = U[3] * U[7] - U[6] * U[4];
    U[5] = U[6] * U[1] - U[0] * U[7];
    U[8] = U[0] * U[4] - U[3] * U[1];
    const double detv = V[0] * (V[4] * V[8] - V[5] * V[7]) - V[1] * (V[3] * V[8] - V[5] * V[6]) +
                        V[2] * (V[3] * V[7] - V[4] * V[6]);
    const double d[3] = {1, 1, detv < 0 ? -1.0 : 1.0};
    double R[9];
    for (int a = 0; a < 3; ++a)
      for (int e = 0; e < 3; ++e)
        R[a * 3 + e] = V[a * 3] * d[0] * U[e * 3] + V[a * 3 + 1] * d[1] * U[e * 3 + 1] +
                       V[a * 3 + 2] * d[2] * U[e * 3 + 2];
    for (int k = 0; k < 9; ++k) m.r[k] = R[k];
    for (int a = 0; a < 3; ++a) {
      double rp = 0;
      for (int e = 0; e < 3; ++e) rp += R[a * 3 + e] * (pb[e] + o.x[e]);
      m.t[a] = qb[a] + o.x[a] - rp;
    }
  } else {
    double C[9], val[3], V[9];
    const int up[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};  // upper-triangle slots
    for (int a = 0; a < 3; ++a)
      for (int e = 0; e < 3; ++e)
        C[a * 3 + e] = (s[22 + up[a][e]] - s[7 + a * 3 + e] - s[7 + e * 3 + a] + s[16 + up[a][e]]) / W;
    jacobi3(C, val, V);
    if (!(val[0] > 0)) return;
    double n[3] = {V[0], V[3], V[6]};
    const double len = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    if (!(len > 0)) return;
    const double sgn = (n[0] * m.n[0] + n[1] * m.n[1] + n[2] * m.n[2]) < 0 ? -1.0 : 1.0;
    for (int a = 0; a < 3; ++a) n[a] *= sgn / len;
    double off = 0;
    for (int a = 0; a < 3; ++a) off -= n[a] * (0.5 * (pb[a] + qb[a]) + o.x[a]);
    for (int a = 0; a < 3; ++a) {
      m.n[a] = n[a];
      m.t[a] = -2 * off * n[a];
      for (int e = 0; e < 3; ++e) m.r[a * 3 + e] = (a == e ? 1.0 : 0.0) - 2 * n[a] * n[e];
    }
    m.offset = off;
  }
}

// patches[set] += 1 for every component root of the set.
__global__ void count_roots(int32_t *parent_all, uint64_t nv, uint64_t sets, unsigned *patches) {
  uint64_t k = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= sets * nv) return;
  const uint64_t set = k / nv;
  int32_t *parent = parent_all + set * nv;
  const int32_t i = int32_t(k % nv);
  if (parent[i] >= 0 && find_root(parent, i) == i) atomicAdd(&patches[set], 1u);
}

}  // namespace

// Unit normal of every face, (b - a) x (c - a) normalised in FP64 as the
// reference's normal test forms it (src/cpu/verification.cpp:71-75), rounded
// to FP32, w = 1.  w = 0 when that FP64 normal is not accurate to well below
// an FP32 unit (|ab x ac| <= 1e-6 |ab| |ac|: its direction error is about
// 1e-16 / sin of the corner angle), and near the reference's cut-off of
// unit() (a cross product of norm <= 1e-14 becomes the zero vector, which
// fails the test): those faces leave their rows to the FP64 decisions.
__global__ void lbvh_face_normals(const double *xyz, uint64_t nv, const int32_t *faces,
                                  uint64_t nf, float4 *fn, double *fn64) {
  const uint64_t f = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  D3 c[3];
  for (int k = 0; k < 3; ++k) {
    const int32_t v = faces[k * nf + f];
    c[k] = D3{xyz[v], xyz[nv + v], xyz[2 * nv + v]};
  }
  const D3 ab = c[1] - c[0], ac = c[2] - c[0], n = cross(ab, ac);
  const D3 u = unit(n);  // the normal test's expression (normal_agrees), once per face
  fn64[3 * f] = u.x, fn64[3 * f + 1] = u.y, fn64[3 * f + 2] = u.z;
  const double n2 = dot(n, n), l2 = dot(ab, ab) * dot(ac, ac);
  if (!(n2 > 1e-12 * l2) || !(n2 > 4e-28)) {
    fn[f] = make_float4(0.f, 0.f, 0.f, 0.f);
    return;
  }
  fn[f] = make_float4(float(u.x), float(u.y), float(u.z), 1.f);
}

Lbvh lbvh_build(Call &call, const double *xyz, const double *vn, uint64_t nv,
                const int32_t *faces, uint64_t nf) {
  Lbvh b;
  b.nv = nv, b.nf = nf, b.faces = faces;
  if (!nf) return b;
  cudaStream_t st = call.stream();
  const uint64_t ni = nf - 1;
  auto pad = [](uint64_t x) { return (x + 255) & ~uint64_t(255); };
  const uint64_t s_xyz = pad(12 * nv), s_child = pad(8 * ni + 8), s_box = pad(48 * ni + 48);
  const uint64_t s_fn = pad(16 * nf), s_order = pad(4 * nv), s_fn64 = pad(24 * nf);
  SYM_CUDA(cudaMalloc(&b.block, 2 * s_xyz + s_child + s_box + s_fn + s_order + s_fn64));
  b.xyz = reinterpret_cast<float *>(b.block);
  b.child = reinterpret_cast<int32_t *>(b.block + s_xyz);
  b.box = reinterpret_cast<float *>(b.block + s_xyz + s_child);
  b.vn = reinterpret_cast<float *>(b.block + s_xyz + s_child + s_box);
  b.fn = reinterpret_cast<float4 *>(b.block + 2 * s_xyz + s_child + s_box);
  b.order = reinterpret_cast<int32_t *>(b.block + 2 * s_xyz + s_child + s_box + s_fn);
  b.fn64 = reinterpret_cast<double *>(b.block + 2 * s_xyz + s_child + s_box + s_fn + s_order);
  lbvh_vertices<<<blocks_for(3 * nv), kThreads, 0, st>>>(xyz, nv, b.xyz);
  check_launch();
  lbvh_vertices<<<blocks_for(3 * nv), kThreads, 0, st>>>(vn, nv, b.vn);
  check_launch();
  lbvh_face_normals<<<blocks_for(nf), kThreads, 0, st>>>(xyz, nv, faces, nf, b.fn, b.fn64);
  check_launch();
  // the mesh box, for the Morton quantisation
  std::vector<float> h(3 * nv);
  SYM_CUDA(cudaMemcpyAsync(h.data(), b.xyz, 12 * nv, cudaMemcpyDeviceToHost, st));
  call.sync();
  float lo[3], hi[3];
  for (int a = 0; a < 3; ++a) {
    auto mm = std::minmax_element(h.begin() + a * nv, h.begin() + (a + 1) * nv);
    lo[a] = *mm.first, hi[a] = *mm.second;
  }
  float ext = std::max({hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2], 1e-30f});
  for (int a = 0; a < 3; ++a) b.scale = std::max({b.scale, std::fabs(lo[a]), std::fabs(hi[a])});
  uint64_t *keys = call.alloc<uint64_t>(nf), *skeys = call.alloc<uint64_t>(nf);
  int32_t *ids = call.alloc<int32_t>(nf), *sids = call.alloc<int32_t>(nf);
  lbvh_keys<<<blocks_for(nf), kThreads, 0, st>>>(b.xyz, nv, faces, nf, make_float3(lo[0], lo[1], lo[2]),
                                                 make_float3(1 / ext, 1 / ext, 1 / ext), keys, ids);
  check_launch();
  radix_sort_pairs(call, keys, ids, skeys, sids, nf, 64);
  {  // the query order of the verification: neighbouring vertices in a warp
    uint64_t *vkeys = call.alloc<uint64_t>(nv), *svkeys = call.alloc<uint64_t>(nv);
    int32_t *vids = call.alloc<int32_t>(nv);
    lbvh_vertex_keys<<<blocks_for(nv), kThreads, 0, st>>>(
        b.xyz, nv, make_float3(lo[0], lo[1], lo[2]), make_float3(1 / ext, 1 / ext, 1 / ext), vkeys,
        vids);
    check_launch();
    call.launched();
    radix_sort_pairs(call, vkeys, vids, svkeys, b.order, nv, 64);
  }
  if (ni) {
    int32_t *parent_in = call.alloc<int32_t>(ni), *parent_leaf = call.alloc<int32_t>(nf);
    unsigned *arrivals = call.alloc<unsigned>(ni);
    SYM_CUDA(cudaMemsetAsync(arrivals, 0, 4 * ni, st));
    lbvh_internal<<<blocks_for(ni), kThreads, 0, st>>>(skeys, int64_t(nf), b.child, parent_in,
                                                        parent_leaf);
    check_launch();
    lbvh_boxes<<<blocks_for(nf), kThreads, 0, st>>>(b.xyz, nv, faces, int64_t(nf), sids, b.child,
                                                     parent_in, parent_leaf, b.box, arrivals);
    check_launch();
  }
  call.launched(ni ? 8 : 6);
  call.sync();
  return b;
}

void lbvh_free(Lbvh &b) {
  if (b.block) cudaFree(b.block);
  b = Lbvh{};
}

namespace {

// `refine` passes of FP64 least-squares refinement of the nc modes' motions
// against the mesh (ICP: forward correspondences under the current motion,
// then the motion that fits them best), on the device; dm is updated in
// place.  `origin` (a point near the mesh) keeps the sums well conditioned.
void refine_motions(Call &call, const BvhView &view, const double *xyz, const double *vn,
                    const double *w, ClusterMotion *dm, uint64_t nc, double tau, int refine,
                    const double origin[3]) {
  const uint64_t nv = view.nv;
  if (refine <= 0 || !nc || !nv || !view.nf) return;
  cudaStream_t st = call.stream();
  const Origin o{{origin[0], origin[1], origin[2]}};
  double *target = call.alloc<double>(nc * nv * 3), *sums = call.alloc<double>(nc * kRefineSums);
  uint8_t *ok = call.alloc<uint8_t>(nc * nv);
  for (int it = 0; it < refine; ++it) {
    refine_pairs<<<blocks_for(nc * nv), kThreads, 0, st>>>(view, xyz, vn, dm, nc, tau,
                                                           float(tau * tau), o, target, ok,
                                                           call.status());
    check_launch();
    refine_sums<<<unsigned(nc), kRefineThreads, 0, st>>>(xyz, w, nv, ok, target, o, sums);
    check_launch();
    refine_solve<<<unsigned((nc + 31) / 32), 32, 0, st>>>(sums, nc, o, dm);
    check_launch();
    call.launched(3);
  }
}

void store_motion(const ClusterMotion &m, sym_cluster_record &r) {
  for (int k = 0; k < 9; ++k) r.rotation[k] = m.r[k];
  for (int k = 0; k < 3; ++k) r.translation[k] = m.t[k], r.plane_normal[k] = m.n[k];
  r.plane_offset = m.offset;
}

}  // namespace

// The reference-order BVH of a resident mesh on the device: the build the
// mesh's load started on a host thread, or, without one, a build from the
// device's vertices and faces.
void ensure_ref_bvh(Call &call, const ResidentSurface &m) {
  RefBvhSource &src = *m.ref;
  if (src.dev.block) return;
  std::unique_ptr<HostBvh> bvh;
  if (src.pending.valid()) {
    bvh = src.pending.get();
  } else {
    std::vector<double> x(3 * m.nv);
    std::vector<int32_t> f(3 * m.nf);
    call.d2h(x.data(), m.xyz, 24 * m.nv);
    call.d2h(f.data(), m.faces, 12 * m.nf);
    call.sync();
    const sym_mesh_view mv{{x.data(), x.data() + m.nv, x.data() + 2 * m.nv, m.nv},
                           {f.data(), f.data() + m.nf, f.data() + 2 * m.nf, m.nf}};
    bvh = std::make_unique<HostBvh>(mv);
  }
  if (2 * bvh->depth + 4 > kRefStack) fail(SYM_RUNTIME_ERROR, "verification: BVH too deep");
  src.dev = ref_bvh_upload(*bvh, call.stream());
}

uint64_t exact_flags(Call &call, const ResidentSurface &m, const ClusterMotion *dm,
                     const sym_cluster_record *records, uint64_t nc, double tau, uint8_t *flags,
                     double *err, uint64_t *fp64_rows) {
  const uint64_t nv = m.nv, rows = nc * 2 * nv;
  cudaStream_t st = call.stream();
  if (fp64_rows) *fp64_rows = 0;
  if (!rows) return 0;
  if (rows >= (uint64_t(1) << 31)) fail(SYM_INVALID_ARGUMENT, "verification: too many queries");
  if (!m.nf) {
    SYM_CUDA(cudaMemsetAsync(flags, 0, rows, st));
    SYM_CUDA(cudaMemsetAsync(err, 0, nc * nv * 8, st));
    return 0;
  }
  const Lbvh &bvh = *m.lbvh;
  std::vector<MotionF> mf(nc);
  for (uint64_t c = 0; c < nc; ++c) {
    const sym_cluster_record &r = records[c];
    for (int k = 0; k < 9; ++k) mf[c].r[k] = float(r.rotation[k]);
    for (int k = 0; k < 3; ++k) mf[c].t[k] = float(r.translation[k]), mf[c].n[k] = float(r.plane_normal[k]);
    mf[c].offset = float(r.plane_offset);
    mf[c].reflection = r.reflection != 0;
  }
  const MotionF *dmf = call.upload(mf.data(), nc);
  RowLists lists;
  lists.forward = call.alloc<uint32_t>(nc * nv);
  lists.faces = call.alloc<int32_t>(nc * nv * kCandidates);
  lists.mark = call.alloc<uint8_t>(rows);
  lists.fp64 = call.alloc<int32_t>(rows);
  lists.reference = call.alloc<int32_t>(rows);
  lists.slot_of = call.alloc<uint32_t>(rows);
  lists.slots = std::min<uint64_t>(rows, uint64_t(1) << 24);  // at most 1 GiB of candidates
  lists.cand = call.alloc<int32_t>(lists.slots * kCandidates);
  lists.counts = call.alloc<unsigned long long>(4);
  uint64_t *listed = call.alloc<uint64_t>(2);
  SYM_CUDA(cudaMemsetAsync(lists.counts, 0, 32, st));
  const BvhView view{bvh.nv, bvh.nf, bvh.faces, bvh.xyz, bvh.child, bvh.box, bvh.fn, bvh.order,
                     bvh.fn64};
  Surface s{m.xyz, nv, m.faces, m.nf, nullptr, nullptr};
  verify_fp32<<<blocks_for(rows), kThreads, 0, st>>>(view, bvh.vn, dmf, nc, float(tau), bvh.scale,
                                                      flags, err, lists, call.status());
  check_launch();
  compact_indices(call, lists.mark, rows, lists.fp64, listed);
  unsigned long long counts[4] = {0, 0, 0, 0};
  call.d2h(counts, lists.counts, 8);
  call.d2h(&counts[1], listed, 8);
  call.sync();
  call.launched();
  if (counts[0]) {
    forward_errors<<<blocks_for(counts[0]), kThreads, 0, st>>>(s, dm, lists, counts[0], err);
    check_launch();
    call.launched();
  }
  if (counts[1]) {
    ensure_ref_bvh(call, m);
    s.nodes = m.ref->dev.nodes, s.ids = m.ref->dev.ids;
    verify_rows_fp64<<<blocks_for(counts[1] * 8), kThreads, 0, st>>>(view, s, m.ref->dev, m.vn, dm, tau,
                                                                  bvh.scale, flags, err, lists,
                                                                  counts[1], call.status());
    check_launch();
    call.launched();
    compact_indices(call, lists.mark, rows, lists.reference, listed + 1);
    call.d2h(&counts[2], listed + 1, 8);
    call.d2h(&counts[3], lists.counts + 3, 8);
    call.sync();
    if (counts[2]) {  // overflowed lists: the wider list first
      verify_rows_wide<<<blocks_for(counts[2]), kThreads, 0, st>>>(
          view, s, m.ref->dev, m.vn, dm, tau, bvh.scale, flags, err, lists, counts[2],
          call.status());
      check_launch();
      call.launched();
      compact_indices(call, lists.mark, rows, lists.reference, listed + 1);
      call.d2h(&counts[2], listed + 1, 8);
      call.d2h(&counts[3], lists.counts + 3, 8);
      call.sync();
    }
  }
  if (fp64_rows) *fp64_rows = counts[1];
  if (counts[2]) {
    verify_listed_ref<<<blocks_for(counts[2]), kThreads, 0, st>>>(s, m.vn, bvh.order, dm, tau,
                                                                   lists, counts[2], flags, err,
                                                                   call.status());
    check_launch();
    call.launched();
  }
  return counts[2] + counts[3];
}

// Coverage, rms and patch counts of the nc modes (sym_detect_fast), after
// `refine` FP64 refinement passes of their motions (written back to
// records); the same coverage, rms and patches as the reference's
// verification of the records.
void verification_fast(Call &call, const ResidentSurface &m, sym_cluster_record *records,
                       uint64_t nc, double tau, int refine, const double origin[3],
                       double *coverage, double *rms, uint32_t *patches, uint64_t *undecided,
                       uint64_t *fp64_rows) {
  const uint64_t nv = m.nv;
  if (undecided) *undecided = 0;
  if (fp64_rows) *fp64_rows = 0;
  if (!nc || !nv) {
    for (uint64_t c = 0; c < nc; ++c) coverage[c] = rms[c] = 0, patches[2 * c] = patches[2 * c + 1] = 0;
    return;
  }
  cudaStream_t st = call.stream();
  std::vector<ClusterMotion> motions(nc);
  for (uint64_t c = 0; c < nc; ++c) motions[c] = cluster_motion(records[c]);
  ClusterMotion *dm = call.upload(motions.data(), nc);
  if (refine > 0 && m.nf) {
    const Lbvh &bvh = *m.lbvh;
    const BvhView view{bvh.nv, bvh.nf, bvh.faces, bvh.xyz, bvh.child, bvh.box, bvh.fn, bvh.order,
                     bvh.fn64};
    refine_motions(call, view, m.xyz, m.vn, m.w, dm, nc, tau, refine, origin);
    call.d2h(motions.data(), dm, nc * sizeof(ClusterMotion));
    call.check_status("transform refinement");
    for (uint64_t c = 0; c < nc; ++c) store_motion(motions[c], records[c]);
  }
  const uint64_t rows = nc * 2 * nv;
  uint8_t *flags = call.alloc<uint8_t>(rows);
  double *err = call.alloc<double>(nc * nv);
  const uint64_t n = exact_flags(call, m, dm, records, nc, tau, flags, err, fp64_rows);
  if (undecided) *undecided = n;
  double *error = call.alloc<double>(nc), *area = call.alloc<double>(nc), *total = call.alloc<double>(1);
  uint64_t *na = call.alloc<uint64_t>(nc);
  tree_sums<<<unsigned(nc + 1), 256, 0, st>>>(flags, err, m.w, nv, nc, error, area, na, total);
  check_launch();
  call.launched();
  int32_t *parent = call.alloc<int32_t>(rows);
  unsigned *dpatch = call.alloc<unsigned>(2 * nc);
  SYM_CUDA(cudaMemsetAsync(dpatch, 0, 8 * nc, st));
  init_parents<<<blocks_for(rows), kThreads, 0, st>>>(flags, rows, parent, nv);
  check_launch();
  unite_edges<<<blocks_for(rows), kThreads, 0, st>>>(m.nbr_off, m.nbr, nv, 2 * nc, parent,
                                                      call.status(), kUniteRetries);
  check_launch();
  count_roots<<<blocks_for(rows), kThreads, 0, st>>>(parent, nv, 2 * nc, dpatch);
  check_launch();
  call.launched(3);
  std::vector<double> herr(nc), harea(nc);
  std::vector<uint64_t> hna(nc);
  std::vector<unsigned> hp(2 * nc);
  double htotal = 0;
  call.d2h(herr.data(), error, nc * 8);
  call.d2h(harea.data(), area, nc * 8);
  call.d2h(hna.data(), na, nc * 8);
  call.d2h(&htotal, total, 8);
  call.d2h(hp.data(), dpatch, 8 * nc);
  call.check_status("verification");
  for (uint64_t c = 0; c < nc; ++c) {
    rms[c] = hna[c] ? std::sqrt(herr[c] / double(hna[c])) : 0;
    coverage[c] = htotal > 0 ? std::min(1.0, harea[c] / htotal) : 0;
    patches[2 * c] = hp[2 * c], patches[2 * c + 1] = hp[2 * c + 1];
  }
}

// The reference's verification of `records` on a resident mesh: side
// lists, patches, coverage and rms identical to verification_core's.
void verification_resident(Call &call, const ResidentSurface &m, const sym_cluster_record *records,
                           uint64_t nc, double tau, std::vector<std::vector<int32_t>> &side,
                           std::vector<std::vector<std::vector<int32_t>>> &patches,
                           std::vector<double> &coverage, std::vector<double> &rms,
                           uint64_t *undecided) {
  const uint64_t nv = m.nv;
  if (undecided) *undecided = 0;
  if (!nc) {
    finish_verification(call, nullptr, nullptr, m.w, m.nbr_off, m.nbr, nv, 0, side, patches,
                        coverage, rms);
    return;
  }
  std::vector<ClusterMotion> motions(nc);
  for (uint64_t c = 0; c < nc; ++c) motions[c] = cluster_motion(records[c]);
  ClusterMotion *dm = call.upload(motions.data(), nc);
  uint8_t *flags = call.alloc<uint8_t>(nc * 2 * nv);
  double *err = call.alloc<double>(nc * nv);
  const uint64_t n = exact_flags(call, m, dm, records, nc, tau, flags, err, nullptr);
  if (undecided) *undecided = n;
  finish_verification(call, flags, err, m.w, m.nbr_off, m.nbr, nv, nc, side, patches, coverage, rms);
}

}  // namespace sym
