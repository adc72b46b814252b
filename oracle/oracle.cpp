// SPDX-License-Identifier: MPL-2.0
//
// ORACLE - test infrastructure only.  This is a CPU restatement of the
// reference (deoksieze/Mitra_algo) CPU backend for the symmetry hot path, used
// by tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg to
// check results.  The GPU library never links, loads or calls it.
//
// Every function follows the reference algorithm operation by operation, in
// FP64, so that results agree bit for bit with the reference's own CPU build
// (compiled without FMA contraction: see oracle/Makefile, -ffp-contract=off).
// Parity is pinned against golden vectors produced by the reference itself
// (tests/golden/make_golden.py, oracle/ref_harness.cpp).
//
// Entry points use the POD views of include/mitra_gb300.h.  Results are
// heap blocks released with oracle_release().
#include "../include/mitra_gb300.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <queue>
#include <random>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

thread_local std::string g_error;

// ----------------------------------------------------------------- vectors
// Arithmetic mirrors src/core/math.cpp:7-16 of the reference: division of a
// vector by a scalar multiplies by the reciprocal, unit() leaves vectors of
// norm <= 1e-14 at zero.
struct V3 {
  double x = 0, y = 0, z = 0;
  double at(int i) const { return i == 0 ? x : (i == 1 ? y : z); }
  double &at(int i) { return i == 0 ? x : (i == 1 ? y : z); }
};
V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 mul(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
V3 divs(V3 a, double s) { return mul(a, 1 / s); }
double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V3 cross(V3 a, V3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
double norm(V3 a) { return std::sqrt(dot(a, a)); }
V3 unit(V3 a) {
  double n = norm(a);
  return n > 1e-14 ? divs(a, n) : V3{};
}
using M3 = std::array<double, 9>; // row-major
V3 xform(const M3 &m, V3 v) {
  return {m[0] * v.x + m[1] * v.y + m[2] * v.z,
          m[3] * v.x + m[4] * v.y + m[5] * v.z,
          m[6] * v.x + m[7] * v.y + m[8] * v.z};
}
M3 transpose(const M3 &m) {
  return {m[0], m[3], m[6], m[1], m[4], m[7], m[2], m[5], m[8]};
}
M3 matmul(const M3 &a, const M3 &b) { // reference math.cpp:34-41 loop order
  M3 r{};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 3; ++k)
        r[i * 3 + j] += a[i * 3 + k] * b[k * 3 + j];
  return r;
}
M3 mirror_matrix(V3 n) { // reference math.cpp:116-121
  M3 r{1, 0, 0, 0, 1, 0, 0, 0, 1};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      r[i * 3 + j] -= 2 * n.at(i) * n.at(j);
  return r;
}
M3 columns(V3 a, V3 b, V3 c) { // frame(): a, b, c are the columns
  return {a.x, b.x, c.x, a.y, b.y, c.y, a.z, b.z, c.z};
}

// Squared distance from p to segment ab (reference math.cpp:75-81).
double segment_d2(V3 p, V3 a, V3 b) {
  V3 d = sub(b, a);
  double l = dot(d, d);
  double t = l > 1e-14 ? std::clamp(dot(sub(p, a), d) / l, 0.0, 1.0) : 0;
  V3 e = sub(p, add(a, mul(d, t)));
  return dot(e, e);
}
// Closest-point region test of Ericson's "Real-Time Collision Detection"
// 5.1.5, with the reference's degenerate-triangle rule (math.cpp:82-112).
double triangle_d2(V3 p, V3 a, V3 b, V3 c) {
  V3 ab = sub(b, a), ac = sub(c, a), ap = sub(p, a);
  V3 nrm = cross(ab, ac);
  if (dot(nrm, nrm) < 1e-14 * 1e-14)
    return std::min({segment_d2(p, a, b), segment_d2(p, a, c),
                     segment_d2(p, b, c)});
  double d1 = dot(ab, ap), d2 = dot(ac, ap);
  if (d1 <= 0 && d2 <= 0)
    return dot(ap, ap);
  V3 bp = sub(p, b);
  double d3 = dot(ab, bp), d4 = dot(ac, bp);
  if (d3 >= 0 && d4 <= d3)
    return dot(bp, bp);
  double vc = d1 * d4 - d3 * d2;
  if (vc <= 0 && d1 >= 0 && d3 <= 0) {
    V3 e = sub(p, add(a, mul(ab, d1 / (d1 - d3))));
    return dot(e, e);
  }
  V3 cp = sub(p, c);
  double d5 = dot(ab, cp), d6 = dot(ac, cp);
  if (d6 >= 0 && d5 <= d6)
    return dot(cp, cp);
  double vb = d5 * d2 - d1 * d6;
  if (vb <= 0 && d2 >= 0 && d6 <= 0) {
    V3 e = sub(p, add(a, mul(ac, d2 / (d2 - d6))));
    return dot(e, e);
  }
  double va = d3 * d6 - d5 * d4;
  if (va <= 0 && (d4 - d3) >= 0 && (d5 - d6) >= 0) {
    V3 e = sub(p, add(b, mul(sub(c, b), (d4 - d3) / ((d4 - d3) + (d5 - d6)))));
    return dot(e, e);
  }
  V3 e = sub(p, add(add(a, mul(ab, vb / (va + vb + vc))),
                    mul(ac, vc / (va + vb + vc))));
  return std::max(0.0, dot(e, e));
}

// ------------------------------------------------------------- view access
V3 point(const sym_points_view &p, uint64_t i) { return {p.x[i], p.y[i], p.z[i]}; }
struct Feat {
  V3 normal, dmin, dmax;
  double kmin, kmax;
  bool valid;
};
Feat feature(const sym_features_view &f, uint64_t i) {
  return {point(f.normal, i), point(f.dmin, i), point(f.dmax, i),
          f.kmin[i],          f.kmax[i],        f.valid[i] != 0};
}
uint64_t row_begin(const sym_csr_view &c, uint64_t r) { return c.offsets[r]; }
uint64_t row_end(const sym_csr_view &c, uint64_t r) { return c.offsets[r + 1]; }

// ---------------------------------------------------------------- storage
// One malloc block per result; the struct's `storage` points at it.
struct Block {
  std::vector<std::pair<void **, size_t>> parts;
  template <class T> void add(T **ptr, uint64_t n) {
    parts.push_back({reinterpret_cast<void **>(ptr), size_t(n) * sizeof(T)});
  }
  void *commit() {
    size_t total = 0;
    for (auto &p : parts)
      total += (p.second + 63) & ~size_t(63);
    char *base = static_cast<char *>(std::malloc(total ? total : 64));
    if (!base)
      throw std::bad_alloc();
    size_t at = 0;
    for (auto &p : parts) {
      *p.first = base + at;
      at += (p.second + 63) & ~size_t(63);
    }
    return base;
  }
};

// -------------------------------------------------------------------- RNG
std::mt19937_64 load_rng(const sym_rng *r) {
  std::stringstream s;
  for (int i = 0; i < 312; ++i)
    s << r->words[i] << ' ';
  s << r->index;
  std::mt19937_64 e;
  s >> e;
  return e;
}
void store_rng(const std::mt19937_64 &e, sym_rng *r) {
  std::stringstream s;
  s << e;
  for (int i = 0; i < 312; ++i)
    s >> r->words[i];
  s >> r->index;
}

// ------------------------------------------------------------- curvature
// Reference src/cpu/curvature.cpp:14-79.
void curvature(const sym_mesh_view &m, const sym_topology_view &g,
               const sym_options &o, const sym_features_out &out) {
  const uint64_t n = m.vertices.count;
  std::vector<M3> tensor(n, M3{});
  std::vector<int> count(n, 0);
  double mean = 0;
  for (uint64_t e = 0; e < g.edge_count; ++e)
    mean += norm(sub(point(m.vertices, g.edges[e].hi),
                     point(m.vertices, g.edges[e].lo)));
  mean /= g.edge_count;
  for (uint64_t e = 0; e < g.edge_count; ++e) {
    const sym_edge &edge = g.edges[e];
    if (edge.face1 < 0)
      continue;
    V3 dir = sub(point(m.vertices, edge.b), point(m.vertices, edge.a));
    double len = norm(dir);
    dir = unit(dir);
    V3 n1 = point(g.face_normals, edge.face0), n2 = point(g.face_normals, edge.face1);
    double beta =
        std::atan2(dot(cross(n1, n2), dir), std::clamp(dot(n1, n2), -1.0, 1.0));
    for (int vertex : {edge.a, edge.b}) {
      ++count[vertex];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
          tensor[vertex][i * 3 + j] += dir.at(i) * dir.at(j) * beta * len / mean;
    }
  }
  for (uint64_t i = 0; i < n; ++i)
    for (double &x : tensor[i])
      x /= std::max(1, count[i]);
  for (int it = 0; it < o.smoothing; ++it) {
    std::vector<M3> next = tensor;
    for (uint64_t i = 0; i < n; ++i) {
      for (uint64_t k = row_begin(g.neighbors, i); k < row_end(g.neighbors, i); ++k)
        for (int c = 0; c < 9; ++c)
          next[i][c] += tensor[g.neighbors.indices[k]][c];
      uint64_t degree = row_end(g.neighbors, i) - row_begin(g.neighbors, i);
      for (double &x : next[i])
        x /= (degree + 1);
    }
    tensor.swap(next);
  }
  for (uint64_t i = 0; i < n; ++i) {
    V3 nv = point(g.normals, i);
    V3 dmin{}, dmax{};
    double kmin = 0, kmax = 0;
    bool valid = false;
    uint64_t degree = row_end(g.neighbors, i) - row_begin(g.neighbors, i);
    if (!(norm(nv) < 0.5 || degree < 3)) {
      V3 axis = std::abs(nv.x) < 0.8 ? V3{1, 0, 0} : V3{0, 1, 0};
      V3 u = unit(cross(nv, axis)), v = cross(nv, u);
      double a = dot(u, xform(tensor[i], u)), b = dot(u, xform(tensor[i], v)),
             c = dot(v, xform(tensor[i], v));
      double angle = 0.5 * std::atan2(2 * b, a - c);
      V3 high = add(mul(u, std::cos(angle)), mul(v, std::sin(angle)));
      V3 low = unit(cross(high, nv));
      double delta = std::hypot(a - c, 2 * b);
      kmin = (a + c - delta) / 2;
      kmax = (a + c + delta) / 2;
      dmin = low;
      dmax = unit(cross(nv, low));
      valid = std::isfinite(kmin) && std::isfinite(kmax) && delta > 1e-10;
    } else {
      nv = V3{}; // untouched rows keep the zero Feature
    }
    out.normal_x[i] = nv.x, out.normal_y[i] = nv.y, out.normal_z[i] = nv.z;
    out.dmin_x[i] = dmin.x, out.dmin_y[i] = dmin.y, out.dmin_z[i] = dmin.z;
    out.dmax_x[i] = dmax.x, out.dmax_y[i] = dmax.y, out.dmax_z[i] = dmax.z;
    out.kmin[i] = kmin, out.kmax[i] = kmax, out.valid[i] = valid;
  }
}

// -------------------------------------------------------------- sampling
// Reference src/core/sampling.cpp:5-24: exponential keys -log(u)/w.
std::vector<int32_t> sample_vertices(const double *w, uint64_t n, double ratio,
                                     std::mt19937_64 &rng) {
  std::vector<std::pair<double, int>> keys;
  for (uint64_t i = 0; i < n; ++i)
    if (w[i] > 0) {
      double u = (static_cast<double>(rng() >> 11) + 0.5) / 9007199254740992.0;
      keys.push_back({-std::log(u) / w[i], static_cast<int>(i)});
    }
  std::sort(keys.begin(), keys.end());
  size_t target =
      std::min(keys.size(), static_cast<size_t>(std::ceil(n * ratio)));
  std::vector<int32_t> s;
  for (size_t i = 0; i < target; ++i)
    s.push_back(keys[i].second);
  std::sort(s.begin(), s.end());
  return s;
}

// ----------------------------------------------------------- votes helpers
struct VoteRow {
  int32_t pair;
  bool reflection;
  M3 rotation;
  V3 translation, normal;
  double offset;
  double desc[12];
};

// --------------------------------------------------------------- surface
// Median-split BVH of the reference (src/cpu/surface.h:12-96): leaves hold at
// most 8 faces, inner nodes split at the median face centroid of the longest
// box axis with std::nth_element, nearest-face search visits the nearer child
// first and keeps the first face reaching the strict minimum.
struct Node {
  V3 lo, hi;
  int left = -1, right = -1, begin = 0, end = 0;
};
class Bvh {
  const sym_mesh_view &mesh;
  std::vector<int> ids;
  std::vector<Node> nodes;
  V3 vtx(int f, int k) const {
    const int32_t *col = k == 0 ? mesh.faces.v0 : (k == 1 ? mesh.faces.v1 : mesh.faces.v2);
    return point(mesh.vertices, col[f]);
  }
  int build(int begin, int end) {
    Node n;
    n.lo = {1e300, 1e300, 1e300};
    n.hi = {-1e300, -1e300, -1e300};
    for (int i = begin; i < end; ++i)
      for (int k = 0; k < 3; ++k) {
        V3 p = vtx(ids[i], k);
        for (int c = 0; c < 3; ++c) {
          n.lo.at(c) = std::min(n.lo.at(c), p.at(c));
          n.hi.at(c) = std::max(n.hi.at(c), p.at(c));
        }
      }
    n.begin = begin;
    n.end = end;
    int index = static_cast<int>(nodes.size());
    nodes.push_back(n);
    if (end - begin > 8) {
      V3 ext = sub(n.hi, n.lo);
      int axis = ext.y > ext.x ? 1 : 0;
      if (ext.z > ext.at(axis))
        axis = 2;
      int mid = (begin + end) / 2;
      auto centroid = [&](int f) {
        return (vtx(f, 0).at(axis) + vtx(f, 1).at(axis) + vtx(f, 2).at(axis)) / 3;
      };
      std::nth_element(ids.begin() + begin, ids.begin() + mid, ids.begin() + end,
                       [&](int a, int b) { return centroid(a) < centroid(b); });
      int l = build(begin, mid), r = build(mid, end);
      nodes[index].left = l;
      nodes[index].right = r;
    }
    return index;
  }
  static double box_d2(V3 p, const Node &n) {
    double s = 0;
    for (int k = 0; k < 3; ++k) {
      double d = std::max({n.lo.at(k) - p.at(k), 0.0, p.at(k) - n.hi.at(k)});
      s += d * d;
    }
    return s;
  }
  void search(int index, V3 p, double &best, int &face) const {
    const Node &n = nodes[index];
    if (box_d2(p, n) > best)
      return;
    if (n.left < 0) {
      for (int i = n.begin; i < n.end; ++i) {
        double d = triangle_d2(p, vtx(ids[i], 0), vtx(ids[i], 1), vtx(ids[i], 2));
        if (d < best) {
          best = d;
          face = ids[i];
        }
      }
      return;
    }
    int first = n.left, second = n.right;
    if (box_d2(p, nodes[first]) > box_d2(p, nodes[second]))
      std::swap(first, second);
    search(first, p, best, face);
    search(second, p, best, face);
  }

public:
  explicit Bvh(const sym_mesh_view &m) : mesh(m) {
    ids.resize(m.faces.count);
    for (size_t i = 0; i < ids.size(); ++i)
      ids[i] = static_cast<int>(i);
    build(0, static_cast<int>(ids.size()));
  }
  std::pair<double, int> nearest(V3 p) const {
    double best = std::numeric_limits<double>::infinity();
    int face = -1;
    search(0, p, best, face);
    return {best, face};
  }
};

// Breadth-first components of the induced neighbour subgraph, seeded in the
// order of `ids` (reference src/cpu/verification.cpp:22-49).
std::vector<std::vector<int32_t>> components(const std::vector<int32_t> &ids,
                                             const sym_topology_view &g) {
  uint64_t n = g.neighbors.rows;
  std::vector<char> allowed(n, 0), seen(n, 0);
  for (int v : ids)
    allowed[v] = 1;
  std::vector<std::vector<int32_t>> result;
  for (int seed : ids) {
    if (seen[seed])
      continue;
    std::queue<int> q;
    q.push(seed);
    seen[seed] = 1;
    std::vector<int32_t> patch;
    while (!q.empty()) {
      int v = q.front();
      q.pop();
      patch.push_back(v);
      for (uint64_t k = row_begin(g.neighbors, v); k < row_end(g.neighbors, v); ++k) {
        int w = g.neighbors.indices[k];
        if (allowed[w] && !seen[w]) {
          seen[w] = 1;
          q.push(w);
        }
      }
    }
    std::sort(patch.begin(), patch.end());
    result.push_back(std::move(patch));
  }
  return result;
}

// ------------------------------------------------------------- clustering
// Reference src/cpu/clustering.cpp:32-208.
struct Desc {
  double v[12] = {};
  int dim = 0;
};
double desc_d2(const Desc &a, const Desc &b) { // clustering.cpp:24-31
  double s = 0;
  for (int i = 0; i < a.dim; ++i) {
    double d = a.v[i] - b.v[i];
    s += d * d;
  }
  return s;
}
struct ClusterRow {
  sym_cluster_record record{};
  std::vector<int32_t> votes;
};

template <class F> sym_status guarded(F f) {
  try {
    f();
    return SYM_OK;
  } catch (const std::invalid_argument &e) {
    g_error = e.what();
    return SYM_INVALID_ARGUMENT;
  } catch (const std::overflow_error &e) {
    g_error = e.what();
    return SYM_OVERFLOW;
  } catch (const std::exception &e) {
    g_error = e.what();
    return SYM_RUNTIME_ERROR;
  }
}

} // namespace

extern "C" {

const char *oracle_last_error(void) { return g_error.c_str(); }
void oracle_release(void *storage) { std::free(storage); }

void oracle_rng_seed(sym_rng *r, uint64_t seed) { store_rng(std::mt19937_64(seed), r); }
uint64_t oracle_rng_next(sym_rng *r) {
  auto e = load_rng(r);
  uint64_t x = e();
  store_rng(e, r);
  return x;
}

// The reference's sample_vertices alone (src/core/sampling.cpp:5-24);
// `out` has room for n ids.
int oracle_sample_vertices(const double *w, uint64_t n, double ratio, sym_rng *r, int32_t *out,
                           uint64_t *count) {
  auto e = load_rng(r);
  auto s = sample_vertices(w, n, ratio, e);
  store_rng(e, r);
  std::copy(s.begin(), s.end(), out);
  *count = s.size();
  return 0;
}

double oracle_triangle_distance2(const double *q) {
  return triangle_d2({q[0], q[1], q[2]}, {q[3], q[4], q[5]}, {q[6], q[7], q[8]},
                     {q[9], q[10], q[11]});
}

sym_status oracle_curvature(const sym_mesh_view *m, const sym_topology_view *g,
                            const sym_options *o, const sym_features_out *out) {
  return guarded([&] { curvature(*m, *g, *o, *out); });
}

sym_status oracle_select(const sym_mesh_view *m, const sym_features_view *f,
                         const double *weights, uint64_t weight_count,
                         const sym_options *o, sym_rng *rng, sym_selection *out) {
  return guarded([&] {
    if (weight_count != m->vertices.count)
      throw std::invalid_argument("SoA component lengths differ");
    auto engine = load_rng(rng);
    auto sample = sample_vertices(weights, weight_count, o->sample_ratio, engine);
    store_rng(engine, rng);
    std::vector<int32_t> pruned;
    for (int32_t i : sample) { // reference selection.cpp:21-27
      Feat p = feature(*f, i);
      double maximum = std::max(std::abs(p.kmin), std::abs(p.kmax));
      if (p.valid && maximum > 1e-10 &&
          std::abs(p.kmin - p.kmax) / maximum > 1 - o->prune)
        pruned.push_back(i);
    }
    Block b;
    b.add(&out->sample, sample.size());
    b.add(&out->pruned, pruned.size());
    out->storage = b.commit();
    out->sample_count = sample.size();
    out->pruned_count = pruned.size();
    std::copy(sample.begin(), sample.end(), out->sample);
    std::copy(pruned.begin(), pruned.end(), out->pruned);
  });
}

sym_status oracle_pairing(const sym_mesh_view *m, const sym_features_view *f,
                          const int32_t *sel, uint64_t count,
                          const sym_model_context *ctx, const sym_options *o,
                          sym_pairs *out) {
  return guarded([&] { // reference pairing.cpp:14-35
    std::vector<int32_t> a, b;
    for (uint64_t x = 0; x < count; ++x)
      for (uint64_t y = x + 1; y < count; ++y) {
        int32_t i = sel[x], j = sel[y];
        Feat p = feature(*f, i), q = feature(*f, j);
        double magnitude = std::max({std::abs(p.kmin), std::abs(p.kmax),
                                     std::abs(q.kmin), std::abs(q.kmax), 1e-10});
        double tolerance = o->pair_threshold * magnitude;
        if (std::abs(p.kmin - q.kmin) > tolerance ||
            std::abs(p.kmax - q.kmax) > tolerance ||
            norm(sub(point(m->vertices, i), point(m->vertices, j))) <
                0.03 * ctx->box_size)
          continue;
        if (a.size() >= o->max_pairs)
          throw std::runtime_error("Pair budget exceeded; lower --sample-ratio "
                                   "or tighten --pair-threshold");
        a.push_back(i);
        b.push_back(j);
      }
    Block blk;
    blk.add(&out->a, a.size());
    blk.add(&out->b, b.size());
    out->storage = blk.commit();
    out->count = a.size();
    std::copy(a.begin(), a.end(), out->a);
    std::copy(b.begin(), b.end(), out->b);
  });
}

sym_status oracle_transformations(const sym_mesh_view *m, const sym_features_view *f,
                                  const sym_pairs_view *pairs,
                                  const sym_model_context *ctx,
                                  const sym_options *o, sym_votes *out) {
  return guarded([&] { // reference transformations.cpp:17-73
    double box = ctx->box_size;
    V3 center{ctx->center[0], ctx->center[1], ctx->center[2]};
    std::vector<VoteRow> rows;
    auto push = [&](const VoteRow &r) {
      if (rows.size() >= o->max_votes)
        throw std::runtime_error("Vote budget exceeded; lower --sample-ratio or "
                                 "tighten --pair-threshold");
      rows.push_back(r);
    };
    for (uint64_t i = 0; i < pairs->count; ++i) {
      int32_t ia = pairs->a[i], ib = pairs->b[i];
      V3 p = point(m->vertices, ia), q = point(m->vertices, ib);
      Feat fa = feature(*f, ia), fb = feature(*f, ib);
      V3 n = unit(sub(q, p));
      int dominant = 0;
      for (int k = 1; k < 3; ++k)
        if (std::abs(n.at(k)) > std::abs(n.at(dominant)))
          dominant = k;
      if (n.at(dominant) < 0)
        n = mul(n, -1);
      double d = -dot(n, divs(add(p, q), 2));
      M3 mirror = mirror_matrix(n);
      if (dot(xform(mirror, fa.normal), fb.normal) > 0.75 &&
          std::abs(dot(xform(mirror, fa.dmin), fb.dmin)) > 0.75) {
        VoteRow r{};
        r.pair = static_cast<int32_t>(i);
        r.reflection = true;
        r.rotation = mirror;
        r.translation = mul(n, -2 * d);
        r.normal = n;
        r.offset = d;
        r.desc[0] = n.x, r.desc[1] = n.y, r.desc[2] = n.z;
        r.desc[3] = (d + dot(n, center)) / box;
        push(r);
      }
      M3 frame_a = columns(fa.dmin, fa.dmax, fa.normal);
      for (double sign : {1.0, -1.0}) {
        M3 frame_b = columns(mul(fb.dmin, sign), mul(fb.dmax, sign), fb.normal);
        M3 rot = matmul(frame_b, transpose(frame_a));
        V3 t = sub(q, xform(rot, p));
        V3 centered = divs(sub(add(xform(rot, center), t), center), box);
        VoteRow r{};
        r.pair = static_cast<int32_t>(i);
        r.reflection = false;
        r.rotation = rot;
        r.translation = t;
        for (int k = 0; k < 9; ++k)
          r.desc[k] = rot[k] / 2;
        r.desc[9] = centered.x, r.desc[10] = centered.y, r.desc[11] = centered.z;
        push(r);
      }
    }
    uint64_t nv = rows.size();
    Block blk;
    blk.add(&out->pair, nv);
    blk.add(&out->kind, nv);
    for (int k = 0; k < 9; ++k)
      blk.add(&out->rotation[k], nv);
    for (int k = 0; k < 3; ++k) {
      blk.add(&out->translation[k], nv);
      blk.add(&out->plane_normal[k], nv);
    }
    blk.add(&out->plane_offset, nv);
    for (int k = 0; k < 12; ++k)
      blk.add(&out->descriptor[k], nv);
    out->storage = blk.commit();
    out->count = nv;
    for (uint64_t v = 0; v < nv; ++v) {
      const VoteRow &r = rows[v];
      out->pair[v] = r.pair;
      out->kind[v] = r.reflection ? SYM_REFLECTION : SYM_RIGID;
      for (int k = 0; k < 9; ++k)
        out->rotation[k][v] = r.rotation[k];
      for (int k = 0; k < 3; ++k) {
        out->translation[k][v] = r.translation.at(k);
        out->plane_normal[k][v] = r.normal.at(k);
      }
      out->plane_offset[v] = r.offset;
      for (int k = 0; k < 12; ++k)
        out->descriptor[k][v] = r.desc[k];
    }
  });
}

// Mean-shift statistics of the last oracle_clustering call on this thread:
// trajectories run and membership evaluations made (votes x iterations).
static thread_local uint64_t g_trajectories = 0, g_evaluations = 0;
void oracle_clustering_stats(uint64_t *trajectories, uint64_t *evaluations) {
  *trajectories = g_trajectories;
  *evaluations = g_evaluations;
}

sym_status oracle_clustering(const sym_votes_view *votes, const sym_model_context *ctx,
                             const sym_options *o, sym_rng *rng, sym_clusters *out) {
  return guarded([&] {
    g_trajectories = g_evaluations = 0;
    auto engine = load_rng(rng);
    const uint64_t q = votes->count;
    const double h = o->bandwidth, h2 = h * h;
    auto desc_of = [&](uint64_t i) {
      Desc d;
      d.dim = votes->kind[i] == SYM_REFLECTION ? 4 : 12;
      for (int k = 0; k < 12; ++k)
        d.v[k] = votes->descriptor[k][i];
      return d;
    };
    std::vector<Desc> centers;
    std::vector<bool> types;
    std::vector<std::map<int, uint64_t>> counters;
    std::vector<bool> visited(q, false);
    uint64_t support_entries = 0;
    int limited = 0;
    while (true) { // driver: clustering.cpp:44-96
      std::vector<int> seeds;
      for (uint64_t i = 0; i < q; ++i)
        if (!visited[i])
          seeds.push_back(static_cast<int>(i));
      if (seeds.empty())
        break;
      int seed = seeds[engine() % seeds.size()];
      bool reflection = votes->kind[seed] == SYM_REFLECTION;
      Desc mean = desc_of(seed);
      // trajectory: clustering.cpp:156-185 with the evaluator of :186-208
      std::map<int, uint64_t> support;
      bool converged = false, exhausted = false;
      ++g_trajectories;
      for (int it = 0; it < o->max_iterations; ++it) {
        double weight = 0;
        Desc sum;
        sum.dim = mean.dim;
        std::vector<int> members;
        for (uint64_t j = 0; j < q; ++j) {
          if ((votes->kind[j] == SYM_REFLECTION) != reflection)
            continue;
          ++g_evaluations;
          Desc x = desc_of(j);
          double dist = desc_d2(mean, x);
          if (dist < h2) {
            double w = 1 - dist / h2;
            weight += w;
            members.push_back(static_cast<int>(j));
            for (int k = 0; k < mean.dim; ++k)
              sum.v[k] += w * x.v[k];
          }
        }
        for (int j : members)
          ++support[j];
        if (weight <= 1e-14) {
          exhausted = true;
          break;
        }
        for (int k = 0; k < sum.dim; ++k)
          sum.v[k] /= weight;
        double movement = desc_d2(mean, sum);
        mean = sum;
        if (movement < 1e-6 * h2) {
          converged = true;
          break;
        }
      }
      for (const auto &e : support)
        visited[e.first] = true;
      if (exhausted)
        visited[seed] = true;
      if (!converged)
        ++limited;
      int merge = -1;
      for (size_t c = 0; c < centers.size(); ++c)
        if (types[c] == reflection && desc_d2(mean, centers[c]) < h2 / 4) {
          merge = static_cast<int>(c);
          break;
        }
      if (merge < 0) {
        centers.push_back(mean);
        types.push_back(reflection);
        support_entries += support.size();
        counters.push_back(std::move(support));
      } else {
        double old = static_cast<double>(counters[merge].size());
        double now = static_cast<double>(support.size());
        if (old + now > 0)
          for (int k = 0; k < mean.dim; ++k)
            centers[merge].v[k] =
                (old * centers[merge].v[k] + now * mean.v[k]) / (old + now);
        size_t before = counters[merge].size();
        for (const auto &e : support)
          counters[merge][e.first] += e.second;
        support_entries += counters[merge].size() - before;
      }
      if (support_entries > 5000000)
        throw std::runtime_error(
            "Mean-shift support budget exceeded; lower --sample-ratio");
      if (centers.size() > 20000)
        throw std::runtime_error("Too many mean-shift modes; increase "
                                 "--bandwidth or lower --sample-ratio");
    }
    // winners: clustering.cpp:97-108
    std::vector<std::vector<int32_t>> members(centers.size());
    std::vector<uint64_t> best(q, 0);
    std::vector<int> winner(q, -1);
    for (size_t c = 0; c < counters.size(); ++c)
      for (const auto &e : counters[c])
        if (e.second > best[e.first]) {
          best[e.first] = e.second;
          winner[e.first] = static_cast<int>(c);
        }
    for (uint64_t i = 0; i < q; ++i)
      if (winner[i] >= 0)
        members[winner[i]].push_back(static_cast<int32_t>(i));
    // decode: clustering.cpp:109-141
    V3 origin{ctx->center[0], ctx->center[1], ctx->center[2]};
    std::vector<ClusterRow> rows;
    for (size_t c = 0; c < centers.size(); ++c) {
      if (members[c].empty())
        continue;
      ClusterRow row;
      row.record.reflection = types[c];
      row.votes = std::move(members[c]);
      const Desc &d = centers[c];
      if (types[c]) {
        V3 n{d.v[0], d.v[1], d.v[2]};
        double length = norm(n);
        V3 pn = unit(n);
        double offset = d.v[3] * ctx->box_size / length - dot(pn, origin);
        M3 r = mirror_matrix(pn);
        V3 t = mul(pn, -2 * offset);
        for (int k = 0; k < 9; ++k)
          row.record.rotation[k] = r[k];
        for (int k = 0; k < 3; ++k) {
          row.record.translation[k] = t.at(k);
          row.record.plane_normal[k] = pn.at(k);
        }
        row.record.plane_offset = offset;
      } else {
        M3 mm{};
        for (int k = 0; k < 9; ++k)
          mm[k] = d.v[k] * 2;
        auto col = [&](int i) { return V3{mm[i], mm[3 + i], mm[6 + i]}; };
        V3 a = unit(col(0)), b = unit(sub(col(1), mul(a, dot(a, col(1)))));
        if (norm(a) < 0.5 || norm(b) < 0.5) {
          int first = row.votes[0];
          for (int k = 0; k < 9; ++k)
            mm[k] = votes->rotation[k][first];
        } else {
          mm = columns(a, b, cross(a, b));
        }
        V3 t{d.v[9], d.v[10], d.v[11]};
        V3 tr = sub(add(mul(t, ctx->box_size), origin), xform(mm, origin));
        for (int k = 0; k < 9; ++k)
          row.record.rotation[k] = mm[k];
        for (int k = 0; k < 3; ++k)
          row.record.translation[k] = tr.at(k);
      }
      rows.push_back(std::move(row));
    }
    std::stable_sort(rows.begin(), rows.end(),
                     [](const ClusterRow &a, const ClusterRow &b) {
                       return a.votes.size() > b.votes.size();
                     });
    if (rows.size() > static_cast<size_t>(o->max_clusters))
      rows.resize(o->max_clusters);
    uint64_t total = 0;
    for (auto &r : rows)
      total += r.votes.size();
    Block blk;
    blk.add(&out->records, rows.size());
    blk.add(&out->vote_offsets, rows.size() + 1);
    blk.add(&out->vote_indices, total);
    out->storage = blk.commit();
    out->count = rows.size();
    out->limited_iterations = limited;
    out->vote_offsets[0] = 0;
    for (size_t c = 0; c < rows.size(); ++c) {
      out->records[c] = rows[c].record;
      std::copy(rows[c].votes.begin(), rows[c].votes.end(),
                out->vote_indices + out->vote_offsets[c]);
      out->vote_offsets[c + 1] = out->vote_offsets[c] + rows[c].votes.size();
    }
    store_rng(engine, rng);
  });
}

sym_status oracle_verification(const sym_mesh_view *m, const sym_topology_view *g,
                               const sym_clusters_view *clusters,
                               const sym_model_context *ctx, const sym_options *o,
                               sym_verification_result *out) {
  return guarded([&] { // reference verification.cpp:50-110
    const uint64_t n = m->vertices.count, nc = clusters->count;
    Bvh surface(*m);
    double tau = o->verify_threshold * ctx->box_size;
    double total = 0;
    for (uint64_t i = 0; i < g->weight_count; ++i)
      total += g->weights[i];
    std::vector<std::vector<int32_t>> sa(nc), sb(nc);
    std::vector<std::vector<std::vector<int32_t>>> pa(nc), pb(nc);
    std::vector<double> coverage(nc), rms(nc);
    auto face_normal = [&](int f) {
      V3 a = point(m->vertices, m->faces.v0[f]), b = point(m->vertices, m->faces.v1[f]),
         c = point(m->vertices, m->faces.v2[f]);
      return unit(cross(sub(b, a), sub(c, a)));
    };
    for (uint64_t ci = 0; ci < nc; ++ci) {
      const sym_cluster_record &c = clusters->records[ci];
      M3 rot, inv;
      for (int k = 0; k < 9; ++k)
        rot[k] = c.rotation[k];
      inv = transpose(rot);
      V3 t{c.translation[0], c.translation[1], c.translation[2]};
      V3 pn{c.plane_normal[0], c.plane_normal[1], c.plane_normal[2]};
      double error = 0, area = 0;
      for (uint64_t i = 0; i < n; ++i) {
        V3 p = point(m->vertices, i), q = add(xform(rot, p), t);
        if (norm(sub(q, p)) < tau * 2)
          continue;
        if (c.reflection && dot(pn, p) + c.plane_offset >= -tau)
          continue;
        auto hit = surface.nearest(q);
        if (hit.first > tau * tau)
          continue;
        if (dot(xform(rot, point(g->normals, i)), face_normal(hit.second)) < 0.5)
          continue;
        sa[ci].push_back(static_cast<int32_t>(i));
        error += hit.first;
        area += g->weights[i];
      }
      for (uint64_t i = 0; i < n; ++i) {
        V3 p = point(m->vertices, i), q = xform(inv, sub(p, t));
        if (norm(sub(q, p)) < tau * 2)
          continue;
        if (c.reflection && dot(pn, p) + c.plane_offset <= tau)
          continue;
        auto hit = surface.nearest(q);
        if (hit.first > tau * tau)
          continue;
        if (dot(xform(inv, point(g->normals, i)), face_normal(hit.second)) < 0.5)
          continue;
        sb[ci].push_back(static_cast<int32_t>(i));
        area += g->weights[i];
      }
      rms[ci] = sa[ci].empty() ? 0 : std::sqrt(error / sa[ci].size());
      coverage[ci] = total > 0 ? std::min(1.0, area / total) : 0;
      pa[ci] = components(sa[ci], *g);
      pb[ci] = components(sb[ci], *g);
    }
    uint64_t na = 0, nb = 0, ra = 0, rb = 0;
    for (uint64_t c = 0; c < nc; ++c) {
      na += sa[c].size(), nb += sb[c].size();
      ra += pa[c].size(), rb += pb[c].size();
    }
    Block blk;
    blk.add(&out->side_a_offsets, nc + 1);
    blk.add(&out->side_b_offsets, nc + 1);
    blk.add(&out->side_a, na);
    blk.add(&out->side_b, nb);
    blk.add(&out->patches_a.groups, nc + 1);
    blk.add(&out->patches_a.offsets, ra + 1);
    blk.add(&out->patches_a.indices, na);
    blk.add(&out->patches_b.groups, nc + 1);
    blk.add(&out->patches_b.offsets, rb + 1);
    blk.add(&out->patches_b.indices, nb);
    blk.add(&out->coverage, nc);
    blk.add(&out->rms, nc);
    out->storage = blk.commit();
    out->cluster_count = nc;
    auto fill_side = [&](std::vector<std::vector<int32_t>> &s, uint64_t *off, int32_t *idx) {
      off[0] = 0;
      for (uint64_t c = 0; c < nc; ++c) {
        std::copy(s[c].begin(), s[c].end(), idx + off[c]);
        off[c + 1] = off[c] + s[c].size();
      }
    };
    fill_side(sa, out->side_a_offsets, out->side_a);
    fill_side(sb, out->side_b_offsets, out->side_b);
    auto fill_patches = [&](std::vector<std::vector<std::vector<int32_t>>> &p,
                            sym_grouped_csr &dst) {
      dst.groups[0] = 0;
      dst.offsets[0] = 0;
      uint64_t row = 0;
      for (uint64_t c = 0; c < nc; ++c) {
        for (auto &patch : p[c]) {
          std::copy(patch.begin(), patch.end(), dst.indices + dst.offsets[row]);
          dst.offsets[row + 1] = dst.offsets[row] + patch.size();
          ++row;
        }
        dst.groups[c + 1] = row;
      }
      dst.rows = row;
    };
    fill_patches(pa, out->patches_a);
    fill_patches(pb, out->patches_b);
    std::copy(coverage.begin(), coverage.end(), out->coverage);
    std::copy(rms.begin(), rms.end(), out->rms);
  });
}

} // extern "C"
