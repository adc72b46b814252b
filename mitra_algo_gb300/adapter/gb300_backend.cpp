// SPDX-License-Identifier: MPL-2.0
//
// gb300_backend.cpp - symmetry::Backend over the GB300 C ABI.
//
// Every reference view (pipeline.h:51-53: borrowed host memory) is passed to
// the library as plain pointers and counts; every library-owned output is
// copied into the reference's SoA containers (storage.h) and released.  The
// reference's RNG consumption is kept: select() and clustering() hand the
// engine's state to the library and take the advanced state back, so the
// engine continues exactly as after the CPU backend's calls.
#include "gb300_backend.h"

#include <cstddef>
#include <cstring>
#include <sstream>
#include <stdexcept>
#include <type_traits>

namespace symmetry {
namespace {

// The ABI's record and edge types are the reference's, byte for byte, so
// their arrays pass without conversion.
static_assert(sizeof(Edge) == sizeof(sym_edge), "Edge layout");
static_assert(offsetof(Edge, lo) == offsetof(sym_edge, lo) &&
                  offsetof(Edge, hi) == offsetof(sym_edge, hi) &&
                  offsetof(Edge, a) == offsetof(sym_edge, a) &&
                  offsetof(Edge, b) == offsetof(sym_edge, b) &&
                  offsetof(Edge, face0) == offsetof(sym_edge, face0) &&
                  offsetof(Edge, face1) == offsetof(sym_edge, face1),
              "Edge field offsets");
static_assert(std::is_standard_layout<ClusterRecord>::value, "ClusterRecord layout");
static_assert(sizeof(ClusterRecord) == sizeof(sym_cluster_record), "ClusterRecord size");
static_assert(sizeof(bool) == sizeof(uint8_t), "ClusterRecord::reflection is one byte");
static_assert(offsetof(ClusterRecord, reflection) == offsetof(sym_cluster_record, reflection) &&
                  offsetof(ClusterRecord, rotation) == offsetof(sym_cluster_record, rotation) &&
                  offsetof(ClusterRecord, translation) == offsetof(sym_cluster_record, translation) &&
                  offsetof(ClusterRecord, plane_normal) ==
                      offsetof(sym_cluster_record, plane_normal) &&
                  offsetof(ClusterRecord, plane_offset) ==
                      offsetof(sym_cluster_record, plane_offset),
              "ClusterRecord field offsets");
static_assert(sizeof(Vec) == 3 * sizeof(double) && sizeof(Mat) == 9 * sizeof(double),
              "Vec / Mat are plain doubles");
static_assert(sizeof(TransformKind) == sizeof(uint8_t) &&
                  uint8_t(TransformKind::Rigid) == SYM_RIGID &&
                  uint8_t(TransformKind::Reflection) == SYM_REFLECTION,
              "TransformKind values");

void check(sym_status s) {
  if (s != SYM_OK) gb300::throw_status(s, sym_last_error());
}

sym_points_view points(PointsView p) { return {p.x.data, p.y.data, p.z.data, p.size()}; }

sym_mesh_view mesh_of(MeshView m) {
  return {points(m.vertices),
          {m.faces.component[0].data, m.faces.component[1].data, m.faces.component[2].data,
           m.faces.size()}};
}

sym_csr_view csr(CsrView c) { return {c.offsets.data, c.size(), c.indices.data}; }

sym_topology_view topology_of(TopologyView t) {
  return {points(t.normals),
          points(t.face_normals),
          t.weights.data,
          t.weights.size(),
          csr(t.neighbors),
          csr(t.incident_faces),
          reinterpret_cast<const sym_edge *>(t.edges.data),
          t.edges.size()};
}

sym_features_view features_of(FeaturesView f) {
  return {points(f.normal), points(f.dmin), points(f.dmax), f.kmin.data, f.kmax.data,
          f.valid.data,     f.size()};
}

sym_options options_of(const Options &o) {
  sym_options c;
  sym_options_default(&c);
  c.sample_ratio = o.sample_ratio;
  c.prune = o.prune;
  c.pair_threshold = o.pair_threshold;
  c.bandwidth = o.bandwidth;
  c.verify_threshold = o.verify_threshold;
  c.smoothing = o.smoothing;
  c.subdivide = o.subdivide;
  c.max_iterations = o.max_iterations;
  c.max_clusters = o.max_clusters;
  c.seed = o.seed;
  c.max_pairs = o.max_pairs;
  c.max_votes = o.max_votes;
  c.patching = o.patching ? 1 : 0;
  return c;
}

sym_model_context model_of(ModelContext c) {
  return {c.box_size, {c.center.x, c.center.y, c.center.z}};
}

sym_votes_view votes_of(VotesView v) {
  sym_votes_view c{};
  c.pair = v.pairs.data;
  c.kind = reinterpret_cast<const uint8_t *>(v.kind.data);
  for (int k = 0; k < 9; ++k) c.rotation[k] = v.rotation.component[k].data;
  const PointsView *tp[2] = {&v.translation, &v.plane_normal};
  const double **cp[2] = {c.translation, c.plane_normal};
  for (int j = 0; j < 2; ++j)
    cp[j][0] = tp[j]->x.data, cp[j][1] = tp[j]->y.data, cp[j][2] = tp[j]->z.data;
  c.plane_offset = v.plane_offset.data;
  for (int k = 0; k < 12; ++k) c.descriptor[k] = v.descriptor.component[k].data;
  c.count = v.size();
  return c;
}

sym_clusters_view clusters_of(ClustersView c) {
  return {reinterpret_cast<const sym_cluster_record *>(c.records.data), c.size(),
          c.votes.offsets.data, c.votes.indices.data};
}

template <class T>
std::vector<T> copy_of(const T *p, uint64_t n) {
  return n ? std::vector<T>(p, p + n) : std::vector<T>{};
}

Csr csr_of(const uint64_t *offsets, const int32_t *indices, uint64_t rows) {
  Csr r;
  r.offsets = copy_of(offsets, rows + 1);
  r.indices = copy_of(indices, r.offsets.back());
  return r;
}

GroupedCsr grouped_of(const sym_grouped_csr &g, uint64_t groups) {
  GroupedCsr r;
  r.groups = copy_of(g.groups, groups + 1);
  r.rows = csr_of(g.offsets, g.indices, g.rows);
  return r;
}

// Owns a library result and releases it on every exit path.
template <class T, void (*Release)(T *)>
struct Owned {
  T value{};
  ~Owned() { Release(&value); }
};

thread_local std::vector<CudaMetric> recorded_metrics;

class Gb300Backend final : public Backend {
public:
  Gb300Backend(bool profile, int device) : profile_(profile) {
    check(sym_context_create(device, &ctx_));
    if (profile_) {
      sym_status s = sym_set_profiling(ctx_, 1);
      if (s != SYM_OK) {
        sym_context_destroy(ctx_);
        gb300::throw_status(s, sym_last_error());
      }
    }
  }
  ~Gb300Backend() override { sym_context_destroy(ctx_); }
  Gb300Backend(const Gb300Backend &) = delete;
  Gb300Backend &operator=(const Gb300Backend &) = delete;

  const char *name() const noexcept override { return sym_backend_name(); }

  Features curvature(MeshView m, TopologyView t, const Options &o) const override {
    Features f;
    f.resize(m.vertices.size());
    const sym_features_out out{f.normal.x.data(), f.normal.y.data(), f.normal.z.data(),
                               f.dmin.x.data(),   f.dmin.y.data(),   f.dmin.z.data(),
                               f.dmax.x.data(),   f.dmax.y.data(),   f.dmax.z.data(),
                               f.kmin.data(),     f.kmax.data(),     f.valid.data(),
                               f.size()};
    const auto mv = mesh_of(m);
    const auto tv = topology_of(t);
    const auto ov = options_of(o);
    run(sym_curvature(ctx_, &mv, &tv, &ov, &out));
    return f;
  }

  Selection select(MeshView m, FeaturesView f, ArrayView<const Scalar> weights,
                   const Options &o, std::mt19937_64 &random) const override {
    const auto mv = mesh_of(m);
    const auto fv = features_of(f);
    const auto ov = options_of(o);
    sym_rng rng = gb300::to_c(random);
    Owned<sym_selection, sym_selection_release> s;
    run(sym_select(ctx_, &mv, &fv, weights.data, weights.size(), &ov, &rng, &s.value));
    gb300::from_c(rng, random);  // the engine advances exactly as the CPU path's
    return {copy_of(s.value.sample, s.value.sample_count),
            copy_of(s.value.pruned, s.value.pruned_count)};
  }

  Pairs pairing(MeshView m, FeaturesView f, ArrayView<const Index> pruned, ModelContext c,
                const Options &o) const override {
    const auto mv = mesh_of(m);
    const auto fv = features_of(f);
    const auto ov = options_of(o);
    const auto cv = model_of(c);
    Owned<sym_pairs, sym_pairs_release> p;
    run(sym_pairing(ctx_, &mv, &fv, pruned.data, pruned.size(), &cv, &ov, &p.value));
    Pairs out;
    out.a = copy_of(p.value.a, p.value.count);
    out.b = copy_of(p.value.b, p.value.count);
    return out;
  }

  Votes transformations(MeshView m, FeaturesView f, PairsView pairs, ModelContext c,
                        const Options &o) const override {
    const auto mv = mesh_of(m);
    const auto fv = features_of(f);
    const auto ov = options_of(o);
    const auto cv = model_of(c);
    const sym_pairs_view pv{pairs.a.data, pairs.b.data, pairs.size()};
    Owned<sym_votes, sym_votes_release> v;
    run(sym_transformations(ctx_, &mv, &fv, &pv, &cv, &ov, &v.value));
    const uint64_t n = v.value.count;
    Votes out;
    out.pairs = copy_of(v.value.pair, n);
    out.kind.resize(n);
    for (uint64_t i = 0; i < n; ++i) out.kind[i] = TransformKind(v.value.kind[i]);
    for (int k = 0; k < 9; ++k) out.rotation.component[k] = copy_of(v.value.rotation[k], n);
    Points *pts[2] = {&out.translation, &out.plane_normal};
    double *const *src[2] = {v.value.translation, v.value.plane_normal};
    for (int j = 0; j < 2; ++j) {
      pts[j]->x = copy_of(src[j][0], n);
      pts[j]->y = copy_of(src[j][1], n);
      pts[j]->z = copy_of(src[j][2], n);
    }
    out.plane_offset = copy_of(v.value.plane_offset, n);
    for (int k = 0; k < 12; ++k) out.descriptor.component[k] = copy_of(v.value.descriptor[k], n);
    return out;
  }

  ClusterOutput clustering(VotesView votes, ModelContext c, const Options &o,
                           std::mt19937_64 &random) const override {
    const auto vv = votes_of(votes);
    const auto cv = model_of(c);
    const auto ov = options_of(o);
    sym_rng rng = gb300::to_c(random);
    Owned<sym_clusters, sym_clusters_release> cl;
    run(sym_clustering(ctx_, &vv, &cv, &ov, &rng, &cl.value));
    gb300::from_c(rng, random);
    const uint64_t n = cl.value.count;
    ClusterOutput out;
    out.clusters.records.resize(n);
    for (uint64_t i = 0; i < n; ++i)
      std::memcpy(static_cast<void *>(&out.clusters.records[i]), &cl.value.records[i],
                  sizeof(ClusterRecord));
    out.clusters.votes = csr_of(cl.value.vote_offsets, cl.value.vote_indices, n);
    out.limited_iterations = cl.value.limited_iterations;
    return out;
  }

  Verification verification(MeshView m, TopologyView t, ClustersView clusters, ModelContext c,
                            const Options &o) const override {
    const auto mv = mesh_of(m);
    const auto tv = topology_of(t);
    const auto kv = clusters_of(clusters);
    const auto cv = model_of(c);
    const auto ov = options_of(o);
    Owned<sym_verification_result, sym_verification_release> r;
    run(sym_verification(ctx_, &mv, &tv, &kv, &cv, &ov, &r.value));
    const uint64_t n = r.value.cluster_count;
    Verification out;
    out.side_a = csr_of(r.value.side_a_offsets, r.value.side_a, n);
    out.side_b = csr_of(r.value.side_b_offsets, r.value.side_b, n);
    out.patches_a = grouped_of(r.value.patches_a, n);
    out.patches_b = grouped_of(r.value.patches_b, n);
    out.coverage = copy_of(r.value.coverage, n);
    out.rms = copy_of(r.value.rms, n);
    return out;
  }

private:
  // Raises a failed call; with profiling, moves the call's metric to the
  // calling thread's list first (the reference records failed stages too).
  void run(sym_status s) const {
    if (profile_) {
      sym_metric m[8];
      uint64_t got;
      while ((got = sym_take_metrics(ctx_, m, 8)) > 0)
        for (uint64_t i = 0; i < got; ++i) recorded_metrics.push_back(gb300::to_cuda_metric(m[i]));
    }
    check(s);
  }

  sym_context *ctx_ = nullptr;
  bool profile_ = false;
};

}  // namespace

namespace gb300 {

[[noreturn]] void throw_status(sym_status status, const std::string &message) {
  std::string m = message.empty() ? "gb300 backend: status " + std::to_string(int(status)) : message;
  switch (status) {
    case SYM_INVALID_ARGUMENT: throw std::invalid_argument(m);
    case SYM_OVERFLOW: throw std::overflow_error(m);
    case SYM_CUDA_ERROR:
    case SYM_NO_DEVICE:
      if (m.compare(0, 6, "CUDA: ") != 0) m = "CUDA: " + m;
      throw std::runtime_error(m);
    default: throw std::runtime_error(m);
  }
}

CudaMetric to_cuda_metric(const sym_metric &m) {
  CudaMetric c;
  c.stage.assign(m.stage, strnlen(m.stage, sizeof(m.stage)));
  c.h2d_bytes = m.h2d_bytes;
  c.d2h_bytes = m.d2h_bytes;
  c.peak_buffer_bytes = m.peak_buffer_bytes;
  c.custom_launches = m.custom_launches;
  c.gpu_interval_ms = m.gpu_interval_ms;
  c.h2d_ms = m.h2d_ms;
  c.d2h_ms = m.d2h_ms;
  c.custom_kernel_ms = m.custom_kernel_ms;
  c.all_buffers_released = m.all_buffers_released != 0;
  return c;
}

sym_rng to_c(const std::mt19937_64 &engine) {
  std::stringstream s;
  s << engine;
  sym_rng r{};
  for (auto &w : r.words) s >> w;
  s >> r.index;
  if (!s) throw std::runtime_error("gb300 backend: unexpected std::mt19937_64 stream format");
  return r;
}

void from_c(const sym_rng &state, std::mt19937_64 &engine) {
  std::stringstream s;
  for (auto w : state.words) s << w << ' ';
  s << state.index;
  s >> engine;
  if (!s) throw std::runtime_error("gb300 backend: engine state rejected");
}

}  // namespace gb300

std::unique_ptr<Backend> make_gb300_backend(bool profile, int device) {
  return std::make_unique<Gb300Backend>(profile, device);
}

std::vector<CudaMetric> take_gb300_metrics() {
  std::vector<CudaMetric> out;
  out.swap(recorded_metrics);
  return out;
}

}  // namespace symmetry
