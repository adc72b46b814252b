// SPDX-License-Identifier: MPL-2.0
// extern "C" entry points of include/mitra_gb300.h.  Each wraps one stage in
// a Call scope and turns exceptions into a status + per-thread message; no
// exception crosses the boundary.
#include "common.cuh"
#include "rng.hpp"
#include "sampling.cuh"

#include <algorithm>
#include <cstdlib>
#include <new>
#include <vector>

namespace sym {
void curvature_host(Call &, const sym_mesh_view &, const sym_topology_view &, const sym_options &,
                    const sym_features_out &);
void select_device(Call &, const sym_mesh_view &, const sym_features_view &, const double *,
                   uint64_t, const sym_options &, sym_rng *, std::vector<int32_t> &,
                   std::vector<int32_t> &);
void pairing_host(Call &, const sym_mesh_view &, const sym_features_view &, const int32_t *,
                  uint64_t, const sym_model_context &, const sym_options &, std::vector<int32_t> &,
                  std::vector<int32_t> &);
void transformations_host(Call &, const sym_mesh_view &, const sym_features_view &,
                          const sym_pairs_view &, const sym_model_context &, const sym_options &,
                          sym_votes &, void *(*)(size_t));
void clustering_host(Call &, const sym_votes_view &, const sym_model_context &,
                     const sym_options &, sym_rng *, sym_clusters &, void *(*)(size_t));
void verification_host(Call &, const sym_mesh_view &, const sym_topology_view &,
                       const sym_clusters_view &, const sym_model_context &, const sym_options &,
                       sym_verification_result &, void *(*)(size_t));
void triangle_distances_host(Call &, const double *, uint64_t, double *);
void wait_selftest_host(Call &, uint64_t);
uint64_t unite_selftest_host(Call &, int);
}  // namespace sym

// Message of the last failing call on this thread (read by sym_last_error).
thread_local std::string sym_error_text;

namespace {

void *host_alloc(size_t bytes) { return std::malloc(bytes); }

template <class F>
sym_status guarded(F &&f) {
  try {
    f();
    return SYM_OK;
  } catch (const sym::Error &e) {
    sym_error_text = e.what();
    return e.status;
  } catch (const std::bad_alloc &) {
    sym_error_text = "host allocation failed";
    return SYM_RUNTIME_ERROR;
  } catch (const std::exception &e) {
    sym_error_text = e.what();
    return SYM_RUNTIME_ERROR;
  }
}

sym_status null_args() {
  sym_error_text = "null argument";
  return SYM_INVALID_ARGUMENT;
}
}  // namespace

extern "C" {

const char *sym_last_error(void) { return sym_error_text.c_str(); }

const char *sym_backend_name(void) { return "gb300"; }

void *sym_context_stream(sym_context *ctx) { return ctx ? static_cast<void *>(ctx->stream) : nullptr; }

void sym_options_default(sym_options *o) {
  *o = sym_options{0.5, 0.85, 0.15, 0.08, 0.025, 3, 0, 100, 20, 42, 200000, 600000, 1};
}

void sym_rng_seed(sym_rng *r, uint64_t seed) { sym::store_rng(std::mt19937_64(seed), r); }

uint64_t sym_rng_next(sym_rng *r) {
  auto e = sym::load_rng(r);
  uint64_t x = e();
  sym::store_rng(e, r);
  return x;
}

void sym_selection_release(sym_selection *s) {
  if (s) std::free(s->storage), *s = sym_selection{};
}
void sym_pairs_release(sym_pairs *p) {
  if (p) std::free(p->storage), *p = sym_pairs{};
}
void sym_votes_release(sym_votes *v) {
  if (v) std::free(v->storage), *v = sym_votes{};
}
void sym_clusters_release(sym_clusters *c) {
  if (c) std::free(c->storage), *c = sym_clusters{};
}
void sym_verification_release(sym_verification_result *v) {
  if (v) std::free(v->storage), *v = sym_verification_result{};
}

sym_status sym_context_create(int device, sym_context **out) {
  if (!out) return null_args();
  *out = nullptr;
  return guarded([&] {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
      cudaGetLastError();
      sym::fail(SYM_NO_DEVICE, "CUDA: no available device");
    }
    if (device < 0 || device >= count) sym::fail(SYM_INVALID_ARGUMENT, "CUDA: device out of range");
    auto ctx = new sym_context();
    try {
      ctx->device = device;
      SYM_CUDA(cudaSetDevice(device));
      SYM_CUDA(cudaFree(nullptr));  // context initialisation outside stage timings
      SYM_CUDA(cudaGetDeviceProperties(&ctx->prop, device));
      SYM_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
      SYM_CUDA(cudaMalloc(&ctx->status, sizeof(int)));
      SYM_CUDA(cudaMallocHost(&ctx->host_status, sizeof(int)));
      SYM_CUDA(cudaEventCreate(&ctx->metrics.begin));
      SYM_CUDA(cudaEventCreate(&ctx->metrics.end));
    } catch (...) {
      sym_context_destroy(ctx);
      throw;
    }
    *out = ctx;
  });
}

void sym_context_destroy(sym_context *ctx) {
  if (!ctx) return;
  for (sym_context *h : ctx->helpers) sym_context_destroy(h);
  ctx->helpers.clear();
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  ctx->arena.release();
  if (ctx->status) cudaFree(ctx->status);
  if (ctx->host_status) cudaFreeHost(ctx->host_status);
  if (ctx->metrics.begin) cudaEventDestroy(ctx->metrics.begin);
  if (ctx->metrics.end) cudaEventDestroy(ctx->metrics.end);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

sym_status sym_set_profiling(sym_context *ctx, int enabled) {
  if (!ctx) return null_args();
  ctx->metrics.enabled = enabled != 0;
  return SYM_OK;
}

uint64_t sym_take_metrics(sym_context *ctx, sym_metric *out, uint64_t capacity) {
  if (!ctx) return 0;
  uint64_t n = std::min<uint64_t>(capacity, ctx->metrics.done.size());
  for (uint64_t i = 0; i < n; ++i) out[i] = ctx->metrics.done[i];
  ctx->metrics.done.erase(ctx->metrics.done.begin(), ctx->metrics.done.begin() + n);
  return n;
}

sym_status sym_curvature(sym_context *ctx, const sym_mesh_view *mesh,
                         const sym_topology_view *topology, const sym_options *options,
                         const sym_features_out *out) {
  if (!ctx || !mesh || !topology || !options || !out) return null_args();
  return guarded([&] {
    sym::Call call(ctx, "curvature");
    sym::curvature_host(call, *mesh, *topology, *options, *out);
  });
}

sym_status sym_select(sym_context *ctx, const sym_mesh_view *mesh,
                      const sym_features_view *features, const double *weights,
                      uint64_t weight_count, const sym_options *options, sym_rng *rng,
                      sym_selection *out) {
  if (!ctx || !mesh || !features || !options || !rng || !out) return null_args();
  *out = sym_selection{};
  return guarded([&] {
    sym::Call call(ctx, "sample_prune");
    std::vector<int32_t> sample, pruned;
    sym::select_device(call, *mesh, *features, weights, weight_count, *options, rng, sample, pruned);
    size_t bytes = (sample.size() + pruned.size()) * 4 + 64;
    char *block = static_cast<char *>(host_alloc(bytes));
    if (!block) throw std::bad_alloc();
    out->storage = block;
    out->sample = reinterpret_cast<int32_t *>(block);
    out->pruned = out->sample + sample.size();
    out->sample_count = sample.size();
    out->pruned_count = pruned.size();
    std::copy(sample.begin(), sample.end(), out->sample);
    std::copy(pruned.begin(), pruned.end(), out->pruned);
  });
}

sym_status sym_sample_vertices(sym_context *ctx, const double *weights, uint64_t count,
                               double ratio, sym_rng *rng, int32_t *sample,
                               uint64_t *sample_count) {
  if (!ctx || !rng || !sample_count || (count && (!weights || !sample))) return null_args();
  return guarded([&] {
    sym::Call call(ctx, "sample");
    double *w = call.upload(weights, count);
    int32_t *d = call.alloc<int32_t>(count);
    const uint64_t n = sym::sample_device(call, w, count, ratio, *rng, d);
    call.d2h(sample, d, n * sizeof(int32_t));
    call.sync();
    *sample_count = n;
  });
}

sym_status sym_pairing(sym_context *ctx, const sym_mesh_view *mesh,
                       const sym_features_view *features, const int32_t *selected,
                       uint64_t selected_count, const sym_model_context *model,
                       const sym_options *options, sym_pairs *out) {
  if (!ctx || !mesh || !features || !model || !options || !out) return null_args();
  *out = sym_pairs{};
  return guarded([&] {
    sym::Call call(ctx, "pairing");
    std::vector<int32_t> a, b;
    sym::pairing_host(call, *mesh, *features, selected, selected_count, *model, *options, a, b);
    char *block = static_cast<char *>(host_alloc(a.size() * 8 + 64));
    if (!block) throw std::bad_alloc();
    out->storage = block;
    out->a = reinterpret_cast<int32_t *>(block);
    out->b = out->a + a.size();
    out->count = a.size();
    std::copy(a.begin(), a.end(), out->a);
    std::copy(b.begin(), b.end(), out->b);
  });
}

sym_status sym_transformations(sym_context *ctx, const sym_mesh_view *mesh,
                               const sym_features_view *features, const sym_pairs_view *pairs,
                               const sym_model_context *model, const sym_options *options,
                               sym_votes *out) {
  if (!ctx || !mesh || !features || !pairs || !model || !options || !out) return null_args();
  *out = sym_votes{};
  return guarded([&] {
    sym::Call call(ctx, "transformation");
    sym::transformations_host(call, *mesh, *features, *pairs, *model, *options, *out, host_alloc);
  });
}

sym_status sym_clustering(sym_context *ctx, const sym_votes_view *votes,
                          const sym_model_context *model, const sym_options *options,
                          sym_rng *rng, sym_clusters *out) {
  if (!ctx || !votes || !model || !options || !rng || !out) return null_args();
  *out = sym_clusters{};
  return guarded([&] {
    sym::Call call(ctx, "mean_shift");
    sym::clustering_host(call, *votes, *model, *options, rng, *out, host_alloc);
  });
}

sym_status sym_verification(sym_context *ctx, const sym_mesh_view *mesh,
                            const sym_topology_view *topology, const sym_clusters_view *clusters,
                            const sym_model_context *model, const sym_options *options,
                            sym_verification_result *out) {
  if (!ctx || !mesh || !topology || !clusters || !model || !options || !out) return null_args();
  *out = sym_verification_result{};
  return guarded([&] {
    sym::Call call(ctx, "verification");
    sym::verification_host(call, *mesh, *topology, *clusters, *model, *options, *out, host_alloc);
  });
}

sym_status sym_triangle_distances(sym_context *ctx, const double *queries, uint64_t count,
                                  double *out) {
  if (!ctx || (count && (!queries || !out))) return null_args();
  return guarded([&] {
    sym::Call call(ctx, "triangle_distances");
    sym::triangle_distances_host(call, queries, count, out);
  });
}

sym_status sym_wait_selftest(sym_context *ctx, int32_t which, uint64_t limit,
                             uint64_t *components) {
  if (!ctx || (which != 0 && which != 1)) return null_args();
  return guarded([&] {
    sym::Call call(ctx, "wait_selftest");
    if (which == 0) {
      sym::wait_selftest_host(call, limit);
    } else {
      const uint64_t roots =
          sym::unite_selftest_host(call, int(std::min<uint64_t>(limit, uint64_t(1) << 30)));
      if (components) *components = roots;
    }
  });
}

}  // extern "C"
