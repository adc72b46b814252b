// SPDX-License-Identifier: MPL-2.0
// Context, workspace arena, call scope and metrics.
#include "common.cuh"

#include <algorithm>
#include <chrono>

namespace sym {

void Arena::release() {
  for (auto &b : blocks_) cudaFree(b.base);
  blocks_.clear();
}

size_t Arena::capacity() const {
  size_t c = 0;
  for (auto &b : blocks_) c += b.size;
  return c;
}

void Arena::reset() {
  // Consolidate into one block sized for the largest call seen so far, so
  // later calls of that size are served without allocating.
  if (blocks_.size() > 1 || (blocks_.size() == 1 && blocks_[0].size < wanted_)) {
    size_t want = std::max(wanted_, capacity());
    release();
    char *p = nullptr;
    cuda_check(cudaMalloc(&p, want), "workspace");
    blocks_.push_back({p, want, 0});
  }
  for (auto &b : blocks_) b.top = 0;
  used_ = 0;
}

void *Arena::take(size_t bytes, size_t align) {
  for (auto &b : blocks_) {
    size_t at = (b.top + align - 1) / align * align;
    if (at + bytes <= b.size) {
      b.top = at + bytes;
      used_ += bytes;
      peak_ = std::max(peak_, used_);
      wanted_ = std::max(wanted_, used_ + 4096);
      return b.base + at;
    }
  }
  size_t grow = std::max<size_t>(bytes + align, std::max<size_t>(capacity(), 64u << 20));
  char *p = nullptr;
  cuda_check(cudaMalloc(&p, grow), "workspace");
  blocks_.push_back({p, grow, bytes});
  used_ += bytes;
  peak_ = std::max(peak_, used_);
  wanted_ = std::max(wanted_, used_ + 4096);
  return p;
}

Call::Call(sym_context *c, const char *stage) : ctx(c), stage_(stage) {
  cuda_check(cudaSetDevice(ctx->device), "cudaSetDevice");
  ctx->arena.reset();
  *ctx->host_status = 0;
  cuda_check(cudaMemsetAsync(ctx->status, 0, sizeof(int), ctx->stream), "status reset");
  ctx->metrics.current = sym_metric{};
  std::strncpy(ctx->metrics.current.stage, stage, sizeof(ctx->metrics.current.stage) - 1);
  if (ctx->metrics.enabled) cudaEventRecord(ctx->metrics.begin, ctx->stream);
}

Call::~Call() {
  if (ctx->metrics.enabled) {
    auto &m = ctx->metrics;
    cudaEventRecord(m.end, ctx->stream);
    if (cudaEventSynchronize(m.end) == cudaSuccess) {
      float ms = 0;
      cudaEventElapsedTime(&ms, m.begin, m.end);
      m.current.gpu_interval_ms = ms;
    }
    m.current.peak_buffer_bytes = ctx->arena.peak();
    m.current.all_buffers_released = 1;  // workspace is reset, never leaked
    m.done.push_back(m.current);
  }
}

void Call::h2d(void *dst, const void *src, size_t bytes) {
  if (!bytes) return;
  cuda_check(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream), "H2D");
  ctx->metrics.current.h2d_bytes += bytes;
}

void Call::d2h(void *dst, const void *src, size_t bytes) {
  if (!bytes) return;
  cuda_check(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
  ctx->metrics.current.d2h_bytes += bytes;
}

void Call::sync() { cuda_check(cudaStreamSynchronize(ctx->stream), "stream sync"); }

void Call::check_status(const char *stage) {
  cuda_check(cudaMemcpyAsync(ctx->host_status, ctx->status, sizeof(int), cudaMemcpyDeviceToHost,
                             ctx->stream),
             "status read");
  sync();
  int s = *ctx->host_status;
  if (s == DS_OK) return;
  std::string where = std::string(stage) + ": ";
  switch (s) {
    case DS_INDEX_RANGE: fail(SYM_INVALID_ARGUMENT, where + "index out of range");
    case DS_NONFINITE: fail(SYM_INVALID_ARGUMENT, where + "non-finite input");
    case DS_EDGE_LOOKUP: fail(SYM_INVALID_ARGUMENT, where + "edge table does not match neighbours");
    case DS_CAPACITY: fail(SYM_RUNTIME_ERROR, where + "device buffer capacity exceeded");
    case DS_SPIN_LIMIT: fail(SYM_DEVICE_TIMEOUT, where + "bounded device loop gave up");
    default: fail(SYM_RUNTIME_ERROR, where + "device status " + std::to_string(s));
  }
}

double *upload_points(Call &call, const sym_points_view &p) {
  double *d = call.alloc<double>(3 * p.count);
  call.h2d(d, p.x, p.count * 8);
  call.h2d(d + p.count, p.y, p.count * 8);
  call.h2d(d + 2 * p.count, p.z, p.count * 8);
  return d;
}

int32_t *upload_faces(Call &call, const sym_faces_view &f) {
  int32_t *d = call.alloc<int32_t>(3 * f.count);
  call.h2d(d, f.v0, f.count * 4);
  call.h2d(d + f.count, f.v1, f.count * 4);
  call.h2d(d + 2 * f.count, f.v2, f.count * 4);
  return d;
}

}  // namespace sym
