// SPDX-License-Identifier: MPL-2.0
// Shared host/device infrastructure of the GB300 symmetry library:
// status errors, the per-context stream + workspace, launch helpers, and FP64
// vector helpers that round like the reference's host math
// (src/core/math.cpp of deoksieze/Mitra_algo).  Every translation unit of the
// exact (parity) path is compiled with --fmad=false so a*b+c is two rounded
// operations, as on the reference's x86 build.
#pragma once
#include "../../include/mitra_gb300.h"

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

namespace sym {

// ------------------------------------------------------------------ errors
struct Error : std::runtime_error {
  sym_status status;
  Error(sym_status s, const std::string &m) : std::runtime_error(m), status(s) {}
};
[[noreturn]] inline void fail(sym_status s, const std::string &m) { throw Error(s, m); }
inline void cuda_check(cudaError_t e, const char *what = nullptr) {
  if (e != cudaSuccess)
    fail(SYM_CUDA_ERROR, std::string("CUDA: ") + cudaGetErrorString(e) +
                             (what ? std::string(" (") + what + ")" : ""));
}
#define SYM_CUDA(x) ::sym::cuda_check((x), #x)

// Device-side status word codes (set by kernels, read by the host).
enum DeviceStatus : int {
  DS_OK = 0,
  DS_INDEX_RANGE = 1,    // an index read from the inputs is out of range
  DS_NONFINITE = 2,      // a value that must be finite is not
  DS_EDGE_LOOKUP = 3,    // the (lo, hi) edge table does not match the rings
  DS_CAPACITY = 4,       // a bounded device buffer would overflow
  DS_SPIN_LIMIT = 5,     // a bounded device loop gave up
};

// ---------------------------------------------------------------- context
// Grow-only device workspace.  A call takes bump allocations from it and
// resets it on entry; blocks are only (re)allocated when a call needs more
// than the workspace holds, so steady-state calls make no cudaMalloc.
class Arena {
public:
  ~Arena() { release(); }
  void reset();
  void *take(size_t bytes, size_t align = 256);
  template <class T> T *alloc(size_t n) { return static_cast<T *>(take(n * sizeof(T))); }
  size_t used() const { return used_; }
  size_t peak() const { return peak_; }
  size_t capacity() const;
  void release();
  // Scoped reuse inside one call: allocations made after mark() are given
  // back by rewind() (loops that allocate per iteration).
  struct Mark {
    std::vector<size_t> tops;
    size_t used;
  };
  Mark mark() const {
    Mark m{{}, used_};
    for (auto &b : blocks_) m.tops.push_back(b.top);
    return m;
  }
  void rewind(const Mark &m) {
    for (size_t i = 0; i < blocks_.size(); ++i) blocks_[i].top = i < m.tops.size() ? m.tops[i] : 0;
    used_ = m.used;
  }

private:
  struct Block {
    char *base;
    size_t size, top;
  };
  std::vector<Block> blocks_;
  size_t used_ = 0, peak_ = 0, wanted_ = 0;
};

struct Metrics {
  bool enabled = false;
  std::vector<sym_metric> done;
  sym_metric current{};
  cudaEvent_t begin = nullptr, end = nullptr;
};

}  // namespace sym

// Message of the last failing ABI call on this thread (sym_last_error).
extern thread_local std::string sym_error_text;

struct sym_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  sym::Arena arena;
  int *status = nullptr;        // device status word (pinned-mapped host copy below)
  int *host_status = nullptr;   // pinned host mirror for cheap reads
  sym::Metrics metrics;
  cudaDeviceProp prop{};
  // contexts of the same device this one runs independent per-mesh work on
  // (the fused batch's modes and verification), created on first use
  std::vector<sym_context *> helpers;
};

namespace sym {

// RAII scope of one ABI call: selects the device, resets the workspace and
// the device status word, and records metrics when profiling is on.
class Call {
public:
  Call(sym_context *ctx, const char *stage);
  ~Call();
  sym_context *ctx;
  cudaStream_t stream() const { return ctx->stream; }
  template <class T> T *alloc(size_t n) { return ctx->arena.alloc<T>(n ? n : 1); }
  // Host <-> device copies on the context stream, counted for metrics.
  void h2d(void *dst, const void *src, size_t bytes);
  void d2h(void *dst, const void *src, size_t bytes);
  template <class T> T *upload(const T *src, size_t n) {
    T *d = alloc<T>(n);
    if (n) h2d(d, src, n * sizeof(T));
    return d;
  }
  void launched(int n = 1) { ctx->metrics.current.custom_launches += n; }
  void sync();
  // Synchronises and turns a nonzero device status word into an Error.
  void check_status(const char *stage);
  int *status() const { return ctx->status; }

private:
  const char *stage_;
};

constexpr int kThreads = 256;
inline unsigned blocks_for(uint64_t n, int threads = kThreads) {
  return static_cast<unsigned>((n + threads - 1) / threads);
}
inline void check_launch() { cuda_check(cudaGetLastError(), "kernel launch"); }

// ------------------------------------------------------------- FP64 math
struct D3 {
  double x, y, z;
};
__host__ __device__ inline D3 d3(double x, double y, double z) { return {x, y, z}; }
__host__ __device__ inline D3 operator+(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__host__ __device__ inline D3 operator-(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__host__ __device__ inline D3 operator*(D3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
// Vec / s multiplies by the reciprocal, as the reference's operator/ does.
__host__ __device__ inline D3 div(D3 a, double s) { return a * (1 / s); }
__host__ __device__ inline double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ inline D3 cross(D3 a, D3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__host__ __device__ inline double norm(D3 a) { return sqrt(dot(a, a)); }
__host__ __device__ inline D3 unit(D3 a) {
  double n = norm(a);
  return n > 1e-14 ? div(a, n) : D3{0, 0, 0};
}
__host__ __device__ inline double comp(D3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
struct M3 {
  double m[9];  // row-major
};
__host__ __device__ inline D3 mul(const M3 &r, D3 v) {
  return {r.m[0] * v.x + r.m[1] * v.y + r.m[2] * v.z, r.m[3] * v.x + r.m[4] * v.y + r.m[5] * v.z,
          r.m[6] * v.x + r.m[7] * v.y + r.m[8] * v.z};
}
__host__ __device__ inline M3 transpose(const M3 &r) {
  return {{r.m[0], r.m[3], r.m[6], r.m[1], r.m[4], r.m[7], r.m[2], r.m[5], r.m[8]}};
}
__host__ __device__ inline M3 columns(D3 a, D3 b, D3 c) {
  return {{a.x, b.x, c.x, a.y, b.y, c.y, a.z, b.z, c.z}};
}
__host__ __device__ inline M3 matmul(const M3 &a, const M3 &b) {
  M3 r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0;
      for (int k = 0; k < 3; ++k) s += a.m[i * 3 + k] * b.m[k * 3 + j];
      r.m[i * 3 + j] = s;
    }
  return r;
}
__host__ __device__ inline M3 mirror(D3 n) {
  M3 r;
  double c[3] = {n.x, n.y, n.z};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r.m[i * 3 + j] = (i == j ? 1.0 : 0.0) - 2 * c[i] * c[j];
  return r;
}
__host__ __device__ inline D3 load3(const double *x, const double *y, const double *z, int64_t i) {
  return {x[i], y[i], z[i]};
}

// -------------------------------------------------------- host utilities
// A CSR view must start at 0, never decrease, and index only [0, columns).
inline void validate_csr(const sym_csr_view &c, uint64_t rows, uint64_t columns, const char *what) {
  if (c.rows != rows) fail(SYM_INVALID_ARGUMENT, "SoA component lengths differ");
  if (!c.offsets || c.offsets[0] != 0) fail(SYM_INVALID_ARGUMENT, std::string("Invalid CSR offsets: ") + what);
  for (uint64_t r = 0; r < rows; ++r)
    if (c.offsets[r + 1] < c.offsets[r]) fail(SYM_INVALID_ARGUMENT, std::string("Invalid CSR offsets: ") + what);
  for (uint64_t k = 0; k < c.offsets[rows]; ++k)
    if (c.indices[k] < 0 || uint64_t(c.indices[k]) >= columns)
      fail(SYM_INVALID_ARGUMENT, std::string("CSR index out of range: ") + what);
}
// Copies of the ABI views' columns into one device buffer, lane-major.
double *upload_points(Call &call, const sym_points_view &p);  // 3 x count
int32_t *upload_faces(Call &call, const sym_faces_view &f);   // 3 x count

}  // namespace sym
