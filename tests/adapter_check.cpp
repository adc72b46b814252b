// SPDX-License-Identifier: MPL-2.0
// Check program for the reference-side adapter (mitra_algo_gb300/adapter):
// built by tests/test_adapter_cpu.py against the reference's headers and
// libmitra_gb300.so.  Prints one "key value" line per fact the test checks;
// exits non-zero on the first failed expectation.
#include "gb300_backend.h"

#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <stdexcept>
#include <string>

using namespace symmetry;

namespace {

int failures = 0;
void expect(bool ok, const char *what) {
  if (!ok) {
    std::printf("FAIL %s\n", what);
    ++failures;
  }
}

template <class E>
void expect_throw(sym_status status, const std::string &message, const std::string &want) {
  try {
    gb300::throw_status(status, message);
  } catch (const E &e) {
    expect(std::string(e.what()) == want, ("message of status " + std::to_string(int(status))).c_str());
    std::printf("status %d %s\n", int(status), e.what());
    return;
  } catch (...) {
  }
  expect(false, ("exception type of status " + std::to_string(int(status))).c_str());
}

}  // namespace

int main() {
  // layout facts (the static_asserts in the adapter hold them at compile time)
  std::printf("cluster_record_size %zu\n", sizeof(ClusterRecord));
  std::printf("cluster_record_offsets %zu %zu %zu %zu %zu\n", offsetof(ClusterRecord, reflection),
              offsetof(ClusterRecord, rotation), offsetof(ClusterRecord, translation),
              offsetof(ClusterRecord, plane_normal), offsetof(ClusterRecord, plane_offset));
  std::printf("edge_size %zu\n", sizeof(Edge));

  // the engine's state crosses the ABI and comes back unchanged, and the
  // library's engine continues the reference's stream
  std::mt19937_64 engine(42);
  engine.discard(1000);
  sym_rng state = gb300::to_c(engine);
  std::mt19937_64 back;
  gb300::from_c(state, back);
  expect(back == engine, "round trip of the engine state");
  bool same = true;
  for (int i = 0; i < 2000; ++i) same = same && sym_rng_next(&state) == engine();
  expect(same, "library draws continue the engine");
  gb300::from_c(state, back);
  expect(back == engine, "state after library draws");
  sym_rng seeded;
  sym_rng_seed(&seeded, 7);
  std::mt19937_64 seven(7);
  gb300::from_c(seeded, back);
  expect(back == seven, "sym_rng_seed equals std::mt19937_64(seed)");
  std::printf("rng ok %d\n", failures == 0);

  // status -> exception type and message, as the reference throws them
  expect_throw<std::invalid_argument>(SYM_INVALID_ARGUMENT, "SoA component lengths differ",
                                      "SoA component lengths differ");
  expect_throw<std::overflow_error>(SYM_OVERFLOW, "CSR size overflow", "CSR size overflow");
  expect_throw<std::runtime_error>(
      SYM_RUNTIME_ERROR, "Pair budget exceeded; lower --sample-ratio or tighten --pair-threshold",
      "Pair budget exceeded; lower --sample-ratio or tighten --pair-threshold");
  expect_throw<std::runtime_error>(SYM_RUNTIME_ERROR, "Mean-shift support budget exceeded",
                                   "Mean-shift support budget exceeded");
  expect_throw<std::runtime_error>(SYM_CUDA_ERROR, "CUDA: out of memory (workspace)",
                                   "CUDA: out of memory (workspace)");
  expect_throw<std::runtime_error>(SYM_CUDA_ERROR, "launch failed", "CUDA: launch failed");
  expect_throw<std::runtime_error>(SYM_NO_DEVICE, "CUDA: no available device",
                                   "CUDA: no available device");
  expect_throw<std::runtime_error>(SYM_DEVICE_TIMEOUT,
                                   "verification: bounded device loop gave up",
                                   "verification: bounded device loop gave up");

  // sym_metric -> CudaMetric, field by field
  sym_metric m{};
  std::strcpy(m.stage, "mean_shift");
  m.h2d_bytes = 11, m.d2h_bytes = 22, m.peak_buffer_bytes = 33, m.custom_launches = 44;
  m.gpu_interval_ms = 1.5, m.h2d_ms = 2.5, m.d2h_ms = 3.5, m.custom_kernel_ms = 4.5;
  m.all_buffers_released = 1;
  CudaMetric c = gb300::to_cuda_metric(m);
  expect(c.stage == "mean_shift" && c.h2d_bytes == 11 && c.d2h_bytes == 22 &&
             c.peak_buffer_bytes == 33 && c.custom_launches == 44 && c.gpu_interval_ms == 1.5 &&
             c.h2d_ms == 2.5 && c.d2h_ms == 3.5 && c.custom_kernel_ms == 4.5 &&
             c.all_buffers_released,
         "metric fields");
  expect(take_gb300_metrics().empty(), "no metrics recorded without a backend call");

  // the factory: a backend on a device, or the reference's CUDA error
  // without one (the same outcome as make_cuda_backend)
  try {
    std::unique_ptr<Backend> b = make_gb300_backend(true);
    expect(std::string(b->name()) == "gb300", "backend name");
    std::printf("factory device %s\n", b->name());
  } catch (const std::runtime_error &e) {
    expect(std::strncmp(e.what(), "CUDA: ", 6) == 0, "no-device message");
    std::printf("factory no_device %s\n", e.what());
  }
  std::printf("failures %d\n", failures);
  return failures ? 1 : 0;
}
