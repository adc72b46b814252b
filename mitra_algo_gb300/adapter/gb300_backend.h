// SPDX-License-Identifier: MPL-2.0
//
// gb300_backend.h - the reference-side adapter of the GB300 library.
//
// Compiled inside the reference project (deoksieze/Mitra_algo), against its
// headers include/symmetry/pipeline.h and include/symmetry/cuda.h, and linked
// with libmitra_gb300.so.  It is a `symmetry::Backend` (pipeline.h:54-69)
// whose six stage methods call the library's C ABI (include/mitra_gb300.h),
// so detect() (src/core/pipeline.cpp:5-52), the CLI's backend switch
// (src/app/main.cpp:122-133) and the reference's stage tests run unchanged
// on the GPU.
#pragma once

#include "mitra_gb300.h"
#include "symmetry/cuda.h"
#include "symmetry/pipeline.h"

#include <memory>
#include <random>
#include <string>
#include <vector>

namespace symmetry {

// The counterpart of make_cuda_backend (include/symmetry/cuda.h:6): a
// backend on CUDA device `device`.  Throws std::runtime_error("CUDA: ...")
// when no device is available, as the reference's factory does.  With
// `profile`, every stage call records a CudaMetric on the calling thread.
std::unique_ptr<Backend> make_gb300_backend(bool profile = false, int device = 0);

// The counterpart of take_cuda_metrics (include/symmetry/cuda.h:15): moves
// out the metrics the gb300 backends recorded on the calling thread.
std::vector<CudaMetric> take_gb300_metrics();

namespace gb300 {

// Rethrows a failed call as the exception the reference throws for the same
// condition: SYM_INVALID_ARGUMENT -> std::invalid_argument, SYM_OVERFLOW ->
// std::overflow_error, everything else (budgets, CUDA errors, timeouts) ->
// std::runtime_error.  `message` is the library's text, which keeps the
// reference's wording ("Pair budget exceeded; ...", "CUDA: ...").
[[noreturn]] void throw_status(sym_status status, const std::string &message);

// sym_metric (the library's per-call record) as the reference's CudaMetric.
CudaMetric to_cuda_metric(const sym_metric &metric);

// std::mt19937_64 <-> the ABI's engine state (the 312 words and the
// position, in the order libstdc++ streams the engine).
sym_rng to_c(const std::mt19937_64 &engine);
void from_c(const sym_rng &state, std::mt19937_64 &engine);

}  // namespace gb300
}  // namespace symmetry
