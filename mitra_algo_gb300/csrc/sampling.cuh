// SPDX-License-Identifier: MPL-2.0
// Area-weighted vertex sampling on the device (sampling.cu) with the host's
// std::mt19937_64 stream and bit-exact sample indices.
#pragma once
#include "common.cuh"

namespace sym {

// The reference's sample_vertices (src/core/sampling.cpp:5-24) over the
// device weights `w` (n entries): one draw of `rng` per positive weight in
// vertex order, key -log(u)/w, the ceil(n * ratio) smallest keys (ties by
// vertex id), ids ascending.  Writes them to `out` (device, room for n) and
// returns their number; `rng` leaves in the state the reference's engine
// has afterwards.  Synchronises the call's stream once.
uint64_t sample_device(Call &call, const double *w, uint64_t n, double ratio, sym_rng &rng,
                       int32_t *out);

}  // namespace sym
