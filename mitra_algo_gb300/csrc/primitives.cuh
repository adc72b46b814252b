// SPDX-License-Identifier: MPL-2.0
// Device-wide primitives: exclusive scan, stable LSD radix sort of
// (uint64 key, int32 value) pairs, stable compaction.  All are deterministic
// and allocate only from the call's workspace.
#pragma once
#include "common.cuh"

namespace sym {

// out[i] = sum(in[0..i)), out[n] = total.  `out` holds n + 1 entries and may
// alias `in` only if in == out is not required: in and out must differ.
void exclusive_scan(Call &call, const uint64_t *in, uint64_t *out, uint64_t n);

// Stable sort of `keys`/`values` by the low `key_bits` bits of the keys
// (8-bit digits).  Results land in keys_out/values_out.
void radix_sort_pairs(Call &call, const uint64_t *keys, const int32_t *values,
                      uint64_t *keys_out, int32_t *values_out, uint64_t n, int key_bits = 64);

// Writes the indices i (ascending) with flags[i] != 0 to `out`
// (capacity n) and their number to *count (device).
void compact_indices(Call &call, const uint8_t *flags, uint64_t n, int32_t *out,
                     uint64_t *count);

// Writes values[i] for flags[i] != 0, in order, to `out`; count to *count.
void compact_values(Call &call, const uint8_t *flags, const int32_t *values, uint64_t n,
                    int32_t *out, uint64_t *count);

// Order-preserving map of a finite double to uint64 (-0 and +0 coincide).
__host__ __device__ inline uint64_t orderable_key(double v) {
  if (v == 0) v = 0.0;  // canonical +0
  uint64_t b;
  memcpy(&b, &v, 8);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

}  // namespace sym
