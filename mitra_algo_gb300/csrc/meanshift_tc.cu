// SPDX-License-Identifier: MPL-2.0
// BF16 tensor-core mean-shift bulk iterations (tcgen05 + TMEM).
#include "common.cuh"

namespace sym {
bool meanshift_bf16_bulk(Call &, const float *, const float *, uint64_t, uint64_t, float *,
                         uint8_t *, uint64_t, float, int, int *, double *) {
  return false;
}
}  // namespace sym
