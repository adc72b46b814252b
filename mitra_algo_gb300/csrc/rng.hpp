// SPDX-License-Identifier: MPL-2.0
// std::mt19937_64 <-> sym_rng (the 312 words and position libstdc++ streams).
#pragma once
#include "../../include/mitra_gb300.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <random>
#include <sstream>
#include <utility>
#include <vector>

namespace sym {

inline std::mt19937_64 load_rng(const sym_rng *r) {
  std::stringstream s;
  for (int i = 0; i < 312; ++i) s << r->words[i] << ' ';
  s << r->index;
  std::mt19937_64 e;
  s >> e;
  return e;
}

inline void store_rng(const std::mt19937_64 &e, sym_rng *r) {
  std::stringstream s;
  s << e;
  for (int i = 0; i < 312; ++i) s >> r->words[i];
  s >> r->index;
}

}  // namespace sym
