// SPDX-License-Identifier: MPL-2.0
// std::mt19937_64 <-> sym_rng (the 312 words and position libstdc++ streams)
// and the host-side area-weighted sampling of the reference
// (src/core/sampling.cpp:5-24), whose indices are an input to the GPU prune.
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

// Weighted sampling without replacement with exponential keys -log(u)/w,
// u = (draw >> 11 + 0.5) / 2^53, smallest keys first, ids returned sorted.
inline std::vector<int32_t> sample_vertices(const double *w, uint64_t n, double ratio,
                                            std::mt19937_64 &rng) {
  std::vector<std::pair<double, int>> keys;
  keys.reserve(n);
  for (uint64_t i = 0; i < n; ++i)
    if (w[i] > 0) {
      double u = (static_cast<double>(rng() >> 11) + 0.5) / 9007199254740992.0;
      keys.push_back({-std::log(u) / w[i], static_cast<int>(i)});
    }
  size_t target = std::min(keys.size(), static_cast<size_t>(std::ceil(n * ratio)));
  std::partial_sort(keys.begin(), keys.begin() + target, keys.end());
  std::vector<int32_t> s(target);
  for (size_t i = 0; i < target; ++i) s[i] = keys[i].second;
  std::sort(s.begin(), s.end());
  return s;
}

}  // namespace sym
