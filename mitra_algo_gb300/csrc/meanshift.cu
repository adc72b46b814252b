// SPDX-License-Identifier: MPL-2.0
// Stage (c): mean-shift clustering in transformation space, reference
// semantics (Epanechnikov weights, 4-D reflection / 12-D rigid descriptors,
// random seeding until every vote is visited).
//
// Reference: src/cpu/clustering.cpp:32-208 (driver + evaluator),
// src/cuda/clustering.cu (the existing GPU path: one block per trajectory,
// launched thousands of times from the host driver).
//
// GB300 design.  A trajectory is a pure function of its seed vote (the
// reference evaluator only reads the seed descriptor and the vote set), so:
//   1. one launch runs the trajectory of EVERY vote as a seed, a warp per
//      seed, and records its final mean, its converged/exhausted flags and
//      its support as a bitmask over same-kind votes;
//   2. the host replays the reference's host loop verbatim (RNG draw per seed,
//      visited set, merge test, budgets) on those results - no device round
//      trip per trajectory;
//   3. one launch re-runs only the trajectories the host loop used and adds
//      each member's per-iteration hit into its cluster's support counts;
//      one launch picks each vote's winning cluster (largest count, first
//      cluster on ties).
// Distances, weights and products are the reference's FP64 expressions (no
// FMA contraction), and the weighted sums add the members' contributions in
// vote order, as the reference's serial loop does: each lane evaluates one
// vote of a group of 32, then every lane adds the members' shuffled weights
// and products in lane order.  The means are therefore the reference's bit
// for bit, and so is every decision that depends on them (d^2 < h^2, the
// stop test, the merge test): no rounding band exists to be checked.
// Memory: seeds run in batches whose support bitmasks fit a fixed device
// budget (the supports go to the host as sparse member lists), and the
// members' hit counts are accumulated over batches of clusters.
#include "common.cuh"
#include "primitives.cuh"
#include "rng.hpp"

#include <algorithm>
#include <cmath>
#include <unordered_map>
#include <vector>

namespace sym {
namespace {

constexpr double kExhausted = 1e-14;  // clustering.cpp:15,169

__global__ void split_kinds(const uint8_t *kind, uint64_t q, uint8_t *is_refl, uint8_t *is_rigid) {
  uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= q) return;
  is_refl[i] = kind[i] == SYM_REFLECTION;
  is_rigid[i] = kind[i] != SYM_REFLECTION;
}

// AoS descriptors of one kind: out[j*D + k] = lanes[k][ids[j]].
template <int D>
__global__ void gather_desc(const double *lanes, uint64_t q, const int32_t *ids, uint64_t n,
                            double *out) {
  uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (j >= n) return;
  int32_t v = ids[j];
  for (int k = 0; k < D; ++k) out[j * D + k] = lanes[uint64_t(k) * q + v];
}

__global__ void round_desc(const double *desc, uint64_t n, float *out) {
  uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) out[i] = float(desc[i]);
}

template <int D>
struct Traj {
  double mean[D];
  bool converged, exhausted;
};

// One trajectory per warp.  RECORD: write the support bitmask row; else add
// every member hit to counts[cluster * n + j].
//
// Culling: `desc32` holds the descriptors rounded to FP32 and `reach` the
// bandwidth plus a bound on how far an FP32 distance can fall below the FP64
// one (the rounding of the mean and of every coordinate, D times 2^-22 of the
// largest coordinate magnitude, and of the FP32 arithmetic).  A vote whose
// FP32 squared distance exceeds reach^2 lies outside the bandwidth in FP64
// as well; only the others take the reference's FP64 test.
template <int D, bool RECORD>
__global__ void __launch_bounds__(128) trajectories(const double *desc, const float *desc32,
                                                    float reach, uint64_t n,
                                                    const int32_t *seeds, const int32_t *cluster,
                                                    uint64_t nseeds, double h2, int max_iter,
                                                    double *final_mean, uint8_t *flags,
                                                    uint32_t *support, uint64_t words,
                                                    uint32_t *counts) {
  uint64_t si = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (si >= nseeds) return;
  int32_t s = seeds[si];
  uint64_t crow = RECORD ? 0 : uint64_t(cluster[si]) * n;
  double mean[D];
  for (int k = 0; k < D; ++k) mean[k] = desc[uint64_t(s) * D + k];
  bool converged = false, exhausted = false;
  const double stop = 1e-6 * h2;
  for (int it = 0; it < max_iter; ++it) {
    double wt = 0, ws[D];  // the same values in every lane
    for (int k = 0; k < D; ++k) ws[k] = 0;
    float mean32[D];
    for (int k = 0; k < D; ++k) mean32[k] = float(mean[k]);
    const float reach2 = reach * reach;
    for (uint64_t base = 0; base < n; base += 32) {
      uint64_t j = base + lane;
      bool in = false;
      double w = 0, x[D];
      for (int k = 0; k < D; ++k) x[k] = 0;
      bool near = false;
      if (j < n) {
        float d32 = 0;
        for (int k = 0; k < D; ++k) {
          const float e = mean32[k] - desc32[j * D + k];
          d32 += e * e;
        }
        near = !(d32 > reach2);
      }
      if (near) {
        double dist = 0;
        for (int k = 0; k < D; ++k) {
          x[k] = desc[j * D + k];
          double d = mean[k] - x[k];
          dist += d * d;
        }
        if (dist < h2) {
          in = true;
          w = 1 - dist / h2;
        }
      }
      const unsigned bits = __ballot_sync(0xffffffffu, in);
      // the members of this group in vote order: weight, then w * x
      for (unsigned m = bits; m; m &= m - 1) {
        const int src = __ffs(int(m)) - 1;
        wt += __shfl_sync(0xffffffffu, w, src);
        for (int k = 0; k < D; ++k) ws[k] += __shfl_sync(0xffffffffu, w * x[k], src);
      }
      if (RECORD) {
        if (lane == 0 && bits) support[si * words + base / 32] |= bits;
      } else if (in) {
        atomicAdd(&counts[crow + j], 1u);
      }
    }
    if (wt <= kExhausted) {
      exhausted = true;
      break;
    }
    double movement = 0;
    for (int k = 0; k < D; ++k) {
      double next = ws[k] / wt;
      double d = mean[k] - next;
      movement += d * d;
      mean[k] = next;
    }
    if (movement < stop) {
      converged = true;
      break;
    }
  }
  if (RECORD && lane == 0) {
    for (int k = 0; k < D; ++k) final_mean[si * D + k] = mean[k];
    flags[si] = uint8_t((converged ? 1 : 0) | (exhausted ? 2 : 0));
  }
}

// Winner per vote over one batch of clusters (in creation order): the
// cluster with the largest count so far, the earliest one on ties (a later
// cluster must count strictly more); best/winner carry over batches.
__global__ void winners(const uint32_t *counts, uint64_t nclusters, uint64_t n,
                        const int32_t *cluster_id, uint32_t *best, int32_t *winner) {
  uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (j >= n) return;
  uint32_t b = best[j];
  int32_t w = winner[j];
  for (uint64_t c = 0; c < nclusters; ++c) {
    uint32_t v = counts[c * n + j];
    if (v > b) b = v, w = cluster_id[c];
  }
  best[j] = b, winner[j] = w;
}

// Device bytes for one batch of seeds' support bitmasks, and for one batch
// of clusters' hit counts.
constexpr uint64_t kBatchBytes = uint64_t(1) << 30;

struct KindData {
  int dim = 0;
  uint64_t n = 0, words = 0;
  std::vector<int32_t> ids;          // global vote id of each local index
  double *desc = nullptr;            // device AoS
  float *desc32 = nullptr;           // the same rounded to FP32
  float reach = 0;                   // the culling radius (trajectories)
  std::vector<double> mean;          // n x dim final means
  std::vector<uint8_t> flags;        // bit0 converged, bit1 exhausted
  std::vector<uint64_t> sup_off;     // n + 1: each seed's support (kind-local
  std::vector<uint32_t> sup_idx;     //   member ids, ascending)
};

template <int D>
void run_all_seeds(Call &call, KindData &k, double h2, int max_iter) {
  if (!k.n) return;
  cudaStream_t st = call.stream();
  k.words = (k.n + 31) / 32;
  const uint64_t batch = std::max<uint64_t>(1, std::min<uint64_t>(k.n, kBatchBytes / (k.words * 4)));
  int32_t *seeds = call.alloc<int32_t>(batch);
  double *mean = call.alloc<double>(batch * D);
  uint8_t *flags = call.alloc<uint8_t>(batch);
  uint32_t *support = call.alloc<uint32_t>(batch * k.words);
  k.mean.resize(k.n * D);
  k.flags.resize(k.n);
  k.sup_off.assign(1, 0);
  k.sup_idx.clear();
  std::vector<int32_t> iota(batch);
  std::vector<uint32_t> rows(batch * k.words);
  for (uint64_t first = 0; first < k.n; first += batch) {
    const uint64_t cnt = std::min(batch, k.n - first);
    for (uint64_t i = 0; i < cnt; ++i) iota[i] = int32_t(first + i);
    call.h2d(seeds, iota.data(), cnt * 4);
    SYM_CUDA(cudaMemsetAsync(support, 0, cnt * k.words * 4, st));
    const unsigned blocks = unsigned((cnt * 32 + 127) / 128);
    trajectories<D, true><<<blocks, 128, 0, st>>>(k.desc, k.desc32, k.reach, k.n, seeds, nullptr,
                                                  cnt, h2, max_iter,
                                                  mean, flags, support, k.words, nullptr);
    check_launch();
    call.launched();
    call.d2h(k.mean.data() + first * D, mean, cnt * D * 8);
    call.d2h(k.flags.data() + first, flags, cnt);
    call.d2h(rows.data(), support, cnt * k.words * 4);
    call.sync();
    for (uint64_t i = 0; i < cnt; ++i) {
      const uint32_t *row = &rows[i * k.words];
      for (uint64_t w = 0; w < k.words; ++w)
        for (uint32_t m = row[w]; m; m &= m - 1)
          k.sup_idx.push_back(uint32_t(w * 32 + __builtin_ctz(m)));
      k.sup_off.push_back(k.sup_idx.size());
    }
  }
}

struct Center {
  double v[12];
  int kind;                    // index into kinds[]
  std::vector<uint64_t> keys;  // union of supports, kind-local bitmask
  uint64_t key_count = 0;
  std::vector<int32_t> seeds;  // kind-local seeds merged into this cluster
};

template <int D>
void count_members(Call &call, KindData &k, const std::vector<Center> &centers, int kind_index,
                   double h2, int max_iter, std::vector<int32_t> &winner_global) {
  std::vector<int32_t> cluster_ids;
  for (size_t c = 0; c < centers.size(); ++c)
    if (centers[c].kind == kind_index) cluster_ids.push_back(int32_t(c));
  if (cluster_ids.empty()) return;
  cudaStream_t st = call.stream();
  const uint64_t batch = std::max<uint64_t>(1, std::min<uint64_t>(cluster_ids.size(),
                                                                   kBatchBytes / (k.n * 4)));
  uint32_t *counts = call.alloc<uint32_t>(batch * k.n);
  uint32_t *best = call.alloc<uint32_t>(k.n);
  int32_t *win = call.alloc<int32_t>(k.n);
  SYM_CUDA(cudaMemsetAsync(best, 0, k.n * 4, st));
  SYM_CUDA(cudaMemsetAsync(win, 0xff, k.n * 4, st));  // -1: no cluster counted the vote
  for (uint64_t first = 0; first < cluster_ids.size(); first += batch) {
    const uint64_t nc = std::min<uint64_t>(batch, cluster_ids.size() - first);
    std::vector<int32_t> seeds, cluster;
    for (uint64_t c = 0; c < nc; ++c)
      for (int32_t s : centers[cluster_ids[first + c]].seeds)
        seeds.push_back(s), cluster.push_back(int32_t(c));
    SYM_CUDA(cudaMemsetAsync(counts, 0, nc * k.n * 4, st));
    int32_t *dseeds = call.upload(seeds.data(), seeds.size());
    int32_t *dcluster = call.upload(cluster.data(), cluster.size());
    int32_t *dids = call.upload(cluster_ids.data() + first, nc);
    const unsigned blocks = unsigned((seeds.size() * 32 + 127) / 128);
    trajectories<D, false><<<blocks, 128, 0, st>>>(k.desc, k.desc32, k.reach, k.n, dseeds,
                                                   dcluster, seeds.size(), h2,
                                                   max_iter, nullptr, nullptr, nullptr, 0, counts);
    check_launch();
    winners<<<blocks_for(k.n), kThreads, 0, st>>>(counts, nc, k.n, dids, best, win);
    check_launch();
    call.launched(2);
  }
  std::vector<int32_t> local(k.n);
  call.d2h(local.data(), win, k.n * 4);
  call.sync();
  for (uint64_t j = 0; j < k.n; ++j) winner_global[k.ids[j]] = local[j];
}

// Index of the centers for the merge test (clustering.cpp:68-73: the first
// center, in creation order, of the same kind within h/2).  A center within
// h/2 lies within h/2 in every coordinate, so on three coordinates it falls
// in one of the 27 cells of pitch slightly above h/2 around the mean; the
// lowest-numbered center among those that pass the reference's test is the
// reference's choice.  Centers with coordinates too large for the grid stay
// in a list that every query scans.
class CenterGrid {
public:
  CenterGrid(double h, const int dims[3]) : scale_(2.0 / h * (1 - 1e-9)) {
    for (int i = 0; i < 3; ++i) dims_[i] = dims[i];
  }
  void insert(int32_t id, const double *v) {
    uint64_t key;
    if (cell(v, 0, 0, 0, key)) map_[key].push_back(id);
    else loose_.push_back(id);
  }
  void erase(int32_t id, const double *v) {
    uint64_t key;
    std::vector<int32_t> &list = cell(v, 0, 0, 0, key) ? map_[key] : loose_;
    list.erase(std::find(list.begin(), list.end(), id));
  }
  template <class Test>
  int32_t first(const double *v, Test &&passes) const {
    int32_t best = -1;
    auto scan = [&](const std::vector<int32_t> &list) {
      for (int32_t id : list)
        if ((best < 0 || id < best) && passes(id)) best = id;
    };
    scan(loose_);
    uint64_t key;
    for (int a = -1; a <= 1; ++a)
      for (int b = -1; b <= 1; ++b)
        for (int c = -1; c <= 1; ++c)
          if (cell(v, a, b, c, key)) {
            auto it = map_.find(key);
            if (it != map_.end()) scan(it->second);
          }
    return best;
  }

private:
  bool cell(const double *v, int a, int b, int c, uint64_t &key) const {
    const int off[3] = {a, b, c};
    key = 0;
    for (int i = 0; i < 3; ++i) {
      const double x = std::floor(v[dims_[i]] * scale_);
      if (!(std::fabs(x) < double(1 << 20))) return false;
      key = (key << 21) | uint64_t(int64_t(x) + off[i] + (1 << 20));
    }
    return true;
  }
  double scale_;
  int dims_[3];
  std::unordered_map<uint64_t, std::vector<int32_t>> map_;
  std::vector<int32_t> loose_;
};

double desc_d2(const double *a, const double *b, int dim) {
  double s = 0;
  for (int i = 0; i < dim; ++i) {
    double d = a[i] - b[i];
    s += d * d;
  }
  return s;
}

}  // namespace

void clustering_host(Call &call, const sym_votes_view &votes, const sym_model_context &ctx,
                     const sym_options &o, sym_rng *rng, sym_clusters &out,
                     void *(*allocate)(size_t)) {
  const uint64_t q = votes.count;
  const double h = o.bandwidth, h2 = h * h;
  if (o.max_iterations < 1) fail(SYM_INVALID_ARGUMENT, "Invalid parameter range; see --help");
  KindData kinds[2];  // 0: reflection (4-D), 1: rigid (12-D)
  kinds[0].dim = 4, kinds[1].dim = 12;
  std::vector<uint8_t> kind_of(q);
  std::vector<int32_t> local_of(q);
  for (uint64_t i = 0; i < q; ++i) {
    int k = votes.kind[i] == SYM_REFLECTION ? 0 : 1;
    kind_of[i] = uint8_t(k);
    local_of[i] = int32_t(kinds[k].ids.size());
    kinds[k].ids.push_back(int32_t(i));
  }
  for (auto &k : kinds) k.n = k.ids.size();
  if (q) {
    double *lanes = call.alloc<double>(12 * q);
    for (int k = 0; k < 12; ++k) call.h2d(lanes + uint64_t(k) * q, votes.descriptor[k], q * 8);
    for (int t = 0; t < 2; ++t) {
      KindData &k = kinds[t];
      if (!k.n) continue;
      int32_t *ids = call.upload(k.ids.data(), k.n);
      k.desc = call.alloc<double>(k.n * k.dim);
      if (k.dim == 4)
        gather_desc<4><<<blocks_for(k.n), kThreads, 0, call.stream()>>>(lanes, q, ids, k.n, k.desc);
      else
        gather_desc<12><<<blocks_for(k.n), kThreads, 0, call.stream()>>>(lanes, q, ids, k.n, k.desc);
      check_launch();
      k.desc32 = call.alloc<float>(k.n * k.dim);
      round_desc<<<blocks_for(k.n * k.dim), kThreads, 0, call.stream()>>>(k.desc, k.n * k.dim,
                                                                         k.desc32);
      check_launch();
      call.launched(2);
      // the culling radius: h plus the FP32 shortfall of a distance (rounding
      // of mean and coordinates, 2^-24 of the largest magnitude each, and of
      // the FP32 sums), each term taken 4 times over
      double mag = 0;
      for (uint64_t j = 0; j < k.n; ++j)
        for (int c = 0; c < k.dim; ++c) mag = std::max(mag, std::fabs(votes.descriptor[c][k.ids[j]]));
      const double reach = h + k.dim * std::ldexp(mag, -22) + (k.dim + 2) * std::ldexp(h, -22);
      k.reach = std::isfinite(mag) && mag < 1e15 ? float(reach * (1 + 1e-6)) : INFINITY;
    }
    run_all_seeds<4>(call, kinds[0], h2, o.max_iterations);
    run_all_seeds<12>(call, kinds[1], h2, o.max_iterations);
    call.sync();
  }

  // ---- the reference driver (clustering.cpp:44-96), replayed on the host
  auto engine = load_rng(rng);
  std::vector<uint64_t> visited((q + 63) / 64, 0);
  uint64_t unvisited = q, support_entries = 0;
  int limited = 0;
  std::vector<Center> centers;
  const int refl_dims[3] = {1, 2, 3}, rigid_dims[3] = {9, 10, 11};
  CenterGrid grids[2] = {CenterGrid(h, refl_dims), CenterGrid(h, rigid_dims)};
  auto visit = [&](uint64_t i) {
    uint64_t &w = visited[i >> 6];
    uint64_t bit = 1ull << (i & 63);
    if (!(w & bit)) w |= bit, --unvisited;
  };
  while (unvisited) {
    uint64_t r = engine() % unvisited;
    uint64_t seed = 0;
    for (uint64_t w = 0;; ++w) {  // r-th unvisited vote, ascending
      uint64_t free_bits = ~visited[w];
      if ((w + 1) * 64 > q) free_bits &= (q % 64 ? (1ull << (q % 64)) - 1 : ~0ull);
      uint64_t c = __builtin_popcountll(free_bits);
      if (r < c) {
        for (; r; --r) free_bits &= free_bits - 1;
        seed = w * 64 + __builtin_ctzll(free_bits);
        break;
      }
      r -= c;
    }
    int t = kind_of[seed];
    KindData &k = kinds[t];
    uint64_t s = uint64_t(local_of[seed]);
    const uint32_t *members = k.sup_idx.data() + k.sup_off[s];
    const uint64_t size = k.sup_off[s + 1] - k.sup_off[s];
    for (uint64_t m = 0; m < size; ++m) visit(uint64_t(k.ids[members[m]]));
    bool converged = k.flags[s] & 1, exhausted = k.flags[s] & 2;
    if (exhausted) visit(seed);
    if (!converged) ++limited;
    const double *mean = &k.mean[s * k.dim];
    const int merge = grids[t].first(mean, [&](int32_t c) {
      return desc_d2(mean, centers[c].v, k.dim) < h2 / 4;
    });
    auto add_keys = [&](Center &c) {  // the support's members into the union
      uint64_t added = 0;
      for (uint64_t m = 0; m < size; ++m) {
        uint64_t &w = c.keys[members[m] >> 6];
        const uint64_t bit = uint64_t(1) << (members[m] & 63);
        if (!(w & bit)) w |= bit, ++added;
      }
      c.key_count += added;
      return added;
    };
    if (merge < 0) {
      Center c;
      for (int i = 0; i < 12; ++i) c.v[i] = i < k.dim ? mean[i] : 0;
      c.kind = t;
      c.keys.assign((k.n + 63) / 64, 0);
      add_keys(c);
      c.seeds.push_back(int32_t(s));
      support_entries += c.key_count;
      grids[t].insert(int32_t(centers.size()), c.v);
      centers.push_back(std::move(c));
    } else {
      Center &c = centers[merge];
      double old = double(c.key_count), now = double(size);
      if (old + now > 0) {
        grids[t].erase(merge, c.v);
        for (int i = 0; i < k.dim; ++i) c.v[i] = (old * c.v[i] + now * mean[i]) / (old + now);
        grids[t].insert(merge, c.v);
      }
      support_entries += add_keys(c);
      c.seeds.push_back(int32_t(s));
    }
    if (support_entries > 5000000)
      fail(SYM_RUNTIME_ERROR, "Mean-shift support budget exceeded; lower --sample-ratio");
    if (centers.size() > 20000)
      fail(SYM_RUNTIME_ERROR, "Too many mean-shift modes; increase --bandwidth or lower --sample-ratio");
  }
  store_rng(engine, rng);

  // ---- support counts and winners (clustering.cpp:97-108) on the GPU
  std::vector<int32_t> winner(q, -1);
  count_members<4>(call, kinds[0], centers, 0, h2, o.max_iterations, winner);
  count_members<12>(call, kinds[1], centers, 1, h2, o.max_iterations, winner);
  std::vector<std::vector<int32_t>> members(centers.size());
  for (uint64_t i = 0; i < q; ++i)
    if (winner[i] >= 0) members[winner[i]].push_back(int32_t(i));

  // ---- decode (clustering.cpp:109-141), stable sort, truncate
  struct Row {
    sym_cluster_record rec;
    std::vector<int32_t> votes;
  };
  std::vector<Row> rows;
  D3 origin{ctx.center[0], ctx.center[1], ctx.center[2]};
  for (size_t c = 0; c < centers.size(); ++c) {
    if (members[c].empty()) continue;
    Row row{};
    row.rec.reflection = centers[c].kind == 0;
    row.votes = std::move(members[c]);
    const double *d = centers[c].v;
    if (row.rec.reflection) {
      D3 n{d[0], d[1], d[2]};
      double length = norm(n);
      D3 pn = unit(n);
      double offset = d[3] * ctx.box_size / length - dot(pn, origin);
      M3 r = mirror(pn);
      D3 t = pn * (-2 * offset);
      for (int i = 0; i < 9; ++i) row.rec.rotation[i] = r.m[i];
      row.rec.translation[0] = t.x, row.rec.translation[1] = t.y, row.rec.translation[2] = t.z;
      row.rec.plane_normal[0] = pn.x, row.rec.plane_normal[1] = pn.y, row.rec.plane_normal[2] = pn.z;
      row.rec.plane_offset = offset;
    } else {
      M3 m;
      for (int i = 0; i < 9; ++i) m.m[i] = d[i] * 2;
      D3 c0{m.m[0], m.m[3], m.m[6]}, c1{m.m[1], m.m[4], m.m[7]};
      D3 a = unit(c0), b = unit(c1 - a * dot(a, c1));
      if (norm(a) < 0.5 || norm(b) < 0.5) {
        int32_t first = row.votes[0];
        for (int i = 0; i < 9; ++i) m.m[i] = votes.rotation[i][first];
      } else {
        m = columns(a, b, cross(a, b));
      }
      D3 t{d[9], d[10], d[11]};
      D3 tr = t * ctx.box_size + origin - mul(m, origin);
      for (int i = 0; i < 9; ++i) row.rec.rotation[i] = m.m[i];
      row.rec.translation[0] = tr.x, row.rec.translation[1] = tr.y, row.rec.translation[2] = tr.z;
    }
    rows.push_back(std::move(row));
  }
  std::stable_sort(rows.begin(), rows.end(),
                   [](const Row &a, const Row &b) { return a.votes.size() > b.votes.size(); });
  if (rows.size() > size_t(o.max_clusters)) rows.resize(o.max_clusters);
  uint64_t total = 0;
  for (auto &r : rows) total += r.votes.size();
  size_t nrec = rows.size();
  size_t bytes = nrec * sizeof(sym_cluster_record) + (nrec + 1) * 8 + total * 4 + 64;
  char *block = static_cast<char *>(allocate(bytes));
  if (!block) fail(SYM_RUNTIME_ERROR, "host allocation failed");
  out.storage = block;
  out.records = reinterpret_cast<sym_cluster_record *>(block);
  out.vote_offsets = reinterpret_cast<uint64_t *>(block + nrec * sizeof(sym_cluster_record));
  out.vote_indices = reinterpret_cast<int32_t *>(out.vote_offsets + nrec + 1);
  out.count = nrec;
  out.limited_iterations = limited;
  out.vote_offsets[0] = 0;
  for (size_t c = 0; c < nrec; ++c) {
    out.records[c] = rows[c].rec;
    std::copy(rows[c].votes.begin(), rows[c].votes.end(), out.vote_indices + out.vote_offsets[c]);
    out.vote_offsets[c + 1] = out.vote_offsets[c] + rows[c].votes.size();
  }
}

}  // namespace sym
