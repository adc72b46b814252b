// SPDX-License-Identifier: MPL-2.0
// Mean-shift of K seeds over a large set of 6-D votes (throughput path, no
// reference counterpart beyond the Epanechnikov update and the stopping
// rules of src/cpu/clustering.cpp:156-208).
//
// Votes are stored 8 values per vote (6 coordinates, |x|^2, padding), sorted
// along a 6-D Morton curve and cut into chunks of kChunk votes with bounding
// boxes.  Seeds are processed in tiles of kChunk active seeds re-sorted along
// the same curve every iteration; a (tile, chunk) pair whose boxes are more
// than the bandwidth apart is skipped, which is exact for Epanechnikov
// weights (they vanish beyond the bandwidth).
#pragma once
#include "common.cuh"

namespace sym {

constexpr int kChunk = 128;  // votes per chunk = seeds per tile

// Seed states.  A seed approaches its mode with plain mean-shift steps
// (kMoving) until its squared step falls under kSwitch2 h^2, then takes
// safeguarded Newton steps on m(x) - x = 0 (kNear) until a Newton step's
// square falls under kNewtonStop2 h^2 (kConverged: a mode whose position is
// well defined).  A Newton step is rejected when the 6x6 system is
// singular, the step is longer than kTrust h or points against the plain
// step (unless it already meets the convergence test): the seed takes the
// plain step instead and tries Newton again at the next iteration
// (kNearRetry1); a second rejection means the density is flat along some
// direction there (a ridge), so the mode has no well-defined position and
// the seed stops (kSettled).  kExhausted: total weight <= 1e-14.
// A seed of the polish still unconverged after kNewtonCap polish iterations
// (Newton steps that keep being accepted without shrinking, or rejected)
// settles too.  The retries matter for the BF16 form, whose approach ends
// within the rounding of its weights: one rejection decided by that
// rounding no longer fixes the seed's fate.
constexpr uint8_t kMoving = 0, kConverged = 1, kExhausted = 2, kNear = 3, kSettled = 4;
constexpr uint8_t kNearRetry1 = 5;  // kNear after one rejected Newton step
__host__ __device__ inline bool is_near(uint8_t s) { return s == kNear || s == kNearRetry1; }
constexpr double kSwitch2 = 4e-4, kNewtonStop2 = 1e-8, kTrust = 0.25;
constexpr int kNewtonCap = 10;
// Floats (or doubles) per partial sum of one seed: sum w (v - x) (6), sum w, pad,
// then for kNear seeds the unweighted in-window sums of d = v - x: sum d
// (6) and sum d d^T (21, upper triangle row by row), pad.
constexpr int kPartial = 40;

// Launch-shape parameters of the mean shift (an autotuner chooses them; the
// defaults are its choice on the benchmark workload).  Each changes only the
// order of FP32 sums, the work split or how often the host looks.
struct Tuning {
  int vote_bits = 8;            // Morton bits per coordinate of the vote order
  int simt_blocks_per_sm = 128; // CTAs per SM the SIMT kernel's grid aims at
  int tc_ctas_per_sm = 1;       // tensor-kernel CTAs per SM for the chunk lists
  int check_interval = 8;       // tensor approach iterations between host checks
};

// The Gaussian kernel of the extension, in base 2 and shifted to reach 0 at
// the cut: w = 2^(-kGauss2 d^2 / h^2) - 2^-kGauss2 for d < h, 0 beyond
// (sigma = h / sqrt(2 kGauss2 ln 2) = h / 3.33), so it is continuous and
// chunk skipping stays exact.  kGauss2 is a power of two: the tensor kernel
// scales its BF16 seed operand by it exactly.
constexpr double kGauss2 = 8.0;

// Chunks per block box: a seed tile whose box lies beyond the bandwidth of
// a block's box skips its kBlockChunks chunks with one test (exact, as the
// chunk tests: the block box holds every vote of its chunks).  Votes of a
// fused batch lie in one cell of vote space per mesh, so a tile's seeds
// (one or two meshes) meet only their own meshes' blocks.
constexpr int kBlockChunks = 256;

// Votes per sub-box: the Newton polish and the support count test each run
// of kSubVotes consecutive votes of a chunk against the warp's seeds before
// evaluating it (exact like the chunk test; the approach keeps whole chunks).
constexpr int kSubVotes = 16, kSubs = kChunk / kSubVotes;
static_assert(kChunk % kSubVotes == 0 && kSubVotes <= 32 && (kSubVotes & (kSubVotes - 1)) == 0,
              "sub-boxes cut chunks into runs of lanes");

struct VoteSet {
  Tuning tuning;
  // weight kernel: 0 Epanechnikov 1 - d^2 / h^2 (the reference's); > 0 the
  // shifted Gaussian 2^(-kernel_k d^2 / h^2) - 2^-kernel_k
  double kernel_k = 0;
  uint64_t q = 0, nchunks = 0;
  float *desc = nullptr;      // q x 8, Morton order
  double *desc64 = nullptr;   // q x 8, same order (only when requested)
  float *cbox = nullptr;      // nchunks x 12: lo[6], hi[6]
  float *sbox = nullptr;      // nchunks x kSubs x 12: the boxes of each chunk's sub-runs
  uint64_t nblocks = 0;       // runs of kBlockChunks consecutive chunks
  float *bbox = nullptr;      // nblocks x 12: the box of each run's chunks
  float *gbox = nullptr;      // 12: box of all votes
  int32_t *order = nullptr;   // sorted position -> original vote
  int32_t *rank = nullptr;    // original vote -> sorted position
};

// Sorts raw votes (q x 8; desc64_raw may be null) into a VoteSet.
VoteSet build_vote_set(Call &call, const float *desc_raw, const double *desc64_raw, uint64_t q,
                       const Tuning &tuning = Tuning());

// Seeds: sorted positions of the seed votes -> initial means (k x 8).
void init_means(Call &call, const VoteSet &v, const int64_t *seed_rank, uint64_t k, float *means);
void init_means(Call &call, const VoteSet &v, const int64_t *seed_rank, uint64_t k, double *means);

// At most max_iter iterations over the active seeds; state[k] in/out
// (kMoving, kNear, kConverged, kExhausted, kSettled).  Approach phase (polish = false):
// only kMoving seeds step, and a seed leaves once it is kNear.  Polish phase
// (polish = true): kMoving and kNear seeds step until converged, settled or
// exhausted.
// Adds the seed-iterations to *seed_iterations and seed-vote evaluations to
// *evals (device counter).
int shift(Call &call, const VoteSet &v, float *means, uint8_t *state, uint64_t k, double h2,
          int max_iter, bool polish, double *seed_iterations, unsigned long long *evals,
          uint32_t *trace = nullptr, int trace_len = 0);
int shift(Call &call, const VoteSet &v, double *means, uint8_t *state, uint64_t k, double h2,
          int max_iter, bool polish, double *seed_iterations, unsigned long long *evals);

// kMoving seeds, Morton-sorted by position when k <= 2048, with their
// number left on the device (nact[0]); an iteration that finds active seeds
// records their number in trace[*iter] (while *iter < trace_cap) and
// increments *iter.  No synchronisation.
void active_seeds_async(Call &call, const VoteSet &v, const float *means, const uint8_t *state,
                        uint64_t k, int32_t *ids, unsigned *nact, unsigned *iter, uint32_t *trace,
                        unsigned trace_cap);

// Number of votes within the bandwidth of each of `nm` points (nm x 8).
void count_within(Call &call, const VoteSet &v, const float *points, uint64_t nm, double h2,
                  unsigned long long *counts);

}  // namespace sym
