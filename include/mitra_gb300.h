/* SPDX-License-Identifier: MPL-2.0
 *
 * mitra_gb300.h - C ABI of the GB300 symmetry hot path.
 *
 * The entry points replace the six stage methods of the reference's
 * `symmetry::Backend` (include/symmetry/pipeline.h:54-69 of deoksieze/Mitra_algo)
 * for one mesh on one GPU: curvature, select, pairing, transformations,
 * clustering and verification.  Every view points at HOST memory, exactly as
 * the reference documents for its backends (pipeline.h:51-53): a call uploads
 * what it needs, runs its sm_103a kernels and returns completed host results.
 *
 * Conventions
 *  - Every function returns a sym_status.  On failure the message of the error
 *    (the same text the reference throws, e.g. "Pair budget exceeded; ...") is
 *    kept per thread and read with sym_last_error().
 *  - Fixed-size outputs (features) are written to caller-owned buffers.
 *    Variable-size outputs (selection, pairs, votes, clusters, verification)
 *    are allocated by the library and released with the matching *_release.
 *  - SoA columns, 32-bit vertex/face/pair/vote ids and 64-bit CSR offsets
 *    follow include/symmetry/storage.h:14-16 of the reference.
 *  - No exceptions, no C++ or torch types cross this boundary.
 */
#ifndef MITRA_GB300_H
#define MITRA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
typedef enum sym_status {
  SYM_OK = 0,
  SYM_INVALID_ARGUMENT = 1, /* reference: std::invalid_argument */
  SYM_RUNTIME_ERROR = 2,    /* reference: std::runtime_error (budgets, ...) */
  SYM_OVERFLOW = 3,         /* reference: std::overflow_error */
  SYM_CUDA_ERROR = 4,       /* reference: runtime_error("CUDA: <msg>") */
  SYM_NO_DEVICE = 5,        /* reference: "CUDA: no available device" */
  SYM_DEVICE_TIMEOUT = 6    /* a bounded device-side wait gave up */
} sym_status;

/* Message of the last failing call made on the calling thread. */
const char *sym_last_error(void);

/* ------------------------------------------------------------ input views */
typedef struct sym_points_view {
  const double *x, *y, *z;
  uint64_t count;
} sym_points_view;

typedef struct sym_faces_view { /* three index columns, reference Faces */
  const int32_t *v0, *v1, *v2;
  uint64_t count;
} sym_faces_view;

typedef struct sym_mesh_view { /* reference MeshView, storage.h:135-138 */
  sym_points_view vertices;
  sym_faces_view faces;
} sym_mesh_view;

typedef struct sym_csr_view { /* reference CsrView, storage.h:143-151 */
  const uint64_t *offsets;
  uint64_t rows; /* offsets has rows + 1 entries */
  const int32_t *indices;
} sym_csr_view;

typedef struct sym_edge { /* reference Edge, pipeline.h:11-13 */
  int32_t lo, hi, a, b, face0, face1;
} sym_edge;

typedef struct sym_topology_view { /* reference TopologyView, pipeline.h:14-20 */
  sym_points_view normals, face_normals;
  const double *weights;
  uint64_t weight_count;
  sym_csr_view neighbors, incident_faces;
  const sym_edge *edges;
  uint64_t edge_count;
} sym_topology_view;

typedef struct sym_features_view { /* reference FeaturesView, storage.h:196-205 */
  sym_points_view normal, dmin, dmax;
  const double *kmin, *kmax;
  const uint8_t *valid;
  uint64_t count;
} sym_features_view;

typedef struct sym_features_out { /* caller-owned, `count` rows each */
  double *normal_x, *normal_y, *normal_z;
  double *dmin_x, *dmin_y, *dmin_z;
  double *dmax_x, *dmax_y, *dmax_z;
  double *kmin, *kmax;
  uint8_t *valid;
  uint64_t count;
} sym_features_out;

typedef struct sym_pairs_view { /* reference PairsView, storage.h:231-235 */
  const int32_t *a, *b;
  uint64_t count;
} sym_pairs_view;

/* Vote kinds follow reference TransformKind (storage.h:296). */
enum { SYM_RIGID = 0, SYM_REFLECTION = 1 };

typedef struct sym_votes_view { /* reference VotesView, storage.h:305-330 */
  const int32_t *pair;
  const uint8_t *kind;
  const double *rotation[9]; /* row-major 3x3 */
  const double *translation[3];
  const double *plane_normal[3];
  const double *plane_offset;
  const double *descriptor[12]; /* 4 used for reflections, 12 for rigid */
  uint64_t count;
} sym_votes_view;

/* Same memory layout as the reference ClusterRecord (storage.h:365-370). */
typedef struct sym_cluster_record {
  uint8_t reflection;
  double rotation[9];
  double translation[3];
  double plane_normal[3];
  double plane_offset;
} sym_cluster_record;

typedef struct sym_clusters_view { /* reference ClustersView, storage.h:383-387 */
  const sym_cluster_record *records;
  uint64_t count;
  const uint64_t *vote_offsets; /* count + 1 */
  const int32_t *vote_indices;
} sym_clusters_view;

typedef struct sym_model_context { /* reference ModelContext, pipeline.h:30-33 */
  double box_size;
  double center[3];
} sym_model_context;

typedef struct sym_options { /* reference Options, options.h:5-12 */
  double sample_ratio, prune, pair_threshold, bandwidth, verify_threshold;
  int32_t smoothing, subdivide, max_iterations, max_clusters;
  uint64_t seed, max_pairs, max_votes;
  int32_t patching;
} sym_options;

/* The reference's defaults (options.h:6-11). */
void sym_options_default(sym_options *out);

/* std::mt19937_64 state: 312 words and the position, in the order libstdc++
 * streams the engine (operator<< / operator>>).  The reference threads one
 * engine through select() and clustering() (pipeline.h:60-66). */
typedef struct sym_rng {
  uint64_t words[312];
  uint64_t index;
} sym_rng;
void sym_rng_seed(sym_rng *rng, uint64_t seed);
uint64_t sym_rng_next(sym_rng *rng);

/* ---------------------------------------------------- library-owned outputs */
typedef struct sym_selection { /* reference Selection, pipeline.h:45-47 */
  int32_t *sample;
  uint64_t sample_count;
  int32_t *pruned;
  uint64_t pruned_count;
  void *storage;
} sym_selection;
void sym_selection_release(sym_selection *s);

typedef struct sym_pairs { /* reference Pairs, storage.h:236-250 */
  int32_t *a, *b;
  uint64_t count;
  void *storage;
} sym_pairs;
void sym_pairs_release(sym_pairs *p);

typedef struct sym_votes { /* reference Votes, storage.h:331-364 */
  int32_t *pair;
  uint8_t *kind;
  double *rotation[9];
  double *translation[3];
  double *plane_normal[3];
  double *plane_offset;
  double *descriptor[12];
  uint64_t count;
  void *storage;
} sym_votes;
void sym_votes_release(sym_votes *v);

typedef struct sym_clusters { /* reference ClusterOutput, pipeline.h:48-51 */
  sym_cluster_record *records;
  uint64_t count;
  uint64_t *vote_offsets; /* count + 1 */
  int32_t *vote_indices;
  int32_t limited_iterations;
  void *storage;
} sym_clusters;
void sym_clusters_release(sym_clusters *c);

typedef struct sym_grouped_csr { /* reference GroupedCsr, storage.h:171-183 */
  uint64_t *groups;      /* cluster_count + 1 row ranges */
  uint64_t *offsets;     /* rows + 1 */
  int32_t *indices;
  uint64_t rows;
} sym_grouped_csr;

typedef struct sym_verification_result { /* reference Verification, storage.h:371-382 */
  uint64_t cluster_count;
  uint64_t *side_a_offsets, *side_b_offsets; /* cluster_count + 1 */
  int32_t *side_a, *side_b;
  sym_grouped_csr patches_a, patches_b;
  double *coverage, *rms;
  void *storage;
} sym_verification_result;
void sym_verification_release(sym_verification_result *v);

/* ------------------------------------------------------------------ context */
/* One context = one device, one stream, one growable device workspace and
 * pinned staging buffers reused across calls.  A context is used by one
 * thread at a time (the reference Backend methods are const but its CUDA
 * backend keeps thread-local metrics: profile.cpp:23-24). */
typedef struct sym_context sym_context;
sym_status sym_context_create(int device, sym_context **out);
void sym_context_destroy(sym_context *ctx);
/* The context's cudaStream_t, for callers that time or order work on it. */
void *sym_context_stream(sym_context *ctx);
/* Name reported by Backend::name() for this backend. */
const char *sym_backend_name(void);

/* ---------------------------------------------------------- stage methods */
/* Backend::curvature (pipeline.h:58; CPU reference src/cpu/curvature.cpp:14-79) */
sym_status sym_curvature(sym_context *ctx, const sym_mesh_view *mesh,
                         const sym_topology_view *topology,
                         const sym_options *options,
                         const sym_features_out *out);

/* The reference's sample_vertices (src/core/sampling.cpp:5-24,
 * include/symmetry/sampling.h:6-7) on the GPU: one draw of `rng` per
 * positive weight in vertex order, exponential keys -log(u)/w, the
 * ceil(count * ratio) smallest (ties by vertex id), ids ascending.  The ids
 * and the engine state left in `rng` are bit-exact with the host function:
 * the engine runs on the device, and keys within a relative 2^-32 of the
 * selection boundary are re-evaluated with the host's std::log.  `weights`
 * (count doubles) and `sample` (room for count ids) are host arrays. */
sym_status sym_sample_vertices(sym_context *ctx, const double *weights, uint64_t count,
                               double ratio, sym_rng *rng, int32_t *sample,
                               uint64_t *sample_count);

/* Backend::select (pipeline.h:59-60; src/cpu/selection.cpp:15-29).  The
 * area-weighted sample (sym_sample_vertices, with `rng`), the anisotropy
 * prune and its stable compaction all run on the GPU. */
sym_status sym_select(sym_context *ctx, const sym_mesh_view *mesh,
                      const sym_features_view *features, const double *weights,
                      uint64_t weight_count, const sym_options *options,
                      sym_rng *rng, sym_selection *out);

/* Backend::pairing (pipeline.h:61-62; src/cpu/pairing.cpp:14-35) */
sym_status sym_pairing(sym_context *ctx, const sym_mesh_view *mesh,
                       const sym_features_view *features,
                       const int32_t *selected, uint64_t selected_count,
                       const sym_model_context *model,
                       const sym_options *options, sym_pairs *out);

/* Backend::transformations (pipeline.h:63-64; src/cpu/transformations.cpp:17-73) */
sym_status sym_transformations(sym_context *ctx, const sym_mesh_view *mesh,
                               const sym_features_view *features,
                               const sym_pairs_view *pairs,
                               const sym_model_context *model,
                               const sym_options *options, sym_votes *out);

/* Backend::clustering (pipeline.h:65-66; src/cpu/clustering.cpp:32-208) */
sym_status sym_clustering(sym_context *ctx, const sym_votes_view *votes,
                          const sym_model_context *model,
                          const sym_options *options, sym_rng *rng,
                          sym_clusters *out);

/* Backend::verification (pipeline.h:67-68; src/cpu/verification.cpp:50-110) */
sym_status sym_verification(sym_context *ctx, const sym_mesh_view *mesh,
                            const sym_topology_view *topology,
                            const sym_clusters_view *clusters,
                            const sym_model_context *model,
                            const sym_options *options,
                            sym_verification_result *out);

/* Test hook for the device point-triangle distance, like the reference's
 * cuda_detail::triangle_distances (src/cuda/verification.cu:266-281).
 * `queries` holds 12 doubles per query: p, a, b, c. */
sym_status sym_triangle_distances(sym_context *ctx, const double *queries,
                                  uint64_t count, double *out);

/* ------------------------------------------------- throughput extension
 * No counterpart in the reference (it processes one mesh per detect() with
 * every stage re-uploading its inputs).  A mesh is loaded once into device
 * memory, then sym_detect_fast runs the whole hot path on it with device-
 * resident intermediates: curvature, prune of the area-weighted sample (the
 * caller's, or drawn on the device by sym_detect_fast_sampled), exact
 * pairing, 6-D rigid votes (axis-angle/2 + centred translation/box, FP32
 * transforms, FP64 log map near pi) or plane votes, a spatially sorted vote
 * set, mean-shift from K seeds with Epanechnikov or exp (Gaussian) weights,
 * mode merging, and verification of the top modes on a device LBVH.  The mean-shift approach phase runs in FP32 (SIMT) or BF16 (tensor
 * cores); both forms then share the same FP32 polish phase (Newton steps near
 * the modes, see sym_meanshift6); a subset of seeds can be re-run in FP64 to
 * report the mode error. */
typedef struct sym_mesh_handle sym_mesh_handle;
/* Uploads the mesh and its topology (the views are read during the call
 * only) and builds the verification LBVH on the device. */
sym_status sym_mesh_load(sym_context *ctx, const sym_mesh_view *mesh,
                         const sym_topology_view *topology,
                         const sym_model_context *model, sym_mesh_handle **out);
/* Waits for all work on the mesh's device, then frees the mesh; any
 * context may have used it, and the loading context may already be
 * destroyed. */
void sym_mesh_free(sym_mesh_handle *handle);

enum { SYM_MS_FP32 = 0, SYM_MS_BF16_REFINED = 1 };
typedef struct sym_fast_options {
  int32_t precision;         /* SYM_MS_FP32 or SYM_MS_BF16_REFINED */
  int32_t seeds;             /* mean-shift seeds K (votes drawn uniformly) */
  uint64_t seed_rng;         /* seed of the seed-drawing std::mt19937_64 */
  int32_t max_iterations;    /* approach-phase iterations (BF16 or FP32) */
  int32_t polish_iterations; /* FP32 polish iterations (both forms) */
  int32_t reference_seeds;   /* seeds re-run in FP64 for the mode error */
  int32_t verify;            /* verify the top modes (max_clusters) */
  /* SYM_RIGID: two rotation + translation votes per pair, 6-D
   * [log(R)/2, (R c + t - c)/box]; SYM_REFLECTION: one plane vote per pair
   * whose mirrored frames agree (the reference's test,
   * transformations.cpp:17-73), [n, (d + n.c)/box] padded to 6-D with
   * zeros, decoded as the reference does (clustering.cpp:117-124) */
  int32_t mode;
  /* 0: every vote.  Otherwise at most about vote_cap votes enter the mean
   * shift: each pair (rigid) or plane vote (reflection) is kept with
   * probability vote_cap / votes by a hash of its index and seed_rng,
   * order preserved (a uniform subsample, the same for every precision) */
  uint64_t vote_cap;
  /* FP64 refinement passes of the verified modes' motions before their
   * verification (0: none): each pass pairs every vertex that supports a
   * mode forward with the closest surface point to its image, then fits the
   * motion to those pairs by weighted least squares (rigid: Kabsch; reflection:
   * the plane through the midpoints, normal along the displacements) --
   * ICP on the device in FP64; the records carry the refined motions */
  int32_t refine;
  /* Launch shapes of the mean shift, 0 for the default (mitra_algo_gb300's
   * autotuner picks them per workload): Morton bits per coordinate of the
   * vote order (1-10, default 8), SIMT CTAs per SM (1-256, default 128),
   * tensor-kernel CTAs per SM for the chunk lists (1-8, default 1), tensor
   * approach iterations between host checks (default 8).  They change the
   * order of FP32 sums and the work split, not the method. */
  int32_t vote_bits, simt_blocks_per_sm, tc_ctas_per_sm, check_interval;
  /* Mean-shift weight kernel: SYM_KERNEL_EPANECHNIKOV (1 - d^2/h^2, the
   * reference's) or SYM_KERNEL_GAUSSIAN (2^(-8 d^2/h^2) - 2^-8 for d < h: a
   * Gaussian with sigma = h/3.33 shifted to reach 0 at the cut; the tensor
   * kernel makes these weights with the MUFU's BF16x2 exponential, the
   * polish takes Newton steps with the Gaussian's Jacobian) */
  int32_t kernel;
} sym_fast_options;
enum { SYM_KERNEL_EPANECHNIKOV = 0, SYM_KERNEL_GAUSSIAN = 1 };

#define SYM_FAST_MAX_CLUSTERS 32
typedef struct sym_fast_result {
  uint64_t sampled, pruned, pairs, votes, modes, clusters;
  int32_t iterations, polish_iterations;
  /* relative error of each mode against FP64, over the reference seeds that
   * converged (Newton, a well-defined mode) in both runs (modes_compared of
   * them); modes_within counts those within 1e-4.  The seeds_* and
   * mode_error_all_* / _settled_ / _unconverged_ fields below cover every
   * reference seed. */
  double mode_error_max, mode_error_mean;
  uint64_t modes_compared, modes_within;
  /* device time per stage: curvature, prune, pairing, votes, vote sort,
   * mean shift, modes, verification */
  double stage_ms[8];
  double mean_shift_pairs; /* seed-vote evaluations actually made */
  double seed_iterations;  /* sum over seeds of the iterations each ran */
  double bulk_ms, polish_ms; /* device time of the two mean-shift phases */
  /* active seeds at the start of the first 320 bulk / polish iterations */
  uint32_t bulk_trace[320], polish_trace[320];
  uint64_t launches, h2d_bytes, d2h_bytes;
  sym_cluster_record records[SYM_FAST_MAX_CLUSTERS];
  uint64_t support[SYM_FAST_MAX_CLUSTERS];
  double coverage[SYM_FAST_MAX_CLUSTERS], rms[SYM_FAST_MAX_CLUSTERS];
  /* connected patches supporting each verified mode (forward, inverse) */
  uint32_t patches[2 * SYM_FAST_MAX_CLUSTERS];
  /* 1 when the mode was formed by Newton-converged seeds (a well-defined
   * position), 0 when only by seeds that settled on a ridge or ran out of
   * iterations */
  uint8_t precise[SYM_FAST_MAX_CLUSTERS];
  /* the BF16 tensor-core kernel alone: launches, summed device time (CUDA
   * events around each launch) and the seed-vote evaluations it made */
  uint64_t tc_launches;
  double tc_kernel_ms, tc_evaluations;
  /* verification queries that the FP32 search and its FP64 rechecks left
   * to the reference-order BVH (an exact FP64 distance tie between faces
   * that disagree on the normal test, or too many candidate faces) */
  uint64_t verify_undecided;
  /* verification queries decided in FP64 because an FP32 test fell within
   * its error band (out of 2 x clusters x vertices) */
  uint64_t verify_fp64_rows;
  /* mode error over every one of the seeds_compared reference seeds (none
   * dropped): max and mean relative error of the final position against the
   * FP64 run's, seeds_within of them within 1e-4; by the pair of final
   * states, modes_compared were Newton-converged in both runs, seeds_settled
   * ended on a ridge (settled) in one or both, seeds_unconverged were still
   * approaching, or lost their weight, in one or both */
  uint64_t seeds_compared, seeds_within, seeds_settled, seeds_unconverged;
  double mode_error_all_max, mode_error_all_mean;
  double mode_error_settled_max, mode_error_unconverged_max;
  /* per reported mode (with reference_seeds > 0): the relative error of its
   * motion [R, t / box] against the FP64 mode that the FP64 mean shift
   * reaches from the same position; with `refine`, the error of the refined
   * motion against the same refinement of the FP64 motion */
  double transform_error[SYM_FAST_MAX_CLUSTERS], transform_error_max;
  double transform_error_refined[SYM_FAST_MAX_CLUSTERS], transform_error_refined_max;
} sym_fast_result;
void sym_fast_options_default(sym_fast_options *out);
/* `sample` is a host array of vertex ids (the area-weighted sample). */
sym_status sym_detect_fast(sym_context *ctx, sym_mesh_handle *mesh,
                           const int32_t *sample, uint64_t sample_count,
                           const sym_options *options,
                           const sym_fast_options *fast, sym_fast_result *out);
/* sym_detect_fast with the sample drawn on the device from the mesh's
 * weights, as the reference's detect() draws it (src/core/pipeline.cpp:25,
 * src/cpu/selection.cpp:20): a std::mt19937_64 seeded with options->seed and
 * sym_sample_vertices' keys -- the same ids, bit-exact.  out->sampled gives
 * their number. */
sym_status sym_detect_fast_sampled(sym_context *ctx, sym_mesh_handle *mesh,
                                   const sym_options *options,
                                   const sym_fast_options *fast, sym_fast_result *out);

/* The refinement and verification of sym_detect_fast on given motions: the
 * `count` records are refined in place by `iterations` passes (see
 * sym_fast_options.refine), then verified with options->verify_threshold;
 * coverage and rms get `count` entries, patches 2 * count (forward, inverse
 * patch counts). */
sym_status sym_refine_transforms(sym_context *ctx, sym_mesh_handle *mesh,
                                 const sym_options *options, sym_cluster_record *records,
                                 uint64_t count, int32_t iterations, double *coverage,
                                 double *rms, uint32_t *patches);

/* Backend::verification (pipeline.h:67-68; src/cpu/verification.cpp:50-110)
 * on a resident mesh: the same side lists, patches, coverage and rms as
 * sym_verification gives for the mesh and records, bit for bit.  The
 * closest-point searches run in FP32 on the mesh's LBVH and every decision
 * is rechecked in FP64 with the reference's expressions; queries whose FP64
 * nearest distance is shared by faces that disagree on the normal test
 * (the reference keeps the face its median-split BVH visits first) go
 * through that BVH, built on the host once per resident mesh when first
 * needed.  `undecided` (may be NULL) receives the number of such queries. */
sym_status sym_verification_resident(sym_context *ctx, sym_mesh_handle *mesh,
                                     const sym_clusters_view *clusters, const sym_options *options,
                                     sym_verification_result *out, uint64_t *undecided);

/* GPU mesh preparation: the reference's prepare() (src/core/prepare.cpp:
 * 102-149) without subdivision (options->subdivide must be 0) and its
 * topology() (prepare.cpp:13-58): option and mesh validation with the
 * reference's messages, the bounding-box diagonal, removal of degenerate
 * faces, face and vertex normals, vertex weights, neighbour ring, incident
 * faces, edge table and vertex centroid, bit-exact with the CPU path.  The
 * outputs are library-owned host arrays (sym_prepared_release). */
typedef struct sym_prepared {
  sym_model_context context;
  uint64_t vertex_count, face_count, edge_count, rejected_faces;
  int32_t *faces[3]; /* the kept faces, face_count rows */
  double *normals[3], *face_normals[3], *weights;
  uint64_t *neighbor_offsets; /* vertex_count + 1 */
  int32_t *neighbor_indices;
  uint64_t *incident_offsets; /* vertex_count + 1 */
  int32_t *incident_indices;
  sym_edge *edges;
  void *storage;
} sym_prepared;
sym_status sym_prepare(sym_context *ctx, const sym_mesh_view *mesh,
                       const sym_options *options, sym_prepared *out);
void sym_prepared_release(sym_prepared *p);
/* sym_prepare straight into a resident mesh (as sym_mesh_load): only the
 * vertices and faces cross from the host. */
sym_status sym_mesh_load_raw(sym_context *ctx, const sym_mesh_view *mesh,
                             const sym_options *options, sym_mesh_handle **out);

/* Batched detection (no reference counterpart; the reference's detect() runs
 * one mesh per call, src/core/pipeline.cpp:27-47).  Runs sym_detect_fast on
 * every item, one host thread per worker context: each worker (its own CUDA
 * stream and workspace) takes the next item in order, so the launches and
 * host round trips of different meshes overlap on the GPU.  The contexts
 * are the caller's (created once with sym_context_create, on the device the
 * meshes were loaded on, and reused across calls so their workspaces stay
 * allocated); no two workers may share one.  Each item's result is the one
 * sym_detect_fast gives for it alone.  Returns SYM_OK when every item
 * succeeded, else the status of the first failing item (each item keeps its
 * own status and message). */
typedef struct sym_batch_item {
  sym_mesh_handle *mesh;
  const int32_t *sample; /* NULL with SYM_SAMPLE_ON_DEVICE: the item runs as */
  uint64_t sample_count; /* sym_detect_fast_sampled (sample from options->seed) */
  const sym_options *options;
  const sym_fast_options *fast;
  sym_fast_result *out; /* caller-owned */
  sym_status status;    /* written by the call */
  char message[256];    /* the item's error message, "" on success */
} sym_batch_item;
#define SYM_SAMPLE_ON_DEVICE UINT64_MAX
sym_status sym_detect_fast_batch(sym_context *const *workers, int32_t worker_count,
                                 sym_batch_item *items, uint64_t count);

/* Fused batched detection (no reference counterpart).  Runs the stages
 * before the mean shift mesh by mesh, then ONE mean shift for every mesh's
 * seeds together -- each mesh's votes are moved to their own cell of a
 * grid in vote space (pitch 8 per coordinate; votes lie within [-2, 2]), so
 * votes of different meshes never weigh on each other's seeds, and every
 * iteration is one launch per kernel for the whole batch -- then the modes
 * and the verification mesh by mesh.  Each item's result is filled as
 * sym_detect_fast fills it (its mean-shift iteration counts are the
 * batch's).  Items must share precision, kernel, iteration counts, launch
 * shape and bandwidth (below 2), and ask for no FP64 reference seeds; at
 * most 4,096 items.  Items may use a sample or SYM_SAMPLE_ON_DEVICE.  An
 * item that fails keeps its status and message and takes no part in the
 * mean shift; the call returns the first failing item's status. */
typedef struct sym_fused_stats {
  uint64_t meshes, votes, seeds;
  int32_t iterations, polish_iterations;
  double seed_iterations, tc_evaluations;
  /* device time (CUDA events): the stages before the mean shift over all
   * meshes, the vote set and seeds, the approach phase, the polish, then
   * modes and verification over all meshes */
  double votes_ms, vote_set_ms, bulk_ms, polish_ms, modes_verification_ms;
  uint64_t tc_launches, launches;
  double tc_kernel_ms;
} sym_fused_stats;
sym_status sym_detect_fast_fused(sym_context *ctx, sym_batch_item *items, uint64_t count,
                                 sym_fused_stats *stats);

/* The mean-shift kernels of sym_detect_fast on their own (no reference
 * counterpart): K seeds over Q 6-D votes (host, q x 6 doubles), seeds are
 * vote indices.  Approach phase (at most max_iterations, in the requested
 * precision: FP32, BF16 tensor cores, or FP64): plain mean-shift steps until a
 * seed's squared step is below 4e-4 h^2 (a step under h/50).  Polish phase (at most
 * polish_iterations, FP32; FP64 for SYM_MS_FP64): safeguarded Newton steps on
 * m(x) = x until a Newton step is below 1e-4 h (converged).  A rejected
 * Newton step (singular system, step longer than h/4 or against the plain
 * step) is replaced by the plain step and Newton is tried once more; the
 * second rejection settles the seed (the density is flat along some
 * direction, the mode has no well-defined position).  Writes
 * the K final means (k x 6), each seed's state (0 still approaching,
 * 1 converged, 2 exhausted, 3 near a mode when the iterations ran out,
 * 4 settled) and the approach / polish iteration counts.  `precision`: SYM_MS_FP32,
 * SYM_MS_BF16_REFINED, or SYM_MS_FP64 (the form used to measure mode
 * errors); `kernel`: SYM_KERNEL_EPANECHNIKOV or SYM_KERNEL_GAUSSIAN (see
 * sym_fast_options). */
enum { SYM_MS_FP64 = 2 };
sym_status sym_meanshift6(sym_context *ctx, const double *votes, uint64_t q,
                          const int64_t *seeds, uint64_t k, double bandwidth,
                          int32_t precision, int32_t max_iterations,
                          int32_t polish_iterations, int32_t kernel, double *means_out,
                          uint8_t *state_out, int32_t *iterations_out);

/* Test hook for the tensor-core path of the BF16 mean-shift: one tile of
 * D = A1 . B1^T (128x128, K=16) and ACC = A2 . B2^T (128x16, K=128) from
 * row-major BF16 inputs (a1, b1: 128 x 16; a2: 128 x 128; b2: 16 x 128), run
 * through the kernel's shared-memory layouts, TMA bulk copy, tcgen05.mma and
 * TMEM loads.  d_out: 128 x 128 floats, acc_out: 128 x 16 floats. */
sym_status sym_tc_selftest(sym_context *ctx, const uint16_t *a1, const uint16_t *b1,
                           const uint16_t *a2, const uint16_t *b2, float *d_out,
                           float *acc_out);

/* Test hook for the throughput path's vote descriptors (the records
 * sym_detect_fast feeds to its mean shift), on host inputs: `positions` and
 * `features` (one row per vertex, as the reference's FeaturesView) and
 * `pairs`.  SYM_RIGID: two records per pair, in the order of the reference's
 * two rigid votes (transformations.cpp:53-70: b's frame with sign +1, then
 * -1), each [log(R)/2, (R c + t - c)/box, |d|^2, 0] in FP32 -- the rotation
 * part is the axis-angle vector of the reference's rotation, the translation
 * part its descriptor[9..11]; SYM_REFLECTION: one record per pair whose
 * mirrored frames agree (the reference's test, transformations.cpp:31-48),
 * [n, (d + n.c)/box, 0, 0, |d|^2, 0].  `out` has room for 16 floats per
 * pair, `pair_of` for 2 ids per pair (the pair of each record); `count`
 * receives the number of records. */
sym_status sym_fast_votes(sym_context *ctx, const sym_points_view *positions,
                          const sym_features_view *features, const sym_pairs_view *pairs,
                          const sym_model_context *model, int32_t mode, float *out,
                          int32_t *pair_of, uint64_t *count);

/* Test hook for the device's bounded waits (no reference counterpart).
 * which = 0: the tensor-core kernels' barrier wait, with a limit of `limit`
 * nanoseconds in place of 2 s, on a barrier nothing signals, in a kernel that
 * holds tensor memory as the mean-shift kernel does; the wait runs out, the
 * kernel frees its tensor memory and returns, and the call returns
 * SYM_DEVICE_TIMEOUT.  which = 1: the verification's union-find retry loop
 * on a path of 64 vertices with at most `limit` retries per union;
 * SYM_DEVICE_TIMEOUT when a union ran out of retries, else SYM_OK with the
 * number of components in *components (may be NULL).  The context stays
 * usable after either. */
sym_status sym_wait_selftest(sym_context *ctx, int32_t which, uint64_t limit,
                             uint64_t *components);

/* ------------------------------------------------ allocation-free prune */
/* No counterpart in the reference: an allocation-free form of the prune half
 * of select() (src/cpu/selection.cpp:20-27, src/cuda/backend.cu:21-30).
 * For callers that must not allocate device memory during a call -- services
 * that size every buffer at start-up, code between allocator checkpoints.
 * Every pointer is a device pointer owned by the caller: `pruned` has room
 * for `count` entries, `*pruned_count` receives the number kept (UINT64_MAX
 * when an entry of `sample` lies outside [0, vertex_count)).  Kept samples
 * come out in sample order, identical to sym_select's `pruned`.  `stream` is
 * a cudaStream_t (NULL: the legacy default stream); the call only enqueues
 * work and returns.
 * Scratch is a fixed 64 KiB array in the library's static device memory, so
 * `count` is limited to sym_prune_static_max_samples() (16,777,216); larger
 * counts are rejected with SYM_INVALID_ARGUMENT.  That array is shared by all
 * calls on a device: calls that may overlap (two streams, two host threads)
 * race and must be ordered by the caller.  sym_prune_static_setup() resolves
 * the array's address for the current device; call it once per device, with
 * that device current, before any stream capture (the first
 * sym_prune_static on a device otherwise does it), and again after the
 * device's context was reset (cudaDeviceReset), which moves the array. */
uint64_t sym_prune_static_max_samples(void);
sym_status sym_prune_static_setup(void);
sym_status sym_prune_static(const int32_t *sample, uint64_t count, const double *kmin,
                            const double *kmax, const uint8_t *valid, uint64_t vertex_count,
                            double prune, int32_t *pruned, uint64_t *pruned_count,
                            void *stream);

/* ------------------------------------------------------- binary tables */
/* No counterpart in the reference, which writes its results as text
 * (export_result, src/io/export.cpp:37-98: features.csv, pairs.csv,
 * votes.csv, descriptors.csv at 17 significant digits, and mesh.off).  Writes
 * the same tables, with the same columns and derived fields (the sampled /
 * pruned flags of each vertex, each vote's cluster -- the last cluster that
 * lists it, -1 for none -- and each descriptor's dimension, 4 for a
 * reflection vote and 12 for a rigid one), into `directory` as binary column
 * files: features.symt, pairs.symt, votes.symt, descriptors.symt,
 * vertices.symt and faces.symt.  A file is a 24-byte header, one 32-byte
 * record per column, then the columns, each starting at a file offset that
 * is a multiple of 64:
 *
 *   char magic[8] = "SYMTAB01"; uint64 rows; uint32 columns; uint32 0;
 *   per column: char name[24] (NUL padded); uint32 type (1 int32,
 *   2 float64, 3 uint8); uint32 0;
 *   then each column's rows, little-endian.
 *
 * The values are the inputs' own bits, so a reader recovers every double
 * exactly; text at 17 significant digits (the reference's format) can be
 * rendered from them byte for byte.  Every id is checked against its range;
 * the directory must exist.  Host memory only: no device work. */
typedef struct sym_export_view {
  sym_mesh_view mesh;           /* the prepared mesh (vertices, faces) */
  sym_features_view features;   /* one row per vertex */
  const int32_t *sample;        /* sampled vertex ids */
  uint64_t sample_count;
  const int32_t *pruned;        /* pruned vertex ids */
  uint64_t pruned_count;
  sym_pairs_view pairs;
  sym_votes_view votes;
  sym_clusters_view clusters;   /* for each vote's cluster column */
} sym_export_view;
sym_status sym_export_tables(const sym_export_view *result, const char *directory);

/* --------------------------------------------------------------- metrics */
/* Per-stage accounting, the fields of the reference CudaMetric
 * (include/symmetry/cuda.h:7-13, src/cuda/profile.cpp). */
typedef struct sym_metric {
  char stage[32];
  uint64_t h2d_bytes, d2h_bytes, peak_buffer_bytes, custom_launches;
  double gpu_interval_ms, h2d_ms, d2h_ms, custom_kernel_ms;
  int32_t all_buffers_released;
} sym_metric;
sym_status sym_set_profiling(sym_context *ctx, int enabled);
/* Moves up to `capacity` collected metrics into `out`; returns how many. */
uint64_t sym_take_metrics(sym_context *ctx, sym_metric *out, uint64_t capacity);

#ifdef __cplusplus
}
#endif
#endif /* MITRA_GB300_H */
