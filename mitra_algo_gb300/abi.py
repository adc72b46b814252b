"""ctypes mirror of include/mitra_gb300.h and the loader of the CUDA library.

The library is built in-tree (``mitra_algo_gb300/_lib/libmitra_gb300.so``) by
``mitra_algo_gb300.build``.  Loading fails loudly when it is missing: there is
no CPU fallback behind these entry points.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

LIB_DIR = Path(__file__).resolve().parent / "_lib"
LIB_PATH = LIB_DIR / "libmitra_gb300.so"

# sym_status
OK, INVALID_ARGUMENT, RUNTIME_ERROR, OVERFLOW, CUDA_ERROR, NO_DEVICE, DEVICE_TIMEOUT = range(7)
RIGID, REFLECTION = 0, 1

_d = C.POINTER(C.c_double)
_i = C.POINTER(C.c_int32)
_u8 = C.POINTER(C.c_uint8)
_u64 = C.POINTER(C.c_uint64)
_f = C.POINTER(C.c_float)


class PointsView(C.Structure):
    _fields_ = [("x", _d), ("y", _d), ("z", _d), ("count", C.c_uint64)]


class FacesView(C.Structure):
    _fields_ = [("v0", _i), ("v1", _i), ("v2", _i), ("count", C.c_uint64)]


class MeshView(C.Structure):
    _fields_ = [("vertices", PointsView), ("faces", FacesView)]


class CsrView(C.Structure):
    _fields_ = [("offsets", _u64), ("rows", C.c_uint64), ("indices", _i)]


class Edge(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("lo", "hi", "a", "b", "face0", "face1")]


class TopologyView(C.Structure):
    _fields_ = [("normals", PointsView), ("face_normals", PointsView),
                ("weights", _d), ("weight_count", C.c_uint64),
                ("neighbors", CsrView), ("incident_faces", CsrView),
                ("edges", C.POINTER(Edge)), ("edge_count", C.c_uint64)]


class FeaturesView(C.Structure):
    _fields_ = [("normal", PointsView), ("dmin", PointsView), ("dmax", PointsView),
                ("kmin", _d), ("kmax", _d), ("valid", _u8), ("count", C.c_uint64)]


class FeaturesOut(C.Structure):
    _fields_ = [(n, _d) for n in ("normal_x", "normal_y", "normal_z", "dmin_x", "dmin_y",
                                  "dmin_z", "dmax_x", "dmax_y", "dmax_z", "kmin", "kmax")] + \
               [("valid", _u8), ("count", C.c_uint64)]


class PairsView(C.Structure):
    _fields_ = [("a", _i), ("b", _i), ("count", C.c_uint64)]


class VotesView(C.Structure):
    _fields_ = [("pair", _i), ("kind", _u8), ("rotation", _d * 9), ("translation", _d * 3),
                ("plane_normal", _d * 3), ("plane_offset", _d), ("descriptor", _d * 12),
                ("count", C.c_uint64)]


class ClusterRecord(C.Structure):
    _fields_ = [("reflection", C.c_uint8), ("rotation", C.c_double * 9),
                ("translation", C.c_double * 3), ("plane_normal", C.c_double * 3),
                ("plane_offset", C.c_double)]


class ClustersView(C.Structure):
    _fields_ = [("records", C.POINTER(ClusterRecord)), ("count", C.c_uint64),
                ("vote_offsets", _u64), ("vote_indices", _i)]


class ExportView(C.Structure):
    _fields_ = [("mesh", MeshView), ("features", FeaturesView), ("sample", _i),
                ("sample_count", C.c_uint64), ("pruned", _i), ("pruned_count", C.c_uint64),
                ("pairs", PairsView), ("votes", VotesView), ("clusters", ClustersView)]


class ModelContext(C.Structure):
    _fields_ = [("box_size", C.c_double), ("center", C.c_double * 3)]


class Options(C.Structure):
    _fields_ = [("sample_ratio", C.c_double), ("prune", C.c_double),
                ("pair_threshold", C.c_double), ("bandwidth", C.c_double),
                ("verify_threshold", C.c_double), ("smoothing", C.c_int32),
                ("subdivide", C.c_int32), ("max_iterations", C.c_int32),
                ("max_clusters", C.c_int32), ("seed", C.c_uint64),
                ("max_pairs", C.c_uint64), ("max_votes", C.c_uint64),
                ("patching", C.c_int32)]


class Rng(C.Structure):
    _fields_ = [("words", C.c_uint64 * 312), ("index", C.c_uint64)]


class Selection(C.Structure):
    _fields_ = [("sample", _i), ("sample_count", C.c_uint64), ("pruned", _i),
                ("pruned_count", C.c_uint64), ("storage", C.c_void_p)]


class PairsOut(C.Structure):
    _fields_ = [("a", _i), ("b", _i), ("count", C.c_uint64), ("storage", C.c_void_p)]


class VotesOut(C.Structure):
    _fields_ = [("pair", _i), ("kind", _u8), ("rotation", _d * 9), ("translation", _d * 3),
                ("plane_normal", _d * 3), ("plane_offset", _d), ("descriptor", _d * 12),
                ("count", C.c_uint64), ("storage", C.c_void_p)]


class ClustersOut(C.Structure):
    _fields_ = [("records", C.POINTER(ClusterRecord)), ("count", C.c_uint64),
                ("vote_offsets", _u64), ("vote_indices", _i),
                ("limited_iterations", C.c_int32), ("storage", C.c_void_p)]


class GroupedCsr(C.Structure):
    _fields_ = [("groups", _u64), ("offsets", _u64), ("indices", _i), ("rows", C.c_uint64)]


class VerificationOut(C.Structure):
    _fields_ = [("cluster_count", C.c_uint64), ("side_a_offsets", _u64),
                ("side_b_offsets", _u64), ("side_a", _i), ("side_b", _i),
                ("patches_a", GroupedCsr), ("patches_b", GroupedCsr),
                ("coverage", _d), ("rms", _d), ("storage", C.c_void_p)]


class Metric(C.Structure):
    _fields_ = [("stage", C.c_char * 32), ("h2d_bytes", C.c_uint64), ("d2h_bytes", C.c_uint64),
                ("peak_buffer_bytes", C.c_uint64), ("custom_launches", C.c_uint64),
                ("gpu_interval_ms", C.c_double), ("h2d_ms", C.c_double), ("d2h_ms", C.c_double),
                ("custom_kernel_ms", C.c_double), ("all_buffers_released", C.c_int32)]


class FastOptions(C.Structure):
    _fields_ = [("precision", C.c_int32), ("seeds", C.c_int32), ("seed_rng", C.c_uint64),
                ("max_iterations", C.c_int32), ("polish_iterations", C.c_int32),
                ("reference_seeds", C.c_int32), ("verify", C.c_int32), ("mode", C.c_int32),
                ("vote_cap", C.c_uint64), ("refine", C.c_int32), ("vote_bits", C.c_int32),
                ("simt_blocks_per_sm", C.c_int32), ("tc_ctas_per_sm", C.c_int32),
                ("check_interval", C.c_int32), ("kernel", C.c_int32)]


FAST_MAX_CLUSTERS = 32


class FastResult(C.Structure):
    _fields_ = [("sampled", C.c_uint64), ("pruned", C.c_uint64), ("pairs", C.c_uint64),
                ("votes", C.c_uint64), ("modes", C.c_uint64), ("clusters", C.c_uint64),
                ("iterations", C.c_int32),
                ("polish_iterations", C.c_int32), ("mode_error_max", C.c_double),
                ("mode_error_mean", C.c_double), ("modes_compared", C.c_uint64),
                ("modes_within", C.c_uint64), ("stage_ms", C.c_double * 8),
                ("mean_shift_pairs", C.c_double), ("seed_iterations", C.c_double),
                ("bulk_ms", C.c_double), ("polish_ms", C.c_double),
                ("bulk_trace", C.c_uint32 * 320), ("polish_trace", C.c_uint32 * 320),
                ("launches", C.c_uint64), ("h2d_bytes", C.c_uint64), ("d2h_bytes", C.c_uint64),
                ("records", ClusterRecord * FAST_MAX_CLUSTERS),
                ("support", C.c_uint64 * FAST_MAX_CLUSTERS),
                ("coverage", C.c_double * FAST_MAX_CLUSTERS),
                ("rms", C.c_double * FAST_MAX_CLUSTERS),
                ("patches", C.c_uint32 * (2 * FAST_MAX_CLUSTERS)),
                ("precise", C.c_uint8 * FAST_MAX_CLUSTERS),
                ("tc_launches", C.c_uint64), ("tc_kernel_ms", C.c_double),
                ("tc_evaluations", C.c_double), ("verify_undecided", C.c_uint64),
                ("verify_fp64_rows", C.c_uint64),
                ("seeds_compared", C.c_uint64), ("seeds_within", C.c_uint64),
                ("seeds_settled", C.c_uint64), ("seeds_unconverged", C.c_uint64),
                ("mode_error_all_max", C.c_double), ("mode_error_all_mean", C.c_double),
                ("mode_error_settled_max", C.c_double), ("mode_error_unconverged_max", C.c_double),
                ("transform_error", C.c_double * FAST_MAX_CLUSTERS), ("transform_error_max", C.c_double),
                ("transform_error_refined", C.c_double * FAST_MAX_CLUSTERS),
                ("transform_error_refined_max", C.c_double)]


class PreparedOut(C.Structure):
    _fields_ = [("context", ModelContext), ("vertex_count", C.c_uint64),
                ("face_count", C.c_uint64), ("edge_count", C.c_uint64),
                ("rejected_faces", C.c_uint64), ("faces", _i * 3), ("normals", _d * 3),
                ("face_normals", _d * 3), ("weights", _d), ("neighbor_offsets", _u64),
                ("neighbor_indices", _i), ("incident_offsets", _u64),
                ("incident_indices", _i), ("edges", C.POINTER(Edge)), ("storage", C.c_void_p)]


class BatchItem(C.Structure):
    _fields_ = [("mesh", C.c_void_p), ("sample", _i), ("sample_count", C.c_uint64),
                ("options", C.POINTER(Options)), ("fast", C.POINTER(FastOptions)),
                ("out", C.POINTER(FastResult)), ("status", C.c_int), ("message", C.c_char * 256)]


class FusedStats(C.Structure):
    _fields_ = [("meshes", C.c_uint64), ("votes", C.c_uint64), ("seeds", C.c_uint64),
                ("iterations", C.c_int32), ("polish_iterations", C.c_int32),
                ("seed_iterations", C.c_double), ("tc_evaluations", C.c_double),
                ("votes_ms", C.c_double), ("vote_set_ms", C.c_double), ("bulk_ms", C.c_double),
                ("polish_ms", C.c_double), ("modes_verification_ms", C.c_double),
                ("tc_launches", C.c_uint64), ("launches", C.c_uint64),
                ("tc_kernel_ms", C.c_double)]


MS_FP32, MS_BF16_REFINED, MS_FP64 = 0, 1, 2
STAGES = ["curvature", "prune", "pairing", "votes", "vote_sort", "mean_shift", "modes",
          "verification"]

P = C.POINTER
# (name, restype, argtypes) of every entry point declared in include/mitra_gb300.h.
PROTOTYPES = [
    ("sym_last_error", C.c_char_p, []),
    ("sym_options_default", None, [P(Options)]),
    ("sym_rng_seed", None, [P(Rng), C.c_uint64]),
    ("sym_rng_next", C.c_uint64, [P(Rng)]),
    ("sym_selection_release", None, [P(Selection)]),
    ("sym_pairs_release", None, [P(PairsOut)]),
    ("sym_votes_release", None, [P(VotesOut)]),
    ("sym_clusters_release", None, [P(ClustersOut)]),
    ("sym_verification_release", None, [P(VerificationOut)]),
    ("sym_context_create", C.c_int, [C.c_int, P(C.c_void_p)]),
    ("sym_context_destroy", None, [C.c_void_p]),
    ("sym_backend_name", C.c_char_p, []),
    ("sym_curvature", C.c_int, [C.c_void_p, P(MeshView), P(TopologyView), P(Options), P(FeaturesOut)]),
    ("sym_select", C.c_int, [C.c_void_p, P(MeshView), P(FeaturesView), _d, C.c_uint64,
                             P(Options), P(Rng), P(Selection)]),
    ("sym_sample_vertices", C.c_int, [C.c_void_p, _d, C.c_uint64, C.c_double, P(Rng), _i,
                                      P(C.c_uint64)]),
    ("sym_pairing", C.c_int, [C.c_void_p, P(MeshView), P(FeaturesView), _i, C.c_uint64,
                              P(ModelContext), P(Options), P(PairsOut)]),
    ("sym_transformations", C.c_int, [C.c_void_p, P(MeshView), P(FeaturesView), P(PairsView),
                                      P(ModelContext), P(Options), P(VotesOut)]),
    ("sym_clustering", C.c_int, [C.c_void_p, P(VotesView), P(ModelContext), P(Options),
                                 P(Rng), P(ClustersOut)]),
    ("sym_verification", C.c_int, [C.c_void_p, P(MeshView), P(TopologyView), P(ClustersView),
                                   P(ModelContext), P(Options), P(VerificationOut)]),
    ("sym_triangle_distances", C.c_int, [C.c_void_p, _d, C.c_uint64, _d]),
    ("sym_mesh_load", C.c_int, [C.c_void_p, P(MeshView), P(TopologyView), P(ModelContext),
                                P(C.c_void_p)]),
    ("sym_mesh_free", None, [C.c_void_p]),
    ("sym_fast_options_default", None, [P(FastOptions)]),
    ("sym_detect_fast", C.c_int, [C.c_void_p, C.c_void_p, _i, C.c_uint64, P(Options),
                                  P(FastOptions), P(FastResult)]),
    ("sym_detect_fast_sampled", C.c_int, [C.c_void_p, C.c_void_p, P(Options), P(FastOptions),
                                          P(FastResult)]),
    ("sym_refine_transforms", C.c_int, [C.c_void_p, C.c_void_p, P(Options), P(ClusterRecord),
                                        C.c_uint64, C.c_int32, _d, _d, P(C.c_uint32)]),
    ("sym_detect_fast_batch", C.c_int, [P(C.c_void_p), C.c_int32, P(BatchItem), C.c_uint64]),
    ("sym_detect_fast_fused", C.c_int, [C.c_void_p, P(BatchItem), C.c_uint64, P(FusedStats)]),
    ("sym_verification_resident", C.c_int, [C.c_void_p, C.c_void_p, P(ClustersView), P(Options),
                                            P(VerificationOut), P(C.c_uint64)]),
    ("sym_prepare", C.c_int, [C.c_void_p, P(MeshView), P(Options), P(PreparedOut)]),
    ("sym_prepared_release", None, [P(PreparedOut)]),
    ("sym_mesh_load_raw", C.c_int, [C.c_void_p, P(MeshView), P(Options), P(C.c_void_p)]),
    ("sym_context_stream", C.c_void_p, [C.c_void_p]),
    ("sym_meanshift6", C.c_int, [C.c_void_p, _d, C.c_uint64, P(C.c_int64), C.c_uint64, C.c_double,
                                 C.c_int32, C.c_int32, C.c_int32, C.c_int32, _d, _u8,
                                 P(C.c_int32)]),
    ("sym_tc_selftest", C.c_int, [C.c_void_p, P(C.c_uint16), P(C.c_uint16), P(C.c_uint16),
                                  P(C.c_uint16), _f, _f]),
    ("sym_wait_selftest", C.c_int, [C.c_void_p, C.c_int32, C.c_uint64, P(C.c_uint64)]),
    ("sym_fast_votes", C.c_int, [C.c_void_p, P(PointsView), P(FeaturesView), P(PairsView),
                                 P(ModelContext), C.c_int32, _f, _i, P(C.c_uint64)]),
    # allocation-free prune: device pointers + a cudaStream_t
    ("sym_prune_static_max_samples", C.c_uint64, []),
    ("sym_prune_static_setup", C.c_int, []),
    ("sym_prune_static", C.c_int, [C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_uint64, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("sym_export_tables", C.c_int, [P(ExportView), C.c_char_p]),
    ("sym_set_profiling", C.c_int, [C.c_void_p, C.c_int]),
    ("sym_take_metrics", C.c_uint64, [C.c_void_p, P(Metric), C.c_uint64]),
]

_LIB = None


def declared_symbols():
    """Names of the functions include/mitra_gb300.h declares."""
    import re
    header = Path(__file__).resolve().parents[1] / "include" / "mitra_gb300.h"
    text = header.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sym_[a-z0-9_]+)\s*\(", text)))


def bind(lib, prototypes=PROTOTYPES, prefix="sym_", rename=None):
    for name, res, args in prototypes:
        target = name if rename is None else rename(name)
        fn = getattr(lib, target)
        fn.restype = res
        fn.argtypes = args
    return lib


def library():
    """The CUDA library, loaded once.  Raises if it has not been built."""
    global _LIB
    if _LIB is None:
        path = Path(os.environ.get("MITRA_GB300_LIB", LIB_PATH))
        if not path.exists():
            raise RuntimeError(
                f"{path} is missing: build the CUDA library first "
                "(python -c 'import __graft_entry__ as g; g.build()')")
        _LIB = bind(C.CDLL(str(path)))
    return _LIB
