"""Python mirror of the reference's ``Backend`` over the GB300 C ABI.

``Gb300Backend`` has the six stage methods of the reference's
``symmetry::Backend`` (deoksieze/Mitra_algo include/symmetry/pipeline.h:54-69)
with the same argument meaning, host-owned results and error behaviour:
``ValueError`` for the reference's ``std::invalid_argument``,
``OverflowError`` for ``std::overflow_error`` and ``RuntimeError`` (message
text included, e.g. "Pair budget exceeded; ...") for ``std::runtime_error``.
Every method runs the hand-written sm_103a kernels of
``_lib/libmitra_gb300.so``; there is no CPU fallback.  ``detect`` strings the
stages together like the reference's ``detect()`` (src/core/pipeline.cpp).
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field

import numpy as np

from . import abi
from .mesh import Prepared, prepare
from .types import (ClusterOutput, Csr, Features, Mesh, ModelContext, Options, Pairs, Rng,
                    Selection, Topology, Verification, Votes, clusters_from_c, pairs_from_c,
                    points_view, selection_from_c, verification_from_c, votes_from_c)


class DeviceTimeout(RuntimeError):
    """A bounded device-side loop gave up (the kernel returned an error
    status instead of spinning)."""


def _raise(status: int):
    msg = abi.library().sym_last_error().decode()
    if status == abi.INVALID_ARGUMENT:
        raise ValueError(msg)
    if status == abi.OVERFLOW:
        raise OverflowError(msg)
    if status == abi.DEVICE_TIMEOUT:
        raise DeviceTimeout(msg)
    raise RuntimeError(msg)


def _check(status: int):
    if status != abi.OK:
        _raise(status)


KERNELS = {"epanechnikov": 0, "gaussian": 1}  # SYM_KERNEL_*
SAMPLE_ON_DEVICE = 2 ** 64 - 1  # SYM_SAMPLE_ON_DEVICE

# sym_fast_options' launch-shape fields, in their order (0 = the default)
TUNING_KEYS = ("vote_bits", "simt_blocks_per_sm", "tc_ctas_per_sm", "check_interval")


class Gb300Backend:
    """The GB300 backend: one device, one stream, one reusable workspace."""

    def __init__(self, device: int = 0, profile: bool = False):
        self._lib = abi.library()
        self._device = device
        self._workers = []  # contexts of sym_detect_fast_batch, created on first use
        ctx = C.c_void_p()
        _check(self._lib.sym_context_create(device, C.byref(ctx)))
        self._ctx = ctx
        if profile:
            _check(self._lib.sym_set_profiling(ctx, 1))

    def close(self):
        for w in getattr(self, "_workers", []):
            self._lib.sym_context_destroy(w)
        self._workers = []
        if getattr(self, "_ctx", None):
            self._lib.sym_context_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def name(self) -> str:
        return self._lib.sym_backend_name().decode()

    # ----------------------------------------------------------- stages
    def curvature(self, mesh: Mesh, topology: Topology, options: Options) -> Features:
        f = Features.zeros(mesh.vertex_count)
        _check(self._lib.sym_curvature(self._ctx, C.byref(mesh.view()), C.byref(topology.view()),
                                       C.byref(options.to_c()), C.byref(f.out_view())))
        return f

    def select(self, mesh: Mesh, features: Features, weights, options: Options,
               rng: Rng) -> Selection:
        w = np.ascontiguousarray(weights, np.float64)
        out = abi.Selection()
        _check(self._lib.sym_select(self._ctx, C.byref(mesh.view()), C.byref(features.view()),
                                    w.ctypes.data_as(C.POINTER(C.c_double)), w.size,
                                    C.byref(options.to_c()), C.byref(rng.state), C.byref(out)))
        try:
            return selection_from_c(out)
        finally:
            self._lib.sym_selection_release(C.byref(out))

    def pairing(self, mesh: Mesh, features: Features, selected, context: ModelContext,
                options: Options) -> Pairs:
        sel = np.ascontiguousarray(selected, np.int32)
        out = abi.PairsOut()
        _check(self._lib.sym_pairing(self._ctx, C.byref(mesh.view()), C.byref(features.view()),
                                     sel.ctypes.data_as(C.POINTER(C.c_int32)), sel.size,
                                     C.byref(context.to_c()), C.byref(options.to_c()),
                                     C.byref(out)))
        try:
            return pairs_from_c(out)
        finally:
            self._lib.sym_pairs_release(C.byref(out))

    def transformations(self, mesh: Mesh, features: Features, pairs: Pairs,
                        context: ModelContext, options: Options) -> Votes:
        out = abi.VotesOut()
        _check(self._lib.sym_transformations(self._ctx, C.byref(mesh.view()),
                                             C.byref(features.view()), C.byref(pairs.view()),
                                             C.byref(context.to_c()), C.byref(options.to_c()),
                                             C.byref(out)))
        try:
            return votes_from_c(out)
        finally:
            self._lib.sym_votes_release(C.byref(out))

    def clustering(self, votes: Votes, context: ModelContext, options: Options,
                   rng: Rng) -> ClusterOutput:
        out = abi.ClustersOut()
        _check(self._lib.sym_clustering(self._ctx, C.byref(votes.view()), C.byref(context.to_c()),
                                        C.byref(options.to_c()), C.byref(rng.state),
                                        C.byref(out)))
        try:
            return clusters_from_c(out)
        finally:
            self._lib.sym_clusters_release(C.byref(out))

    def verification(self, mesh: Mesh, topology: Topology, clusters: ClusterOutput,
                     context: ModelContext, options: Options) -> Verification:
        view, keep = clusters.view()
        out = abi.VerificationOut()
        _check(self._lib.sym_verification(self._ctx, C.byref(mesh.view()),
                                          C.byref(topology.view()), C.byref(view),
                                          C.byref(context.to_c()), C.byref(options.to_c()),
                                          C.byref(out)))
        del keep
        try:
            return verification_from_c(out)
        finally:
            self._lib.sym_verification_release(C.byref(out))

    def verification_resident(self, mesh: "ResidentMesh", clusters: ClusterOutput,
                              options: Options):
        """Backend::verification on a resident mesh (sym_verification_resident):
        the same result as verification() on the mesh's host arrays; also
        returns how many queries went to the reference-order BVH."""
        view, keep = clusters.view()
        out = abi.VerificationOut()
        undecided = C.c_uint64(0)
        _check(self._lib.sym_verification_resident(self._ctx, mesh.handle, C.byref(view),
                                                   C.byref(options.to_c()), C.byref(out),
                                                   C.byref(undecided)))
        del keep
        try:
            return verification_from_c(out), int(undecided.value)
        finally:
            self._lib.sym_verification_release(C.byref(out))

    def triangle_distances(self, queries) -> np.ndarray:
        q = np.ascontiguousarray(queries, np.float64).reshape(-1)
        n = q.size // 12
        out = np.zeros(n)
        _check(self._lib.sym_triangle_distances(self._ctx, q.ctypes.data_as(C.POINTER(C.c_double)),
                                                n, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    # ------------------------------------------- throughput extension
    @property
    def stream_handle(self) -> int:
        """The context's cudaStream_t as an integer."""
        return int(self._lib.sym_context_stream(self._ctx) or 0)

    def load_mesh(self, prepared: Prepared) -> "ResidentMesh":
        return ResidentMesh(self, prepared)

    def prepare(self, mesh: Mesh, options: Options) -> Prepared:
        """The reference's prepare() (no subdivision) on the GPU, sym_prepare:
        bit-exact with mesh.prepare."""
        view = mesh.view()
        out = abi.PreparedOut()
        _check(self._lib.sym_prepare(self._ctx, C.byref(view), C.byref(options.to_c()),
                                     C.byref(out)))
        try:
            nv, nf, ne = int(out.vertex_count), int(out.face_count), int(out.edge_count)

            def arr(ptr, n, dtype):
                return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True) if n else \
                    np.zeros(0, dtype)
            faces = np.stack([arr(out.faces[k], nf, np.int32) for k in range(3)])
            normals = np.stack([arr(out.normals[k], nv, np.float64) for k in range(3)])
            fnorm = np.stack([arr(out.face_normals[k], nf, np.float64) for k in range(3)])
            weights = arr(out.weights, nv, np.float64)
            noff = arr(out.neighbor_offsets, nv + 1, np.uint64)
            nidx = arr(out.neighbor_indices, int(noff[-1]), np.int32)
            ioff = arr(out.incident_offsets, nv + 1, np.uint64)
            iidx = arr(out.incident_indices, int(ioff[-1]), np.int32)
            edges = np.ctypeslib.as_array(C.cast(out.edges, C.POINTER(C.c_int32)),
                                          shape=(ne * 6,)).reshape(ne, 6).copy() if ne else \
                np.zeros((0, 6), np.int32)
            ctx = ModelContext(float(out.context.box_size), tuple(float(c) for c in out.context.center))
            return Prepared(Mesh(mesh.vertices.copy(), faces),
                            Topology(normals, fnorm, weights, Csr(noff, nidx), Csr(ioff, iidx), edges),
                            ctx, int(out.rejected_faces))
        finally:
            self._lib.sym_prepared_release(C.byref(out))

    def load_mesh_raw(self, mesh: Mesh, options: Options) -> "ResidentMesh":
        """A resident mesh prepared on the GPU (sym_mesh_load_raw): only the
        vertices and faces cross from the host."""
        return ResidentMesh(self, None, raw=(mesh, options))

    @staticmethod
    def _fast_options(precision, seeds, seed_rng, max_iterations, polish_iterations,
                      reference_seeds, verify, mode="rigid", vote_cap=0, refine=0, tuning=None,
                      kernel="epanechnikov"):
        if mode not in ("rigid", "reflection"):
            raise ValueError(f"unknown detection mode {mode!r}")
        t = dict(tuning or {})
        unknown = set(t) - set(TUNING_KEYS)
        if unknown:
            raise ValueError(f"unknown tuning parameters {sorted(unknown)}")
        return abi.FastOptions(abi.MS_BF16_REFINED if precision == "bf16" else abi.MS_FP32, seeds,
                               seed_rng, max_iterations, polish_iterations, reference_seeds,
                               1 if verify else 0, 1 if mode == "reflection" else 0,
                               int(vote_cap), int(refine), *(int(t.get(k, 0)) for k in TUNING_KEYS),
                               KERNELS[kernel])

    def detect_fast(self, mesh: "ResidentMesh", sample, options: Options, precision="bf16",
                    seeds=2048, seed_rng=7, max_iterations=100, polish_iterations=100,
                    reference_seeds=0, verify=True, mode="rigid", vote_cap=0,
                    refine=0, tuning=None, kernel="epanechnikov") -> dict:
        """Throughput pipeline on a resident mesh (no reference counterpart);
        mode "rigid" (rotation + translation votes) or "reflection" (plane
        votes); vote_cap > 0 subsamples the votes that enter the mean shift
        to about that many; refine > 0 runs that many FP64 ICP passes on the
        verified modes' motions; `tuning` sets the mean shift's launch
        shapes (keys TUNING_KEYS, see autotune.py); kernel "epanechnikov"
        (the reference's weights) or "gaussian" (2^(-8 d^2/h^2) - 2^-8, zero
        at the cut h).  `sample` None draws the
        area-weighted sample on the device from options.seed, as detect()
        does (sym_detect_fast_sampled)."""
        fo = self._fast_options(precision, seeds, seed_rng, max_iterations, polish_iterations,
                                reference_seeds, verify, mode, vote_cap, refine, tuning, kernel)
        res = abi.FastResult()
        if sample is None:
            _check(self._lib.sym_detect_fast_sampled(self._ctx, mesh.handle,
                                                     C.byref(options.to_c()), C.byref(fo),
                                                     C.byref(res)))
            return self._fast_dict(res)
        sample = np.ascontiguousarray(sample, np.int32)
        _check(self._lib.sym_detect_fast(self._ctx, mesh.handle,
                                         sample.ctypes.data_as(C.POINTER(C.c_int32)), sample.size,
                                         C.byref(options.to_c()), C.byref(fo), C.byref(res)))
        return self._fast_dict(res)

    def refine_transforms(self, mesh: "ResidentMesh", options: Options, records,
                          iterations: int) -> dict:
        """sym_refine_transforms: `records` = [(reflection, rotation (9),
        translation (3), plane_normal (3), plane_offset), ...] refined by
        `iterations` FP64 ICP passes against the resident mesh, then
        verified.  Returns the refined motions with coverage, rms, patches."""
        n = len(records)
        recs = (abi.ClusterRecord * max(n, 1))()
        for r, (refl, rot, tr, nrm, off) in zip(recs, records):
            r.reflection = int(refl)
            for k in range(9):
                r.rotation[k] = float(rot[k])
            for k in range(3):
                r.translation[k] = float(tr[k])
                r.plane_normal[k] = float(nrm[k])
            r.plane_offset = float(off)
        cov, rms = np.zeros(max(n, 1)), np.zeros(max(n, 1))
        patches = np.zeros(2 * max(n, 1), np.uint32)
        _check(self._lib.sym_refine_transforms(
            self._ctx, mesh.handle, C.byref(options.to_c()), recs, n, int(iterations),
            cov.ctypes.data_as(C.POINTER(C.c_double)), rms.ctypes.data_as(C.POINTER(C.c_double)),
            patches.ctypes.data_as(C.POINTER(C.c_uint32))))
        return {"rotation": np.array([list(r.rotation) for r in recs[:n]]).reshape(n, 9),
                "translation": np.array([list(r.translation) for r in recs[:n]]).reshape(n, 3),
                "plane_normal": np.array([list(r.plane_normal) for r in recs[:n]]).reshape(n, 3),
                "plane_offset": np.array([r.plane_offset for r in recs[:n]]),
                "coverage": cov[:n], "rms": rms[:n],
                "patches": [(int(patches[2 * i]), int(patches[2 * i + 1])) for i in range(n)]}

    def sample_vertices(self, weights, ratio: float, rng: Rng) -> np.ndarray:
        """sym_sample_vertices: the reference's sample_vertices
        (src/core/sampling.cpp:5-24) on the GPU; advances `rng` like it."""
        w = np.ascontiguousarray(weights, np.float64)
        out = np.empty(max(1, w.size), np.int32)
        count = C.c_uint64()
        _check(self._lib.sym_sample_vertices(self._ctx, w.ctypes.data_as(C.POINTER(C.c_double)),
                                             w.size, float(ratio), C.byref(rng.state),
                                             out.ctypes.data_as(C.POINTER(C.c_int32)),
                                             C.byref(count)))
        return out[:count.value].copy()

    def detect_fast_fused(self, jobs, precision="bf16", seeds=2048, seed_rng=7,
                          max_iterations=100, polish_iterations=100, verify=True,
                          mode="rigid", tuning=None, kernel="epanechnikov", refine=0):
        """sym_detect_fast_fused over `jobs` = [(ResidentMesh, sample, Options), ...]
        (a sample None is drawn on the device; `mode` may be one mode for all
        or a list, one per job): one mean shift for every mesh's seeds.
        Returns (one result dict per job as detect_fast gives it, the batch's
        statistics)."""
        modes = mode if isinstance(mode, (list, tuple)) else [mode] * len(jobs)
        keep = []
        items = (abi.BatchItem * max(len(jobs), 1))()
        results = [abi.FastResult() for _ in jobs]
        for it, (mesh, sample, options), res, md in zip(items, jobs, results, modes):
            fo = self._fast_options(precision, seeds, seed_rng, max_iterations, polish_iterations,
                                    0, verify, md, refine=refine, tuning=tuning, kernel=kernel)
            opts = options.to_c()
            keep += [fo, opts]
            it.mesh = mesh.handle
            if sample is None:
                it.sample = None
                it.sample_count = SAMPLE_ON_DEVICE
            else:
                sample = np.ascontiguousarray(sample, np.int32)
                keep.append(sample)
                it.sample = sample.ctypes.data_as(C.POINTER(C.c_int32))
                it.sample_count = sample.size
            it.options = C.pointer(opts)
            it.fast = C.pointer(fo)
            it.out = C.pointer(res)
        stats = abi.FusedStats()
        _check(self._lib.sym_detect_fast_fused(self._ctx, items, len(jobs), C.byref(stats)))
        return ([self._fast_dict(r) for r in results],
                {f: getattr(stats, f) for f, _ in abi.FusedStats._fields_})

    def detect_fast_batch(self, jobs, workers=4, precision="bf16", seeds=2048, seed_rng=7,
                          max_iterations=100, polish_iterations=100, verify=True,
                          mode="rigid", tuning=None) -> list:
        """sym_detect_fast_batch over `jobs` = [(ResidentMesh, sample, Options), ...]
        (a sample None is drawn on the device, as detect_fast does it):
        `workers` meshes in flight at a time, each on its own context (stream
        and workspace), the contexts kept for later calls.  Returns one result
        dict per job, as detect_fast gives it."""
        while len(self._workers) < workers:
            w = C.c_void_p()
            _check(self._lib.sym_context_create(self._device, C.byref(w)))
            self._workers.append(w)
        fo = self._fast_options(precision, seeds, seed_rng, max_iterations, polish_iterations, 0,
                                verify, mode, tuning=tuning)
        keep = []
        items = (abi.BatchItem * len(jobs))()
        results = [abi.FastResult() for _ in jobs]
        for it, (mesh, sample, options), res in zip(items, jobs, results):
            opts = options.to_c()
            keep.append(opts)
            it.mesh = mesh.handle
            if sample is None:  # drawn on the device from options.seed
                it.sample = None
                it.sample_count = SAMPLE_ON_DEVICE
            else:
                sample = np.ascontiguousarray(sample, np.int32)
                keep.append(sample)
                it.sample = sample.ctypes.data_as(C.POINTER(C.c_int32))
                it.sample_count = sample.size
            it.options = C.pointer(opts)
            it.fast = C.pointer(fo)
            it.out = C.pointer(res)
        pool = (C.c_void_p * workers)(*[w.value for w in self._workers[:workers]])
        _check(self._lib.sym_detect_fast_batch(pool, workers, items, len(jobs)))
        return [self._fast_dict(r) for r in results]

    @staticmethod
    def _fast_dict(res) -> dict:
        n = int(res.clusters)
        out = {k: getattr(res, k) for k in ("sampled", "pruned", "pairs", "votes", "modes",
                                            "clusters", "iterations", "polish_iterations",
                                            "mode_error_max",
                                            "mode_error_mean", "modes_compared", "modes_within",
                                            "mean_shift_pairs",
                                            "seed_iterations", "launches", "h2d_bytes",
                                            "d2h_bytes", "bulk_ms", "polish_ms")}
        out["bulk_trace"] = [int(x) for x in res.bulk_trace][:max(0, res.iterations)]
        out["polish_trace"] = [int(x) for x in res.polish_trace][:max(0, res.polish_iterations)]
        out["stage_ms"] = dict(zip(abi.STAGES, list(res.stage_ms)))
        out["support"] = list(res.support)[:n]
        out["coverage"] = list(res.coverage)[:n]
        out["rms"] = list(res.rms)[:n]
        out["patches"] = [(res.patches[2 * i], res.patches[2 * i + 1]) for i in range(n)]
        out["precise"] = [bool(res.precise[i]) for i in range(n)]
        out["tc_launches"] = int(res.tc_launches)
        out["tc_kernel_ms"] = float(res.tc_kernel_ms)
        out["tc_evaluations"] = float(res.tc_evaluations)
        out["verify_undecided"] = int(res.verify_undecided)
        out["verify_fp64_rows"] = int(res.verify_fp64_rows)
        for k in ("seeds_compared", "seeds_within", "seeds_settled", "seeds_unconverged"):
            out[k] = int(getattr(res, k))
        for k in ("mode_error_all_max", "mode_error_all_mean", "mode_error_settled_max",
                  "mode_error_unconverged_max", "transform_error_max",
                  "transform_error_refined_max"):
            out[k] = float(getattr(res, k))
        out["transform_error"] = list(res.transform_error)[:n]
        out["transform_error_refined"] = list(res.transform_error_refined)[:n]
        out["rotation"] = [list(res.records[i].rotation) for i in range(n)]
        out["translation"] = [list(res.records[i].translation) for i in range(n)]
        out["reflection"] = [bool(res.records[i].reflection) for i in range(n)]
        out["plane_normal"] = [list(res.records[i].plane_normal) for i in range(n)]
        out["plane_offset"] = [float(res.records[i].plane_offset) for i in range(n)]
        return out

    def meanshift6(self, votes, seeds, bandwidth, precision="fp32", max_iterations=100,
                   polish_iterations=100, kernel="epanechnikov"):
        """Mean-shift of the seed votes over 6-D votes (q x 6); returns the
        final means (k x 6), per-seed state and the (approach, polish)
        iteration counts.  precision: "fp32" (FP32 approach), "bf16" (BF16
        tensor-core approach), both followed by the same FP32 polish, or
        "fp64" (both phases in FP64); kernel "epanechnikov" or "gaussian"."""
        v = np.ascontiguousarray(votes, np.float64).reshape(-1, 6)
        s = np.ascontiguousarray(seeds, np.int64)
        means = np.zeros((s.size, 6))
        state = np.zeros(s.size, np.uint8)
        iters = (C.c_int32 * 2)()
        code = {"fp32": abi.MS_FP32, "bf16": abi.MS_BF16_REFINED, "fp64": abi.MS_FP64}[precision]
        _check(self._lib.sym_meanshift6(self._ctx, v.ctypes.data_as(C.POINTER(C.c_double)),
                                        v.shape[0], s.ctypes.data_as(C.POINTER(C.c_int64)), s.size,
                                        bandwidth, code, max_iterations, polish_iterations,
                                        KERNELS[kernel],
                                        means.ctypes.data_as(C.POINTER(C.c_double)),
                                        state.ctypes.data_as(C.POINTER(C.c_uint8)), iters))
        return means, state, (iters[0], iters[1])

    def fast_votes(self, mesh: Mesh, features: Features, pairs: Pairs, context: ModelContext,
                   mode="rigid"):
        """The throughput path's FP32 vote records for `pairs` (sym_fast_votes):
        (records (q, 8) float32, pair index of each record (q,))."""
        if mode not in ("rigid", "reflection"):
            raise ValueError(f"unknown detection mode {mode!r}")
        n = len(pairs)
        out = np.zeros((max(2 * n, 1), 8), np.float32)
        pair_of = np.zeros(max(2 * n, 1), np.int32)
        count = C.c_uint64(0)
        pts = points_view(mesh.vertices)
        _check(self._lib.sym_fast_votes(self._ctx, C.byref(pts), C.byref(features.view()),
                                        C.byref(pairs.view()), C.byref(context.to_c()),
                                        1 if mode == "reflection" else 0,
                                        out.ctypes.data_as(C.POINTER(C.c_float)),
                                        pair_of.ctypes.data_as(C.POINTER(C.c_int32)),
                                        C.byref(count)))
        q = int(count.value)
        return out[:q].copy(), pair_of[:q].copy()

    def wait_selftest(self, which: str, limit: int):
        """sym_wait_selftest: which = "tensor" (the tensor kernels' barrier
        wait, limit in ns) or "union" (the verification's union-find retries);
        raises DeviceTimeout when the wait runs out, else returns the
        union-find's component count (None for "tensor")."""
        comps = C.c_uint64(0)
        _check(self._lib.sym_wait_selftest(self._ctx, {"tensor": 0, "union": 1}[which],
                                           int(limit), C.byref(comps)))
        return int(comps.value) if which == "union" else None

    def tc_selftest(self, a1, b1, a2, b2):
        """Tensor-core path check: returns (A1 . B1^T, A2 . B2^T) computed by
        tcgen05 from BF16 bit patterns (uint16 arrays 128x16, 128x16, 128x128,
        16x128)."""
        arrs = [np.ascontiguousarray(x, np.uint16) for x in (a1, b1, a2, b2)]
        d = np.zeros((128, 128), np.float32)
        acc = np.zeros((128, 16), np.float32)
        p16 = C.POINTER(C.c_uint16)
        _check(self._lib.sym_tc_selftest(self._ctx, *[x.ctypes.data_as(p16) for x in arrs],
                                         d.ctypes.data_as(C.POINTER(C.c_float)),
                                         acc.ctypes.data_as(C.POINTER(C.c_float))))
        return d, acc

    def take_metrics(self):
        buf = (abi.Metric * 64)()
        n = self._lib.sym_take_metrics(self._ctx, buf, 64)
        return [{f: (getattr(buf[i], f).decode() if f == "stage" else getattr(buf[i], f))
                 for f, _ in abi.Metric._fields_} for i in range(n)]


@dataclass
class Result:
    """Reference ``Result`` (pipeline.h:72-81)."""
    prepared: Prepared
    options: Options
    features: Features = None
    sample: np.ndarray = None
    pruned: np.ndarray = None
    pairs: Pairs = None
    votes: Votes = None
    clusters: ClusterOutput = None
    verification: Verification = None
    timings: list = field(default_factory=list)


def detect(mesh: Mesh, options: Options, backend, progress=None) -> Result:
    """Reference ``detect`` (src/core/pipeline.cpp:5-52): prepare, then the six
    stages in order with one RNG threaded through select and clustering."""
    clock = time.perf_counter()
    p = prepare(mesh, options)
    r = Result(p, options)

    def timed(stage):
        nonlocal clock
        now = time.perf_counter()
        r.timings.append((stage, (now - clock) * 1e3))
        if progress:
            progress(stage, r.timings[-1][1])
        clock = now

    rng = Rng(options.seed, getattr(backend, "_lib", None))
    timed("prepare")
    r.features = backend.curvature(p.mesh, p.topology, options)
    timed("curvature")
    s = backend.select(p.mesh, r.features, p.topology.weights, options, rng)
    r.sample, r.pruned = s.sample, s.pruned
    timed("sample_prune")
    r.pairs = backend.pairing(p.mesh, r.features, r.pruned, p.context, options)
    timed("pairing")
    r.votes = backend.transformations(p.mesh, r.features, r.pairs, p.context, options)
    timed("transformation")
    r.clusters = backend.clustering(r.votes, p.context, options, rng)
    timed("mean_shift")
    if options.patching:
        r.verification = backend.verification(p.mesh, p.topology, r.clusters, p.context, options)
    timed("verification")
    return r


class ResidentMesh:
    """A prepared mesh uploaded once to the device (sym_mesh_load)."""

    def __init__(self, backend: Gb300Backend, prepared: Prepared, raw=None):
        self._lib = backend._lib
        self._backend = backend  # its context outlives the mesh
        self.prepared = prepared
        h = C.c_void_p()
        if raw is not None:  # prepared on the GPU from the raw mesh
            mesh, options = raw
            self._raw = mesh
            view = mesh.view()
            _check(self._lib.sym_mesh_load_raw(backend._ctx, C.byref(view),
                                               C.byref(options.to_c()), C.byref(h)))
        else:
            self._views = (prepared.mesh.view(), prepared.topology.view(),
                           prepared.context.to_c())
            _check(self._lib.sym_mesh_load(backend._ctx, C.byref(self._views[0]),
                                           C.byref(self._views[1]), C.byref(self._views[2]),
                                           C.byref(h)))
        self.handle = h

    @property
    def vertex_count(self) -> int:
        m = self._raw if self.prepared is None else self.prepared.mesh
        return int(m.vertex_count)

    def bytes(self) -> int:
        """Host-to-device bytes of one load."""
        if self.prepared is None:
            return int(self._raw.vertices.nbytes + self._raw.faces.nbytes)
        p = self.prepared
        return int(p.mesh.vertices.nbytes + p.mesh.faces.nbytes + p.topology.normals.nbytes +
                   p.topology.face_normals.nbytes + p.topology.weights.nbytes +
                   p.topology.neighbors.offsets.nbytes + p.topology.neighbors.indices.nbytes +
                   np.asarray(p.topology.edges).nbytes)

    def close(self):
        if self.handle:
            self._lib.sym_mesh_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
