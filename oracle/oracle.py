"""ORACLE - test infrastructure only.

ctypes wrapper of oracle/_build/liboracle.so (the CPU restatement of the
reference's CPU backend, oracle/oracle.cpp) with the method names of the
reference's ``Backend`` (include/symmetry/pipeline.h:54-69), plus a runner
for the reference's own CPU library (oracle/_ref/ref_harness) where it has
been built.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg use this module, to check results.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile
from pathlib import Path

import numpy as np

from mitra_algo_gb300 import abi
from mitra_algo_gb300.types import (ClusterOutput, Features, Mesh, ModelContext, Options,
                                    Pairs, Rng, Topology, Votes, clusters_from_c,
                                    pairs_from_c, selection_from_c, verification_from_c,
                                    votes_from_c)

from . import symd

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
REF_HARNESS = HERE / "_ref" / "ref_harness"


def reference_tree():
    """The reference's source tree, or None where it is absent: the
    MITRA_REFERENCE_DIR environment variable, else the default that
    oracle/Makefile's recipe records (REF)."""
    path = os.environ.get("MITRA_REFERENCE_DIR")
    if not path:
        try:
            path = subprocess.run(["make", "-s", "--no-print-directory", "-C", str(HERE),
                                   "print-ref"], check=True, capture_output=True,
                                  text=True).stdout.strip()
        except (OSError, subprocess.CalledProcessError):
            return None
    tree = Path(path)
    return tree if (tree / "include" / "symmetry").is_dir() else None


_P = C.POINTER
_PROTOS = [
    ("oracle_last_error", C.c_char_p, []),
    ("oracle_release", None, [C.c_void_p]),
    ("oracle_rng_seed", None, [_P(abi.Rng), C.c_uint64]),
    ("oracle_rng_next", C.c_uint64, [_P(abi.Rng)]),
    ("oracle_triangle_distance2", C.c_double, [_P(C.c_double)]),
    ("oracle_sample_vertices", C.c_int, [_P(C.c_double), C.c_uint64, C.c_double, _P(abi.Rng),
                                         _P(C.c_int32), _P(C.c_uint64)]),
    ("oracle_curvature", C.c_int, [_P(abi.MeshView), _P(abi.TopologyView), _P(abi.Options),
                                   _P(abi.FeaturesOut)]),
    ("oracle_select", C.c_int, [_P(abi.MeshView), _P(abi.FeaturesView), _P(C.c_double),
                                C.c_uint64, _P(abi.Options), _P(abi.Rng), _P(abi.Selection)]),
    ("oracle_pairing", C.c_int, [_P(abi.MeshView), _P(abi.FeaturesView), _P(C.c_int32),
                                 C.c_uint64, _P(abi.ModelContext), _P(abi.Options),
                                 _P(abi.PairsOut)]),
    ("oracle_transformations", C.c_int, [_P(abi.MeshView), _P(abi.FeaturesView),
                                         _P(abi.PairsView), _P(abi.ModelContext),
                                         _P(abi.Options), _P(abi.VotesOut)]),
    ("oracle_clustering", C.c_int, [_P(abi.VotesView), _P(abi.ModelContext), _P(abi.Options),
                                    _P(abi.Rng), _P(abi.ClustersOut)]),
    ("oracle_clustering_stats", None, [_P(C.c_uint64), _P(C.c_uint64)]),
    ("oracle_verification", C.c_int, [_P(abi.MeshView), _P(abi.TopologyView),
                                      _P(abi.ClustersView), _P(abi.ModelContext),
                                      _P(abi.Options), _P(abi.VerificationOut)]),
]

_lib = None


def build(reference=False):
    """Compile the oracle (and, when the reference tree is present and
    `reference` is set, the reference harness) with oracle/Makefile."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    tree = reference_tree() if reference else None
    if tree:
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF={tree}"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        _lib = C.CDLL(str(LIB))
        for name, res, args in _PROTOS:
            fn = getattr(_lib, name)
            fn.restype, fn.argtypes = res, args
    return _lib


class OracleError(Exception):
    pass


def _check(status):
    if status == abi.OK:
        return
    msg = lib().oracle_last_error().decode()
    if status == abi.INVALID_ARGUMENT:
        raise ValueError(msg)
    if status == abi.OVERFLOW:
        raise OverflowError(msg)
    raise RuntimeError(msg)


class OracleRng(Rng):
    def __init__(self, seed: int = 42):
        self.state = abi.Rng()
        self._lib = None
        lib().oracle_rng_seed(C.byref(self.state), C.c_uint64(seed))

    def next(self):
        return int(lib().oracle_rng_next(C.byref(self.state)))


def rng(seed=42) -> Rng:
    return OracleRng(seed)


class OracleBackend:
    """CPU restatement of the reference CpuBackend (src/cpu/backend.cpp:5-32)."""

    def name(self):
        return "oracle-cpu"

    def curvature(self, mesh: Mesh, topo: Topology, options: Options) -> Features:
        f = Features.zeros(mesh.vertex_count)
        _check(lib().oracle_curvature(C.byref(mesh.view()), C.byref(topo.view()),
                                      C.byref(options.to_c()), C.byref(f.out_view())))
        return f

    def sample_vertices(self, weights, ratio: float, rng: Rng) -> np.ndarray:
        """The reference's sample_vertices (src/core/sampling.cpp:5-24)."""
        w = np.ascontiguousarray(weights, np.float64)
        out = np.empty(max(1, w.size), np.int32)
        count = C.c_uint64()
        lib().oracle_sample_vertices(w.ctypes.data_as(_P(C.c_double)), w.size, float(ratio),
                                     C.byref(rng.state), out.ctypes.data_as(_P(C.c_int32)),
                                     C.byref(count))
        return out[:count.value].copy()

    def select(self, mesh: Mesh, features: Features, weights, options: Options, rng: Rng):
        w = np.ascontiguousarray(weights, np.float64)
        out = abi.Selection()
        _check(lib().oracle_select(C.byref(mesh.view()), C.byref(features.view()),
                                   w.ctypes.data_as(_P(C.c_double)), w.size,
                                   C.byref(options.to_c()), C.byref(rng.state), C.byref(out)))
        try:
            return selection_from_c(out)
        finally:
            lib().oracle_release(out.storage)

    def pairing(self, mesh: Mesh, features: Features, selected, context: ModelContext,
                options: Options) -> Pairs:
        sel = np.ascontiguousarray(selected, np.int32)
        out = abi.PairsOut()
        _check(lib().oracle_pairing(C.byref(mesh.view()), C.byref(features.view()),
                                    sel.ctypes.data_as(_P(C.c_int32)), sel.size,
                                    C.byref(context.to_c()), C.byref(options.to_c()),
                                    C.byref(out)))
        try:
            return pairs_from_c(out)
        finally:
            lib().oracle_release(out.storage)

    def transformations(self, mesh: Mesh, features: Features, pairs: Pairs,
                        context: ModelContext, options: Options) -> Votes:
        out = abi.VotesOut()
        _check(lib().oracle_transformations(C.byref(mesh.view()), C.byref(features.view()),
                                            C.byref(pairs.view()), C.byref(context.to_c()),
                                            C.byref(options.to_c()), C.byref(out)))
        try:
            return votes_from_c(out)
        finally:
            lib().oracle_release(out.storage)

    def clustering(self, votes: Votes, context: ModelContext, options: Options,
                   rng: Rng) -> ClusterOutput:
        out = abi.ClustersOut()
        _check(lib().oracle_clustering(C.byref(votes.view()), C.byref(context.to_c()),
                                       C.byref(options.to_c()), C.byref(rng.state),
                                       C.byref(out)))
        try:
            return clusters_from_c(out)
        finally:
            lib().oracle_release(out.storage)

    @staticmethod
    def clustering_stats():
        t, e = C.c_uint64(), C.c_uint64()
        lib().oracle_clustering_stats(C.byref(t), C.byref(e))
        return int(t.value), int(e.value)

    def verification(self, mesh: Mesh, topo: Topology, clusters: ClusterOutput,
                     context: ModelContext, options: Options):
        view, keep = clusters.view()
        out = abi.VerificationOut()
        _check(lib().oracle_verification(C.byref(mesh.view()), C.byref(topo.view()),
                                         C.byref(view), C.byref(context.to_c()),
                                         C.byref(options.to_c()), C.byref(out)))
        del keep
        try:
            return verification_from_c(out)
        finally:
            lib().oracle_release(out.storage)

    @staticmethod
    def triangle_distance2(p, a, b, c):
        q = np.ascontiguousarray(np.concatenate([p, a, b, c]), np.float64)
        return float(lib().oracle_triangle_distance2(q.ctypes.data_as(_P(C.c_double))))


# ------------------------------------------------------- reference harness
def reference_available() -> bool:
    return REF_HARNESS.exists()


def run_reference(mode: str, arrays: dict) -> dict:
    """Run the reference's own CPU library (oracle/_ref/ref_harness) in
    `mode` on the named input arrays and return its named outputs."""
    if not REF_HARNESS.exists():
        raise FileNotFoundError("the reference harness has not been built (make -C oracle ref)")
    with tempfile.TemporaryDirectory() as d:
        src, dst = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
        symd.write(src, arrays)
        subprocess.run([str(REF_HARNESS), mode, src, dst], check=True)
        return symd.read(dst)
