"""Host data model of the symmetry hot path, in the reference's SoA layout.

Each class mirrors one storage type of the reference
(deoksieze/Mitra_algo include/symmetry/storage.h and pipeline.h): points are
(3, n) float64 arrays (one contiguous column per coordinate, like
``Points``), index columns are int32 (``Index``), CSR offsets uint64
(``Offset``).  ``ctypes`` views over these arrays are what the C ABI
(include/mitra_gb300.h) consumes, so no copy is made on the way in.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, replace

import numpy as np

from . import abi


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a if shape is None else a.reshape(shape)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _u64(a):
    return np.ascontiguousarray(a, dtype=np.uint64)


def _ptr(a, ctype):
    return a.ctypes.data_as(C.POINTER(ctype)) if a is not None and a.size else None


def points_view(p: np.ndarray) -> abi.PointsView:
    """View of a (3, n) float64 array (reference PointsView)."""
    n = p.shape[1] if p.ndim == 2 else 0
    return abi.PointsView(_ptr(p[0], C.c_double) if n else None,
                          _ptr(p[1], C.c_double) if n else None,
                          _ptr(p[2], C.c_double) if n else None, n)


@dataclass
class Options:
    """Reference ``Options`` (include/symmetry/options.h:5-12) with its defaults."""
    sample_ratio: float = 0.5
    prune: float = 0.85
    pair_threshold: float = 0.15
    bandwidth: float = 0.08
    verify_threshold: float = 0.025
    smoothing: int = 3
    subdivide: int = 0
    max_iterations: int = 100
    max_clusters: int = 20
    seed: int = 42
    max_pairs: int = 200000
    max_votes: int = 600000
    patching: bool = True

    def to_c(self) -> abi.Options:
        return abi.Options(self.sample_ratio, self.prune, self.pair_threshold,
                           self.bandwidth, self.verify_threshold, self.smoothing,
                           self.subdivide, self.max_iterations, self.max_clusters,
                           self.seed, self.max_pairs, self.max_votes,
                           1 if self.patching else 0)

    def with_(self, **kw) -> "Options":
        return replace(self, **kw)


@dataclass
class ModelContext:
    """Reference ``ModelContext`` (pipeline.h:30-33)."""
    box_size: float = 0.0
    center: tuple = (0.0, 0.0, 0.0)

    def to_c(self) -> abi.ModelContext:
        return abi.ModelContext(self.box_size, (C.c_double * 3)(*self.center))


@dataclass
class Mesh:
    """Reference ``Mesh``: vertices (3, n) float64, faces (3, f) int32."""
    vertices: np.ndarray
    faces: np.ndarray

    def __post_init__(self):
        self.vertices = _f64(self.vertices)
        self.faces = _i32(self.faces)
        if self.vertices.ndim != 2 or self.vertices.shape[0] != 3:
            raise ValueError("vertices must be (3, n)")
        if self.faces.ndim != 2 or self.faces.shape[0] != 3:
            raise ValueError("faces must be (3, f)")

    @property
    def vertex_count(self):
        return self.vertices.shape[1]

    def view(self) -> abi.MeshView:
        f = self.faces
        nf = f.shape[1]
        faces = abi.FacesView(_ptr(f[0], C.c_int32) if nf else None,
                              _ptr(f[1], C.c_int32) if nf else None,
                              _ptr(f[2], C.c_int32) if nf else None, nf)
        return abi.MeshView(points_view(self.vertices), faces)


@dataclass
class Csr:
    """Reference ``Csr``: uint64 offsets (rows + 1) and int32 indices."""
    offsets: np.ndarray
    indices: np.ndarray

    def __post_init__(self):
        self.offsets = _u64(self.offsets)
        self.indices = _i32(self.indices)

    @property
    def rows(self):
        return self.offsets.size - 1

    def row(self, i):
        return self.indices[self.offsets[i]:self.offsets[i + 1]]

    def view(self) -> abi.CsrView:
        return abi.CsrView(_ptr(self.offsets, C.c_uint64), self.rows,
                           _ptr(self.indices, C.c_int32))

    @staticmethod
    def from_rows(rows):
        off = np.zeros(len(rows) + 1, np.uint64)
        off[1:] = np.cumsum([len(r) for r in rows]) if rows else []
        idx = np.concatenate([np.asarray(r, np.int32) for r in rows]) if rows else np.zeros(0, np.int32)
        return Csr(off, idx)


@dataclass
class Topology:
    """Reference ``Topology`` (pipeline.h:21-29); edges are (e, 6) int32 rows
    ``lo, hi, a, b, face0, face1``."""
    normals: np.ndarray
    face_normals: np.ndarray
    weights: np.ndarray
    neighbors: Csr
    incident_faces: Csr
    edges: np.ndarray

    def view(self) -> abi.TopologyView:
        e = np.ascontiguousarray(self.edges, dtype=np.int32).reshape(-1, 6)
        self.edges = e
        return abi.TopologyView(points_view(self.normals), points_view(self.face_normals),
                                _ptr(self.weights, C.c_double), self.weights.size,
                                self.neighbors.view(), self.incident_faces.view(),
                                e.ctypes.data_as(C.POINTER(abi.Edge)) if e.size else None,
                                e.shape[0])


@dataclass
class Features:
    """Reference ``Features``: normal/dmin/dmax (3, n), kmin/kmax, valid (uint8)."""
    normal: np.ndarray
    dmin: np.ndarray
    dmax: np.ndarray
    kmin: np.ndarray
    kmax: np.ndarray
    valid: np.ndarray

    @staticmethod
    def zeros(n):
        return Features(np.zeros((3, n)), np.zeros((3, n)), np.zeros((3, n)),
                        np.zeros(n), np.zeros(n), np.zeros(n, np.uint8))

    def __len__(self):
        return self.kmin.size

    def view(self) -> abi.FeaturesView:
        for k in ("normal", "dmin", "dmax"):
            setattr(self, k, _f64(getattr(self, k)))
        self.kmin, self.kmax = _f64(self.kmin), _f64(self.kmax)
        self.valid = np.ascontiguousarray(self.valid, dtype=np.uint8)
        return abi.FeaturesView(points_view(self.normal), points_view(self.dmin),
                                points_view(self.dmax), _ptr(self.kmin, C.c_double),
                                _ptr(self.kmax, C.c_double), _ptr(self.valid, C.c_uint8),
                                self.kmin.size)

    def out_view(self) -> abi.FeaturesOut:
        n = self.kmin.size
        cols = [self.normal[0], self.normal[1], self.normal[2], self.dmin[0], self.dmin[1],
                self.dmin[2], self.dmax[0], self.dmax[1], self.dmax[2], self.kmin, self.kmax]
        return abi.FeaturesOut(*[_ptr(c, C.c_double) for c in cols],
                               _ptr(self.valid, C.c_uint8), n)


@dataclass
class Selection:
    sample: np.ndarray
    pruned: np.ndarray


@dataclass
class Pairs:
    a: np.ndarray
    b: np.ndarray

    def __post_init__(self):
        self.a, self.b = _i32(self.a), _i32(self.b)

    def __len__(self):
        return self.a.size

    def view(self) -> abi.PairsView:
        return abi.PairsView(_ptr(self.a, C.c_int32), _ptr(self.b, C.c_int32), self.a.size)


@dataclass
class Votes:
    """Reference ``Votes``: pair, kind (0 rigid, 1 reflection), rotation (9, q),
    translation (3, q), plane_normal (3, q), plane_offset (q), descriptor (12, q)."""
    pair: np.ndarray
    kind: np.ndarray
    rotation: np.ndarray
    translation: np.ndarray
    plane_normal: np.ndarray
    plane_offset: np.ndarray
    descriptor: np.ndarray

    def __len__(self):
        return self.pair.size

    def view(self) -> abi.VotesView:
        self.pair = _i32(self.pair)
        self.kind = np.ascontiguousarray(self.kind, dtype=np.uint8)
        for k in ("rotation", "translation", "plane_normal", "plane_offset", "descriptor"):
            setattr(self, k, _f64(getattr(self, k)))
        v = abi.VotesView()
        v.pair = _ptr(self.pair, C.c_int32)
        v.kind = _ptr(self.kind, C.c_uint8)
        for k in range(9):
            v.rotation[k] = _ptr(self.rotation[k], C.c_double)
        for k in range(3):
            v.translation[k] = _ptr(self.translation[k], C.c_double)
            v.plane_normal[k] = _ptr(self.plane_normal[k], C.c_double)
        v.plane_offset = _ptr(self.plane_offset, C.c_double)
        for k in range(12):
            v.descriptor[k] = _ptr(self.descriptor[k], C.c_double)
        v.count = self.pair.size
        return v


@dataclass
class ClusterOutput:
    """Reference ``ClusterOutput``: records, CSR of member votes,
    limited_iterations."""
    reflection: np.ndarray      # (c,) uint8
    rotation: np.ndarray        # (c, 9)
    translation: np.ndarray     # (c, 3)
    plane_normal: np.ndarray    # (c, 3)
    plane_offset: np.ndarray    # (c,)
    votes: Csr
    limited_iterations: int = 0

    def __len__(self):
        return self.reflection.size

    def records(self):
        n = len(self)
        recs = (abi.ClusterRecord * max(n, 1))()
        for i in range(n):
            recs[i].reflection = int(self.reflection[i])
            for k in range(9):
                recs[i].rotation[k] = float(self.rotation[i, k])
            for k in range(3):
                recs[i].translation[k] = float(self.translation[i, k])
                recs[i].plane_normal[k] = float(self.plane_normal[i, k])
            recs[i].plane_offset = float(self.plane_offset[i])
        return recs

    def view(self):
        recs = self.records()
        v = abi.ClustersView(recs, len(self), _ptr(self.votes.offsets, C.c_uint64),
                             _ptr(self.votes.indices, C.c_int32))
        return v, recs


@dataclass
class Verification:
    """Reference ``Verification``: per-cluster side CSRs, grouped patch CSRs,
    coverage and rms."""
    side_a: Csr
    side_b: Csr
    patches_a_groups: np.ndarray
    patches_a: Csr
    patches_b_groups: np.ndarray
    patches_b: Csr
    coverage: np.ndarray
    rms: np.ndarray


# ------------------------------------------------------------ result copies
def _arr(ptr, n, dtype):
    if n == 0 or not ptr:
        return np.zeros(0, dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


def selection_from_c(s: abi.Selection) -> Selection:
    return Selection(_arr(s.sample, s.sample_count, np.int32), _arr(s.pruned, s.pruned_count, np.int32))


def pairs_from_c(p: abi.PairsOut) -> Pairs:
    return Pairs(_arr(p.a, p.count, np.int32), _arr(p.b, p.count, np.int32))


def votes_from_c(v: abi.VotesOut) -> Votes:
    n = v.count
    return Votes(_arr(v.pair, n, np.int32), _arr(v.kind, n, np.uint8),
                 np.stack([_arr(v.rotation[k], n, np.float64) for k in range(9)]) if n else np.zeros((9, 0)),
                 np.stack([_arr(v.translation[k], n, np.float64) for k in range(3)]) if n else np.zeros((3, 0)),
                 np.stack([_arr(v.plane_normal[k], n, np.float64) for k in range(3)]) if n else np.zeros((3, 0)),
                 _arr(v.plane_offset, n, np.float64),
                 np.stack([_arr(v.descriptor[k], n, np.float64) for k in range(12)]) if n else np.zeros((12, 0)))


def clusters_from_c(c: abi.ClustersOut) -> ClusterOutput:
    n = c.count
    refl = np.zeros(n, np.uint8)
    rot = np.zeros((n, 9))
    tr = np.zeros((n, 3))
    pn = np.zeros((n, 3))
    off = np.zeros(n)
    for i in range(n):
        r = c.records[i]
        refl[i] = r.reflection
        rot[i] = list(r.rotation)
        tr[i] = list(r.translation)
        pn[i] = list(r.plane_normal)
        off[i] = r.plane_offset
    offsets = _arr(c.vote_offsets, n + 1, np.uint64) if n else np.zeros(1, np.uint64)
    total = int(offsets[-1]) if n else 0
    return ClusterOutput(refl, rot, tr, pn, off, Csr(offsets, _arr(c.vote_indices, total, np.int32)),
                         int(c.limited_iterations))


def verification_from_c(v: abi.VerificationOut) -> Verification:
    n = v.cluster_count

    def side(off_ptr, idx_ptr):
        off = _arr(off_ptr, n + 1, np.uint64) if True else None
        if off.size == 0:
            off = np.zeros(1, np.uint64)
        return Csr(off, _arr(idx_ptr, int(off[-1]), np.int32))

    def patches(g: abi.GroupedCsr):
        groups = _arr(g.groups, n + 1, np.uint64)
        if groups.size == 0:
            groups = np.zeros(1, np.uint64)
        offsets = _arr(g.offsets, g.rows + 1, np.uint64)
        return groups, Csr(offsets, _arr(g.indices, int(offsets[-1]) if offsets.size else 0, np.int32))

    ga, pa = patches(v.patches_a)
    gb, pb = patches(v.patches_b)
    return Verification(side(v.side_a_offsets, v.side_a), side(v.side_b_offsets, v.side_b),
                        ga, pa, gb, pb, _arr(v.coverage, n, np.float64), _arr(v.rms, n, np.float64))


class Rng:
    """``std::mt19937_64`` state as libstdc++ streams it (312 words + index),
    carried between select() and clustering() like the reference's engine."""

    def __init__(self, seed: int = 42, lib=None):
        self.state = abi.Rng()
        self._lib = lib
        (lib or abi.library()).sym_rng_seed(C.byref(self.state), C.c_uint64(seed))

    def next(self) -> int:
        return int((self._lib or abi.library()).sym_rng_next(C.byref(self.state)))

    def words(self):
        return np.array(list(self.state.words), np.uint64), int(self.state.index)

    def copy(self) -> "Rng":
        r = Rng.__new__(Rng)
        r.state = abi.Rng()
        C.memmove(C.byref(r.state), C.byref(self.state), C.sizeof(abi.Rng))
        r._lib = self._lib
        return r

    def __eq__(self, other):
        return bytes(self.state) == bytes(other.state)

    def text(self) -> str:
        """The engine as ``operator<<`` writes it."""
        return " ".join(str(w) for w in self.state.words) + " " + str(self.state.index)
