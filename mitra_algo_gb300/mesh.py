"""Mesh preparation and seeded synthetic meshes (host pre-step of the path).

``prepare`` restates the reference's host pre-step
(deoksieze/Mitra_algo src/core/prepare.cpp:13-149) in vectorised numpy with
the same FP64 operation order, so the topology it returns is bit-identical to
the reference's (pinned by tests/golden).  It builds the ``Topology`` the
GPU stages consume: face and vertex normals, area weights, the sorted
(lo, hi) edge table, neighbour and incident-face CSRs, plus ``ModelContext``.

The generators build the seeded inputs of the benchmark workloads: a mirrored
Gaussian-bump heightfield and a bump-displaced icosphere with a 5-fold motif
and a partial translated copy.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .types import Csr, Mesh, ModelContext, Options, Topology

EPS = 1e-14


@dataclass
class Prepared:
    mesh: Mesh
    topology: Topology
    context: ModelContext
    rejected_faces: int = 0
    nonmanifold_edges: int = 0
    orientation_conflicts: int = 0


def validate_options(o: Options):
    """Reference validate_options (src/core/prepare.cpp:85-101)."""
    imax = 2 ** 31 - 1
    if o.max_pairs > imax or o.max_votes > imax:
        raise ValueError("Pair/vote budgets exceed 32-bit ID capacity")
    ok = (0 < o.sample_ratio <= 1 and 0 < o.prune < 1 and 0 < o.pair_threshold <= 1
          and 0 < o.bandwidth <= 2 and 0 < o.verify_threshold < 0.5
          and 0 <= o.smoothing <= 1000 and 0 <= o.subdivide <= 3
          and 1 <= o.max_iterations <= 10000 and 1 <= o.max_clusters <= 1000
          and o.max_pairs >= 1 and o.max_votes >= 1)
    if not ok:
        raise RuntimeError("Invalid parameter range; see --help")


def _cross(a, b):
    return np.stack([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2],
                     a[0] * b[1] - a[1] * b[0]])


def _norm(a):
    return np.sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2])


def _unit(a):
    n = _norm(a)
    with np.errstate(divide="ignore", invalid="ignore"):
        r = a * (1.0 / n)  # Vec / s multiplies by the reciprocal (math.cpp:11)
    return np.where(n > EPS, r, 0.0)


def _subdivide(v: np.ndarray, f: np.ndarray):
    """Midpoint subdivision, reference prepare.cpp:60-84 (first-use vertex order)."""
    if f.shape[1] > 500000:
        raise RuntimeError("Subdivision face budget exceeded")
    verts = [tuple(p) for p in v.T]
    mid = {}

    def midpoint(a, b):
        key = (a, b) if a < b else (b, a)
        got = mid.get(key)
        if got is not None:
            return got
        idx = len(verts)
        pa, pb = verts[a], verts[b]
        verts.append(tuple((pa[k] + pb[k]) * 0.5 for k in range(3)))
        mid[key] = idx
        return idx

    out = []
    for f0, f1, f2 in f.T.tolist():
        a = midpoint(f0, f1)
        b = midpoint(f1, f2)
        c = midpoint(f2, f0)
        out += [(f0, a, c), (a, f1, b), (c, b, f2), (a, b, c)]
    return np.array(verts, np.float64).T.copy(), np.array(out, np.int32).T.copy()


def prepare(mesh: Mesh, options: Options | None = None) -> Prepared:
    """Reference ``prepare`` (src/core/prepare.cpp:102-149)."""
    o = options or Options()
    validate_options(o)
    v, f = mesh.vertices, mesh.faces
    n = v.shape[1]
    if n == 0 or f.shape[1] == 0:
        raise RuntimeError("Mesh is empty")
    if n > 2 ** 31 - 1 or f.shape[1] > 2 ** 31 - 1:
        raise RuntimeError("Mesh exceeds 32-bit index capacity")
    if not np.all(np.isfinite(v)):
        raise RuntimeError("Non-finite coordinate")
    d = v.max(axis=1) - v.min(axis=1)
    box = math.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
    if box < 1e-14:
        raise RuntimeError("Mesh has zero extent")
    if np.any(f < 0) or np.any(f >= n):
        raise RuntimeError("Face index out of range")
    p0, p1, p2 = v[:, f[0]], v[:, f[1]], v[:, f[2]]
    area2 = _norm(_cross(p1 - p0, p2 - p0))
    keep = ~(area2 <= 1e-14 * box * box)
    rejected = int(np.count_nonzero(~keep))
    f = np.ascontiguousarray(f[:, keep])
    if f.shape[1] == 0:
        raise RuntimeError("No nondegenerate triangles")
    for _ in range(o.subdivide):
        v, f = _subdivide(v, f)
    prepared_mesh = Mesh(v, f)
    topo, nonmanifold, conflicts = topology(prepared_mesh)
    n = v.shape[1]
    center = np.array([np.cumsum(v[k])[-1] for k in range(3)]) * (1.0 / n)
    return Prepared(prepared_mesh, topo, ModelContext(box, tuple(float(c) for c in center)),
                    rejected, nonmanifold, conflicts)


def topology(m: Mesh):
    """Reference topology() (src/core/prepare.cpp:13-58)."""
    v, f = m.vertices, m.faces
    n, nf = v.shape[1], f.shape[1]
    p0, p1, p2 = v[:, f[0]], v[:, f[1]], v[:, f[2]]
    fn = _cross(p1 - p0, p2 - p0)
    area = _norm(fn) / 2
    fn = _unit(fn)
    corners = f.T.reshape(-1)                       # (face, k) order
    normals = np.zeros((3, n))
    for k in range(3):
        np.add.at(normals[k], corners, np.repeat(fn[k], 3))
    weights = np.zeros(n)
    np.add.at(weights, corners, np.repeat(area / 3, 3))
    normals = _unit(normals)
    # directed corner edges a -> b = f[k] -> f[(k+1)%3]
    a = corners.astype(np.int64)
    b = np.roll(f, -1, axis=0).T.reshape(-1).astype(np.int64)
    face_of = np.repeat(np.arange(nf, dtype=np.int64), 3)
    # neighbours: sorted unique ring
    src = np.concatenate([a, b])
    dst = np.concatenate([b, a])
    ring = np.unique(src * n + dst)
    nbr_off = np.zeros(n + 1, np.uint64)
    np.cumsum(np.bincount(ring // n, minlength=n), out=nbr_off[1:])
    neighbors = Csr(nbr_off, (ring % n).astype(np.int32))
    # incident faces: per vertex in (face, k) order
    order = np.argsort(corners, kind="stable")
    inc_off = np.zeros(n + 1, np.uint64)
    np.cumsum(np.bincount(corners, minlength=n), out=inc_off[1:])
    incident = Csr(inc_off, face_of[order].astype(np.int32))
    # edges: std::map over (lo, hi) with faces in insertion order
    lo, hi = np.minimum(a, b), np.maximum(a, b)
    key = lo * n + hi
    order = np.argsort(key, kind="stable")
    sk = key[order]
    starts = np.flatnonzero(np.r_[True, sk[1:] != sk[:-1]])
    counts = np.diff(np.r_[starts, sk.size])
    first = order[starts]
    has2 = counts >= 2
    second = np.where(has2, order[np.minimum(starts + 1, sk.size - 1)], -1)
    nonmanifold = int(np.count_nonzero(counts > 2))
    conflicts = int(np.count_nonzero((counts == 2) & (a[first] != b[np.maximum(second, 0)])))
    edges = np.stack([lo[first], hi[first], a[first], b[first], face_of[first],
                      np.where(has2, face_of[np.maximum(second, 0)], -1)], axis=1).astype(np.int32)
    if nonmanifold or conflicts:
        raise RuntimeError("Mesh must have manifold edges and consistent face winding; "
                           "repair input mesh first")
    return Topology(normals, fn, weights, neighbors, incident, edges), nonmanifold, conflicts


# ---------------------------------------------------------------- generators
def _grid_faces(nx, ny, mirror_split=True):
    """Two triangles per cell, counter-clockwise seen from +z; cells left of
    the middle column use the other diagonal so the split is mirror
    symmetric about x = 0."""
    faces = []
    for j in range(ny - 1):
        for i in range(nx - 1):
            v00, v10 = j * nx + i, j * nx + i + 1
            v01, v11 = (j + 1) * nx + i, (j + 1) * nx + i + 1
            if mirror_split and 2 * i + 1 < nx - 1:
                faces += [(v00, v10, v01), (v10, v11, v01)]
            else:
                faces += [(v00, v10, v11), (v00, v11, v01)]
    return np.array(faces, np.int32).T.copy()


def mirrored_heightfield(size=128, bumps=8, seed=0):
    """Height field on [-1,1]^2 with `bumps` Gaussian bumps (amplitude
    U[0.05,0.2], sigma U[0.08,0.3], seeded centres) mirrored so that
    z(x, y) = z(-x, y)."""
    rng = np.random.default_rng(seed)
    amp = rng.uniform(0.05, 0.2, bumps)
    sig = rng.uniform(0.08, 0.3, bumps)
    cen = rng.uniform(-0.8, 0.8, (bumps, 2))
    idx = np.arange(size, dtype=np.float64)
    coord = (2 * idx - (size - 1)) / (size - 1)   # exactly antisymmetric
    x, y = np.meshgrid(coord, coord)
    z = np.zeros_like(x)
    for a, s, (cx, cy) in zip(amp, sig, cen):
        z += a * (np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2 * s * s))
                  + np.exp(-((-x - cx) ** 2 + (y - cy) ** 2) / (2 * s * s)))
    verts = np.stack([x.ravel(), y.ravel(), z.ravel()])
    return Mesh(verts, _grid_faces(size, size))


def icosphere(level):
    t = (1 + 5 ** 0.5) / 2
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t),
         (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
         (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
         (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = np.array(v, np.float64)
    verts /= np.linalg.norm(verts, axis=1, keepdims=True)
    faces = np.array(f, np.int64)
    for _ in range(level):
        e = np.concatenate([faces[:, [0, 1]], faces[:, [1, 2]], faces[:, [2, 0]]])
        e.sort(axis=1)
        uniq, inv = np.unique(e, axis=0, return_inverse=True)
        inv = inv.reshape(-1)
        mids = verts[uniq[:, 0]] + verts[uniq[:, 1]]
        mids /= np.linalg.norm(mids, axis=1, keepdims=True)
        base = verts.shape[0]
        verts = np.concatenate([verts, mids])
        nfc = faces.shape[0]
        ab, bc, ca = (inv[:nfc] + base, inv[nfc:2 * nfc] + base, inv[2 * nfc:] + base)
        a, b, c = faces[:, 0], faces[:, 1], faces[:, 2]
        faces = np.concatenate([np.stack([a, ab, ca], 1), np.stack([ab, b, bc], 1),
                                np.stack([ca, bc, c], 1), np.stack([ab, bc, ca], 1)])
    return verts, faces.astype(np.int32)


def motif_sphere(level=6, bumps=12, folds=5, partial_shift=0.4, noise=1e-3, seed=0):
    """Icosphere subdivided `level` times, radially displaced by a seeded
    motif of `bumps` Gaussian bumps (amplitude 0.03-0.1) repeated `folds`
    times about z, plus a partial copy (the cap z > 0.35) translated by
    `partial_shift` along x; Gaussian vertex noise of `noise` x bbox
    diagonal."""
    rng = np.random.default_rng(seed)
    verts, faces = icosphere(level)
    amp = rng.uniform(0.03, 0.1, bumps)
    sig = rng.uniform(0.08, 0.2, bumps)
    lon = rng.uniform(0, 2 * np.pi / folds, bumps)
    lat = rng.uniform(-1.2, 1.2, bumps)
    r = np.ones(verts.shape[0])
    for k in range(folds):
        for a, s, lo, la in zip(amp, sig, lon + 2 * np.pi * k / folds, lat):
            c = np.array([np.cos(la) * np.cos(lo), np.cos(la) * np.sin(lo), np.sin(la)])
            d2 = np.sum((verts - c) ** 2, axis=1)
            r += a * np.exp(-d2 / (2 * s * s))
    verts = verts * r[:, None]
    cent = verts[faces].mean(axis=1)
    cap = faces[cent[:, 2] > 0.35]
    used = np.unique(cap)
    remap = -np.ones(verts.shape[0], np.int64)
    remap[used] = np.arange(used.size) + verts.shape[0]
    copy = verts[used] + np.array([partial_shift, 0, 0])
    verts = np.concatenate([verts, copy])
    faces = np.concatenate([faces, remap[cap]]).astype(np.int32)
    diag = np.linalg.norm(verts.max(0) - verts.min(0))
    verts = verts + rng.normal(0, noise * diag, verts.shape)
    return Mesh(verts.T.copy(), faces.T.copy())


def motif_torus(R=1.0, r=0.3, nu=1000, nv=500, copies=12, mirrored=2, bumps=6, noise=0.0,
                seed=0):
    """Torus (tube radius r around a circle of radius R in the xy-plane) on an
    nu x nv grid (2 nu nv triangles; 1,000 x 500 gives 1e6), displaced along
    the tube normal by `copies` copies of one seeded motif of `bumps` Gaussian
    bumps (amplitude 0.01-0.03, width 0.03-0.08 in tube arc length): each
    copy sits at a seeded angle about z (a rotation of the torus onto
    itself), the last `mirrored` of them reflected through the xy-plane;
    Gaussian vertex noise of `noise` x bbox diagonal."""
    rng = np.random.default_rng(seed)
    amp = rng.uniform(0.01, 0.03, bumps)
    sig = rng.uniform(0.03, 0.08, bumps)
    du = rng.uniform(-0.15, 0.15, bumps)      # motif offsets: angle about z
    dv = rng.uniform(-0.6, 0.6, bumps)        # angle around the tube
    base_v = rng.uniform(-1.2, 1.2, copies)  # where each copy sits around the tube
    at_u = (np.arange(copies) + rng.uniform(0.1, 0.9, copies)) * (2 * np.pi / copies)
    u = 2 * np.pi * np.arange(nu) / nu
    v = 2 * np.pi * np.arange(nv) / nv
    U, V = np.meshgrid(u, v, indexing="ij")
    disp = np.zeros_like(U)
    for c in range(copies):
        sgn = -1.0 if c >= copies - mirrored else 1.0
        for a, s, ou, ov in zip(amp, sig, du, dv):
            cu, cv = at_u[c] + ou, sgn * (base_v[c] + ov) if sgn < 0 else base_v[c] + ov
            eu = np.angle(np.exp(1j * (U - cu))) * R       # arc lengths, wrapped
            ev = np.angle(np.exp(1j * (V - cv))) * r
            disp += a * np.exp(-(eu * eu + ev * ev) / (2 * s * s))
    rad = r + disp
    x = (R + rad * np.cos(V)) * np.cos(U)
    y = (R + rad * np.cos(V)) * np.sin(U)
    z = rad * np.sin(V)
    verts = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
    i = np.arange(nu)[:, None]
    j = np.arange(nv)[None, :]
    a = (i * nv + j).ravel()
    b = (((i + 1) % nu) * nv + j).ravel()
    c2 = (((i + 1) % nu) * nv + (j + 1) % nv).ravel()
    d = (i * nv + (j + 1) % nv).ravel()
    faces = np.concatenate([np.stack([a, b, c2], 1), np.stack([a, c2, d], 1)]).astype(np.int32)
    if noise:
        diag = np.linalg.norm(verts.max(0) - verts.min(0))
        verts = verts + rng.normal(0, noise * diag, verts.shape)
    return Mesh(verts.T.copy(), faces.T.copy())


def _vertex_normals(verts: np.ndarray, faces: np.ndarray) -> np.ndarray:
    """Area-weighted vertex normals (n, 3) of vertices (n, 3), faces (f, 3)."""
    a, b, c = verts[faces[:, 0]], verts[faces[:, 1]], verts[faces[:, 2]]
    fn = np.cross(b - a, c - a)
    vn = np.zeros_like(verts)
    for k in range(3):
        np.add.at(vn, faces[:, k], fn)
    return vn / np.maximum(np.linalg.norm(vn, axis=1, keepdims=True), 1e-300)


def add_random_bumps(mesh: Mesh, share: float, seed: int, amp=(0.02, 0.06)) -> Mesh:
    """Unsymmetric relief over about `share` of the surface: Gaussian bumps
    along the vertex normals at seeded vertices, each of width a tenth of
    the bounding-box diagonal, as many as cover that share of the vertices."""
    rng = np.random.default_rng(seed)
    v = mesh.vertices.T.copy()
    f = mesh.faces.T
    n = _vertex_normals(v, f)
    diag = float(np.linalg.norm(v.max(0) - v.min(0)))
    sig = 0.1 * diag
    disp = np.zeros(len(v))
    covered = np.zeros(len(v), bool)
    for _ in range(200):
        if covered.mean() >= share:
            break
        c = v[rng.integers(len(v))]
        d2 = ((v - c) ** 2).sum(1)
        disp += rng.uniform(*amp) * diag * np.exp(-d2 / (2 * sig * sig))
        covered |= d2 < (1.5 * sig) ** 2
    return Mesh((v + n * disp[:, None]).T.copy(), mesh.faces.copy())


def add_noise(mesh: Mesh, sigma: float, seed: int) -> Mesh:
    """Gaussian vertex noise of `sigma` times the bounding-box diagonal."""
    if sigma <= 0:
        return mesh
    v = mesh.vertices
    diag = float(np.linalg.norm(v.max(1) - v.min(1)))
    return Mesh(v + np.random.default_rng(seed).normal(0, sigma * diag, v.shape), mesh.faces.copy())


def uneven_batch(count=256, seed=0):
    """The uneven batch: `count` seeded meshes, an even mix of
    motif icospheres, motif tori and mirrored height fields, vertex counts
    log-uniform in 2k-60k (the nearest icosphere level; grid sizes for the
    others), each with 1-4 planted symmetries (rotations about z of a
    repeated motif, rotated or mirrored copies of a motif, or the height
    field's mirror plane) and Gaussian noise sigma uniform in [0, 5e-3] of
    the diagonal.  Returns [(mesh, mode, planted), ...] with mode "rigid" or
    "reflection"."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        kind = ("sphere", "torus", "height")[i % 3]
        target = float(np.exp(rng.uniform(np.log(2000), np.log(60000))))
        planted = int(rng.integers(1, 5))
        noise = float(rng.uniform(0.0, 5e-3))
        if kind == "sphere":
            level = int(np.clip(np.round(np.log(target / 10) / np.log(4)), 4, 6))
            mesh = motif_sphere(level=level, bumps=int(rng.integers(6, 13)), folds=planted + 1,
                                partial_shift=float(rng.uniform(0.2, 0.5)), noise=noise,
                                seed=1000 + i)
            mode = "rigid"
        elif kind == "torus":
            nu = max(24, int(np.sqrt(2 * target)))
            mesh = motif_torus(nu=nu, nv=max(12, nu // 2), copies=planted + 1,
                               mirrored=int(rng.integers(0, 2)), noise=noise, seed=1000 + i)
            mode = "rigid"
        else:
            mesh = add_noise(mirrored_heightfield(size=max(32, int(np.sqrt(target))),
                                                  bumps=int(rng.integers(4, 9)), seed=1000 + i),
                             noise, 2000 + i)
            planted, mode = 1, "reflection"
        out.append((mesh, mode, planted))
    return out


def stress_batch(count=64, seed=1):
    """The stress batch: `count` seeded meshes of 1e5-1e6
    triangles (log-uniform), half reflection (mirrored height fields) and
    half rigid (motif tori with rotated copies), with unsymmetric random
    bumps over about 30% of each surface, so that most pairs vote for no
    symmetry.  Returns [(mesh, mode), ...]."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        tris = float(np.exp(rng.uniform(np.log(1e5), np.log(1e6))))
        if i % 2:
            size = int(np.sqrt(tris / 2)) + 1
            mesh = mirrored_heightfield(size=size, bumps=int(rng.integers(5, 10)), seed=3000 + i)
            mode = "reflection"
        else:
            nu = int(np.sqrt(tris))
            mesh = motif_torus(nu=nu, nv=max(12, nu // 2), copies=int(rng.integers(3, 7)),
                               mirrored=0, noise=0.0, seed=3000 + i)
            mode = "rigid"
        out.append((add_random_bumps(mesh, 0.3, 4000 + i), mode))
    return out
