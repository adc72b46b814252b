"""Shared conversions between golden archives and the host data model."""
import hashlib

import numpy as np

from mitra_algo_gb300.types import (ClusterOutput, Csr, Features, Mesh, ModelContext, Options,
                                    Topology, Votes)

FEATURE_LANES = ["nx", "ny", "nz", "dminx", "dminy", "dminz", "dmaxx", "dmaxy", "dmaxz"]


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def options_from(d, prefix=""):
    o = Options()
    for k in ["sample_ratio", "prune", "pair_threshold", "bandwidth", "verify_threshold"]:
        if prefix + k in d:
            setattr(o, k, float(d[prefix + k][0]))
    for k in ["smoothing", "subdivide", "max_iterations", "max_clusters"]:
        if prefix + k in d:
            setattr(o, k, int(d[prefix + k][0]))
    for k in ["seed", "max_pairs", "max_votes"]:
        if prefix + k in d:
            setattr(o, k, int(d[prefix + k][0]))
    if prefix + "patching" in d:
        o.patching = bool(d[prefix + "patching"][0])
    return o


def mesh_from(d, prefix=""):
    return Mesh(np.stack([d[prefix + "vx"], d[prefix + "vy"], d[prefix + "vz"]]),
                np.stack([d[prefix + "f0"], d[prefix + "f1"], d[prefix + "f2"]]))


def points_only_mesh(d):
    return Mesh(np.stack([d["vx"], d["vy"], d["vz"]]), np.zeros((3, 0), np.int32))


def features_from(d, n):
    z = np.zeros(n)
    lane = lambda k: d[k] if k in d else z  # noqa: E731
    return Features(np.stack([lane("nx"), lane("ny"), lane("nz")]),
                    np.stack([lane("dminx"), lane("dminy"), lane("dminz")]),
                    np.stack([lane("dmaxx"), lane("dmaxy"), lane("dmaxz")]),
                    lane("kmin").astype(np.float64), lane("kmax").astype(np.float64),
                    (d["valid"] if "valid" in d else np.zeros(n, np.uint8)).astype(np.uint8))


def votes_from(d):
    q = d["vote_pair"].size
    return Votes(d["vote_pair"], d["vote_kind"],
                 np.stack([d[f"rot{k}"] for k in range(9)]) if q else np.zeros((9, 0)),
                 np.stack([d["tx"], d["ty"], d["tz"]]) if q else np.zeros((3, 0)),
                 np.stack([d["pnx"], d["pny"], d["pnz"]]) if q else np.zeros((3, 0)),
                 d["poff"], np.stack([d[f"desc{k}"] for k in range(12)]) if q else np.zeros((12, 0)))


def clusters_from(d):
    refl = d["cl_reflection"]
    n = refl.size
    offsets = d["cl_vote_offsets"] if "cl_vote_offsets" in d else np.zeros(n + 1, np.uint64)
    indices = d["cl_vote_indices"] if "cl_vote_indices" in d else np.zeros(0, np.int32)
    return ClusterOutput(refl, d["cl_rotation"].reshape(n, 9), d["cl_translation"].reshape(n, 3),
                         d["cl_plane_normal"].reshape(n, 3), d["cl_plane_offset"],
                         Csr(offsets, indices))


def topology_from(d):
    return Topology(np.stack([d["vnx"], d["vny"], d["vnz"]]), np.stack([d["fnx"], d["fny"], d["fnz"]]),
                    d["weights"], Csr(d["nbr_offsets"], d["nbr_indices"]),
                    Csr(d["inc_offsets"], d["inc_indices"]), d["edges"].reshape(-1, 6))


def context_from(d):
    c = d["center"] if "center" in d else np.zeros(3)
    return ModelContext(float(d["box_size"][0]), tuple(float(x) for x in c))


def feature_arrays(f: Features):
    return {"nx": f.normal[0], "ny": f.normal[1], "nz": f.normal[2], "dminx": f.dmin[0],
            "dminy": f.dmin[1], "dminz": f.dmin[2], "dmaxx": f.dmax[0], "dmaxy": f.dmax[1],
            "dmaxz": f.dmax[2], "kmin": f.kmin, "kmax": f.kmax, "valid": f.valid}


def vote_arrays(v: Votes):
    out = {"vote_pair": v.pair, "vote_kind": v.kind, "tx": v.translation[0], "ty": v.translation[1],
           "tz": v.translation[2], "pnx": v.plane_normal[0], "pny": v.plane_normal[1],
           "pnz": v.plane_normal[2], "poff": v.plane_offset}
    for k in range(9):
        out[f"rot{k}"] = v.rotation[k]
    for k in range(12):
        out[f"desc{k}"] = v.descriptor[k]
    return out


def topology_arrays(t: Topology):
    return {"vnx": t.normals[0], "vny": t.normals[1], "vnz": t.normals[2],
            "fnx": t.face_normals[0], "fny": t.face_normals[1], "fnz": t.face_normals[2],
            "weights": t.weights, "nbr_offsets": t.neighbors.offsets,
            "nbr_indices": t.neighbors.indices, "inc_offsets": t.incident_faces.offsets,
            "inc_indices": t.incident_faces.indices,
            "edges": np.ascontiguousarray(t.edges, np.int32).reshape(-1)}


def same_array(got, want, name=""):
    got = np.asarray(got)
    want = np.asarray(want)
    assert got.shape == want.shape, (name, got.shape, want.shape)
    assert got.tobytes() == want.astype(got.dtype).tobytes() or np.array_equal(got, want), name


def cluster_arrays(c: ClusterOutput):
    return {"cl_reflection": c.reflection, "cl_rotation": c.rotation.reshape(-1),
            "cl_translation": c.translation.reshape(-1),
            "cl_plane_normal": c.plane_normal.reshape(-1), "cl_plane_offset": c.plane_offset,
            "cl_vote_offsets": c.votes.offsets, "cl_vote_indices": c.votes.indices}


def verification_arrays(v):
    return {"ver_side_a_offsets": v.side_a.offsets, "ver_side_a": v.side_a.indices,
            "ver_side_b_offsets": v.side_b.offsets, "ver_side_b": v.side_b.indices,
            "ver_patches_a_groups": v.patches_a_groups, "ver_patches_a_offsets": v.patches_a.offsets,
            "ver_patches_a_indices": v.patches_a.indices, "ver_patches_b_groups": v.patches_b_groups,
            "ver_patches_b_offsets": v.patches_b.offsets, "ver_patches_b_indices": v.patches_b.indices,
            "ver_coverage": v.coverage, "ver_rms": v.rms}


def lattice_clustering_votes(spacing):
    """Votes on lattices of pitch `spacing`: rigid votes on a 13 x 13 grid
    in descriptor entries 9 and 10 and reflection votes on a chain of 25 in
    entry 3.  With the pitch at the bandwidth, a seed's lattice neighbours
    lie at a squared distance within a few units of rounding of h^2, so the
    reference's strict d^2 < h^2 decides by the FP64 rounding of the
    distances.  Columns as the golden fixtures store votes."""
    rigid = [(i, j) for i in range(13) for j in range(13)]
    refl = list(range(25))
    q = len(rigid) + len(refl)
    kind = np.array([0] * len(rigid) + [1] * len(refl), np.uint8)
    rot = np.zeros((9, q))
    desc = np.zeros((12, q))
    tr = np.zeros((3, q))
    pn = np.zeros((3, q))
    off = np.zeros(q)
    ident = np.eye(3).reshape(-1)
    for v, (i, j) in enumerate(rigid):
        rot[:, v] = ident
        desc[:9, v] = ident / 2
        desc[9, v] = 0.2 + i * spacing
        desc[10, v] = -0.1 + j * spacing
        tr[:, v] = [desc[9, v] * 10, desc[10, v] * 10, 0]
    for u, i in enumerate(refl):
        v = len(rigid) + u
        rot[:, v] = np.diag([-1.0, 1, 1]).reshape(-1)
        pn[:, v] = [1, 0, 0]
        off[v] = 0.5 + i * spacing * 10
        tr[:, v] = [-2 * off[v], 0, 0]
        desc[:4, v] = [1, 0, 0, 0.05 + i * spacing]
    return {"vote_pair": np.arange(q, dtype=np.int32), "vote_kind": kind,
            **{f"rot{k}": rot[k] for k in range(9)}, "tx": tr[0], "ty": tr[1], "tz": tr[2],
            "pnx": pn[0], "pny": pn[1], "pnz": pn[2], "poff": off,
            **{f"desc{k}": desc[k] for k in range(12)}}


def _mix64(z):
    """splitmix64 finaliser on uint64 arrays (wrapping integer arithmetic,
    the same bits on every machine)."""
    z = z + np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def large_clustering_votes(q=100_000, modes=8, outliers=200, seed=7):
    """A large vote set, regenerated bit for bit anywhere from integers:
    `modes` clusters (the first 3 reflection votes, the others rigid) with
    offsets uniform in [-0.005, 0.005) in every descriptor entry, and
    `outliers` votes spread over a wide range.  Uniform values are 20-bit
    integers over 2^20, exact in FP64.  Columns as the golden fixtures store
    votes."""
    with np.errstate(over="ignore"):
        i = np.arange(q, dtype=np.uint64)
        base = np.uint64(seed) * np.uint64(0x632BE59BD9B4E019)

        def uniform(k):  # (q,) values k/2^20 in [0, 1), stream k
            z = _mix64(i * np.uint64(16) + np.uint64(k) + base)
            return (z >> np.uint64(44)).astype(np.float64) / 1048576.0
        mode = (i % np.uint64(modes)).astype(np.int64)
        outlier = np.zeros(q, bool)
        outlier[(_mix64(i + base) % np.uint64(q)).astype(np.int64)[:outliers]] = True
        kind = (mode < 3).astype(np.uint8)
        desc = np.zeros((12, q))
        for k in range(12):
            desc[k] = (uniform(k) - 0.5) * 0.01
        ident = np.eye(3).reshape(-1)
        rot = np.zeros((9, q))
        for k in range(9):
            rot[k] = np.where(kind == 1, np.diag([-1.0, 1, 1]).reshape(-1)[k], ident[k])
        centre = 0.25 * mode
        desc[3] = np.where(kind == 1, 0.1 + centre + desc[3], desc[3])
        desc[:3] = np.where(kind == 1, np.array([[1.0], [0.0], [0.0]]) + desc[:3], desc[:3])
        for k in range(9):
            desc[k] = np.where(kind == 0, ident[k] / 2 + desc[k], desc[k])
        desc[9] = np.where(kind == 0, centre + desc[9], desc[9])
        wide = (uniform(12) - 0.5) * 40.0
        desc[9] = np.where(outlier & (kind == 0), wide, desc[9])
        desc[3] = np.where(outlier & (kind == 1), wide, desc[3])
        desc[4:] = np.where(kind == 1, 0.0, desc[4:])
        tr = np.zeros((3, q))
        tr[0] = np.where(kind == 0, desc[9] * 10, -2 * desc[3] * 10)
        pn = np.zeros((3, q))
        pn[0] = np.where(kind == 1, 1.0, 0.0)
        off = np.where(kind == 1, desc[3] * 10, 0.0)
    return {"vote_pair": np.arange(q, dtype=np.int32), "vote_kind": kind,
            **{f"rot{k}": rot[k] for k in range(9)}, "tx": tr[0], "ty": tr[1], "tz": tr[2],
            "pnx": pn[0], "pny": pn[1], "pnz": pn[2], "poff": off,
            **{f"desc{k}": desc[k] for k in range(12)}}
