#!/usr/bin/env python3
"""Generate the golden fixtures under tests/golden/ from the reference itself.

Runs the reference's own CPU library (deoksieze/Mitra_algo src/core + src/cpu,
compiled from the read-only reference tree by ``make -C oracle ref``) through
oracle/ref_harness.cpp on:

* the reference's example meshes (examples/*.off, 132/132/198/66 vertices)
  with the options of its CLI comparison tests (tests/compare_cuda.py:29-31:
  sample ratio 1 and 0.5, pair threshold 0.08, verify threshold 0.01),
  dumping every stage of detect();
* a mirrored Gaussian-bump heightfield of 128x128 vertices (the
  reflection-mode workload: 2,000 samples, pair threshold 0.05, bandwidth
  0.02);
* stage-level cases shaped like the reference's own stage tests
  (tests/cuda_pairing.cpp, cuda_backend.cpp, cuda_clustering.cpp,
  cuda_verification.cpp, geometry.cpp).

Inputs and outputs are stored together (np.savez_compressed), so the fixtures
need neither the reference nor this script at test time.  Large FP64 arrays
are stored as SHA-256 digests of their bytes: the oracle is bit-exact, so a
digest comparison is an exact comparison.

Usage:  python tests/golden/make_golden.py   (needs the reference tree: the
        MITRA_REFERENCE_DIR environment variable, else oracle/Makefile's REF)
"""
from __future__ import annotations

import hashlib
import math
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

sys.path.insert(0, str(ROOT / "tests"))

from helpers import large_clustering_votes, lattice_clustering_votes  # noqa: E402
from mitra_algo_gb300.mesh import mirrored_heightfield  # noqa: E402
from oracle import oracle, symd  # noqa: E402

OUT = Path(__file__).resolve().parent
EXAMPLES = (oracle.reference_tree() or Path("reference-tree-not-found")) / "examples"


def digest(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def read_off(path):
    tokens = []
    for line in Path(path).read_text().splitlines():
        tokens += line.split("#")[0].split()
    assert tokens[0] == "OFF"
    nv, nf = int(tokens[1]), int(tokens[2])
    at = 4
    v = np.array(tokens[at:at + 3 * nv], np.float64).reshape(nv, 3).T.copy()
    at += 3 * nv
    faces = []
    for _ in range(nf):
        k = int(tokens[at])
        poly = [int(t) for t in tokens[at + 1:at + 1 + k]]
        at += 1 + k
        faces += [(poly[0], poly[i], poly[i + 1]) for i in range(1, k - 1)]
    return v, np.array(faces, np.int32).T.copy()


def options(**kw):
    out = {}
    for k, v in kw.items():
        if k in ("seed", "max_pairs", "max_votes"):
            out[k] = np.array([v], np.uint64)
        else:
            out[k] = np.array([float(v)])
    return out


def mesh_arrays(v, f):
    return {"vx": v[0], "vy": v[1], "vz": v[2], "f0": f[0], "f1": f[1], "f2": f[2]}


def save(name, arrays):
    clean = {}
    for k, val in arrays.items():
        clean[k] = np.asarray(val)
    np.savez_compressed(OUT / f"{name}.npz", **clean)
    size = (OUT / f"{name}.npz").stat().st_size
    print(f"{name}.npz  {size / 1024:.0f} KiB")


def text(arrays, key):
    return symd.text(arrays, key) if key in arrays else ""


# ------------------------------------------------------------- detect runs
DIGESTED = ["vnx", "vny", "vnz", "fnx", "fny", "fnz", "weights", "nbr_offsets", "nbr_indices",
            "inc_offsets", "inc_indices", "edges", "nx", "ny", "nz", "dminx", "dminy", "dminz",
            "dmaxx", "dmaxy", "dmaxz", "kmin", "kmax", "valid"] + \
           [f"rot{k}" for k in range(9)] + ["tx", "ty", "tz", "pnx", "pny", "pnz", "poff"] + \
           [f"desc{k}" for k in range(12)]


def detect_fixture(name, v, f, opts, keep_full):
    inputs = {**mesh_arrays(v, f), **opts}
    out = oracle.run_reference("detect", inputs)
    record = {f"in_{k}": val for k, val in inputs.items()}
    for k, val in out.items():
        if k.startswith("rng_") or k in ("error", "error_kind"):
            record[k] = np.array(symd.text(out, k))
        elif keep_full or k not in DIGESTED:
            record[k] = val
        if k in DIGESTED:
            record[f"sha_{k}"] = np.array(digest(val))
    save(name, record)
    return out


def examples():
    for scene in ["reflection", "rigid", "partial", "single"]:
        v, f = read_off(EXAMPLES / f"{scene}.off")
        for ratio in [1, 0.5]:
            tag = "1" if ratio == 1 else "05"
            detect_fixture(f"detect_{scene}_{tag}", v, f,
                           options(sample_ratio=ratio, pair_threshold=0.08,
                                   verify_threshold=0.01), keep_full=True)


def heightfield():
    m = mirrored_heightfield(128, 8, seed=0)
    out = detect_fixture("detect_heightfield", m.vertices, m.faces,
                         options(sample_ratio=2000 / 16384, pair_threshold=0.05,
                                 bandwidth=0.02), keep_full=False)
    print("  heightfield stage ms:", np.round(out["stage_ms"], 1),
          "pairs", out["pair_a"].size, "votes", out["vote_pair"].size)


def export_cases():
    """The reference's own text export (detect() then export_result(),
    src/io/export.cpp:37-189) of the eight example runs: SHA-256 and size of
    features.csv, pairs.csv, votes.csv, descriptors.csv and mesh.off."""
    import tempfile
    record = {}
    for scene in ["reflection", "rigid", "partial", "single"]:
        v, f = read_off(EXAMPLES / f"{scene}.off")
        for ratio in [1, 0.5]:
            name = f"{scene}_{'1' if ratio == 1 else '05'}"
            with tempfile.TemporaryDirectory() as d:
                out = oracle.run_reference("export", {
                    **mesh_arrays(v, f), "dir": str(Path(d) / "csv"),
                    **options(sample_ratio=ratio, pair_threshold=0.08, verify_threshold=0.01)})
                for file in EXPORT_FILES:
                    data = (Path(d) / "csv" / file).read_bytes()
                    record[f"{name}:{file}:sha"] = np.array(hashlib.sha256(data).hexdigest())
                    record[f"{name}:{file}:bytes"] = np.array(len(data))
            print(f"  export {name}: {int(out['pairs'][0])} pairs, {int(out['votes'][0])} votes, "
                  f"export_result {out['export_ms'][0]:.2f} ms")
    save("export_text", record)


EXPORT_FILES = ("features.csv", "pairs.csv", "votes.csv", "descriptors.csv", "mesh.off")


# ------------------------------------------------------------- stage cases
def pairing_cases():
    """Shaped like the reference's tests/cuda_pairing.cpp:42-127."""
    cases = []

    def fixture(count):
        i = np.arange(count, dtype=np.float64)
        pos = np.stack([i, (np.arange(count) % 7) * 0.1, (np.arange(count) % 11) * 0.2])
        return pos, np.full(count, 0.5), np.full(count, 1.0), np.arange(count, dtype=np.int32)

    pos, kmin, kmax, sel = fixture(513)
    cases.append(("dense", pos, kmin, kmax, sel, 0.15, 2000000, 1.0))
    cases.append(("dense_exact_budget", pos, kmin, kmax, sel, 0.15, 513 * 512 // 2, 1.0))
    cases.append(("dense_over_budget", pos, kmin, kmax, sel, 0.15, 513 * 512 // 2 - 1, 1.0))
    rng = np.random.default_rng(123)
    pos, kmin, kmax, sel = fixture(777)
    kmin = rng.uniform(-2, 2, 777)
    kmax = rng.uniform(-2, 2, 777)
    kmin[::13] = 0
    kmax[::17] = 1e-12
    sel = rng.permutation(777).astype(np.int32)
    for t in [1e-8, 0.01, 0.15, 0.7, np.nextafter(1.0, 0.0), 1.0]:
        cases.append((f"random_t{t!r}", pos, kmin, kmax, sel, t, 2000000, 1.0))
    dup = np.concatenate([sel, sel[:1]])
    cases.append(("random_duplicate", pos, kmin, kmax, dup, 0.7, 2000000, 1.0))
    pos, kmin, kmax, sel = fixture(12)
    curv = np.array([0.75, 1, np.nextafter(0.75, 0), -0.75, -1, 0, -0.0, 1e-12, -1e-12, 1e-10,
                     1e200, 1e200])
    pos[:, 0] = 0
    pos[:, 1] = [0.03, 0, 0]
    pos[:, 2] = [np.nextafter(0.03, 0), 0, 0]
    for t in [0.25, 0.5, 1.0]:
        cases.append((f"boundary_t{t}", pos, curv, curv.copy(), sel, t, 2000000, 1.0))
    for t in [0.01, 0.15, 0.5, 0.9, np.nextafter(1.0, 0.0)]:
        pos, _, _, sel = fixture(4)
        target = 1 / (1 - t)
        k = np.array([1, target, np.nextafter(target, 0), np.nextafter(target, np.inf)])
        cases.append((f"edge_t{t!r}", pos, k, k.copy(), sel, t, 2000000, 1.0))
    pos, _, _, sel = fixture(2)
    k = np.array([1, 13510798882111490.0])
    cases.append(("rounded", pos, k, k.copy(), sel, np.nextafter(1.0, 0.0), 2000000, 1.0))
    pos, _, _, sel = fixture(20)
    zk = np.where(np.arange(20) % 2 == 1, -0.0, 0.0)
    cases.append(("signed_zeros", pos, zk, np.zeros(20), sel, 0.15, 2000000, 1.0))
    # clustered curvature keys (the reference's isolated pairing benchmark shape,
    # benchmarks/pairing.cpp:14-24, at 2,000 points)
    n = 2000
    i = np.arange(n)
    pos = np.stack([i.astype(float), (i % 7).astype(float), (i % 11).astype(float)])
    k = ((i * 37) % 100 + 1).astype(float)
    cases.append(("key_groups", pos, k, 2 * k, i.astype(np.int32), 1e-6, 600000, 1.0))
    record = {}
    for idx, (name, pos, kmin, kmax, sel, t, budget, box) in enumerate(cases):
        inputs = {"vx": pos[0], "vy": pos[1], "vz": pos[2], "kmin": kmin, "kmax": kmax,
                  "selected": sel, "box_size": np.array([box]),
                  **options(pair_threshold=t, max_pairs=budget)}
        out = oracle.run_reference("pairing", inputs)
        p = f"c{idx}_"
        record[p + "name"] = np.array(name)
        for k, val in inputs.items():
            record[p + "in_" + k] = val
        record[p + "pair_a"] = out.get("pair_a", np.zeros(0, np.int32))
        record[p + "pair_b"] = out.get("pair_b", np.zeros(0, np.int32))
        record[p + "error"] = np.array(text(out, "error"))
        print(f"  pairing {name}: {record[p + 'pair_a'].size} pairs {text(out, 'error')[:30]}")
    record["count"] = np.array(len(cases))
    save("stage_pairing", record)


def oblique_mirror_fixture():
    """Points mirrored across an oblique plane with nearly zero first normal
    component (shape of the reference's tests/cuda_backend.cpp:60-88)."""
    def unit(a):
        return a / np.linalg.norm(a)

    n = unit(np.array([1e-16, 1.0, 2.0]))
    d = unit(np.cross(n, [1.0, 0, 0]))
    mirror = np.eye(3) - 2 * np.outer(n, n)
    verts = []
    for i in range(514):
        p = np.array([i * 0.01, -2 - 0.001 * i, 0.13])
        verts += [p, mirror @ p]
    verts = np.array(verts).T.copy()
    cnt = verts.shape[1]
    normal = np.zeros((3, cnt))
    dmin = np.zeros((3, cnt))
    dmax = np.zeros((3, cnt))
    for i in range(cnt):
        nn, mm = n.copy(), d.copy()
        if i % 4 == 3:
            mm = -mm
        if i % 2:
            nn, mm = mirror @ nn, mirror @ mm
        normal[:, i], dmin[:, i], dmax[:, i] = nn, mm, np.cross(nn, mm)
    pairs_a = np.array(sum([[2 * i, 2 * i + 1] for i in range(514)], []), np.int32)
    pairs_b = np.array(sum([[2 * i + 1, 2 * i] for i in range(514)], []), np.int32)
    return verts, normal, dmin, dmax, pairs_a, pairs_b, n, d


def transformation_cases():
    verts, normal, dmin, dmax, pa, pb, n, d = oblique_mirror_fixture()
    cnt = verts.shape[1]
    base = {"vx": verts[0], "vy": verts[1], "vz": verts[2], "box_size": np.array([20.0]),
            "center": np.array([3.0, -1.0, 2.0])}

    def feats(normal, dmin, dmax, kmin, kmax, valid):
        return {"nx": normal[0], "ny": normal[1], "nz": normal[2], "dminx": dmin[0],
                "dminy": dmin[1], "dminz": dmin[2], "dmaxx": dmax[0], "dmaxy": dmax[1],
                "dmaxz": dmax[2], "kmin": kmin, "kmax": kmax, "valid": valid}

    ones = np.ones(cnt, np.uint8)
    cases = [("mirror", feats(normal, dmin, dmax, np.full(cnt, 0.2), np.ones(cnt), ones), pa, pb,
              600000)]
    mixed_n, mixed_x = normal.copy(), dmax.copy()
    for i in range(1, cnt, 4):
        mixed_n[:, i] = n
        mixed_x[:, i] = np.cross(n, dmin[:, i])
    f_mixed = feats(mixed_n, dmin, mixed_x, np.full(cnt, 0.2), np.ones(cnt), ones)
    cases.append(("mixed", f_mixed, pa, pb, 600000))
    par = feats(np.tile(n[:, None], cnt), np.tile(d[:, None], cnt),
                np.tile(np.cross(n, d)[:, None], cnt), np.full(cnt, 0.2), np.ones(cnt), ones)
    cases.append(("parallel", par, pa, pb, 600000))
    cases.append(("same_point", par, np.array([0], np.int32), np.array([0], np.int32), 600000))
    zero = {k: v.copy() for k, v in par.items()}
    for k in ["nx", "ny", "nz", "dminx", "dminy", "dminz", "dmaxx", "dmaxy", "dmaxz"]:
        zero[k][0] = 0
    cases.append(("zero_directions", zero, np.array([0], np.int32), np.array([0], np.int32), 600000))
    cases.append(("budget", f_mixed, pa, pb, 1))
    record = {}
    for idx, (name, f, a, b, budget) in enumerate(cases):
        inputs = {**base, **f, "pair_a": a, "pair_b": b, **options(max_votes=budget)}
        out = oracle.run_reference("transformations", inputs)
        p = f"c{idx}_"
        record[p + "name"] = np.array(name)
        for k, val in inputs.items():
            record[p + "in_" + k] = val
        for k, val in out.items():
            record[p + k] = np.array(symd.text(out, k)) if k.startswith("error") else val
        if "error" not in out:
            record[p + "error"] = np.array("")
        print(f"  transformations {name}: {out.get('vote_pair', np.zeros(0)).size} votes "
              f"{text(out, 'error')[:30]}")
    record["count"] = np.array(len(cases))
    save("stage_transformations", record)


def clustering_votes(count):
    """Alternating reflection/rigid votes around four modes with sin jitter
    (shape of the reference's tests/cuda_clustering.cpp:12-18)."""
    q = count
    refl = (np.arange(q) % 2).astype(np.uint8)
    d = 3 + ((np.arange(q) % 4) // 2) * 2 + 0.001 * np.sin(np.arange(q))
    rot = np.zeros((9, q))
    desc = np.zeros((12, q))
    tr = np.zeros((3, q))
    pn = np.zeros((3, q))
    off = np.zeros(q)
    mirror = np.diag([-1.0, 1, 1]).reshape(-1)
    ident = np.eye(3).reshape(-1)
    for i in range(q):
        if refl[i]:
            rot[:, i] = mirror
            tr[:, i] = [-2 * d[i], 0, 0]
            pn[:, i] = [1, 0, 0]
            off[i] = d[i]
            desc[:4, i] = [1, 0, 0, d[i] / 10]
        else:
            rot[:, i] = ident
            tr[:, i] = [d[i], 0, 0]
            desc[:9, i] = ident / 2
            desc[9, i] = d[i] / 10
    return {"vote_pair": np.arange(q, dtype=np.int32), "vote_kind": refl,
            **{f"rot{k}": rot[k] for k in range(9)}, "tx": tr[0], "ty": tr[1], "tz": tr[2],
            "pnx": pn[0], "pny": pn[1], "pnz": pn[2], "poff": off,
            **{f"desc{k}": desc[k] for k in range(12)}}


def clustering_cases():
    """The shape of tests/cuda_clustering.cpp:12-18 at four sizes, then
    votes on lattices whose pitch is the bandwidth and the bandwidth times
    1 +- 1e-15: neighbours at a squared distance within a few units of
    rounding of h^2, where the reference's strict d^2 < h^2 is decided by
    the FP64 rounding."""
    record = {}
    idx = 0

    def add(name, votes, **opts):
        nonlocal idx
        inputs = {**votes, "box_size": np.array([10.0]), "center": np.zeros(3), **options(**opts)}
        out = oracle.run_reference("clustering", inputs)
        p = f"c{idx}_"
        record[p + "name"] = np.array(name)
        for k, val in inputs.items():
            record[p + "in_" + k] = val
        for k, val in out.items():
            record[p + k] = np.array(symd.text(out, k)) if k.startswith(("rng", "error")) else val
        print(f"  clustering {name}: {out['cl_reflection'].size} clusters")
        idx += 1

    for count in [0, 1, 64, 2048]:
        for iters in [1, 100]:
            add(f"votes{count}_iters{iters}", clustering_votes(count), bandwidth=0.03,
                max_clusters=4, max_iterations=iters, seed=42)
    for name, scale in (("lattice_h", 1.0), ("lattice_h_plus", 1 + 1e-15),
                        ("lattice_h_minus", 1 - 1e-15)):
        add(name, lattice_clustering_votes(0.03 * scale), bandwidth=0.03, max_clusters=50,
            max_iterations=100, seed=42)
    record["count"] = np.array(idx)
    save("stage_clustering", record)


def clustering_large_case():
    """100,000 votes regenerated from integers by
    tests/helpers.py:large_clustering_votes (not stored): the reference's
    memberships (as a digest), cluster sizes, records, RNG state."""
    votes = large_clustering_votes()
    inputs = {**votes, "box_size": np.array([10.0]), "center": np.zeros(3),
              **options(bandwidth=0.03, max_clusters=20, max_iterations=100, seed=42)}
    out = oracle.run_reference("clustering", inputs)
    rec = {"votes": np.array(votes["vote_kind"].size), "generator_seed": np.array(7),
           "bandwidth": np.array(0.03), "max_clusters": np.array(20),
           "max_iterations": np.array(100), "seed": np.array(42),
           "sha_cl_vote_indices": np.array(digest(out["cl_vote_indices"]))}
    for k, val in out.items():
        if k == "cl_vote_indices":
            continue
        rec[k] = np.array(symd.text(out, k)) if k.startswith(("rng", "error")) else val
    print(f"  clustering large: {out['cl_reflection'].size} clusters")
    save("stage_clustering_large", rec)


def verification_cases():
    """Known transforms on the example meshes plus a stationary cluster
    (shape of the reference's tests/cuda_verification.cpp:18-78)."""
    record = {}
    idx = 0
    for scene in ["reflection", "rigid", "partial"]:
        v, f = read_off(EXAMPLES / f"{scene}.off")
        if scene == "rigid":
            a = 0.65
            rot = [math.cos(a), -math.sin(a), 0, math.sin(a), math.cos(a), 0, 0, 0, 1]
            rec = dict(refl=0, rot=rot, tr=[3.2, 0.3, 0.2], pn=[0, 0, 0], off=0)
        else:
            rec = dict(refl=1, rot=[-1, 0, 0, 0, 1, 0, 0, 0, 1], tr=[0, 0, 0], pn=[1, 0, 0], off=0)
        inputs = {**mesh_arrays(v, f), **options(verify_threshold=0.01),
                  "cl_reflection": np.array([rec["refl"], 0], np.uint8),
                  "cl_rotation": np.array(rec["rot"] + [1, 0, 0, 0, 1, 0, 0, 0, 1], float),
                  "cl_translation": np.array(rec["tr"] + [0, 0, 0], float),
                  "cl_plane_normal": np.array(rec["pn"] + [0, 0, 0], float),
                  "cl_plane_offset": np.array([rec["off"], 0.0])}
        out = oracle.run_reference("verification", inputs)
        p = f"c{idx}_"
        record[p + "name"] = np.array(scene)
        for k, val in inputs.items():
            record[p + "in_" + k] = val
        for k, val in out.items():
            record[p + k] = val
        print(f"  verification {scene}: side_a {out['ver_side_a'].size}")
        idx += 1
    record["count"] = np.array(idx)
    save("stage_verification", record)


def select_cases():
    """Sampling + pruning fixtures (shape of tests/cuda_backend.cpp:144-198)."""
    verts, normal, dmin, dmax, *_ = oblique_mirror_fixture()
    cnt = verts.shape[1]
    i = np.arange(cnt)
    valid = (i % 7 != 0).astype(np.uint8)
    kmin = np.where(i % 5 == 0, 1.0, 0.2)
    kmax = np.ones(cnt)
    kmin[i % 11 == 0] = 1e-12
    kmax[i % 11 == 0] = 1e-12
    weights = np.where(i % 13 == 0, 0.0, 1.0)
    cases = [(f"ratio{r}", kmin, kmax, valid, weights, r, 0.85) for r in [1.0, 0.5, 0.001]]
    kb = np.where(i % 3 == 0, 0.75, np.where(i % 3 == 1, np.nextafter(0.75, 0), -1.0))
    cases.append(("prune_boundary", kb, np.ones(cnt), np.ones(cnt, np.uint8), np.ones(cnt), 1.0, 0.75))
    cases.append(("none_valid", kb, np.ones(cnt), np.zeros(cnt, np.uint8), np.ones(cnt), 1.0, 0.75))
    cases.append(("zero_weights", kb, np.ones(cnt), np.ones(cnt, np.uint8), np.zeros(cnt), 1.0, 0.75))
    record = {}
    for idx, (name, kmn, kmx, val, w, ratio, prune) in enumerate(cases):
        inputs = {"vx": verts[0], "vy": verts[1], "vz": verts[2], "kmin": kmn, "kmax": kmx,
                  "valid": val, "weights": w, **options(sample_ratio=ratio, prune=prune, seed=42)}
        out = oracle.run_reference("select", inputs)
        p = f"c{idx}_"
        record[p + "name"] = np.array(name)
        for k, v in inputs.items():
            record[p + "in_" + k] = v
        record[p + "sample"] = out["sample"]
        record[p + "pruned"] = out["pruned"]
        record[p + "rng_after_select"] = np.array(symd.text(out, "rng_after_select"))
        print(f"  select {name}: sample {out['sample'].size} pruned {out['pruned'].size}")
    record["count"] = np.array(len(cases))
    save("stage_select", record)


def sampling_draw_logs(n, seed=42):
    """-log(u) of the first n draws of std::mt19937_64(seed), u as
    src/core/sampling.cpp:12-13 forms it."""
    r = oracle.rng(seed)
    return np.array([-math.log(((r.next() >> 11) + 0.5) / 9007199254740992.0)
                     for _ in range(n)])


def sampling_cases():
    """Area-weighted sampling alone (src/core/sampling.cpp:5-24) through the
    reference's select(): mixed weights (zero, negative, NaN and infinite
    ones), ratio edges, all-zero weights, and keys packed closer than 2^-32
    of each other around the selection boundary (weights -log(u) (1 + i
    2^-46), so the keys fall in i order, 128 ulps apart)."""
    g = np.random.default_rng(2024)
    mixed = g.lognormal(0.0, 1.0, 6000)
    mixed[::10] = 0.0
    mixed[3::17] = -1.0
    mixed[5], mixed[7] = np.nan, np.inf
    uniform = g.uniform(0.5, 2.0, 1000)
    tight = sampling_draw_logs(4000) * (1.0 + np.arange(4000) * 2.0 ** -46)
    cases = [("mixed_weights", mixed, 0.3), ("ratio_one", uniform, 1.0),
             ("ratio_tiny", uniform, 0.001), ("ratio_zero", uniform, 0.0),
             ("all_zero", np.zeros(500), 0.5), ("tight_keys", tight, 0.4)]
    record = {}
    for idx, (name, w, ratio) in enumerate(cases):
        n = w.size
        inputs = {"vx": np.zeros(n), "vy": np.zeros(n), "vz": np.zeros(n),
                  "valid": np.ones(n, np.uint8), "kmin": np.full(n, 0.1), "kmax": np.ones(n),
                  "weights": w, **options(sample_ratio=ratio, seed=42)}
        out = oracle.run_reference("select", inputs)
        p = f"c{idx}_"
        record[p + "name"] = np.array(name)
        record[p + "in_weights"] = w
        record[p + "in_sample_ratio"] = inputs["sample_ratio"]
        record[p + "in_seed"] = inputs["seed"]
        record[p + "sample"] = out["sample"]
        record[p + "rng_after_select"] = np.array(symd.text(out, "rng_after_select"))
        print(f"  sampling {name}: sample {out['sample'].size} of {n}")
    record["count"] = np.array(len(cases))
    save("stage_sampling", record)


def triangle_cases():
    """Point-triangle distances: the reference's geometry.cpp KATs and 1,024
    random queries with degenerate triangles (cuda_verification.cpp:79-100)."""
    q = [[0.2, 0.3, 2, 0, 0, 0, 1, 0, 0, 0, 1, 0], [2, 0, 0, 0, 0, 0, 1, 0, 0, 0, 1, 0],
         [-1, -1, 0, 0, 0, 0, 1, 0, 0, 0, 1, 0], [1, 1, 0, 0, 0, 0, 1, 0, 0, 0, 1, 0],
         [0.5, 1, 0, 0, 0, 0, 1, 0, 0, 1, 0, 0], [1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0]]
    rng = np.random.default_rng(12)
    for i in range(1024):
        p, a, b, c = (rng.uniform(-3, 3, 3) for _ in range(4))
        if i % 5 == 0:
            c = a.copy()
        if i % 7 == 0:
            b = a.copy()
            c = a.copy()
        if i % 11 == 0:
            p = a.copy()
        q.append(list(p) + list(a) + list(b) + list(c))
    queries = np.array(q, np.float64).reshape(-1)
    out = oracle.run_reference("triangles", {"queries": queries})
    save("stage_triangles", {"queries": queries, "distances": out["distances"]})


def rng_case():
    out = oracle.run_reference("rng", options(seed=42))
    save("stage_rng", {"rng_seeded": np.array(symd.text(out, "rng_seeded")),
                       "draws": out["draws"],
                       "rng_after_draws": np.array(symd.text(out, "rng_after_draws"))})


if __name__ == "__main__":
    oracle.build(reference=True)
    if sys.argv[1:] == ["clustering"]:  # only the clustering fixtures
        clustering_cases()
        clustering_large_case()
        sys.exit(0)
    rng_case()
    triangle_cases()
    select_cases()
    sampling_cases()
    pairing_cases()
    transformation_cases()
    clustering_cases()
    clustering_large_case()
    verification_cases()
    examples()
    export_cases()
    heightfield()
