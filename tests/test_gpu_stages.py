"""GPU parity of every stage against the reference's golden outputs and the
oracle, through the C ABI.  Cases follow the reference's own stage tests
(tests/cuda_curvature.cpp, cuda_backend.cpp, cuda_pairing.cpp,
cuda_clustering.cpp, cuda_verification.cpp of deoksieze/Mitra_algo).

Tolerances: pair sets, vote geometry (FP64, same operation order),
selections, memberships, sides, patches and coverage are bit-exact; curvature
features use the reference's own CPU/GPU bound 1e-10 (its libm transcendental
functions differ from CUDA's in the last ulp); cluster centres 1e-10 and rms
1e-12 x box as in the reference's tests."""
import numpy as np
import pytest

from conftest import golden_cases, load_golden
from helpers import (cluster_arrays, clusters_from, context_from, features_from, mesh_from,
                     options_from, points_only_mesh, same_array, topology_from,
                     verification_arrays, vote_arrays, votes_from)
from mitra_algo_gb300.mesh import prepare
from mitra_algo_gb300.types import Mesh, ModelContext, Options, Pairs, Rng
from oracle import oracle

pytestmark = pytest.mark.gpu

EXAMPLES = ["reflection_1", "rigid_1", "partial_1", "single_1"]


@pytest.fixture(scope="module")
def gpu():
    from mitra_algo_gb300 import Gb300Backend
    b = Gb300Backend(0)
    yield b
    b.close()


def close(a, b, tol=1e-10):
    a, b = np.asarray(a, float), np.asarray(b, float)
    assert a.shape == b.shape
    assert np.all(np.isfinite(b))
    assert np.all(np.abs(a - b) <= tol * (1 + np.abs(a))), np.max(np.abs(a - b))


def check_features(ref, got):
    same_array(got.valid, ref.valid, "valid")
    close(ref.kmin, got.kmin)
    close(ref.kmax, got.kmax)
    close(ref.normal, got.normal)
    v = ref.valid.astype(bool)
    dmin = np.abs(np.sum(ref.dmin[:, v] * got.dmin[:, v], axis=0))
    dmax = np.abs(np.sum(ref.dmax[:, v] * got.dmax[:, v], axis=0))
    assert np.all(dmin > 1 - 1e-10) and np.all(dmax > 1 - 1e-10)
    assert np.all(got.kmin[v] <= got.kmax[v])


# ---------------------------------------------------------------- curvature
@pytest.mark.parametrize("name", EXAMPLES + ["heightfield"])
@pytest.mark.parametrize("smoothing", [0, 3, 7])
def test_curvature(gpu, oracle_backend, name, smoothing):
    g = load_golden(f"detect_{name}")
    o = options_from(g, "in_").with_(smoothing=smoothing)
    p = prepare(mesh_from(g, "in_"), o)
    ref = oracle_backend.curvature(p.mesh, p.topology, o)
    got = gpu.curvature(p.mesh, p.topology, o)
    check_features(ref, got)
    again = gpu.curvature(p.mesh, p.topology, o)
    same_array(again.kmin, got.kmin)
    same_array(again.dmin, got.dmin)


def test_curvature_matches_reference_golden(gpu):
    g = load_golden("detect_reflection_1")
    o = options_from(g, "in_")
    p = prepare(mesh_from(g, "in_"), o)
    got = gpu.curvature(p.mesh, topology_from(g), o)
    check_features(features_from(g, p.mesh.vertex_count), got)


def test_curvature_planar_is_invalid(gpu):
    m = Mesh(np.array([[0, 1, 1, 0], [0, 0, 1, 1], [0, 0, 0, 0]], float),
             np.array([[0, 0], [1, 2], [2, 3]]))
    o = Options()
    p = prepare(m, o)
    f = gpu.curvature(p.mesh, p.topology, o)
    assert not f.valid.any() and not f.kmin.any() and not f.kmax.any()


# ------------------------------------------------------------------- select
@pytest.mark.parametrize("case", golden_cases("stage_select"), ids=lambda c: c["name"])
def test_select(gpu, case):
    d = case["in"]
    mesh = points_only_mesh(d)
    f = features_from(d, mesh.vertex_count)
    rng = Rng(int(d["seed"][0]))
    s = gpu.select(mesh, f, d["weights"], options_from(d), rng)
    same_array(s.sample, case["out"]["sample"], "sample")
    same_array(s.pruned, case["out"]["pruned"], "pruned")
    assert rng.text() == str(case["out"]["rng_after_select"])


# ------------------------------------------------------------------ pairing
@pytest.mark.parametrize("case", golden_cases("stage_pairing"), ids=lambda c: c["name"])
def test_pairing(gpu, case):
    d = case["in"]
    mesh = points_only_mesh(d)
    f = features_from(d, mesh.vertex_count)
    o = options_from(d)
    if str(case["out"]["error"]):
        with pytest.raises(RuntimeError, match="budget"):
            gpu.pairing(mesh, f, d["selected"], context_from(d), o)
        return
    p = gpu.pairing(mesh, f, d["selected"], context_from(d), o)
    same_array(p.a, case["out"]["pair_a"], "a")
    same_array(p.b, case["out"]["pair_b"], "b")
    again = gpu.pairing(mesh, f, d["selected"], context_from(d), o)
    same_array(again.a, p.a)
    same_array(again.b, p.b)


def test_pairing_random_vs_oracle(gpu, oracle_backend):
    rng = np.random.default_rng(7)
    n = 3000
    pos = rng.uniform(-1, 1, (3, n))
    k0 = rng.normal(0, 1, n)
    f = features_from({"kmin": k0, "kmax": k0 + rng.uniform(0, 0.5, n)}, n)
    mesh = Mesh(pos, np.zeros((3, 0), np.int32))
    sel = rng.permutation(n)[:2500].astype(np.int32)
    for t in [0.02, 0.1, 0.3]:
        o = Options(pair_threshold=t, max_pairs=10 ** 7)
        ref = oracle_backend.pairing(mesh, f, sel, ModelContext(1.0), o)
        got = gpu.pairing(mesh, f, sel, ModelContext(1.0), o)
        same_array(got.a, ref.a)
        same_array(got.b, ref.b)


def test_pairing_rejects_invalid(gpu):
    n = 513
    mesh = Mesh(np.stack([np.arange(n, dtype=float), np.zeros(n), np.zeros(n)]),
                np.zeros((3, 0), np.int32))
    f = features_from({"kmin": np.full(n, 0.5), "kmax": np.ones(n)}, n)
    sel = np.arange(n, dtype=np.int32)
    o = Options()
    for ctx, t in [(ModelContext(0.0), 0.15), (ModelContext(float("nan")), 0.15),
                   (ModelContext(1.0), 0.0), (ModelContext(1.0), float("nan")),
                   (ModelContext(1.0), 1.1)]:
        with pytest.raises(ValueError):
            gpu.pairing(mesh, f, sel, ctx, o.with_(pair_threshold=t))
    for bad in [-1, n]:
        s2 = sel.copy()
        s2[0] = bad
        with pytest.raises(ValueError):
            gpu.pairing(mesh, f, s2, ModelContext(1.0), o)
    f.kmin[0] = np.nan
    with pytest.raises(ValueError):
        gpu.pairing(mesh, f, sel, ModelContext(1.0), o)


def test_pairing_sparse_65536(gpu):
    n = 65536
    mesh = Mesh(np.zeros((3, n)), np.zeros((3, 0), np.int32))
    k = np.arange(1, n + 1, dtype=float)
    f = features_from({"kmin": k, "kmax": k}, n)
    o = Options(pair_threshold=1e-10, max_pairs=1)
    p = gpu.pairing(mesh, f, np.arange(n, dtype=np.int32), ModelContext(1.0), o)
    assert len(p) == 0


def test_pairing_empty_and_single(gpu):
    mesh = Mesh(np.zeros((3, 1)), np.zeros((3, 0), np.int32))
    f = features_from({"kmin": np.ones(1), "kmax": np.ones(1)}, 1)
    for sel in [np.zeros(0, np.int32), np.zeros(1, np.int32)]:
        assert len(gpu.pairing(mesh, f, sel, ModelContext(1.0), Options())) == 0


# ---------------------------------------------------------- transformations
@pytest.mark.parametrize("case", golden_cases("stage_transformations"), ids=lambda c: c["name"])
def test_transformations(gpu, case):
    d = case["in"]
    mesh = points_only_mesh(d)
    f = features_from(d, mesh.vertex_count)
    pairs = Pairs(d["pair_a"], d["pair_b"])
    if str(case["out"]["error"]):
        with pytest.raises(RuntimeError, match="budget"):
            gpu.transformations(mesh, f, pairs, context_from(d), options_from(d))
        return
    v = gpu.transformations(mesh, f, pairs, context_from(d), options_from(d))
    for k, arr in vote_arrays(v).items():
        same_array(arr, case["out"][k], k)


def test_transformations_rejects_invalid(gpu):
    d = golden_cases("stage_transformations")[0]["in"]
    mesh = points_only_mesh(d)
    f = features_from(d, mesh.vertex_count)
    pairs = Pairs(d["pair_a"], d["pair_b"])
    o = options_from(d)
    for ctx in [ModelContext(0.0), ModelContext(float("nan"))]:
        with pytest.raises(ValueError):
            gpu.transformations(mesh, f, pairs, ctx, o)
    for bad in [-1, mesh.vertex_count]:
        with pytest.raises(ValueError):
            gpu.transformations(mesh, f, Pairs([bad], [0]), context_from(d), o)
    assert len(gpu.transformations(Mesh(np.zeros((3, 0)), np.zeros((3, 0), np.int32)),
                                   features_from({}, 0), Pairs([], []), ModelContext(), o)) == 0


# --------------------------------------------------------------- clustering
@pytest.mark.parametrize("case", golden_cases("stage_clustering"), ids=lambda c: c["name"])
def test_clustering(gpu, case):
    d = case["in"]
    votes = votes_from(d)
    rng = Rng(int(d["seed"][0]))
    c = gpu.clustering(votes, context_from(d), options_from(d), rng)
    want = case["out"]
    assert rng.text() == str(want["rng_after_clustering"])
    assert c.limited_iterations == int(want["limited_iterations"][0])
    same_array(c.votes.offsets, want["cl_vote_offsets"], "offsets")
    same_array(c.votes.indices, want["cl_vote_indices"], "indices")
    same_array(c.reflection, want["cl_reflection"], "reflection")
    # the means add the members in the reference's order, so the cluster
    # records are the reference's bit for bit
    for k in ["cl_rotation", "cl_translation", "cl_plane_normal", "cl_plane_offset"]:
        same_array(cluster_arrays(c)[k], want[k], k)
    rng2 = Rng(int(d["seed"][0]))
    again = gpu.clustering(votes, context_from(d), options_from(d), rng2)
    same_array(again.votes.indices, c.votes.indices)
    same_array(again.rotation, c.rotation)


def test_clustering_large(gpu):
    """100,000 votes (regenerated from integers, tests/helpers.py): the
    reference's memberships, cluster order, records and RNG state; the
    trajectories of every vote run in seed batches of bounded device
    memory."""
    from helpers import digest, large_clustering_votes
    g = load_golden("stage_clustering_large")
    votes = large_clustering_votes(int(g["votes"]), seed=int(g["generator_seed"]))
    o = Options(bandwidth=float(g["bandwidth"]), max_clusters=int(g["max_clusters"]),
                max_iterations=int(g["max_iterations"]))
    rng = Rng(int(g["seed"]))
    c = gpu.clustering(votes_from(votes), ModelContext(10.0, (0.0, 0.0, 0.0)), o, rng)
    got = cluster_arrays(c)
    assert digest(got["cl_vote_indices"]) == str(g["sha_cl_vote_indices"])
    for k in ("cl_vote_offsets", "cl_reflection", "cl_rotation", "cl_translation",
              "cl_plane_normal", "cl_plane_offset"):
        same_array(got[k], g[k], k)
    assert c.limited_iterations == int(g["limited_iterations"][0])
    assert rng.text() == str(g["rng_after_clustering"])


# ------------------------------------------------------------- verification
@pytest.mark.parametrize("case", golden_cases("stage_verification"), ids=lambda c: c["name"])
def test_verification(gpu, case):
    d = case["in"]
    o = options_from(d)
    p = prepare(mesh_from(d), o)
    v = gpu.verification(p.mesh, p.topology, clusters_from(d), p.context, o)
    got = verification_arrays(v)
    for k, arr in got.items():
        if k == "ver_rms":
            assert np.all(np.abs(arr - case["out"][k]) < 1e-12 * p.context.box_size)
        else:
            same_array(arr, case["out"][k], k)
    assert v.side_a.row(0)[0] == 0
    assert v.side_a.row(1).size == 0 and v.side_b.row(1).size == 0
    again = gpu.verification(p.mesh, p.topology, clusters_from(d), p.context, o)
    same_array(again.patches_a.indices, v.patches_a.indices)


def test_triangle_distances(gpu):
    g = load_golden("stage_triangles")
    got = gpu.triangle_distances(g["queries"])
    ref = g["distances"]
    assert np.all(np.isfinite(got))
    assert np.all(np.abs(got - ref) <= 1e-12 * (1 + ref))
    assert gpu.triangle_distances(np.zeros(0)).size == 0


# ---------------------------------------------------- full detect() fixtures
@pytest.mark.parametrize("name", ["reflection_1", "reflection_05", "rigid_1", "rigid_05",
                                  "partial_1", "partial_05", "single_1", "single_05",
                                  "heightfield"])
def test_detect_stages_against_reference(gpu, name):
    """Each GPU stage on the reference's own inputs against the reference's
    outputs from a full detect() run."""
    g = load_golden(f"detect_{name}")
    o = options_from(g, "in_")
    p = prepare(mesh_from(g, "in_"), o)
    topo = topology_from(g) if "vnx" in g else p.topology
    f = oracle.OracleBackend().curvature(p.mesh, topo, o) if "nx" not in g else \
        features_from(g, p.mesh.vertex_count)
    rng = Rng(o.seed)
    s = gpu.select(p.mesh, f, topo.weights, o, rng)
    same_array(s.sample, g["sample"], "sample")
    same_array(s.pruned, g["pruned"], "pruned")
    assert rng.text() == str(g["rng_after_select"])
    pairs = gpu.pairing(p.mesh, f, g["pruned"], p.context, o)
    same_array(pairs.a, g["pair_a"], "pair_a")
    same_array(pairs.b, g["pair_b"], "pair_b")
    v = gpu.transformations(p.mesh, f, pairs, p.context, o)
    got = vote_arrays(v)
    if "desc0" in g:
        for k, arr in got.items():
            same_array(arr, g[k], k)
        ref_votes = votes_from(g)
    else:
        ref_votes = oracle.OracleBackend().transformations(p.mesh, f, pairs, p.context, o)
        for k, arr in vote_arrays(ref_votes).items():
            same_array(got[k], arr, k)
    c = gpu.clustering(ref_votes, p.context, o, rng)
    assert rng.text() == str(g["rng_after_clustering"])
    same_array(c.votes.offsets, g["cl_vote_offsets"], "cl offsets")
    same_array(c.votes.indices, g["cl_vote_indices"], "cl indices")
    assert c.limited_iterations == int(g["limited_iterations"][0])
    ver = gpu.verification(p.mesh, topo, clusters_from(g), p.context, o)
    for k, arr in verification_arrays(ver).items():
        if k == "ver_rms":
            assert np.all(np.abs(arr - g[k]) < 1e-12 * p.context.box_size)
        else:
            same_array(arr, g[k], k)
