"""Pins the oracle (and the host-side prepare) to golden vectors produced by the
reference's own CPU library (tests/golden/make_golden.py).  Every comparison is
bit-exact: the oracle restates the reference operation by operation."""
import numpy as np
import pytest

from conftest import golden_cases, load_golden
from helpers import (cluster_arrays, context_from, digest, feature_arrays, features_from,
                     mesh_from, options_from, points_only_mesh, same_array, topology_arrays,
                     topology_from, verification_arrays, vote_arrays, votes_from)
from mitra_algo_gb300.mesh import prepare
from mitra_algo_gb300.types import Pairs
from oracle import oracle

DETECT = ["reflection_1", "reflection_05", "rigid_1", "rigid_05", "partial_1", "partial_05",
          "single_1", "single_05", "heightfield"]


def check(got: dict, golden: dict):
    for k, v in got.items():
        if k in golden:
            same_array(v, golden[k], k)
        elif f"sha_{k}" in golden:
            assert digest(np.ascontiguousarray(v, dtype=v.dtype)) == str(golden[f"sha_{k}"]), k
        else:
            raise AssertionError(f"golden has no {k}")


def test_rng_matches_std_mt19937_64():
    g = load_golden("stage_rng")
    r = oracle.rng(42)
    assert r.text() == str(g["rng_seeded"])
    draws = [r.next() for _ in range(1000)]
    assert np.array_equal(np.array(draws, np.uint64), g["draws"])
    assert r.text() == str(g["rng_after_draws"])


def test_triangle_distances(oracle_backend):
    g = load_golden("stage_triangles")
    q = g["queries"].reshape(-1, 12)
    got = np.array([oracle_backend.triangle_distance2(r[0:3], r[3:6], r[6:9], r[9:12]) for r in q])
    same_array(got, g["distances"])
    # the reference's known answers (tests/geometry.cpp:14-20)
    assert np.allclose(got[:6], [4, 1, 2, 0.5, 1, 1], atol=1e-10)


@pytest.mark.parametrize("case", golden_cases("stage_select"), ids=lambda c: c["name"])
def test_select(case, oracle_backend):
    d = case["in"]
    mesh = points_only_mesh(d)
    f = features_from(d, mesh.vertex_count)
    rng = oracle.rng(int(d["seed"][0]))
    s = oracle_backend.select(mesh, f, d["weights"], options_from(d), rng)
    same_array(s.sample, case["out"]["sample"], "sample")
    same_array(s.pruned, case["out"]["pruned"], "pruned")
    assert rng.text() == str(case["out"]["rng_after_select"])


@pytest.mark.parametrize("case", golden_cases("stage_sampling"), ids=lambda c: c["name"])
def test_sampling(case, oracle_backend):
    d = case["in"]
    rng = oracle.rng(int(d["seed"][0]))
    got = oracle_backend.sample_vertices(d["weights"], float(d["sample_ratio"][0]), rng)
    same_array(got, case["out"]["sample"], "sample")
    assert rng.text() == str(case["out"]["rng_after_select"])


@pytest.mark.parametrize("case", golden_cases("stage_pairing"), ids=lambda c: c["name"])
def test_pairing(case, oracle_backend):
    d = case["in"]
    mesh = points_only_mesh(d)
    f = features_from(d, mesh.vertex_count)
    o = options_from(d)
    err = str(case["out"]["error"])
    if err:
        with pytest.raises(RuntimeError, match="budget"):
            oracle_backend.pairing(mesh, f, d["selected"], context_from(d), o)
        return
    p = oracle_backend.pairing(mesh, f, d["selected"], context_from(d), o)
    same_array(p.a, case["out"]["pair_a"], "a")
    same_array(p.b, case["out"]["pair_b"], "b")


@pytest.mark.parametrize("case", golden_cases("stage_transformations"), ids=lambda c: c["name"])
def test_transformations(case, oracle_backend):
    d = case["in"]
    mesh = points_only_mesh(d)
    f = features_from(d, mesh.vertex_count)
    pairs = Pairs(d["pair_a"], d["pair_b"])
    if str(case["out"]["error"]):
        with pytest.raises(RuntimeError, match="budget"):
            oracle_backend.transformations(mesh, f, pairs, context_from(d), options_from(d))
        return
    v = oracle_backend.transformations(mesh, f, pairs, context_from(d), options_from(d))
    check(vote_arrays(v), case["out"])


@pytest.mark.parametrize("case", golden_cases("stage_clustering"), ids=lambda c: c["name"])
def test_clustering(case, oracle_backend):
    d = case["in"]
    rng = oracle.rng(int(d["seed"][0]))
    c = oracle_backend.clustering(votes_from(d), context_from(d), options_from(d), rng)
    check(cluster_arrays(c), case["out"])
    assert c.limited_iterations == int(case["out"]["limited_iterations"][0])
    assert rng.text() == str(case["out"]["rng_after_clustering"])


def test_clustering_large(oracle_backend):
    """100,000 regenerated votes (tests/helpers.py:large_clustering_votes)
    against the reference's clustering of them."""
    from helpers import digest, large_clustering_votes
    from mitra_algo_gb300.types import ModelContext, Options
    g = load_golden("stage_clustering_large")
    votes = large_clustering_votes(int(g["votes"]), seed=int(g["generator_seed"]))
    o = Options(bandwidth=float(g["bandwidth"]), max_clusters=int(g["max_clusters"]),
                max_iterations=int(g["max_iterations"]))
    rng = oracle.rng(int(g["seed"]))
    c = oracle_backend.clustering(votes_from(votes), ModelContext(10.0, (0.0, 0.0, 0.0)), o, rng)
    got = cluster_arrays(c)
    assert digest(got["cl_vote_indices"]) == str(g["sha_cl_vote_indices"])
    for k in ("cl_vote_offsets", "cl_reflection", "cl_rotation", "cl_translation",
              "cl_plane_normal", "cl_plane_offset"):
        assert np.array_equal(got[k], g[k]), k
    assert c.limited_iterations == int(g["limited_iterations"][0])
    assert rng.text() == str(g["rng_after_clustering"])


@pytest.mark.parametrize("case", golden_cases("stage_verification"), ids=lambda c: c["name"])
def test_verification(case, oracle_backend):
    d = case["in"]
    o = options_from(d)
    p = prepare(mesh_from(d), o)
    clusters = __import__("helpers").clusters_from(d)
    v = oracle_backend.verification(p.mesh, p.topology, clusters, p.context, o)
    check(verification_arrays(v), case["out"])


@pytest.mark.parametrize("name", DETECT)
def test_detect_stages(name, oracle_backend):
    """prepare + every oracle stage against a full reference detect() run."""
    g = load_golden(f"detect_{name}")
    o = options_from(g, "in_")
    p = prepare(mesh_from(g, "in_"), o)
    check(topology_arrays(p.topology), g)
    same_array(p.mesh.vertices[0], g["vx"], "vx")
    assert p.context.box_size == float(g["box_size"][0])
    same_array(np.array(p.context.center), g["center"], "center")
    # each stage runs on the reference's own inputs, so a mismatch is local
    topo = topology_from(g) if "vnx" in g else p.topology
    f = oracle_backend.curvature(p.mesh, topo, o)
    check(feature_arrays(f), g)
    ref_f = features_from(g, p.mesh.vertex_count) if "nx" in g else f
    rng = oracle.rng(o.seed)
    s = oracle_backend.select(p.mesh, ref_f, topo.weights, o, rng)
    same_array(s.sample, g["sample"], "sample")
    same_array(s.pruned, g["pruned"], "pruned")
    assert rng.text() == str(g["rng_after_select"])
    pairs = oracle_backend.pairing(p.mesh, ref_f, g["pruned"], p.context, o)
    same_array(pairs.a, g["pair_a"], "pair_a")
    same_array(pairs.b, g["pair_b"], "pair_b")
    v = oracle_backend.transformations(p.mesh, ref_f, pairs, p.context, o)
    check(vote_arrays(v), g)
    ref_v = votes_from(g) if "desc0" in g else v
    c = oracle_backend.clustering(ref_v, p.context, o, rng)
    check(cluster_arrays(c), g)
    assert c.limited_iterations == int(g["limited_iterations"][0])
    assert rng.text() == str(g["rng_after_clustering"])
    ver = oracle_backend.verification(p.mesh, topo, c, p.context, o)
    check(verification_arrays(ver), g)
