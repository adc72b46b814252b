"""The throughput pipeline (sym_mesh_load + sym_detect_fast, no reference
counterpart) on the 256-seed motif-sphere case: it finds the planted 5-fold
rotation about z, its LBVH verification (FP32 decisions, FP64 rechecks) gives
the patch counts, coverage and rms of the exact verification
(sym_verification, the reference's algorithm) of the same modes, and the
BF16-refined and FP32 forms report the same top modes.

Tolerances: patch counts equal; coverage and rms within 1e-12 relative (the
throughput path sums in a fixed tree instead of the reference's serial
order; the reference's own CPU/GPU comparison allows 2e-10,
tests/compare_cuda.py:20-21); top modes of the two mean-shift forms agree
to 1e-4 relative (the mode-error target)."""
import numpy as np
import pytest

from mitra_algo_gb300.mesh import motif_sphere, prepare
from mitra_algo_gb300.types import ClusterOutput, Csr, Options, Rng

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fast():
    from mitra_algo_gb300 import Gb300Backend
    gpu = Gb300Backend(0)
    mesh = motif_sphere(level=5, bumps=12, folds=5, partial_shift=0.4, noise=1e-3, seed=0)
    opts = Options(sample_ratio=5000 / mesh.vertex_count, pair_threshold=0.25, bandwidth=0.1,
                   max_pairs=2 * 10 ** 7, max_votes=5 * 10 ** 7, max_clusters=8)
    p = prepare(mesh, opts)
    f = gpu.curvature(p.mesh, p.topology, opts)
    sample = gpu.select(p.mesh, f, p.topology.weights, opts, Rng(opts.seed)).sample
    resident = gpu.load_mesh(p)
    runs = {pr: gpu.detect_fast(resident, sample, opts, precision=pr, seeds=256,
                                max_iterations=300, polish_iterations=30)
            for pr in ("bf16", "fp32")}
    yield gpu, p, opts, runs
    resident.close()
    gpu.close()


def rotation_angle_axis(r):
    r = np.asarray(r).reshape(3, 3)
    angle = np.arccos(np.clip((np.trace(r) - 1) / 2, -1, 1))
    axis = np.array([r[2, 1] - r[1, 2], r[0, 2] - r[2, 0], r[1, 0] - r[0, 1]])
    return angle, axis / max(np.linalg.norm(axis), 1e-300)


def test_finds_the_five_fold_rotation(fast):
    _, _, _, runs = fast
    r = runs["bf16"]
    assert r["clusters"] > 0 and r["pairs"] > 0 and r["votes"] > 0
    hits = []
    for rot, cov in zip(r["rotation"], r["coverage"]):
        angle, axis = rotation_angle_axis(rot)
        k = angle / (2 * np.pi / 5)
        if abs(axis[2]) > 0.99 and abs(k - round(k)) < 0.05 and round(k) in (1, 2):
            hits.append(cov)
    assert hits and max(hits) > 0.3, (hits, r["coverage"])


def test_fast_verification_matches_exact(fast):
    gpu, p, opts, runs = fast
    r = runs["bf16"]
    n = r["clusters"]
    clusters = ClusterOutput(np.zeros(n, np.uint8), np.array(r["rotation"]),
                             np.array(r["translation"]), np.zeros((n, 3)), np.zeros(n),
                             Csr(np.zeros(n + 1, np.uint64), np.zeros(0, np.int32)))
    exact = gpu.verification(p.mesh, p.topology, clusters, p.context, opts)
    assert np.allclose(r["coverage"], exact.coverage, rtol=1e-12, atol=0), (r["coverage"], exact.coverage)
    assert np.allclose(r["rms"], exact.rms, rtol=1e-12, atol=0), (r["rms"], exact.rms)
    pa = np.diff(exact.patches_a_groups.astype(np.int64))
    pb = np.diff(exact.patches_b_groups.astype(np.int64))
    got = np.array(r["patches"]).reshape(n, 2)
    assert np.array_equal(got[:, 0], pa) and np.array_equal(got[:, 1], pb), \
        (got.tolist(), pa.tolist(), pb.tolist())


def test_forms_agree_on_the_top_modes(fast):
    _, _, _, runs = fast
    b, f = runs["bf16"], runs["fp32"]
    assert b["pairs"] == f["pairs"] and b["votes"] == f["votes"]
    # every strongly supported FP32 mode with a well-defined position
    # (Newton-converged seeds) has a BF16-refined mode within 1e-4; modes on
    # ridges of the vote set (e.g. the base sphere's continuous rotations)
    # have no such position, and modes of a seed or two may land in either
    # run's basin
    strong = 0.5 * max(f["support"])
    top = [i for i, (ok, sup) in enumerate(zip(f["precise"], f["support"])) if ok and sup >= strong]
    assert top and f["precise"][0]
    mb = [np.concatenate([np.ravel(r), t])
          for r, t, ok in zip(b["rotation"], b["translation"], b["precise"]) if ok]
    for i in top:
        mf = np.concatenate([np.ravel(f["rotation"][i]), f["translation"][i]])
        err = min(np.linalg.norm(m - mf) / np.linalg.norm(mf) for m in mb)
        assert err <= 1e-4, (i, err)


def test_every_reference_seed_and_mode_is_reported(fast):
    """With reference seeds, every one of them is compared with its FP64 run
    (none dropped: Newton-converged in both, settled on a ridge, or
    unconverged), and every reported mode's motion carries its error against
    the FP64 mode reached from the same position: within 1e-4 for modes
    formed by Newton-converged seeds (measured: under 5e-6), finite for
    ridge modes, whose FP64 restart may slide along the ridge."""
    gpu, p, opts, _ = fast
    resident = gpu.load_mesh(p)
    r = gpu.detect_fast(resident, None, opts, precision="bf16", seeds=256, max_iterations=300,
                        polish_iterations=30, reference_seeds=64, refine=2)
    resident.close()
    assert r["seeds_compared"] == 64
    assert r["modes_compared"] + r["seeds_settled"] + r["seeds_unconverged"] == 64
    assert r["mode_error_all_max"] >= r["mode_error_max"]
    assert r["seeds_within"] >= r["modes_within"]
    n = r["clusters"]
    assert n > 0 and len(r["transform_error"]) == n and len(r["transform_error_refined"]) == n
    assert all(np.isfinite(r["transform_error"])) and all(np.isfinite(r["transform_error_refined"]))
    for err, precise in zip(r["transform_error"], r["precise"]):
        if precise:
            assert err <= 1e-4, (err, r["transform_error"])
    assert r["transform_error_max"] == max(r["transform_error"])


# --------------------------------------------------------- reflection mode
# The mirrored height field (128 x 128 grid, 8 bumps mirrored in x, 2,000
# samples, 5% curvature tolerance, bandwidth 0.02) has one plane of symmetry,
# x = 0; reflection mode votes one plane per pair whose mirrored frames agree.

@pytest.fixture(scope="module")
def refl():
    from mitra_algo_gb300 import Gb300Backend
    from mitra_algo_gb300.mesh import mirrored_heightfield
    gpu = Gb300Backend(0)
    mesh = mirrored_heightfield(size=128, bumps=8, seed=0)
    opts = Options(sample_ratio=2000 / mesh.vertex_count, pair_threshold=0.05, bandwidth=0.02,
                   max_pairs=10 ** 7, max_votes=2 * 10 ** 7, max_clusters=8)
    p = prepare(mesh, opts)
    f = gpu.curvature(p.mesh, p.topology, opts)
    sample = gpu.select(p.mesh, f, p.topology.weights, opts, Rng(opts.seed)).sample
    resident = gpu.load_mesh(p)
    runs = {pr: gpu.detect_fast(resident, sample, opts, precision=pr, seeds=512,
                                max_iterations=100, polish_iterations=30, mode="reflection")
            for pr in ("bf16", "fp32")}
    yield gpu, p, opts, runs
    resident.close()
    gpu.close()


def test_reflection_finds_the_mirror_plane(refl):
    _, p, _, runs = refl
    for pr, r in runs.items():
        assert r["clusters"] > 0 and r["votes"] > 0, pr
        assert all(r["reflection"]), pr
        n, off = np.array(r["plane_normal"][0]), r["plane_offset"][0]
        assert abs(abs(n[0]) - 1) < 1e-3 and abs(off) < 1e-3 * p.context.box_size, (pr, n, off)
        assert r["coverage"][0] > 0.5, (pr, r["coverage"])


def test_reflection_forms_agree(refl):
    _, _, _, runs = refl
    b, f = runs["bf16"], runs["fp32"]
    assert b["pairs"] == f["pairs"] and b["votes"] == f["votes"]
    pb = np.concatenate([b["plane_normal"][0], [b["plane_offset"][0]]])
    pf = np.concatenate([f["plane_normal"][0], [f["plane_offset"][0]]])
    assert np.linalg.norm(pb - pf) <= 1e-4 * np.linalg.norm(pf), (pb, pf)


def test_reflection_fast_verification_matches_exact(refl):
    gpu, p, opts, runs = refl
    r = runs["bf16"]
    n = r["clusters"]
    clusters = ClusterOutput(np.ones(n, np.uint8), np.array(r["rotation"]),
                             np.array(r["translation"]), np.array(r["plane_normal"]),
                             np.array(r["plane_offset"]),
                             Csr(np.zeros(n + 1, np.uint64), np.zeros(0, np.int32)))
    exact = gpu.verification(p.mesh, p.topology, clusters, p.context, opts)
    assert np.allclose(r["coverage"], exact.coverage, rtol=1e-12, atol=0), (r["coverage"], exact.coverage)
    assert np.allclose(r["rms"], exact.rms, rtol=1e-12, atol=0), (r["rms"], exact.rms)
    got = np.array(r["patches"]).reshape(n, 2)
    assert np.array_equal(got[:, 0], np.diff(exact.patches_a_groups.astype(np.int64)))
    assert np.array_equal(got[:, 1], np.diff(exact.patches_b_groups.astype(np.int64)))


def test_vote_cap_subsamples_uniformly_and_deterministically(fast):
    gpu, p, opts, runs = fast
    full = runs["bf16"]["votes"]
    cap = full // 4
    sample = gpu.select(p.mesh, gpu.curvature(p.mesh, p.topology, opts), p.topology.weights, opts,
                        Rng(opts.seed)).sample
    resident = gpu.load_mesh(p)
    kw = dict(seeds=128, max_iterations=60, polish_iterations=10, vote_cap=cap)
    a = gpu.detect_fast(resident, sample, opts, precision="bf16", **kw)
    b = gpu.detect_fast(resident, sample, opts, precision="bf16", **kw)
    c = gpu.detect_fast(resident, sample, opts, precision="fp32", **kw)
    resident.close()
    assert a["pairs"] == runs["bf16"]["pairs"]          # every pair is still formed
    assert abs(a["votes"] - cap) <= 0.02 * cap            # ~cap votes enter the mean shift
    assert a["votes"] == b["votes"] == c["votes"]         # the same subsample every run
    assert a["rotation"] == b["rotation"] and a["support"] == b["support"]


@pytest.mark.parametrize("precision", ["bf16", "fp32"])
def test_gaussian_kernel_pipeline(fast, precision):
    """The pipeline with the shifted Gaussian kernel (exp weights): the
    same pairs and votes, the compared modes within 1e-4 of the FP64 run of
    the same seeds (a BF16 approach may leave one seed in 50 at a nearby
    fixed point: measured 101 of 102 within, the other at 2.8e-4), and the
    planted 5-fold rotation among the top modes."""
    gpu, p, opts, runs = fast
    resident = gpu.load_mesh(p)
    r = gpu.detect_fast(resident, None, opts, precision=precision, seeds=256, max_iterations=300,
                        polish_iterations=30, reference_seeds=128, kernel="gaussian")
    resident.close()
    assert r["pairs"] == runs[precision]["pairs"] and r["votes"] == runs[precision]["votes"]
    assert r["modes_compared"] >= 10
    spare = 0 if precision == "fp32" else max(1, r["modes_compared"] // 50)
    assert r["modes_within"] >= r["modes_compared"] - spare, r["mode_error_max"]
    assert r["mode_error_max"] < 1e-3
    hits = []
    for rot in r["rotation"]:
        angle, axis = rotation_angle_axis(rot)
        k = angle / (2 * np.pi / 5)
        hits.append(abs(axis[2]) > 0.99 and abs(k - round(k)) < 0.05 and round(k) in (1, 2))
    assert any(hits)
