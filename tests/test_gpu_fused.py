"""Fused batched detection (sym_detect_fast_fused, no reference
counterpart): the stages before the mean shift run mesh by mesh, then one
mean shift serves every mesh's seeds, each mesh's votes moved to their own
cell of vote space.  Against sym_detect_fast on each mesh alone: the same
samples, pairs and votes (exact), and every strongly supported mode with a
well-defined position (Newton-converged seeds) found again within 2e-4
relative -- each run's modes are held to 1e-4 of FP64 (the mode-error
target), so two runs may differ by twice that: the fused run's FP32 sums go
in another order, its BF16 tiles hold other seeds."""
import numpy as np
import pytest

from mitra_algo_gb300.mesh import mirrored_heightfield, motif_sphere, prepare
from mitra_algo_gb300.types import Options

pytestmark = pytest.mark.gpu

BANDWIDTH = 0.1


@pytest.fixture(scope="module")
def batch():
    from mitra_algo_gb300 import Gb300Backend
    gpu = Gb300Backend(0)
    meshes = [(motif_sphere(level=4, bumps=8, folds=5, partial_shift=0.3, noise=1e-3, seed=1),
               "rigid", 0.25),
              (motif_sphere(level=5, bumps=10, folds=3, partial_shift=0.4, noise=5e-4, seed=2),
               "rigid", 0.25),
              (mirrored_heightfield(size=64, bumps=5, seed=3), "reflection", 0.05),
              (motif_sphere(level=4, bumps=6, folds=4, partial_shift=0.25, noise=0.0, seed=4),
               "rigid", 0.25)]
    jobs, modes = [], []
    for mesh, mode, threshold in meshes:
        o = Options(sample_ratio=min(1.0, 3000 / mesh.vertex_count), pair_threshold=threshold,
                    bandwidth=BANDWIDTH, max_pairs=10 ** 7, max_votes=2 * 10 ** 7, max_clusters=6)
        jobs.append((gpu.load_mesh(prepare(mesh, o)), None, o))
        modes.append(mode)
    yield gpu, jobs, modes
    for m, _, _ in jobs:
        m.close()
    gpu.close()


def motion(r, i):
    return np.concatenate([np.ravel(r["rotation"][i]), r["translation"][i]])


@pytest.mark.parametrize("precision", ["bf16", "fp32"])
def test_fused_equals_single_mesh_runs(batch, precision):
    gpu, jobs, modes = batch
    kw = dict(precision=precision, seeds=256, max_iterations=300, polish_iterations=30)
    fused, stats = gpu.detect_fast_fused(jobs, mode=modes, **kw)
    assert stats["meshes"] == len(jobs) and stats["seeds"] == sum(min(256, f["votes"]) for f in fused)
    assert stats["votes"] == sum(f["votes"] for f in fused)
    for (mesh, sample, o), mode, f in zip(jobs, modes, fused):
        alone = gpu.detect_fast(mesh, sample, o, mode=mode, **kw)
        for k in ("sampled", "pruned", "pairs", "votes"):
            assert f[k] == alone[k], k
        assert f["clusters"] > 0
        strong = 0.5 * max(alone["support"])
        found = [motion(f, i) for i in range(f["clusters"]) if f["precise"][i]]
        for i in range(alone["clusters"]):
            if not (alone["precise"][i] and alone["support"][i] >= strong):
                continue
            want = motion(alone, i)
            err = min(np.linalg.norm(m - want) / np.linalg.norm(want) for m in found)
            assert err <= 2e-4, (mode, i, err)


def test_fused_rejects_mixed_bandwidths(batch):
    gpu, jobs, modes = batch
    (m0, s0, o0), rest = jobs[0], jobs[1:]
    other = Options(**{**o0.__dict__, "bandwidth": BANDWIDTH * 2})
    with pytest.raises(ValueError):
        gpu.detect_fast_fused([(m0, s0, other)] + rest, mode=modes)


def test_uneven_batch_fused(batch):
    """Twelve meshes of the uneven batch (2k-60k vertices, rigid and
    reflection mixed, samples drawn on the device): the same pairs and votes
    as the single-mesh runs, and every strongly supported Newton-converged
    mode found again (12 modes reported, so that the strong ones are not
    cut by the cap on the reported count).  "Strongly supported" here also
    means at least 50 votes within the
    bandwidth: with 1,500 samples some of these meshes' vote sets are so
    sparse that most seeds end in modes of a handful of votes, whose
    positions are noise."""
    from mitra_algo_gb300.mesh import uneven_batch
    gpu = batch[0]
    jobs, modes = [], []
    for mesh, mode, _ in uneven_batch(12, seed=5):
        o = Options(sample_ratio=min(1.0, 1500 / mesh.vertex_count),
                    pair_threshold=0.25 if mode == "rigid" else 0.05, bandwidth=BANDWIDTH,
                    max_pairs=10 ** 7, max_votes=2 * 10 ** 7, max_clusters=12)
        jobs.append((gpu.load_mesh_raw(mesh, o), None, o))
        modes.append(mode)
    try:
        kw = dict(precision="bf16", seeds=128, max_iterations=300, polish_iterations=30)
        fused, _ = gpu.detect_fast_fused(jobs, mode=modes, **kw)
        for (mesh, _, o), mode, f in zip(jobs, modes, fused):
            alone = gpu.detect_fast(mesh, None, o, mode=mode, **kw)
            for k in ("sampled", "pruned", "pairs", "votes"):
                assert f[k] == alone[k], k
            strong = max(0.5 * max(alone["support"], default=0), 50)
            found = [motion(f, i) for i in range(f["clusters"]) if f["precise"][i]]
            for i in range(alone["clusters"]):
                if alone["precise"][i] and alone["support"][i] >= strong:
                    want = motion(alone, i)
                    err = min(np.linalg.norm(m - want) / np.linalg.norm(want) for m in found)
                    assert err <= 2e-4, (mode, i, err)
    finally:
        for m, _, _ in jobs:
            m.close()


def test_fused_reports_a_failing_item(batch):
    """An item whose sample holds an out-of-range vertex fails with the
    reference's message while the others are processed, and the context
    (with its helper contexts) serves the next fused call unchanged."""
    gpu, jobs, modes = batch
    kw = dict(precision="bf16", seeds=64, max_iterations=60, polish_iterations=20)
    (m0, _, o0) = jobs[0]
    bad = np.array([0, m0.prepared.mesh.vertex_count], np.int32)
    with pytest.raises(Exception, match="sample vertex index out of range"):
        gpu.detect_fast_fused([jobs[1], (m0, bad, o0), jobs[2]], mode=[modes[1], modes[0], modes[2]],
                              **kw)
    again, _ = gpu.detect_fast_fused(jobs[1:3], mode=modes[1:3], **kw)
    first, _ = gpu.detect_fast_fused(jobs[1:3], mode=modes[1:3], **kw)
    for a, b in zip(again, first):
        for k in ("sampled", "pairs", "votes", "clusters", "support"):
            assert a[k] == b[k], k
