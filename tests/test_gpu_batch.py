"""Batched detection (sym_detect_fast_batch, no reference counterpart): a
batch of uneven motif meshes run three at a time on separate worker contexts
gives, mesh by mesh, exactly the results of sym_detect_fast run alone (every
mesh's computation is independent of the others and deterministic), and a
failing item reports its own error."""
import numpy as np
import pytest

from mitra_algo_gb300.mesh import motif_sphere, prepare
from mitra_algo_gb300.types import Options, Rng

pytestmark = pytest.mark.gpu

KEYS = ("pruned", "pairs", "votes", "modes", "clusters", "iterations", "polish_iterations",
        "support", "rotation", "translation", "coverage", "rms", "patches", "precise")


@pytest.fixture(scope="module")
def batch():
    from mitra_algo_gb300 import Gb300Backend
    gpu = Gb300Backend(0)
    jobs, meshes = [], []
    for i, (level, folds) in enumerate([(4, 3), (5, 5), (4, 4), (5, 2), (4, 5)]):
        mesh = motif_sphere(level=level, bumps=8, folds=folds, partial_shift=0.3, noise=1e-3,
                            seed=10 + i)
        opts = Options(sample_ratio=min(1.0, 3000 / mesh.vertex_count), pair_threshold=0.25,
                       bandwidth=0.1, max_pairs=10 ** 7, max_votes=2 * 10 ** 7, max_clusters=8)
        p = prepare(mesh, opts)
        f = gpu.curvature(p.mesh, p.topology, opts)
        sample = gpu.select(p.mesh, f, p.topology.weights, opts, Rng(opts.seed)).sample
        resident = gpu.load_mesh(p)
        meshes.append(resident)
        jobs.append((resident, sample, opts))
    yield gpu, jobs
    for m in meshes:
        m.close()
    gpu.close()


def same(a, b):
    for k in KEYS:
        assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), k


def test_batch_equals_single_runs(batch):
    gpu, jobs = batch
    kw = dict(precision="bf16", seeds=256, max_iterations=100, polish_iterations=30)
    alone = [gpu.detect_fast(m, s, o, **kw) for m, s, o in jobs]
    together = gpu.detect_fast_batch(jobs, workers=3, **kw)
    assert len(together) == len(jobs)
    for a, b in zip(alone, together):
        assert a["pairs"] > 0 and a["votes"] > 0
        same(a, b)
    # the worker contexts are kept: a second call gives the same results again
    again = gpu.detect_fast_batch(jobs, workers=3, **kw)
    for a, b in zip(alone, again):
        same(a, b)


def test_batch_fp32_form(batch):
    gpu, jobs = batch
    kw = dict(precision="fp32", seeds=128, max_iterations=60, polish_iterations=20)
    alone = [gpu.detect_fast(m, s, o, **kw) for m, s, o in jobs[:3]]
    together = gpu.detect_fast_batch(jobs[:3], workers=2, **kw)
    for a, b in zip(alone, together):
        same(a, b)


def test_batch_reports_a_failing_item(batch):
    gpu, jobs = batch
    mesh, sample, opts = jobs[0]
    bad = np.array(sample, np.int32)
    bad[0] = mesh.prepared.mesh.vertex_count  # out of range
    with pytest.raises(Exception, match="sample vertex index out of range"):
        gpu.detect_fast_batch([jobs[1], (mesh, bad, opts), jobs[2]], workers=2, seeds=64,
                              max_iterations=20, polish_iterations=5)


def test_batch_items_may_sample_on_the_device(batch):
    """An item without a sample draws it on the device from its options'
    seed (sym_detect_fast_sampled): the results equal detect_fast with the
    sample None, and also with the host-drawn sample of the fixture."""
    gpu, jobs = batch
    kw = dict(precision="bf16", seeds=128, max_iterations=60, polish_iterations=20)
    alone = [gpu.detect_fast(m, None, o, **kw) for m, _, o in jobs[:3]]
    with_host_sample = [gpu.detect_fast(m, s, o, **kw) for m, s, o in jobs[:3]]
    together = gpu.detect_fast_batch([(m, None, o) for m, _, o in jobs[:3]], workers=2, **kw)
    for a, b, c in zip(alone, together, with_host_sample):
        same(a, b)
        same(a, c)
        assert a["sampled"] == b["sampled"] > 0
