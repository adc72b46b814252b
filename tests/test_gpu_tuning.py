"""Launch-shape parameters of the mean shift (sym_fast_options vote_bits,
simt_blocks_per_sm, tc_ctas_per_sm, check_interval) and the autotuner on the
GPU: the host-check interval changes nothing in the results; the other
shapes keep the pair and vote sets and every compared mode within 1e-4 of
FP64; the tuner returns one of the candidate shapes, no slower than the
defaults."""
import numpy as np
import pytest

from mitra_algo_gb300.autotune import CANDIDATES, autotune
from mitra_algo_gb300.mesh import motif_sphere, prepare
from mitra_algo_gb300.types import Options

pytestmark = pytest.mark.gpu

KEYS = ("pairs", "votes", "modes", "clusters", "iterations", "polish_iterations", "support",
        "rotation", "translation", "coverage", "rms", "patches")


@pytest.fixture(scope="module")
def job():
    from mitra_algo_gb300 import Gb300Backend
    gpu = Gb300Backend(0)
    mesh = motif_sphere(level=5, bumps=10, folds=5, partial_shift=0.3, noise=1e-3, seed=21)
    o = Options(sample_ratio=min(1.0, 4000 / mesh.vertex_count), pair_threshold=0.25,
                bandwidth=0.1, max_pairs=10 ** 7, max_votes=2 * 10 ** 7, max_clusters=8)
    resident = gpu.load_mesh(prepare(mesh, o))
    yield gpu, resident, o
    resident.close()
    gpu.close()


KW = dict(seeds=512, max_iterations=200, polish_iterations=30)


def test_check_interval_changes_nothing(job):
    gpu, mesh, o = job
    a = gpu.detect_fast(mesh, None, o, precision="bf16", **KW)
    for interval in (1, 4, 16):
        b = gpu.detect_fast(mesh, None, o, precision="bf16", tuning={"check_interval": interval},
                            **KW)
        for k in KEYS:
            assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), (interval, k)


@pytest.mark.parametrize("precision", ["bf16", "fp32"])
@pytest.mark.parametrize("tuning", [{"vote_bits": 6}, {"vote_bits": 9},
                                    {"simt_blocks_per_sm": 32}, {"simt_blocks_per_sm": 256},
                                    {"tc_ctas_per_sm": 3}])
def test_shapes_keep_the_results(job, precision, tuning):
    gpu, mesh, o = job
    base = gpu.detect_fast(mesh, None, o, precision=precision, **KW)
    r = gpu.detect_fast(mesh, None, o, precision=precision, tuning=tuning, reference_seeds=128,
                        **KW)
    assert r["pairs"] == base["pairs"] and r["votes"] == base["votes"]
    assert r["modes_compared"] >= 10
    assert r["modes_within"] == r["modes_compared"], r["mode_error_max"]


def test_out_of_range_shape_is_rejected(job):
    gpu, mesh, o = job
    with pytest.raises(Exception, match="tuning parameter out of range"):
        gpu.detect_fast(mesh, None, o, tuning={"vote_bits": 11}, **KW)


def test_autotune_picks_a_candidate(job):
    gpu, mesh, o = job
    r = autotune(gpu, mesh, None, o, precision="bf16", repeats=1, **KW)
    for k, v in r["tuning"].items():
        assert v in CANDIDATES[k]
    assert r["ms"] <= r["default_ms"]
