"""Area-weighted sampling on the GPU (sym_sample_vertices, and the sample
inside sym_select and sym_detect_fast_sampled) against the reference's
sample_vertices (src/core/sampling.cpp:5-24): the same ids and the same
std::mt19937_64 state afterwards, bit for bit -- on the golden cases made by
the reference itself, on random weights with zero, negative, NaN and infinite
entries, from every kind of engine position, and on keys packed inside the
band where the device log is not trusted (exact ties included)."""
import math

import numpy as np
import pytest

from conftest import golden_cases
from helpers import same_array
from mitra_algo_gb300.mesh import motif_sphere, prepare
from mitra_algo_gb300.types import Options, Rng
from oracle import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from mitra_algo_gb300 import Gb300Backend
    g = Gb300Backend(0)
    yield g
    g.close()


@pytest.fixture(scope="module")
def ref():
    return oracle.OracleBackend()


def same_as_oracle(gpu, ref, w, ratio, seed=42, advance=0):
    a, b = Rng(seed), oracle.rng(seed)
    for _ in range(advance):
        a.next()
        b.next()
    got = gpu.sample_vertices(w, ratio, a)
    want = ref.sample_vertices(w, ratio, b)
    same_array(got, want, "sample")
    assert a.text() == b.text()
    return got


@pytest.mark.parametrize("case", golden_cases("stage_sampling"), ids=lambda c: c["name"])
def test_golden_sampling(gpu, case):
    d = case["in"]
    rng = Rng(int(d["seed"][0]))
    got = gpu.sample_vertices(d["weights"], float(d["sample_ratio"][0]), rng)
    same_array(got, case["out"]["sample"], "sample")
    assert rng.text() == str(case["out"]["rng_after_select"])


def random_weights(n, seed):
    g = np.random.default_rng(seed)
    w = g.lognormal(0.0, 1.5, n)
    if n > 20:
        w[g.choice(n, n // 8, replace=False)] = 0.0
        w[g.choice(n, n // 20, replace=False)] = -g.uniform(0, 1, n // 20)
        w[1], w[3] = np.nan, np.inf
    return w


@pytest.mark.parametrize("n", [0, 1, 2, 997, 100_000])
@pytest.mark.parametrize("ratio", [1.0, 0.5, 0.013, 0.0])
def test_random_weights(gpu, ref, n, ratio):
    same_as_oracle(gpu, ref, random_weights(n, n + 1), ratio, seed=n + 7)


@pytest.mark.parametrize("advance", [1, 155, 156, 311, 312, 313, 624, 1000])
def test_engine_positions(gpu, ref, advance):
    """The engine enters at every kind of position: inside a block of 312
    words, at its end (the next draw regenerates), and just after one."""
    same_as_oracle(gpu, ref, random_weights(3000, advance), 0.4, seed=advance, advance=advance)


def draw_logs(n, seed):
    r = oracle.rng(seed)
    return np.array([-math.log(((r.next() >> 11) + 0.5) / 9007199254740992.0)
                     for _ in range(n)])


def test_exact_ties(gpu, ref):
    """Weights equal to -log(u) of each vertex's own draw: on the host every
    key is exactly 1.0 and the reference keeps the lowest ids; the device
    keys are 1 within an ulp, so all of them fall in the band and the host
    orders them."""
    n = 5000
    w = draw_logs(n, 42)
    got = same_as_oracle(gpu, ref, w, 0.3)
    assert np.array_equal(got, np.arange(1500))


def test_tight_keys_around_the_boundary(gpu, ref):
    n = 20_000
    w = draw_logs(n, 5) * (1.0 + (np.arange(n) % 1000) * 2.0 ** -44)
    same_as_oracle(gpu, ref, w, 0.25, seed=5)


def test_large(gpu, ref):
    same_as_oracle(gpu, ref, random_weights(2_000_000, 11), 0.37, seed=3)


def test_ratio_must_be_a_number(gpu):
    with pytest.raises(Exception, match="sample ratio"):
        gpu.sample_vertices(np.ones(10), float("nan"), Rng(1))


def test_detect_fast_sampled_equals_the_host_sample():
    """sym_detect_fast_sampled draws the sample detect() would draw
    (std::mt19937_64(options.seed), pipeline.cpp:25) and then runs exactly
    as sym_detect_fast on that sample."""
    from mitra_algo_gb300 import Gb300Backend
    gpu = Gb300Backend(0)
    mesh = motif_sphere(level=4, bumps=8, folds=5, partial_shift=0.3, noise=1e-3, seed=8)
    opts = Options(sample_ratio=min(1.0, 3000 / mesh.vertex_count), pair_threshold=0.25,
                   bandwidth=0.1, max_pairs=10 ** 7, max_votes=2 * 10 ** 7, max_clusters=8,
                   seed=1234)
    p = prepare(mesh, opts)
    sample = oracle.OracleBackend().sample_vertices(p.topology.weights, opts.sample_ratio,
                                                    oracle.rng(opts.seed))
    kw = dict(precision="bf16", seeds=256, max_iterations=60, polish_iterations=20)
    for resident in (gpu.load_mesh(p), gpu.load_mesh_raw(mesh, opts)):
        a = gpu.detect_fast(resident, sample, opts, **kw)
        b = gpu.detect_fast(resident, None, opts, **kw)
        assert b["sampled"] == len(sample) == a["sampled"]
        for k in ("pruned", "pairs", "votes", "modes", "clusters", "support", "rotation",
                  "translation", "coverage", "rms", "patches"):
            assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), k
        resident.close()
    gpu.close()
