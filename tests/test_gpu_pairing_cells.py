"""Pairing of a large sample (at least 65,536 selected vertices), where the
kmin-sorted samples are cut into cells re-sorted by kmax and each source
tests only the candidates inside both curvature windows.  The pairs of a
random subset of sources are checked against the reference's acceptance
test (src/cpu/pairing.cpp:22-28) evaluated in FP64 over every later
ordinal with numpy: the same partners, in ordinal order, and the whole
pair list is sorted by (source ordinal, partner ordinal)."""
import numpy as np
import pytest

from helpers import features_from
from mitra_algo_gb300.types import Mesh, ModelContext, Options

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from mitra_algo_gb300 import Gb300Backend
    b = Gb300Backend(0)
    yield b
    b.close()


def accepted_partners(a, sel, pos, k0, k1, t, min_dist):
    """Ordinals b > a the reference accepts for source ordinal a (its FP64
    expressions: tolerance t * max(|k|, 1e-10), then the distance test)."""
    va, vb = sel[a], sel[a + 1:]
    m = np.maximum.reduce([np.full(vb.size, abs(k0[va])), np.full(vb.size, abs(k1[va])),
                           np.abs(k0[vb]), np.abs(k1[vb]), np.full(vb.size, 1e-10)])
    tol = t * m
    ok = (np.abs(k0[va] - k0[vb]) <= tol) & (np.abs(k1[va] - k1[vb]) <= tol)
    d = pos[:, vb] - pos[:, [va]]
    dist = np.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
    ok &= ~(dist < min_dist)
    return a + 1 + np.nonzero(ok)[0]


@pytest.mark.parametrize("t", [0.02, 0.04])
def test_large_sample_pairs(gpu, t):
    rng = np.random.default_rng(11)
    n = 80_000
    pos = rng.uniform(-1, 1, (3, n))
    k0 = rng.normal(0, 1, n)
    k0[: n // 8] = np.round(k0[: n // 8], 2)  # many equal kmin keys
    k1 = k0 + rng.uniform(0, 0.5, n)
    f = features_from({"kmin": k0, "kmax": k1}, n)
    mesh = Mesh(pos, np.zeros((3, 0), np.int32))
    sel = rng.permutation(n)[:70_000].astype(np.int32)
    o = Options(pair_threshold=t, max_pairs=10 ** 9)
    got = gpu.pairing(mesh, f, sel, ModelContext(1.0), o)
    ordinal = np.empty(n, np.int64)
    ordinal[sel] = np.arange(sel.size)
    ga, gb = ordinal[got.a], ordinal[got.b]
    assert np.all((ga[1:] > ga[:-1]) | ((ga[1:] == ga[:-1]) & (gb[1:] > gb[:-1])))
    starts = np.searchsorted(ga, np.arange(sel.size + 1))
    for a in rng.choice(sel.size, 200, replace=False):
        want = accepted_partners(int(a), sel, pos, k0, k1, t, 0.03)
        have = gb[starts[a]:starts[a + 1]]
        assert np.array_equal(have, want), (int(a), have.size, want.size)
