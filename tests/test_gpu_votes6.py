"""The throughput path's FP32 vote records (sym_fast_votes: the kernels
sym_detect_fast runs) against the FP64 restatement of oracle/votes6.py
applied to the reference's own votes for the same pairs (the oracle's
transformations, bit-exact with the reference's CPU library).

Tolerance: 1e-5 relative per record, |d32 - d64| / |d64| over the 6
descriptor entries -- the "pair transforms within 1e-5 relative" contract of
the FP32 vote path.  Random pairs of a curved mesh put about a tenth of the
rotations within the FP64 band near pi (c = (tr R - 1)/2 <= -0.99), and the
test requires such votes to be present."""
import numpy as np
import pytest

from mitra_algo_gb300.mesh import motif_sphere, prepare
from mitra_algo_gb300.types import Options, Pairs
from oracle.votes6 import plane6, rigid6, votes_in_order

pytestmark = pytest.mark.gpu

REL = 1e-5


@pytest.fixture(scope="module")
def gpu():
    from mitra_algo_gb300 import Gb300Backend
    g = Gb300Backend(0)
    yield g
    g.close()


@pytest.fixture(scope="module")
def case(oracle_backend):
    mesh = motif_sphere(level=4, bumps=10, folds=5, partial_shift=0.35, noise=1e-3, seed=3)
    o = Options(max_votes=10 ** 7, max_pairs=10 ** 7)
    p = prepare(mesh, o)
    f = oracle_backend.curvature(p.mesh, p.topology, o)
    valid = np.flatnonzero(f.valid)
    g = np.random.default_rng(8)
    a = g.choice(valid, 40000)
    b = g.choice(valid, 40000)
    keep = a != b
    pairs = Pairs(a[keep], b[keep])
    votes = oracle_backend.transformations(p.mesh, f, pairs, p.context, o)
    return p, f, pairs, votes


def relative(got, want):
    return np.linalg.norm(got - want, axis=1) / np.linalg.norm(want, axis=1)


def test_rigid_records_match_fp64(gpu, case):
    p, f, pairs, votes = case
    rec, pair_of = gpu.fast_votes(p.mesh, f, pairs, p.context, "rigid")
    rigid, _ = votes_in_order(votes)
    assert len(rec) == 2 * len(pairs) == rigid.size
    assert np.array_equal(pair_of, votes.pair[rigid])
    R = votes.rotation[:, rigid].T
    want = rigid6(R, votes.descriptor[:, rigid].T)
    err = relative(rec[:, :6].astype(np.float64), want)
    c = (R[:, 0] + R[:, 4] + R[:, 8] - 1) / 2
    near_pi = c <= -0.99
    assert near_pi.sum() >= 200, near_pi.sum()
    assert err.max() <= REL, (err.max(), int(err.argmax()), bool(near_pi[err.argmax()]))
    assert err[near_pi].max() <= REL
    n2 = (rec[:, :6].astype(np.float64) ** 2).sum(1)
    assert np.abs(rec[:, 6] - n2).max() <= 1e-5 * n2.max()
    assert not rec[:, 7].any()


def test_plane_records_match_fp64(gpu, case):
    p, f, pairs, votes = case
    rec, pair_of = gpu.fast_votes(p.mesh, f, pairs, p.context, "reflection")
    _, refl = votes_in_order(votes)
    # the same pairs vote for a plane (the reference's FP64 test)
    assert np.array_equal(pair_of, votes.pair[refl])
    want = plane6(votes.descriptor[:, refl].T)
    err = relative(rec[:, :6].astype(np.float64), want)
    assert err.max() <= REL, err.max()


def test_empty_and_invalid_pairs(gpu, case):
    p, f, pairs, _ = case
    rec, pair_of = gpu.fast_votes(p.mesh, f, Pairs(np.zeros(0, np.int32), np.zeros(0, np.int32)),
                                  p.context)
    assert rec.shape == (0, 8) and pair_of.size == 0
    with pytest.raises(ValueError):
        gpu.fast_votes(p.mesh, f, Pairs(np.array([0]), np.array([p.mesh.vertex_count])), p.context)
