"""The FP64 mean-shift restatement of the throughput extension on CPU:
clusters are found, the Newton phase lands on fixed points of the
mean-shift map, and the stopping rules behave."""
import numpy as np

from oracle.meanshift6 import CONVERGED, clustered_votes, meanshift6, solve6


def shift_target(votes, m, h):
    d2 = ((votes - m) ** 2).sum(1)
    w = np.where(d2 < h * h, 1 - d2 / (h * h), 0.0)
    return (w @ votes) / w.sum()


def test_restatement_finds_cluster_centres():
    votes, centers = clustered_votes(clusters=3, per_cluster=500, noise=2000, seed=1)
    start = np.min(np.linalg.norm(votes[:, None, :] - centers[None], axis=2), axis=1)
    seeds = np.flatnonzero(start < 0.02)[:20]
    means, state, it = meanshift6(votes, seeds, 0.06, 200, 200)
    assert np.all(state == CONVERGED)
    near = np.min(np.linalg.norm(means[:, None, :] - centers[None], axis=2), axis=1)
    assert np.all(near < 0.005)
    # converged means are fixed points of the mean-shift map to ~1e-4 h
    for m in means:
        assert np.linalg.norm(shift_target(votes, m, 0.06) - m) < 1e-4 * 0.06
    assert sum(it) < 60


def test_isolated_seed_converges_in_place():
    votes = np.array([[0.0] * 6, [1.0] * 6])
    means, state, it = meanshift6(votes, [0], 0.1, 10, 10)
    assert state[0] == CONVERGED and it == (1, 1) and np.allclose(means[0], 0)


def test_solve6_matches_numpy():
    rng = np.random.default_rng(2)
    M = np.eye(6) + 0.3 * rng.normal(size=(6, 6))
    b = rng.normal(size=6)
    assert np.allclose(solve6(M, b), np.linalg.solve(M, b), rtol=1e-12, atol=1e-12)
    assert solve6(np.zeros((6, 6)), b) is None


def gauss_target(votes, m, h):
    d2 = ((votes - m) ** 2).sum(1)
    w = np.where(d2 < h * h, np.exp2(-8.0 * d2 / (h * h)) - 2.0 ** -8, 0.0)
    return (w @ votes) / w.sum()


def test_gaussian_restatement_converges_to_fixed_points():
    """Shifted Gaussian kernel: seeds near the cluster centres converge
    with the Gaussian Newton steps to fixed points of the Gaussian map."""
    votes, centers = clustered_votes(clusters=3, per_cluster=500, noise=2000, seed=1)
    start = np.min(np.linalg.norm(votes[:, None, :] - centers[None], axis=2), axis=1)
    seeds = np.flatnonzero(start < 0.02)[:20]
    means, state, it = meanshift6(votes, seeds, 0.06, 200, 200, kernel="gaussian")
    assert np.all(state == CONVERGED)
    near = np.min(np.linalg.norm(means[:, None, :] - centers[None], axis=2), axis=1)
    assert np.all(near < 0.005)
    for m in means:
        assert np.linalg.norm(gauss_target(votes, m, 0.06) - m) < 1e-4 * 0.06
