"""The FP64 mean-shift restatement of the throughput extension on CPU:
clusters are found and the stopping rules behave."""
import numpy as np

from oracle.meanshift6 import clustered_votes, meanshift6


def test_restatement_finds_cluster_centres():
    votes, centers = clustered_votes(clusters=3, per_cluster=500, noise=2000, seed=1)
    start = np.min(np.linalg.norm(votes[:, None, :] - centers[None], axis=2), axis=1)
    seeds = np.flatnonzero(start < 0.02)[:20]
    means, state, _ = meanshift6(votes, seeds, 0.06, 200)
    assert np.all(state == 1)
    near = np.min(np.linalg.norm(means[:, None, :] - centers[None], axis=2), axis=1)
    assert np.all(near < 0.005)


def test_isolated_seed_converges_in_place():
    votes = np.array([[0.0] * 6, [1.0] * 6])
    means, state, it = meanshift6(votes, [0], 0.1, 10)
    assert state[0] == 1 and it == 1 and np.allclose(means[0], 0)
