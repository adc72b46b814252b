"""ORACLE - test infrastructure only.  FP64 restatement of the K-seed
mean-shift of the throughput extension (no reference counterpart; parity
unpinned): Epanechnikov weights w = 1 - d^2/h^2 for d^2 < h^2, and the
reference's stopping rules (src/cpu/clustering.cpp:169-181): a seed is
exhausted when its total weight is <= 1e-14 and converged when its squared
movement is below 1e-6 h^2."""
import numpy as np


def meanshift6(votes, seeds, bandwidth, max_iterations=100, block=64):
    x = np.ascontiguousarray(votes, np.float64).reshape(-1, 6)
    means = x[np.asarray(seeds, np.int64)].copy()
    state = np.zeros(len(means), np.uint8)
    h2 = bandwidth * bandwidth
    iterations = 0
    for _ in range(max_iterations):
        act = np.flatnonzero(state == 0)
        if act.size == 0:
            break
        iterations += 1
        for b in range(0, act.size, block):
            ids = act[b:b + block]
            m = means[ids]
            d2 = ((x[None, :, :] - m[:, None, :]) ** 2).sum(-1)
            w = np.where(d2 < h2, 1 - d2 / h2, 0.0)
            tot = w.sum(1)
            exhausted = tot <= 1e-14
            nxt = (w @ x) / np.where(exhausted, 1, tot)[:, None]
            move = ((m - nxt) ** 2).sum(1)
            upd = ~exhausted
            means[ids[upd]] = nxt[upd]
            state[ids[exhausted]] = 2
            state[ids[upd & (move < 1e-6 * h2)]] = 1
    return means, state, iterations


def clustered_votes(clusters=6, per_cluster=3000, noise=30000, sigma=0.01, seed=0):
    """Seeded 6-D votes: Gaussian clusters plus uniform background."""
    rng = np.random.default_rng(seed)
    centers = rng.uniform(-1, 1, (clusters, 6))
    parts = [c + rng.normal(0, sigma, (per_cluster, 6)) for c in centers]
    parts.append(rng.uniform(-1.5, 1.5, (noise, 6)))
    v = np.concatenate(parts)
    return v[rng.permutation(len(v))], centers
