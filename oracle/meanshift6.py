"""ORACLE - test infrastructure only.  FP64 restatement of the K-seed
mean-shift of the throughput extension (no reference counterpart; parity
unpinned).

Epanechnikov weights w = 1 - d^2/h^2 for d^2 < h^2 (kernel "epanechnikov"),
or the shifted Gaussian w = 2^(-8 d^2/h^2) - 2^-8 for d^2 < h^2 (kernel
"gaussian": zero at the cut).  A seed takes plain mean-shift steps m(x) - x until its squared
step is below 4e-4 h^2 (a step under h/50), then safeguarded Newton steps on m(x) = x:
    (I - J) s = m(x) - x,   J = 2 / (h^2 sum w) * (sum d d^T - (m - x) (sum d)^T)
with d = v - x over the votes within the bandwidth (Epanechnikov), or
    J = 2 k ln2 / (h^2 sum w) * (sum g d d^T - (m - x) (sum g d)^T)
with g = w + 2^-k = 2^(-k d^2/h^2), k = 8 (Gaussian: dw/dx = 2 k ln2 g d / h^2).  A Newton step is taken
when the 6x6 system is regular (pivots above 1e-12), |s| <= h/4 and
s.(m - x) > 0 (or the step already meets the convergence test); otherwise the
plain step is taken and Newton is tried once more at the next iteration; at
the second rejection the density is flat along some direction (a ridge, no
well-defined mode position) and the seed stops (settled).  A seed of the
polish not converged after 10 polish iterations settles too.  Stopping rules: exhausted when the total weight is <= 1e-14
(the reference's rule, src/cpu/clustering.cpp:169-181), converged when a
Newton step's square is below 1e-8 h^2.  States: 0 approaching,
1 converged, 2 exhausted, 3 near a mode, 4 settled.
"""
import numpy as np

MOVING, CONVERGED, EXHAUSTED, NEAR, SETTLED = 0, 1, 2, 3, 4
NEAR1 = 5  # near after one rejected Newton step (reported as NEAR)
SWITCH2, NEWTON_STOP2, TRUST, NEWTON_CAP = 4e-4, 1e-8, 0.25, 10
GAUSS_K = 8.0  # base-2 exponent scale of the Gaussian kernel


def weights(d2, h2, kernel):
    inside = d2 < h2
    if kernel == "gaussian":
        return np.where(inside, np.exp2(-GAUSS_K * (d2 / h2)) - 2.0 ** -GAUSS_K, 0.0)
    return np.where(inside, 1 - d2 / h2, 0.0)


def solve6(M, b, tiny=1e-12):
    """b <- M^-1 b by Gaussian elimination with partial pivoting (the order
    of the device solver); None when a pivot is below `tiny`."""
    M = np.array(M, np.float64)
    b = np.array(b, np.float64)
    for c in range(6):
        piv = c + int(np.argmax(np.abs(M[c:, c])))
        if not abs(M[piv, c]) > tiny:
            return None
        if piv != c:
            M[[c, piv]] = M[[piv, c]]
            b[[c, piv]] = b[[piv, c]]
        for r in range(c + 1, 6):
            f = M[r, c] / M[c, c]
            M[r, c:] -= f * M[c, c:]
            b[r] -= f * b[c]
    for c in range(5, -1, -1):
        b[c] = (b[c] - M[c, c + 1:] @ b[c + 1:]) / M[c, c]
    return b


def newton_seed(x, m, w, tot, delta, move, h2, polish_it, kernel="epanechnikov", state=NEAR):
    """The kNear step of one seed (in `state`: NEAR or NEAR1) from its
    weights w over all votes x (polish_it: the polish iteration, -1 in the
    approach phase)."""
    inside = w > 0
    di = x[inside] - m
    if kernel == "gaussian":
        gi = (w[inside] + 2.0 ** -GAUSS_K)[:, None]
        sd = (gi * di).sum(0)
        g = 2.0 * GAUSS_K * np.log(2.0) / (h2 * tot)
        M = np.eye(6) - g * ((gi * di).T @ di - np.outer(delta, sd))
    else:
        sd = di.sum(0)
        g = 2.0 / (h2 * tot)
        M = np.eye(6) - g * (di.T @ di - np.outer(delta, sd))
    s = solve6(M, delta)
    if (s is not None and np.all(np.isfinite(s)) and s @ s <= TRUST * TRUST * h2
            and (s @ delta > 0 or s @ s < NEWTON_STOP2 * h2)):
        if s @ s < NEWTON_STOP2 * h2:
            return m + s, CONVERGED
        return m + s, SETTLED if polish_it >= NEWTON_CAP else state
    return m + delta, NEAR1 if polish_it < NEWTON_CAP and state == NEAR else SETTLED


def meanshift6(votes, seeds, bandwidth, max_iterations=100, polish_iterations=100, block=64,
               kernel="epanechnikov"):
    """Approach phase (at most max_iterations; kMoving seeds only, a seed
    leaves once it is near a mode), then the polish phase (at most
    polish_iterations; kMoving and kNear seeds).  Returns the means, the
    states and the (approach, polish) iteration counts."""
    x = np.ascontiguousarray(votes, np.float64).reshape(-1, 6)
    means = x[np.asarray(seeds, np.int64)].copy()
    state = np.zeros(len(means), np.uint8)
    h2 = bandwidth * bandwidth
    counts = []
    for phase, budget in ((False, max_iterations), (True, polish_iterations)):
        counts.append(_phase(x, means, state, h2, budget, phase, block, kernel))
    state[state == NEAR1] = NEAR
    return means, state, tuple(counts)


def _phase(x, means, state, h2, budget, polish, block, kernel):
    iterations = 0
    for it in range(budget):
        near = (state == NEAR) | (state == NEAR1)
        act = np.flatnonzero((state == MOVING) | (near & polish))
        if act.size == 0:
            break
        iterations += 1
        for b in range(0, act.size, block):
            ids = act[b:b + block]
            m = means[ids]
            d2 = ((x[None, :, :] - m[:, None, :]) ** 2).sum(-1)
            w = weights(d2, h2, kernel)
            tot = w.sum(1)
            safe = np.where(tot <= 1e-14, 1.0, tot)
            delta = (w @ x) / safe[:, None] - m
            move = (delta * delta).sum(1)
            for j, i in enumerate(ids):
                if tot[j] <= 1e-14:
                    state[i] = EXHAUSTED
                elif state[i] == MOVING:
                    means[i] = m[j] + delta[j]
                    if move[j] < SWITCH2 * h2:
                        state[i] = NEAR
                else:
                    means[i], state[i] = newton_seed(x, m[j], w[j], tot[j], delta[j], move[j], h2,
                                                     it if polish else -1, kernel, state[i])
    return iterations


def clustered_votes(clusters=6, per_cluster=3000, noise=30000, sigma=0.01, seed=0):
    """Seeded 6-D votes: Gaussian clusters plus uniform background."""
    rng = np.random.default_rng(seed)
    centers = rng.uniform(-1, 1, (clusters, 6))
    parts = [c + rng.normal(0, sigma, (per_cluster, 6)) for c in centers]
    parts.append(rng.uniform(-1.5, 1.5, (noise, 6)))
    v = np.concatenate(parts)
    return v[rng.permutation(len(v))], centers
