"""GPU mean-shift of the throughput extension against its FP64 restatement
(oracle/meanshift6.py).  Tolerances: FP64 kernels 1e-9 relative (same
iteration, summation order differs), FP32 1e-5, BF16-refined (BF16 bulk,
FP32 polish with Newton steps) 1e-4 - the <=1e-4 mode-error target."""
import numpy as np
import pytest

from oracle.meanshift6 import clustered_votes, meanshift6

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from mitra_algo_gb300 import Gb300Backend
    b = Gb300Backend(0)
    yield b
    b.close()


@pytest.fixture(scope="module")
def case():
    votes, centers = clustered_votes()
    rng = np.random.default_rng(3)
    seeds = np.sort(rng.choice(len(votes), 300, replace=False))
    ref, state, _ = meanshift6(votes, seeds, 0.06, 200, 200)
    return votes, seeds, ref, state


def rel(a, b):
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("fp32", 1e-5)])
def test_meanshift6_matches_fp64(gpu, case, precision, tol):
    """FP64 and FP32 follow the restatement's trajectories: every seed ends in
    the same state at the same place."""
    votes, seeds, ref, ref_state = case
    means, state, iters = gpu.meanshift6(votes, seeds, 0.06, precision, 200, 200)
    assert np.array_equal(state, ref_state)
    err = rel(means, ref)
    assert np.max(err) <= tol, (precision, np.max(err), iters)


def test_meanshift6_bf16_mode_error(gpu, case):
    """BF16 approach + FP32 polish: every mode that is well defined (Newton-
    converged) in both runs lies within 1e-4 of the FP64 mode."""
    votes, seeds, ref, ref_state = case
    means, state, iters = gpu.meanshift6(votes, seeds, 0.06, "bf16", 200, 200)
    assert np.array_equal(state == 2, ref_state == 2)
    both = (state == 1) & (ref_state == 1)
    assert both.sum() >= 0.9 * (ref_state == 1).sum()
    err = rel(means[both], ref[both])
    assert np.max(err) <= 1e-4, (np.max(err), iters)


@pytest.fixture(scope="module")
def gauss_case():
    votes, centers = clustered_votes()
    rng = np.random.default_rng(4)
    seeds = np.sort(rng.choice(len(votes), 300, replace=False))
    ref, state, _ = meanshift6(votes, seeds, 0.06, 200, 200, kernel="gaussian")
    return votes, seeds, ref, state


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("fp32", 1e-5)])
def test_gaussian_kernel_matches_fp64(gpu, gauss_case, precision, tol):
    """The shifted Gaussian kernel (exp weights, Gaussian Newton steps):
    FP64 and FP32 follow the restatement's trajectories."""
    votes, seeds, ref, ref_state = gauss_case
    means, state, iters = gpu.meanshift6(votes, seeds, 0.06, precision, 200, 200,
                                         kernel="gaussian")
    assert np.array_equal(state, ref_state)
    err = rel(means, ref)
    assert np.max(err) <= tol, (precision, np.max(err), iters)


def test_gaussian_kernel_bf16_mode_error(gpu, gauss_case):
    """BF16 weights from the MUFU's BF16x2 exponential in the tensor kernel,
    FP32 Gaussian polish: every mode converged in both runs within 1e-4."""
    votes, seeds, ref, ref_state = gauss_case
    means, state, iters = gpu.meanshift6(votes, seeds, 0.06, "bf16", 200, 200, kernel="gaussian")
    both = (state == 1) & (ref_state == 1)
    assert both.sum() >= 0.9 * (ref_state == 1).sum()
    err = rel(means[both], ref[both])
    assert np.max(err) <= 1e-4, (np.max(err), iters)


def test_meanshift6_finds_the_clusters(gpu):
    votes, centers = clustered_votes(seed=5)
    seeds = np.arange(0, len(votes), 97)
    means, state, _ = gpu.meanshift6(votes, seeds, 0.06, "fp32", 200)
    near = np.min(np.linalg.norm(means[:, None, :] - centers[None], axis=2), axis=1)
    # seeds that started inside a cluster end at its centre (sigma 0.01 blob)
    start = np.min(np.linalg.norm(votes[seeds][:, None, :] - centers[None], axis=2), axis=1)
    inside = start < 0.03
    assert inside.sum() > 20
    assert np.all(near[inside] < 0.005)


def test_meanshift6_deterministic(gpu, case):
    votes, seeds, _, _ = case
    a = gpu.meanshift6(votes, seeds, 0.06, "fp32", 200)[0]
    b = gpu.meanshift6(votes, seeds, 0.06, "fp32", 200)[0]
    assert np.array_equal(a, b)


def test_meanshift6_rejects_bad_seeds(gpu, case):
    votes = case[0]
    with pytest.raises(ValueError):
        gpu.meanshift6(votes, [len(votes)], 0.06)
    with pytest.raises(ValueError):
        gpu.meanshift6(votes, [0], 0.0)
