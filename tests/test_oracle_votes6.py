"""The FP64 restatement of the 6-D vote descriptors (oracle/votes6.py) on
CPU, pinned to the reference's own votes: on every rigid vote of the golden
fixtures (written by the reference's CPU library) the log map inverts the
reference's rotation (exp(log R) = R) and the translation part is the
reference's descriptor[9..11]; on known rotations, near 0 and pi included,
the log map returns the angle and axis they were made from."""
import numpy as np
import pytest

from conftest import golden_cases, load_golden
from helpers import votes_from
from oracle.votes6 import exp_map, log_map, plane6, rigid6, votes_in_order


def golden_vote_sets():
    sets = [(f"stage_transformations/{c['name']}", c["out"]) for c in
            golden_cases("stage_transformations") if "rot0" in c["out"]]
    for name in ("detect_rigid_05", "detect_rigid_1", "detect_reflection_1", "detect_partial_1",
                 "detect_heightfield"):
        g = load_golden(name)
        if "rot0" in g and g["vote_pair"].size:
            sets.append((name, g))
    return sets


@pytest.mark.parametrize("name,d", golden_vote_sets(), ids=[n for n, _ in golden_vote_sets()])
def test_log_map_inverts_the_reference_rotations(name, d):
    v = votes_from(d)
    rigid, refl = votes_in_order(v)
    assert rigid.size or refl.size
    if rigid.size:
        R = v.rotation[:, rigid].T
        w = log_map(R)
        assert np.all(np.linalg.norm(w, axis=1) <= np.pi + 1e-12)
        # the round trip holds for proper rotations; votes of vertices without
        # principal directions (the zero_directions case) carry R = 0, whose
        # antisymmetric part is zero, so their rotation part is 0
        M = R.reshape(-1, 3, 3)
        proper = np.abs(np.einsum("qji,qjk->qik", M, M) - np.eye(3)).max(axis=(1, 2)) < 1e-9
        assert np.abs(exp_map(w[proper]) - R[proper]).max(initial=0) < 1e-12
        assert not w[~proper].any()
        d6 = rigid6(R, v.descriptor[:, rigid].T)
        assert np.array_equal(d6[:, 3:], v.descriptor[9:12, rigid].T)
        assert np.array_equal(d6[:, :3], w / 2)
    if refl.size:
        p6 = plane6(v.descriptor[:, refl].T)
        assert np.array_equal(p6[:, :4], v.descriptor[:4, refl].T)
        assert not p6[:, 4:].any()


def test_log_map_of_known_rotations():
    g = np.random.default_rng(5)
    axes = g.normal(size=(600, 3))
    axes /= np.linalg.norm(axes, axis=1, keepdims=True)
    angles = np.concatenate([np.pi - 10.0 ** g.uniform(-12, -0.3, 300),
                             10.0 ** g.uniform(-12, 0.4, 300)])
    w = axes * angles[:, None]
    got = log_map(exp_map(w))
    assert np.abs(got - w).max() < 1e-9
    # exactly pi: the axis up to its sign
    at_pi = log_map(exp_map(axes[:20] * np.pi))
    assert np.allclose(np.abs(np.einsum("ij,ij->i", at_pi, axes[:20])), np.pi, atol=1e-12)
