"""ORACLE - test infrastructure only.

FP64 restatement of the throughput path's vote descriptors (no reference
counterpart; the reference votes with 12-D rigid and 4-D plane descriptors,
src/cpu/transformations.cpp:17-73).  The throughput path describes the same
votes in 6-D:

* rigid vote (rotation R, translation t of the reference's vote): the
  axis-angle vector of R halved, then the reference's own centred
  translation (R c + t - c) / box, i.e. its descriptor[9..11];
* plane vote: the reference's 4-D plane descriptor [n, (d + n.c) / box],
  zero-padded to 6-D.

So the 6-D descriptor of a rigid vote is a function of the reference's vote
record, and tests compare the GPU's FP32 records with this restatement
applied to the reference's (or the oracle's bit-exact) FP64 votes.
"""
from __future__ import annotations

import numpy as np


def log_map(rotation) -> np.ndarray:
    """Axis-angle vectors w (q, 3) of rotations given row-major (q, 9):
    |w| = theta in [0, pi], R = exp([w]x).  theta = atan2(|s| / 2, c) with
    c = (tr R - 1) / 2 and s = (R21 - R12, R02 - R20, R10 - R01) =
    2 sin(theta) n; the axis is s / |s|, and within 0.9 of c = -1 (near pi,
    where s vanishes) the normalised column of the symmetric part
    (R + R^T) / 2 - c I = (1 - c) n n^T with the largest diagonal entry,
    signed like s."""
    R = np.asarray(rotation, np.float64).reshape(-1, 3, 3)
    c = (R[:, 0, 0] + R[:, 1, 1] + R[:, 2, 2] - 1.0) / 2.0
    s = np.stack([R[:, 2, 1] - R[:, 1, 2], R[:, 0, 2] - R[:, 2, 0], R[:, 1, 0] - R[:, 0, 1]], 1)
    sn = np.linalg.norm(s, axis=1)
    theta = np.arctan2(sn / 2.0, c)
    with np.errstate(divide="ignore", invalid="ignore"):
        w = np.where(sn[:, None] > 0, s * (theta / np.where(sn > 0, sn, 1.0))[:, None], 0.0)
    near = c < -0.9
    if near.any():
        Rn = R[near]
        sym = (Rn + np.transpose(Rn, (0, 2, 1))) / 2.0
        cn = c[near]
        k = np.argmax(np.stack([sym[:, 0, 0], sym[:, 1, 1], sym[:, 2, 2]], 1), axis=1)
        rows = np.arange(len(Rn))
        col = sym[rows, :, k] - np.eye(3)[k] * cn[:, None]  # (1 - c) n_k n
        n = col / np.linalg.norm(col, axis=1, keepdims=True)
        flip = np.einsum("ij,ij->i", n, s[near]) < 0
        n[flip] *= -1.0
        w[near] = n * theta[near][:, None]
    return w


def exp_map(w) -> np.ndarray:
    """Rotations (q, 9) row-major of axis-angle vectors w (q, 3) (Rodrigues)."""
    w = np.asarray(w, np.float64).reshape(-1, 3)
    th = np.linalg.norm(w, axis=1)
    with np.errstate(divide="ignore", invalid="ignore"):
        a = np.where(th > 1e-8, np.sin(th) / np.where(th > 0, th, 1.0), 1.0 - th * th / 6.0)
        b = np.where(th > 1e-8, (1.0 - np.cos(th)) / np.where(th > 0, th * th, 1.0),
                     0.5 - th * th / 24.0)
    K = np.zeros((len(w), 3, 3))
    K[:, 0, 1], K[:, 0, 2], K[:, 1, 2] = -w[:, 2], w[:, 1], -w[:, 0]
    K[:, 1, 0], K[:, 2, 0], K[:, 2, 1] = w[:, 2], -w[:, 1], w[:, 0]
    R = np.eye(3)[None] + a[:, None, None] * K + b[:, None, None] * (K @ K)
    return R.reshape(-1, 9)


def rigid6(rotation, descriptor) -> np.ndarray:
    """6-D descriptors (q, 6) of rigid votes from the reference's records:
    rotation (q, 9) row-major and the 12-D descriptor (q, 12), whose last
    three entries are the centred translation (transformations.cpp:56-69)."""
    d = np.asarray(descriptor, np.float64).reshape(-1, 12)
    return np.concatenate([log_map(rotation) / 2.0, d[:, 9:12]], axis=1)


def plane6(descriptor) -> np.ndarray:
    """6-D descriptors (q, 6) of plane votes: the reference's 4-D plane
    descriptor (transformations.cpp:41-48) and two zeros."""
    d = np.asarray(descriptor, np.float64).reshape(-1, 12)
    return np.concatenate([d[:, :4], np.zeros((len(d), 2))], axis=1)


def votes_in_order(votes):
    """The reference's votes split by kind, keeping their order:
    (rigid indices, reflection indices)."""
    kind = np.asarray(votes.kind)
    return np.flatnonzero(kind == 0), np.flatnonzero(kind == 1)
