"""ORACLE - test infrastructure only.  FP64 restatement of one pass of the
transform refinement of sym_refine_transforms / sym_fast_options.refine (no
reference counterpart, so parity is unpinned: this is an independent FP64
statement of the same method, used to check the device's).

One pass: every vertex that supports the motion forward -- the verification
tests of src/cpu/verification.cpp:22-110 (its image at least 2 tau away, on
the far side of a reflection plane, within tau of the surface, transformed
normal within 60 degrees of the nearest face's) -- is paired with the closest
point of its nearest face (brute force over all faces here; the region tests
of Ericson, Real-Time Collision Detection, 2005, section 5.1.5), then the
motion is fitted to the pairs by weighted least squares (vertex weights):
Kabsch for a rigid motion, and for a reflection the plane through the
weighted mean of the midpoints with its normal along the top eigenvector of
the displacements' second moment.
"""
from __future__ import annotations

import numpy as np


def closest_on_segments(p, a, b):
    """Closest points of segments ab to points p (the clamp of the
    reference's segment distance, src/core/math.cpp: the parameter is used
    only when the segment's squared length exceeds 1e-14, the reference's
    eps; otherwise the closest point is a)."""
    d = b - a
    ln = np.einsum("ij,ij->i", d, d)
    with np.errstate(divide="ignore", invalid="ignore"):
        t = np.where(ln > 1e-14, np.einsum("ij,ij->i", p - a, d) / np.where(ln > 1e-14, ln, 1.0), 0.0)
    return a + d * np.clip(t, 0.0, 1.0)[:, None]


def closest_on_triangles(p, a, b, c):
    """Closest points of triangles (a, b, c) to points p, all (m, 3): the
    region tests, and for a triangle without area (|ab x ac|^2 < 1e-28) the
    nearest of its three segments."""
    ab, ac, ap = b - a, c - a, p - a
    bp, cp = p - b, p - c
    dot = lambda x, y: np.einsum("ij,ij->i", x, y)  # noqa: E731
    d1, d2, d3, d4, d5, d6 = dot(ab, ap), dot(ac, ap), dot(ab, bp), dot(ac, bp), dot(ab, cp), dot(ac, cp)
    vc, vb, va = d1 * d4 - d3 * d2, d5 * d2 - d1 * d6, d3 * d6 - d5 * d4
    with np.errstate(divide="ignore", invalid="ignore"):
        den = va + vb + vc
        out = a + ab * (vb / den)[:, None] + ac * (vc / den)[:, None]
        e_bc = b + (c - b) * ((d4 - d3) / ((d4 - d3) + (d5 - d6)))[:, None]
        e_ac = a + ac * (d2 / (d2 - d6))[:, None]
        e_ab = a + ab * (d1 / (d1 - d3))[:, None]
    # region tests in the order they are made; the first that holds wins
    choices = [
        ((d1 <= 0) & (d2 <= 0), a),
        ((d3 >= 0) & (d4 <= d3), b),
        ((vc <= 0) & (d1 >= 0) & (d3 <= 0), e_ab),
        ((d6 >= 0) & (d5 <= d6), c),
        ((vb <= 0) & (d2 >= 0) & (d6 <= 0), e_ac),
        ((va <= 0) & ((d4 - d3) >= 0) & ((d5 - d6) >= 0), e_bc),
    ]
    taken = np.zeros(len(p), bool)
    for cond, val in choices:
        use = cond & ~taken
        out = np.where(use[:, None], val, out)
        taken |= use
    n = np.cross(ab, ac)
    flat = dot(n, n) < 1e-14 * 1e-14
    if flat.any():
        s = [closest_on_segments(p, a, b), closest_on_segments(p, a, c),
             closest_on_segments(p, b, c)]
        e = [((p - x) ** 2).sum(1) for x in s]
        m01 = np.where(e[1] < e[0], 1, 0)
        pick = np.where(e[2] < np.where(m01 == 1, e[1], e[0]), 2, m01)
        seg = np.stack(s)[pick, np.arange(len(p))]
        out = np.where(flat[:, None], seg, out)
    return out


def refine_pass(xyz, vn, w, faces, motion: dict, tau: float) -> dict:
    """One refinement pass of `motion` = {reflection, rotation (9),
    translation (3), plane_normal (3), plane_offset} on a mesh given as
    xyz (3, n), vn (3, n), w (n,), faces (3, f)."""
    R = np.asarray(motion["rotation"], float).reshape(3, 3)
    t = np.asarray(motion["translation"], float)
    refl = bool(motion["reflection"])
    p = xyz.T
    q = p @ R.T + t
    keep = ((q - p) ** 2).sum(1) >= 4 * tau * tau
    if refl:
        keep &= p @ np.asarray(motion["plane_normal"], float) + motion["plane_offset"] < -tau
    A, B, C = (xyz[:, faces[k]].T for k in range(3))
    fn = np.cross(B - A, C - A)
    fl = np.linalg.norm(fn, axis=1)
    idx = np.flatnonzero(keep)
    src, dst = [], []
    for lo in range(0, len(idx), 64):
        ids = idx[lo:lo + 64]
        m, f = len(ids), len(A)
        qq = np.repeat(q[ids], f, axis=0)
        cp = closest_on_triangles(qq, np.tile(A, (m, 1)), np.tile(B, (m, 1)), np.tile(C, (m, 1)))
        d2 = ((cp - qq) ** 2).sum(1).reshape(m, f)
        best = d2.argmin(1)
        for j, i in enumerate(ids):
            k = best[j]
            if not d2[j, k] < tau * tau or not fl[k] > 0:
                continue
            rn = R @ vn[:, i]
            if rn @ fn[k] / fl[k] < 0.5:
                continue
            src.append(i)
            dst.append(cp[j * f + k])
    if len(src) < 3:
        return dict(motion)
    src = np.array(src)
    P, Q, W = p[src], np.array(dst), w[src]
    sw = W.sum()
    pb, qb = (W[:, None] * P).sum(0) / sw, (W[:, None] * Q).sum(0) / sw
    out = dict(motion)
    if not refl:
        H = ((P - pb) * W[:, None]).T @ (Q - qb) / sw
        U, S, Vt = np.linalg.svd(H)
        V = Vt.T
        d = np.sign(np.linalg.det(V @ U.T)) or 1.0
        Rn = V @ np.diag([1.0, 1.0, d]) @ U.T
        out["rotation"] = Rn.reshape(-1)
        out["translation"] = qb - Rn @ pb
    else:
        D = Q - P
        Cm = (D * W[:, None]).T @ D / sw
        _, vecs = np.linalg.eigh(Cm)
        n = vecs[:, -1]
        if n @ np.asarray(motion["plane_normal"], float) < 0:
            n = -n
        off = -n @ (0.5 * (pb + qb))
        out["plane_normal"] = n
        out["plane_offset"] = off
        out["rotation"] = (np.eye(3) - 2 * np.outer(n, n)).reshape(-1)
        out["translation"] = -2 * off * n
    return out
