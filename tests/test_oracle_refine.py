"""The FP64 restatement of the transform refinement (oracle/refine.py) on
CPU: its closest points are the nearest points of the triangles (checked
against dense barycentric sampling, degenerate triangles included), and the
exact motion of a shape and its rigid or mirrored copy is a fixed point of a
refinement pass."""
import numpy as np
import pytest

from mitra_algo_gb300.mesh import prepare
from mitra_algo_gb300.types import Options
from oracle.refine import closest_on_triangles, refine_pass


def test_closest_points_are_nearest():
    g = np.random.default_rng(3)
    m = 400
    a, b, c = (g.normal(size=(m, 3)) for _ in range(3))
    c[::7] = a[::7] + 0.5 * (b[::7] - a[::7])  # collinear corners
    b[::11] = a[::11]                          # two equal corners
    p = g.normal(size=(m, 3)) * 2
    q = closest_on_triangles(p, a, b, c)
    u, v = np.meshgrid(np.linspace(0, 1, 101), np.linspace(0, 1, 101))
    keep = u + v <= 1
    u, v = u[keep], v[keep]
    for i in range(m):
        pts = a[i] + np.outer(u, b[i] - a[i]) + np.outer(v, c[i] - a[i])
        best = np.min(((pts - p[i]) ** 2).sum(1))
        got = ((q[i] - p[i]) ** 2).sum()
        assert got <= best + 1e-9, i
        # the point lies on the triangle: its distance is attained by a sample nearby
        assert np.min(((pts - q[i]) ** 2).sum(1)) < 1e-3


@pytest.mark.parametrize("kind", ["rigid", "reflection"])
def test_exact_motion_is_a_fixed_point(kind):
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parent))
    from test_gpu_refine import two_copies
    mesh, truth = two_copies(kind)
    o = Options()
    p = prepare(mesh, o)
    tau = o.verify_threshold * p.context.box_size
    got = refine_pass(p.mesh.vertices, p.topology.normals, p.topology.weights, p.mesh.faces,
                      truth, tau)
    assert np.abs(np.asarray(got["rotation"]) - truth["rotation"]).max() < 1e-9
    assert np.abs(np.asarray(got["translation"]) - truth["translation"]).max() < 1e-9
