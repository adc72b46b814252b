"""The seeded batch generators (mesh.uneven_batch: 2k-60k-vertex meshes; mesh.stress_batch: 1e5-1e6 triangles):
deterministic, with vertex and triangle counts inside their stated ranges,
valid faces and the stated mode mix."""
import numpy as np

from mitra_algo_gb300.mesh import add_noise, add_random_bumps, motif_torus, stress_batch, uneven_batch


def test_uneven_batch_is_seeded_and_in_range():
    a = uneven_batch(6, seed=3)
    b = uneven_batch(6, seed=3)
    assert [m for _, m, _ in a] == ["rigid", "rigid", "reflection"] * 2
    for (ma, mode, planted), (mb, _, _) in zip(a, b):
        assert np.array_equal(ma.vertices, mb.vertices) and np.array_equal(ma.faces, mb.faces)
        assert 1 <= planted <= 4
        assert 900 <= ma.vertex_count <= 70000, ma.vertex_count
        assert ma.faces.min() >= 0 and ma.faces.max() < ma.vertex_count
        assert np.isfinite(ma.vertices).all()


def test_stress_batch_sizes_and_modes():
    batch = stress_batch(2, seed=1)
    assert [m for _, m in batch] == ["rigid", "reflection"]
    for mesh, _ in batch:
        assert 0.9e5 <= mesh.faces.shape[1] <= 1.1e6, mesh.faces.shape
        assert mesh.faces.max() < mesh.vertex_count


def test_relief_and_noise_move_vertices_only():
    mesh = motif_torus(nu=40, nv=20, copies=3, mirrored=0, seed=5)
    bumped = add_random_bumps(mesh, 0.3, seed=2)
    assert np.array_equal(bumped.faces, mesh.faces)
    moved = np.linalg.norm(bumped.vertices - mesh.vertices, axis=0) > 1e-6 * 1.3
    assert 0.2 <= moved.mean() <= 1.0
    assert add_noise(mesh, 0.0, 1) is mesh
    noisy = add_noise(mesh, 1e-3, 1)
    assert np.array_equal(noisy.faces, mesh.faces) and not np.array_equal(noisy.vertices, mesh.vertices)
