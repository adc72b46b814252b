"""GPU mesh preparation (sym_prepare / sym_mesh_load_raw) against the host
restatement of the reference's prepare() (src/core/prepare.cpp:102-149) and
topology() (prepare.cpp:13-58): every output bit-exact, the same error
messages, and a mesh prepared on the GPU detects exactly like one prepared on
the host."""
import numpy as np
import pytest

from mitra_algo_gb300.mesh import mirrored_heightfield, motif_sphere, prepare
from mitra_algo_gb300.types import Mesh, Options, Rng

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from mitra_algo_gb300 import Gb300Backend
    g = Gb300Backend(0)
    yield g
    g.close()


def with_degenerate_faces(mesh):
    """Appends a zero-area face (a repeated vertex) and a sliver of three
    collinear vertices, both to be rejected."""
    v = mesh.vertices
    n = v.shape[1]
    extra = np.stack([v[:, 0], v[:, 0] + 1e-3 * (v[:, 1] - v[:, 0]),
                      v[:, 0] + 2e-3 * (v[:, 1] - v[:, 0])], axis=1)
    verts = np.concatenate([v, extra], axis=1)
    faces = np.concatenate([mesh.faces, np.array([[0, 0, 1], [n, n + 1, n + 2]], np.int32).T],
                           axis=1)
    return Mesh(verts, faces)


MESHES = {
    "sphere_l4": lambda: motif_sphere(level=4, bumps=8, folds=5, partial_shift=0.3, noise=1e-3,
                                      seed=3),
    "sphere_l5": lambda: motif_sphere(level=5, bumps=12, folds=4, partial_shift=0.4, noise=2e-3,
                                      seed=4),
    "heightfield": lambda: mirrored_heightfield(size=64, bumps=6, seed=2),
    "degenerate": lambda: with_degenerate_faces(mirrored_heightfield(size=32, bumps=3, seed=5)),
}


@pytest.mark.parametrize("name", sorted(MESHES))
def test_gpu_prepare_is_bit_exact(gpu, name):
    mesh = MESHES[name]()
    opts = Options()
    host, dev = prepare(mesh, opts), gpu.prepare(mesh, opts)
    assert dev.context.box_size == host.context.box_size
    assert tuple(dev.context.center) == tuple(host.context.center)
    assert dev.rejected_faces == host.rejected_faces
    np.testing.assert_array_equal(dev.mesh.faces, host.mesh.faces)
    t, u = dev.topology, host.topology
    for a, b in ((t.normals, u.normals), (t.face_normals, u.face_normals),
                 (t.weights, u.weights)):
        assert np.array_equal(a, b, equal_nan=True)
    np.testing.assert_array_equal(t.neighbors.offsets, u.neighbors.offsets)
    np.testing.assert_array_equal(t.neighbors.indices, u.neighbors.indices)
    np.testing.assert_array_equal(t.incident_faces.offsets, u.incident_faces.offsets)
    np.testing.assert_array_equal(t.incident_faces.indices, u.incident_faces.indices)
    np.testing.assert_array_equal(np.asarray(t.edges).reshape(-1, 6),
                                  np.asarray(u.edges).reshape(-1, 6))


def test_degenerate_faces_are_rejected(gpu):
    mesh = MESHES["degenerate"]()
    dev = gpu.prepare(mesh, Options())
    assert dev.rejected_faces == 2


@pytest.mark.parametrize("case,message", [
    ("empty", "Mesh is empty"),
    ("nonfinite", "Non-finite coordinate"),
    ("index", "Face index out of range"),
    ("flat", "Mesh has zero extent"),
    ("nonmanifold", "manifold edges"),
    ("options", "Invalid parameter range"),
])
def test_gpu_prepare_errors(gpu, case, message):
    base = mirrored_heightfield(size=8, bumps=1, seed=1)
    v, f = base.vertices.copy(), base.faces.copy()
    opts = Options()
    if case == "empty":
        mesh = Mesh(v, np.zeros((3, 0), np.int32))
    elif case == "nonfinite":
        v[2, 5] = np.nan
        mesh = Mesh(v, f)
    elif case == "index":
        f[1, 3] = v.shape[1]
        mesh = Mesh(v, f)
    elif case == "flat":
        mesh = Mesh(np.zeros_like(v), f)
    elif case == "nonmanifold":  # a third face on the edge of face 0
        a, b = f[0, 0], f[1, 0]
        mesh = Mesh(np.concatenate([v, [[0.5], [0.5], [1.0]]], axis=1),
                    np.concatenate([f, [[a], [b], [v.shape[1]]]], axis=1))
    else:
        mesh = Mesh(v, f)
        opts = Options(bandwidth=3.0)
    with pytest.raises(Exception, match=message):
        gpu.prepare(mesh, opts)


def test_raw_load_detects_like_host_prepare(gpu):
    mesh = motif_sphere(level=4, bumps=8, folds=5, partial_shift=0.3, noise=1e-3, seed=8)
    opts = Options(sample_ratio=min(1.0, 3000 / mesh.vertex_count), pair_threshold=0.25,
                   bandwidth=0.1, max_pairs=10 ** 7, max_votes=2 * 10 ** 7, max_clusters=8)
    p = prepare(mesh, opts)
    f = gpu.curvature(p.mesh, p.topology, opts)
    sample = gpu.select(p.mesh, f, p.topology.weights, opts, Rng(opts.seed)).sample
    host_loaded, raw_loaded = gpu.load_mesh(p), gpu.load_mesh_raw(mesh, opts)
    kw = dict(precision="bf16", seeds=256, max_iterations=60, polish_iterations=20)
    a = gpu.detect_fast(host_loaded, sample, opts, **kw)
    b = gpu.detect_fast(raw_loaded, sample, opts, **kw)
    for k in ("pairs", "votes", "modes", "clusters", "support", "rotation", "translation",
              "coverage", "rms", "patches"):
        assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), k
    host_loaded.close()
    raw_loaded.close()
