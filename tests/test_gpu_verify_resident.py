"""Backend::verification on a resident mesh (sym_verification_resident: FP32
LBVH search, FP64 rechecks, the reference-order BVH for FP64 ties) against
sym_verification (the exact path, identical to the reference's CPU
verification) and against the reference's own outputs.

Integer and FP64 results must be identical: side lists, patch lists and
their order, coverage and rms, bit for bit.  The motions cover the
reference's examples (its own clusters), the throughput path's modes,
perturbed and random rigid motions, and an exact mirror of a grid height
field, which maps vertices onto vertices: images at distance 0 from several
faces at once, the case where the nearest face is decided by the
reference's traversal order."""
import numpy as np
import pytest

from conftest import load_golden
from helpers import clusters_from, mesh_from, options_from, same_array, verification_arrays
from mitra_algo_gb300.mesh import mirrored_heightfield, motif_sphere, prepare
from mitra_algo_gb300.types import ClusterOutput, Csr, Options, Rng

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from mitra_algo_gb300 import Gb300Backend
    g = Gb300Backend(0)
    yield g
    g.close()


def records(rigid=(), planes=()):
    """ClusterOutput of rigid motions [(R (3x3), t)] and planes [(n, offset)]."""
    refl, rot, tr, nrm, off = [], [], [], [], []
    for R, t in rigid:
        refl.append(0), rot.append(np.ravel(R)), tr.append(t), nrm.append(np.zeros(3)), off.append(0.0)
    for n, d in planes:
        n = np.asarray(n, float) / np.linalg.norm(n)
        refl.append(1), rot.append(np.ravel(np.eye(3) - 2 * np.outer(n, n)))
        tr.append(-2 * d * n), nrm.append(n), off.append(float(d))
    k = len(refl)
    return ClusterOutput(np.array(refl, np.uint8), np.array(rot).reshape(k, 9),
                         np.array(tr).reshape(k, 3), np.array(nrm).reshape(k, 3),
                         np.array(off, float), Csr(np.zeros(k + 1, np.uint64), np.zeros(0, np.int32)))


def rotation(axis, angle):
    k = np.asarray(axis, float) / np.linalg.norm(axis)
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + np.sin(angle) * K + (1 - np.cos(angle)) * K @ K


def assert_identical(got, want):
    g, w = verification_arrays(got), verification_arrays(want)
    for k in w:
        same_array(g[k], w[k], k)


def compare(gpu, p, o, clusters):
    resident = gpu.load_mesh(p)
    try:
        got, undecided = gpu.verification_resident(resident, clusters, o)
        again, _ = gpu.verification_resident(resident, clusters, o)
    finally:
        resident.close()
    want = gpu.verification(p.mesh, p.topology, clusters, p.context, o)
    assert_identical(got, want)
    assert_identical(again, want)
    return got, undecided


@pytest.mark.parametrize("name", ["reflection_1", "reflection_05", "rigid_1", "rigid_05",
                                  "partial_1", "partial_05", "single_1", "single_05",
                                  "heightfield"])
def test_reference_examples(gpu, name):
    g = load_golden(f"detect_{name}")
    o = options_from(g, "in_")
    p = prepare(mesh_from(g, "in_"), o)
    got, _ = compare(gpu, p, o, clusters_from(g))
    ref = verification_arrays(got)
    for k in ref:  # the reference's own verification of its clusters
        if k in g and k != "ver_rms":
            same_array(ref[k], g[k], k)
    if "ver_rms" in g:
        assert np.all(np.abs(ref["ver_rms"] - g["ver_rms"]) < 1e-12 * p.context.box_size)


def test_motif_sphere_modes_and_random_motions(gpu):
    mesh = motif_sphere(level=5, bumps=12, folds=5, partial_shift=0.4, noise=1e-3, seed=0)
    o = Options(sample_ratio=5000 / mesh.vertex_count, pair_threshold=0.25, bandwidth=0.1,
                max_pairs=2 * 10 ** 7, max_votes=5 * 10 ** 7, max_clusters=8)
    p = prepare(mesh, o)
    resident = gpu.load_mesh(p)
    r = gpu.detect_fast(resident, None, o, precision="bf16", seeds=256, max_iterations=300,
                        polish_iterations=30, verify=False)
    resident.close()
    g = np.random.default_rng(12)
    rigid = [(np.reshape(R, (3, 3)), np.asarray(t)) for R, t in zip(r["rotation"], r["translation"])]
    for k in (1, 2):  # the planted 5-fold rotation, exact and perturbed
        R = rotation((0, 0, 1), 2 * np.pi * k / 5)
        c = np.asarray(p.context.center)
        rigid.append((R, c - R @ c))
        rigid.append((rotation((0.01, -0.02, 1), 2 * np.pi * k / 5 + 1e-3), c - R @ c + 1e-3))
    for _ in range(6):
        rigid.append((rotation(g.normal(size=3), g.uniform(0, np.pi)), g.normal(size=3) * 0.2))
    compare(gpu, p, o, records(rigid=rigid, planes=[((1, 0, 0), 0.0), ((0.3, 1, 0.1), 0.05)]))


def test_exact_mirror_of_a_grid(gpu):
    mesh = mirrored_heightfield(size=64, bumps=5, seed=2)
    o = Options(verify_threshold=0.02)
    p = prepare(mesh, o)
    planes = [((1, 0, 0), 0.0), ((1, 0, 0), 1e-3), ((1, 1e-3, 0), 0.0), ((0, 1, 0), 0.0)]
    got, undecided = compare(gpu, p, o, records(planes=planes))
    assert got.coverage[0] > 0.9  # the exact mirror is verified nearly everywhere


def test_noisy_torus_with_slivers(gpu):
    """A torus whose vertex noise makes a tenth of its faces slivers (smallest
    angle under 13 degrees, as on the 1e6-triangle benchmark torus) under
    rotations about its axis: nearly every image lies on the surface, and
    many near the edge lines of several faces."""
    from mitra_algo_gb300.mesh import motif_torus
    mesh = motif_torus(R=1.0, r=0.3, nu=160, nv=80, copies=6, mirrored=1, noise=3e-3, seed=7)
    o = Options(verify_threshold=0.01)
    p = prepare(mesh, o)
    c = np.asarray(p.context.center)
    rigid = []
    for k in (1, 2, 3):
        R = rotation((0, 0, 1), 2 * np.pi * k / 6)
        rigid.append((R, c - R @ c))
    R = rotation((0, 0, 1), 0.37)
    rigid.append((R, c - R @ c))
    rigid.append((rotation((0.02, 0.01, 1), 1.1), c - rotation((0.02, 0.01, 1), 1.1) @ c + 2e-3))
    got, undecided = compare(gpu, p, o, records(rigid=rigid, planes=[((1, 0, 0), 0.0)]))
    assert max(got.coverage) > 0.5


def fan_pair_mesh(valences, shift=5.0, gap=4.0):
    """For each valence N, two identical cones: an apex with N triangles to a
    rim whose heights alternate, the second cone `shift` along x from the
    first; cones of different N lie `gap` apart along y."""
    from mitra_algo_gb300.types import Mesh
    verts, faces = [], []
    for row, n in enumerate(valences):
        for copy in range(2):
            base = len(verts)
            o = np.array([shift * copy, gap * row, 0.0])
            verts.append(o + [0.0, 0.0, 0.3])
            for k in range(n):
                a = 2 * np.pi * k / n
                verts.append(o + [np.cos(a), np.sin(a), 0.25 if k % 2 else -0.25])
            for k in range(n):
                faces.append([base, base + 1 + k, base + 1 + (k + 1) % n])
    return Mesh(np.array(verts).T.copy(), np.array(faces, np.int32).T.copy())


def test_high_valence_fans(gpu):
    """Images landing exactly on a vertex of 24, 40 or 80 faces: every face
    at the FP64 minimum is a candidate, more than the 16-entry lists hold,
    so the queries take the 64-entry list (24, 40) or the reference-order
    search (80); the faces' normals alternate, so the ties are decided by
    the reference's visiting order."""
    mesh = fan_pair_mesh((24, 40, 80))
    o = Options(verify_threshold=0.01)
    p = prepare(mesh, o)
    got, undecided = compare(gpu, p, o, records(rigid=[(np.eye(3), (5.0, 0.0, 0.0)),
                                                       (np.eye(3), (5.0, 1e-9, 0.0))]))
    assert got.coverage[0] > 0 and undecided > 0


def test_empty_cluster_list(gpu):
    mesh = motif_sphere(level=3, bumps=4, folds=3, partial_shift=0.3, noise=0.0, seed=1)
    o = Options()
    p = prepare(mesh, o)
    got, undecided = compare(gpu, p, o, records())
    assert undecided == 0 and got.coverage.size == 0
