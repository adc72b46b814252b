"""FP64 refinement of detected motions (sym_refine_transforms and
sym_fast_options.refine; no reference counterpart): one pass on the device
equals the FP64 restatement in oracle/refine.py; repeated passes move a
perturbed motion toward the true one on meshes made of a shape and an exact
rigid or mirrored copy of it; refinement inside sym_detect_fast keeps the
pipeline's other results and moves the modes toward the exact motion."""
import numpy as np
import pytest

from mitra_algo_gb300.mesh import icosphere, mirrored_heightfield, prepare
from mitra_algo_gb300.types import Mesh, Options
from oracle.refine import refine_pass

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from mitra_algo_gb300 import Gb300Backend
    g = Gb300Backend(0)
    yield g
    g.close()


def rotation(axis, angle):
    k = np.asarray(axis, float) / np.linalg.norm(axis)
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + np.sin(angle) * K + (1 - np.cos(angle)) * K @ K


def bumpy_sphere(level=3):
    v, f = icosphere(level)
    r = np.ones(len(v))
    for c, a, s in (((0.6, 0.3, 0.74), 0.25, 0.3), ((-0.5, 0.7, 0.1), 0.15, 0.25),
                    ((0.1, -0.8, -0.6), 0.2, 0.35)):
        r += a * np.exp(-((v - np.array(c)) ** 2).sum(1) / (2 * s * s))
    return v * r[:, None], f


def two_copies(kind):
    """The shape and its image: a rigid motion (rotation 0.65 rad about
    (1, 2, 3) and a shift of 3.2 along x), or the mirror in the plane x = 2."""
    v, f = bumpy_sphere()
    if kind == "rigid":
        R, t = rotation((1, 2, 3), 0.65), np.array([3.2, 0.3, 0.2])
        w, g = v @ R.T + t, f
        truth = dict(reflection=0, rotation=R.reshape(-1), translation=t,
                     plane_normal=np.zeros(3), plane_offset=0.0)
    else:
        n, off = np.array([1.0, 0, 0]), -2.0
        R = np.eye(3) - 2 * np.outer(n, n)
        w, g = v @ R.T - 2 * off * n, f[:, ::-1]  # a mirror reverses the winding
        truth = dict(reflection=1, rotation=R.reshape(-1), translation=-2 * off * n,
                     plane_normal=n, plane_offset=off)
    verts = np.concatenate([v, w])
    faces = np.concatenate([f, g + len(v)])
    return Mesh(verts.T.copy(), faces.T.copy()), truth


def perturbed(truth, scale):
    m = dict(truth)
    if truth["reflection"]:
        n = truth["plane_normal"] + scale * np.array([0.0, 0.8, -0.6])
        n /= np.linalg.norm(n)
        off = truth["plane_offset"] + scale
        m.update(plane_normal=n, plane_offset=off, rotation=(np.eye(3) - 2 * np.outer(n, n)).reshape(-1),
                 translation=-2 * off * n)
    else:
        dR = rotation((0.3, -1, 0.5), scale)
        m.update(rotation=(dR @ truth["rotation"].reshape(3, 3)).reshape(-1),
                 translation=truth["translation"] + scale * np.array([1.0, -2.0, 1.0]))
    return m


def record(m):
    return (m["reflection"], m["rotation"], m["translation"], m["plane_normal"], m["plane_offset"])


def motion_error(a, b):
    return (np.abs(np.asarray(a["rotation"]) - np.asarray(b["rotation"])).max(),
            np.abs(np.asarray(a["translation"]) - np.asarray(b["translation"])).max())


@pytest.mark.parametrize("kind", ["rigid", "reflection"])
def test_one_pass_equals_the_fp64_restatement(gpu, kind):
    mesh, truth = two_copies(kind)
    o = Options()
    p = prepare(mesh, o)
    start = perturbed(truth, 3e-3)
    resident = gpu.load_mesh(p)
    got = gpu.refine_transforms(resident, o, [record(start)], 1)
    resident.close()
    tau = o.verify_threshold * p.context.box_size
    want = refine_pass(p.mesh.vertices, p.topology.normals, p.topology.weights, p.mesh.faces,
                       start, tau)
    dev = dict(rotation=got["rotation"][0], translation=got["translation"][0])
    # the device picks each vertex's nearest face by an FP32 search, so where
    # two faces are equally near to within FP32 it can take the other one,
    # whose closest point differs slightly: agreement to 1e-6, not to FP64
    # rounding (measured: 5e-8)
    er, et = motion_error(dev, want)
    assert er < 1e-6 and et < 1e-6, (er, et)
    if kind == "reflection":
        assert np.abs(got["plane_normal"][0] - want["plane_normal"]).max() < 1e-6
        assert abs(got["plane_offset"][0] - want["plane_offset"]) < 1e-6
    # the pass moved the motion toward the truth
    assert motion_error(dev, truth)[0] < motion_error(start, truth)[0]


@pytest.mark.parametrize("kind", ["rigid", "reflection"])
def test_passes_recover_the_exact_motion(gpu, kind):
    mesh, truth = two_copies(kind)
    o = Options()
    p = prepare(mesh, o)
    start = perturbed(truth, 3e-3)
    resident = gpu.load_mesh(p)
    before = gpu.refine_transforms(resident, o, [record(start)], 0)
    few = gpu.refine_transforms(resident, o, [record(start)], 3)
    many = gpu.refine_transforms(resident, o, [record(start)], 30)
    resident.close()
    err = [motion_error(dict(rotation=r["rotation"][0], translation=r["translation"][0]), truth)
           for r in (before, few, many)]
    assert err[0] == motion_error(start, truth)  # zero passes: the motion as given
    assert err[2][0] < err[1][0] < err[0][0] and err[2][1] < err[1][1] < err[0][1], err
    # point-to-point passes converge slowly along the sphere's sliding
    # rotation, fast everywhere else
    if kind == "reflection":
        assert err[2][0] < 0.01 * err[0][0] and err[2][1] < 0.01 * err[0][1], err
    else:
        assert err[2][1] < 0.1 * err[0][1], err
    assert many["rms"][0] < before["rms"][0]
    assert many["coverage"][0] >= before["coverage"][0]


def test_refinement_inside_detect_fast(gpu):
    """Reflection mode on the mirrored height field (mirror image in x = 0):
    refinement passes leave pairs, votes and mode counts as they were and
    bring the top plane closer to x = 0."""
    mesh = mirrored_heightfield(size=96, bumps=6, seed=4)
    o = Options(sample_ratio=3000 / mesh.vertex_count, pair_threshold=0.05, bandwidth=0.02,
                max_pairs=10 ** 7, max_votes=10 ** 7, max_clusters=4)
    p = prepare(mesh, o)
    resident = gpu.load_mesh(p)
    kw = dict(precision="bf16", seeds=256, max_iterations=100, polish_iterations=30,
              mode="reflection")
    a = gpu.detect_fast(resident, None, o, **kw)
    b = gpu.detect_fast(resident, None, o, refine=10, **kw)
    resident.close()
    for k in ("pairs", "votes", "modes", "clusters", "support"):
        assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), k
    na, nb = np.asarray(a["plane_normal"][0]), np.asarray(b["plane_normal"][0])
    ea = np.abs(np.abs(na) - np.array([1.0, 0, 0])).max() + abs(a["plane_offset"][0])
    eb = np.abs(np.abs(nb) - np.array([1.0, 0, 0])).max() + abs(b["plane_offset"][0])
    assert eb <= ea + 1e-12, (ea, eb)


def test_one_pass_with_faces_without_area(gpu):
    """Faces without area among the correspondences (each repeats a corner
    of a face of the copy, so its cross product is exactly zero): the
    device's closest point on such a face is the nearest of its segments,
    as in the FP64 restatement, and one pass still equals it."""
    import dataclasses
    mesh, truth = two_copies("rigid")
    o = Options()
    p = prepare(mesh, o)
    f = p.mesh.faces
    pick = np.arange(f.shape[1] // 2, f.shape[1], 5)  # faces of the copy
    extra = np.stack([f[0, pick], f[0, pick], f[1, pick]])
    faces = np.concatenate([f, extra], axis=1).astype(np.int32)
    fn = np.concatenate([p.topology.face_normals, np.zeros((3, extra.shape[1]))], axis=1)
    q = dataclasses.replace(p, mesh=Mesh(p.mesh.vertices, faces),
                            topology=dataclasses.replace(p.topology, face_normals=fn))
    start = perturbed(truth, 3e-3)
    resident = gpu.load_mesh(q)
    got = gpu.refine_transforms(resident, o, [record(start)], 1)
    resident.close()
    tau = o.verify_threshold * p.context.box_size
    want = refine_pass(q.mesh.vertices, q.topology.normals, q.topology.weights, q.mesh.faces,
                       start, tau)
    er, et = motion_error(dict(rotation=got["rotation"][0], translation=got["translation"][0]), want)
    assert er < 1e-6 and et < 1e-6, (er, et)
