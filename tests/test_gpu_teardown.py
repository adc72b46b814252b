"""A resident mesh freed after the context that loaded it is destroyed
(as at interpreter exit, where finalizers run in any order): sym_mesh_free
does not use the loading context."""
import pytest

from mitra_algo_gb300.mesh import motif_sphere
from mitra_algo_gb300.types import Options

pytestmark = pytest.mark.gpu


def test_mesh_freed_after_its_context():
    from mitra_algo_gb300 import Gb300Backend
    gpu = Gb300Backend(0)
    mesh = motif_sphere(level=3, bumps=4, folds=3, partial_shift=0.3, noise=1e-3, seed=2)
    o = Options(sample_ratio=1.0, pair_threshold=0.25, bandwidth=0.1, max_clusters=4)
    resident = gpu.load_mesh_raw(mesh, o)
    r = gpu.detect_fast(resident, None, o, seeds=64, max_iterations=40, polish_iterations=10)
    assert r["votes"] > 0
    gpu.close()        # the loading context first
    resident.close()   # then the mesh
    again = Gb300Backend(0)
    resident = again.load_mesh_raw(mesh, o)
    assert again.detect_fast(resident, None, o, seeds=64, max_iterations=40,
                             polish_iterations=10)["votes"] == r["votes"]
    resident.close()
    again.close()
