"""The GPU stages' results of the reference's eight example runs (each stage
on the reference's own inputs, as in the stage tests), exported as binary
tables (sym_export_tables) and rendered as text, are byte-identical with the
files the reference's export_result wrote (src/io/export.cpp:37-98)."""
import hashlib

import pytest

from conftest import load_golden
from helpers import features_from, mesh_from, options_from, votes_from
from mitra_algo_gb300.export import export_tables, render_text
from mitra_algo_gb300.mesh import prepare
from mitra_algo_gb300.types import Rng

pytestmark = pytest.mark.gpu

CASES = [f"{s}_{r}" for s in ("reflection", "rigid", "partial", "single") for r in ("1", "05")]
FILES = ("features.csv", "pairs.csv", "votes.csv", "descriptors.csv", "mesh.off")


@pytest.fixture(scope="module")
def gpu():
    from mitra_algo_gb300 import Gb300Backend
    g = Gb300Backend(0)
    yield g
    g.close()


@pytest.mark.parametrize("name", CASES)
def test_gpu_results_export_like_the_reference(gpu, name, tmp_path):
    g = load_golden(f"detect_{name}")
    o = options_from(g, "in_")
    p = prepare(mesh_from(g, "in_"), o)
    f = features_from(g, p.mesh.vertex_count)
    rng = Rng(o.seed)
    s = gpu.select(p.mesh, f, p.topology.weights, o, rng)
    pairs = gpu.pairing(p.mesh, f, s.pruned, p.context, o)
    votes = gpu.transformations(p.mesh, f, pairs, p.context, o)
    clusters = gpu.clustering(votes_from(g), p.context, o, rng)
    export_tables(tmp_path / "bin", p.mesh, f, s.sample, s.pruned, pairs, votes, clusters)
    render_text(tmp_path / "bin", tmp_path / "text")
    want = load_golden("export_text")
    for file in FILES:
        data = (tmp_path / "text" / file).read_bytes()
        assert hashlib.sha256(data).hexdigest() == str(want[f"{name}:{file}:sha"]), file
