"""Binary result tables (sym_export_tables, host code, no GPU): the tables of
the reference's eight example runs, exported from the reference's own stage
outputs and rendered as text, are byte-identical with the files the
reference's export_result wrote for the same runs (src/io/export.cpp:37-98);
the tables read back bit-exact; bad ids are rejected."""
import hashlib

import numpy as np
import pytest

from conftest import load_golden
from helpers import clusters_from, features_from, mesh_from, votes_from
from mitra_algo_gb300.export import export_tables, read_tables, render_text
from mitra_algo_gb300.types import Pairs

CASES = [f"{s}_{r}" for s in ("reflection", "rigid", "partial", "single") for r in ("1", "05")]
FILES = ("features.csv", "pairs.csv", "votes.csv", "descriptors.csv", "mesh.off")


def golden_result(name):
    g = load_golden(f"detect_{name}")
    mesh = mesh_from(g)
    return (g, mesh, features_from(g, mesh.vertex_count), g["sample"], g["pruned"],
            Pairs(g["pair_a"], g["pair_b"]), votes_from(g), clusters_from(g))


@pytest.mark.parametrize("name", CASES)
def test_text_matches_the_reference(name, tmp_path):
    g, *result = golden_result(name)
    export_tables(tmp_path / "bin", *result)
    render_text(tmp_path / "bin", tmp_path / "text")
    want = load_golden("export_text")
    for file in FILES:
        data = (tmp_path / "text" / file).read_bytes()
        assert len(data) == int(want[f"{name}:{file}:bytes"]), file
        assert hashlib.sha256(data).hexdigest() == str(want[f"{name}:{file}:sha"]), file


def test_tables_read_back_exactly(tmp_path):
    g, mesh, f, sample, pruned, pairs, votes, clusters = golden_result("partial_1")
    export_tables(tmp_path, mesh, f, sample, pruned, pairs, votes, clusters)
    t = read_tables(tmp_path)
    assert np.array_equal(t["pairs"]["a"], pairs.a) and np.array_equal(t["pairs"]["b"], pairs.b)
    for k, lane in enumerate(("x", "y", "z")):
        assert t["vertices"][lane].tobytes() == mesh.vertices[k].tobytes()
        assert t["features"]["n" + lane].tobytes() == f.normal[k].tobytes()
    assert np.array_equal(t["faces"]["c"], mesh.faces[2])
    assert t["votes"]["r12"].tobytes() == votes.rotation[5].tobytes()
    assert t["descriptors"]["component11"].tobytes() == votes.descriptor[11].tobytes()
    assert np.array_equal(np.flatnonzero(t["features"]["sampled"]), np.sort(sample))
    want = np.full(len(votes), -1)
    for c in range(len(clusters)):
        lo, hi = clusters.votes.offsets[c], clusters.votes.offsets[c + 1]
        want[clusters.votes.indices[lo:hi]] = c
    assert np.array_equal(t["votes"]["cluster"], want)
    assert np.array_equal(t["descriptors"]["dimension"], np.where(votes.kind == 1, 4, 12))


def test_bad_ids_are_rejected(tmp_path):
    g, mesh, f, sample, pruned, pairs, votes, clusters = golden_result("single_05")
    bad = np.array(sample, np.int32)
    bad[0] = mesh.vertex_count
    with pytest.raises(RuntimeError, match="sample index out of range"):
        export_tables(tmp_path, mesh, f, bad, pruned, pairs, votes, clusters)
    a = np.array(pairs.a)
    a[-1] = -1
    with pytest.raises(RuntimeError, match="pair index out of range"):
        export_tables(tmp_path, mesh, f, sample, pruned, Pairs(a, pairs.b), votes, clusters)


def test_empty_result_exports_headers_only(tmp_path):
    """No pairs, votes or clusters: the tables have zero rows and the text
    files hold the reference's header lines only (features and the mesh
    still list every vertex)."""
    g, mesh, f, sample, pruned, pairs, votes, clusters = golden_result("single_05")
    empty_pairs = Pairs(np.zeros(0, np.int32), np.zeros(0, np.int32))
    empty_votes = votes_from({**g, "vote_pair": np.zeros(0, np.int32),
                              "vote_kind": np.zeros(0, np.uint8), "poff": np.zeros(0)})
    from mitra_algo_gb300.types import ClusterOutput, Csr
    no_clusters = ClusterOutput(np.zeros(0, np.uint8), np.zeros((0, 9)), np.zeros((0, 3)),
                                np.zeros((0, 3)), np.zeros(0),
                                Csr(np.zeros(1, np.uint64), np.zeros(0, np.int32)))
    export_tables(tmp_path / "bin", mesh, f, sample, pruned, empty_pairs, empty_votes, no_clusters)
    t = read_tables(tmp_path / "bin")
    assert len(t["pairs"]["a"]) == 0 and len(t["votes"]["pair"]) == 0
    assert len(t["features"]["x"]) == mesh.vertex_count
    render_text(tmp_path / "bin", tmp_path / "text")
    assert (tmp_path / "text" / "pairs.csv").read_text() == "pair,a,b\n"
    assert (tmp_path / "text" / "votes.csv").read_text().count("\n") == 1
    assert (tmp_path / "text" / "descriptors.csv").read_text().startswith("vote,dimension,component0")
    lines = (tmp_path / "text" / "features.csv").read_text().splitlines()
    assert len(lines) == mesh.vertex_count + 1
