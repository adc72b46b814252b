"""The C ABI header is plain C (it compiles as C99 with warnings as errors)
and every structure of the ctypes binding (mitra_algo_gb300/abi.py) has the
size and field offsets of its C declaration (include/mitra_gb300.h), so the
binding and a C caller read the same bytes."""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import pytest

from mitra_algo_gb300 import abi

ROOT = Path(__file__).resolve().parents[1]

PAIRS = {  # ctypes structure -> C type
    "PointsView": "sym_points_view", "FacesView": "sym_faces_view", "MeshView": "sym_mesh_view",
    "CsrView": "sym_csr_view", "Edge": "sym_edge", "TopologyView": "sym_topology_view",
    "FeaturesView": "sym_features_view", "FeaturesOut": "sym_features_out",
    "PairsView": "sym_pairs_view", "VotesView": "sym_votes_view",
    "ClusterRecord": "sym_cluster_record", "ClustersView": "sym_clusters_view",
    "ExportView": "sym_export_view", "ModelContext": "sym_model_context",
    "Options": "sym_options", "Rng": "sym_rng", "Selection": "sym_selection",
    "PairsOut": "sym_pairs", "VotesOut": "sym_votes", "ClustersOut": "sym_clusters",
    "GroupedCsr": "sym_grouped_csr", "VerificationOut": "sym_verification_result",
    "Metric": "sym_metric", "FastOptions": "sym_fast_options", "FastResult": "sym_fast_result",
    "PreparedOut": "sym_prepared", "BatchItem": "sym_batch_item",
}


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("abi")
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "mitra_gb300.h"',
             "int main(void) {"]
    for py, ct in PAIRS.items():
        lines.append(f'  printf("{py} size %zu\\n", sizeof({ct}));')
        for name, *_ in getattr(abi, py)._fields_:
            lines.append(f'  printf("{py} {name} %zu\\n", offsetof({ct}, {name}));')
    lines += ["  return 0;", "}"]
    src = d / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = d / "layout"
    subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic",
                    f"-I{ROOT / 'include'}", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {tuple(line.split()[:2]): int(line.split()[2]) for line in out.splitlines()}


@pytest.mark.parametrize("py", sorted(PAIRS))
def test_struct_layout_matches_the_header(c_layout, py):
    cls = getattr(abi, py)
    assert C.sizeof(cls) == c_layout[(py, "size")], py
    for name, *_ in cls._fields_:
        assert getattr(cls, name).offset == c_layout[(py, name)], (py, name)
