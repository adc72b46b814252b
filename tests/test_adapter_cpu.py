"""The reference-side adapter (mitra_algo_gb300/adapter: Gb300Backend, a
symmetry::Backend over the C ABI) compiled against the reference's own
headers (include/symmetry/pipeline.h, cuda.h, storage.h) and linked with
libmitra_gb300.so, on CPU.  The compile itself checks, by static_assert, that
sym_cluster_record and sym_edge have the layout of the reference's
ClusterRecord and Edge; the program then checks the engine-state round trip,
the status -> exception mapping (types and messages, "budget" included), the
metrics mapping and the factory's "CUDA: ..." error without a device.

The reference tree comes from MITRA_REFERENCE_DIR, else from oracle/Makefile's
recipe default; the test is skipped where neither names a tree."""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import pytest

from mitra_algo_gb300 import abi
from oracle import oracle

ROOT = Path(__file__).resolve().parents[1]
ADAPTER = ROOT / "mitra_algo_gb300" / "adapter"


@pytest.fixture(scope="module")
def check_program(tmp_path_factory):
    tree = oracle.reference_tree()
    if tree is None:
        pytest.skip("reference source tree not available (set MITRA_REFERENCE_DIR)")
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    from mitra_algo_gb300 import build
    lib = build.build()
    exe = tmp_path_factory.mktemp("adapter") / "adapter_check"
    cmd = [cxx, "-std=c++17", "-O1", "-Wall", "-Werror", f"-I{ADAPTER}", f"-I{ROOT / 'include'}",
           f"-I{tree / 'include'}", str(ADAPTER / "gb300_backend.cpp"),
           str(ROOT / "tests" / "adapter_check.cpp"), f"-L{lib.parent}", "-lmitra_gb300",
           f"-Wl,-rpath,{lib.parent}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.fixture(scope="module")
def facts(check_program):
    r = subprocess.run([str(check_program)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    out = {}
    for line in r.stdout.splitlines():
        key, _, value = line.partition(" ")
        out.setdefault(key, []).append(value)
    return out


def test_cluster_record_layout_matches_the_ctypes_binding(facts):
    assert int(facts["cluster_record_size"][0]) == C.sizeof(abi.ClusterRecord)
    offsets = [int(x) for x in facts["cluster_record_offsets"][0].split()]
    assert offsets == [getattr(abi.ClusterRecord, f).offset for f in
                       ("reflection", "rotation", "translation", "plane_normal", "plane_offset")]
    assert int(facts["edge_size"][0]) == 24


def test_engine_state_round_trip(facts):
    assert facts["rng"] == ["ok 1"]


def test_status_maps_to_reference_exceptions(facts):
    got = {int(v.split(" ", 1)[0]): v.split(" ", 1)[1] for v in facts["status"]}
    assert "budget" in got[abi.RUNTIME_ERROR]  # the reference's tests grep for it
    assert got[abi.CUDA_ERROR].startswith("CUDA: ")
    assert got[5] == "CUDA: no available device"


def test_factory_without_device_raises_the_cuda_error(facts):
    kind, _, message = facts["factory"][0].partition(" ")
    if kind == "no_device":
        assert message.startswith("CUDA: ")
    else:
        assert message == "gb300"


def test_no_failures(facts):
    assert facts["failures"] == ["0"]
