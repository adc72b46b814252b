"""CPU-side checks of the C ABI library: it builds for sm_103a, loads, and
exports exactly what include/mitra_gb300.h declares; host-only entry points
behave like the reference (options defaults, std::mt19937_64 state) and a
missing GPU is reported like the reference's "no device" error."""
import ctypes as C
import subprocess

import numpy as np
import pytest

from conftest import load_golden
from mitra_algo_gb300 import abi
from mitra_algo_gb300.types import Options, Rng


@pytest.fixture(scope="module")
def lib():
    from mitra_algo_gb300 import build
    build.build()
    return abi.library()


def test_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", str(abi.LIB_PATH)], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T sym_" in line}
    declared = set(abi.declared_symbols())
    assert declared == exported
    for name, _, _ in abi.PROTOTYPES:
        assert name in declared


def test_library_is_sm103a_only(lib):
    out = subprocess.run(["cuobjdump", "--list-elf", str(abi.LIB_PATH)], capture_output=True,
                         text=True).stdout
    assert "sm_103a" in out


def test_options_default_matches_reference(lib):
    o = abi.Options()
    lib.sym_options_default(C.byref(o))
    d = Options()
    for name, _ in abi.Options._fields_:
        assert getattr(o, name) == (int(getattr(d, name)) if name == "patching" else getattr(d, name))


def test_rng_matches_std_mt19937_64(lib):
    g = load_golden("stage_rng")
    r = Rng(42)
    assert r.text() == str(g["rng_seeded"])
    assert np.array_equal(np.array([r.next() for _ in range(1000)], np.uint64), g["draws"])
    assert r.text() == str(g["rng_after_draws"])


def test_no_device_is_reported(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    ctx = C.c_void_p()
    status = lib.sym_context_create(0, C.byref(ctx))
    assert status == abi.NO_DEVICE
    assert lib.sym_last_error().decode() == "CUDA: no available device"
    assert not ctx.value
