"""sym_prune_static (allocation-free prune, scratch in static device memory)
against the regular entry point sym_select, through the C ABI.

Integer selection: the kept samples must be identical to sym_select's
`pruned`, in the same order, on every call.  The file name sorts last so the
test also runs after every other GPU test has used the library."""
import ctypes as C

import numpy as np
import pytest

from conftest import golden_cases
from helpers import features_from, options_from, points_only_mesh
from mitra_algo_gb300 import abi
from mitra_algo_gb300.types import Features, Mesh, Options, Rng

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def gpu():
    from mitra_algo_gb300 import Gb300Backend
    b = Gb300Backend(0)
    yield b
    b.close()


def prune_static(sample, features, prune, vertex_count=None):
    """Two back-to-back sym_prune_static calls on torch's current stream;
    returns both (kept ids, kept count) results."""
    lib = abi.library()
    dev = torch.device("cuda", 0)
    d_sample = torch.from_numpy(np.ascontiguousarray(sample, np.int32)).to(dev)
    d_kmin = torch.from_numpy(np.ascontiguousarray(features.kmin, np.float64)).to(dev)
    d_kmax = torch.from_numpy(np.ascontiguousarray(features.kmax, np.float64)).to(dev)
    d_valid = torch.from_numpy(np.ascontiguousarray(features.valid, np.uint8)).to(dev)
    n = len(features) if vertex_count is None else vertex_count
    stream = torch.cuda.current_stream(dev).cuda_stream
    assert lib.sym_prune_static_setup() == abi.OK, lib.sym_last_error()
    results = []
    for _ in range(2):
        d_pruned = torch.full((max(len(sample), 1),), -7, dtype=torch.int32, device=dev)
        d_count = torch.full((1,), 12345, dtype=torch.int64, device=dev)
        status = lib.sym_prune_static(d_sample.data_ptr(), len(sample), d_kmin.data_ptr(),
                                      d_kmax.data_ptr(), d_valid.data_ptr(), n, prune,
                                      d_pruned.data_ptr(), d_count.data_ptr(), stream)
        assert status == abi.OK, lib.sym_last_error()
        torch.cuda.synchronize(dev)
        count = int(d_count.cpu().numpy().view(np.uint64)[0])
        kept = d_pruned.cpu().numpy()
        results.append((kept, count))
    return results


@pytest.mark.parametrize("case", golden_cases("stage_select"), ids=lambda c: c["name"])
def test_matches_select_on_golden_cases(gpu, case):
    d = case["in"]
    mesh = points_only_mesh(d)
    f = features_from(d, mesh.vertex_count)
    o = options_from(d)
    s = gpu.select(mesh, f, d["weights"], o, Rng(int(d["seed"][0])))
    want = case["out"]["pruned"]  # the reference's own select() on this case
    assert np.array_equal(s.pruned, want)
    for kept, count in prune_static(case["out"]["sample"], f, o.prune):
        assert count == len(want)
        assert np.array_equal(kept[:count], want)
        assert np.all(kept[count:] == -7)  # nothing written past the kept entries


def test_call_allocates_no_device_memory(gpu):
    """The defining property: a call (after the set-up) takes no device
    memory.  The device's free memory is read right before and right after
    a call whose inputs and outputs were allocated beforehand."""
    lib = abi.library()
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(3)
    n = 200_000
    d_sample = torch.from_numpy(rng.integers(0, n, n // 2).astype(np.int32)).to(dev)
    d_kmin = torch.from_numpy(rng.normal(size=n)).to(dev)
    d_kmax = torch.from_numpy(rng.normal(size=n)).to(dev)
    d_valid = torch.ones(n, dtype=torch.uint8, device=dev)
    d_pruned = torch.empty(n // 2, dtype=torch.int32, device=dev)
    d_count = torch.empty(1, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    assert lib.sym_prune_static_setup() == abi.OK, lib.sym_last_error()

    def call():
        assert lib.sym_prune_static(d_sample.data_ptr(), n // 2, d_kmin.data_ptr(),
                                    d_kmax.data_ptr(), d_valid.data_ptr(), n, 0.85,
                                    d_pruned.data_ptr(), d_count.data_ptr(),
                                    stream) == abi.OK, lib.sym_last_error()
        torch.cuda.synchronize(dev)

    call()  # first call: kernels loaded
    for _ in range(2):
        free_before, _ = torch.cuda.mem_get_info(dev)
        call()
        free_after, _ = torch.cuda.mem_get_info(dev)
        assert free_after == free_before
    assert 0 < int(d_count.cpu()[0]) <= n // 2


def test_matches_select_many_tiles(gpu):
    # 3M vertices, about 2.7M samples: thousands of 1024-sample tiles
    rng = np.random.default_rng(11)
    n = 3_000_000
    f = Features.zeros(n)
    f.kmin = rng.normal(size=n) * rng.choice([0.0, 1e-12, 1.0, 50.0], size=n)
    f.kmax = f.kmin + rng.normal(size=n) * rng.choice([0.0, 0.1, 1.0], size=n)
    f.valid = (rng.random(n) < 0.9).astype(np.uint8)
    mesh = Mesh(rng.random((3, n)), np.zeros((3, 0), np.int32))
    o = Options(sample_ratio=0.9, prune=0.6)
    s = gpu.select(mesh, f, np.ones(n), o, Rng(5))
    assert len(s.sample) > 1_000_000 and 0 < len(s.pruned) < len(s.sample)
    for kept, count in prune_static(s.sample, f, o.prune):
        assert count == len(s.pruned)
        assert np.array_equal(kept[:count], s.pruned)


def test_empty_sample(gpu):
    f = Features.zeros(4)
    for kept, count in prune_static(np.zeros(0, np.int32), f, 0.85):
        assert count == 0


def test_out_of_range_index_reported(gpu):
    f = Features.zeros(8)
    f.kmin[:] = 1.0
    f.kmax[:] = 3.0
    f.valid[:] = 1
    for kept, count in prune_static(np.array([0, 1, 8, 2], np.int32), f, 0.85):
        assert count == 2**64 - 1


def test_rejects_counts_beyond_the_static_limit(gpu):
    lib = abi.library()
    limit = lib.sym_prune_static_max_samples()
    assert limit == 1 << 24
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    status = lib.sym_prune_static(dummy, limit + 1, dummy, dummy, dummy, 10, 0.85, dummy, dummy,
                                  None)
    assert status == abi.INVALID_ARGUMENT
    assert b"static scratch limit" in lib.sym_last_error()
