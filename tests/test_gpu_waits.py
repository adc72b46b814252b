"""The device's bounded waits, made to run out without a fault (the failure
is made on the device by a wait that nothing satisfies, with a short limit):

* the tensor-core kernels' barrier wait -- a kernel holding tensor memory
  waits on an mbarrier nothing signals with a limit of 50 microseconds in
  place of 2 s; the call reports SYM_DEVICE_TIMEOUT (DeviceTimeout) well
  within a second, the kernel freed its tensor memory, and a tensor-core
  call on the same context afterwards is correct;
* the verification's union-find retry loop -- with no retries every union
  gives up and the call reports SYM_DEVICE_TIMEOUT; with the regular limit
  the 64-vertex path is one component; a verification on the same context
  afterwards equals the reference's golden output."""
import time

import numpy as np
import pytest

from conftest import golden_cases
from helpers import clusters_from, mesh_from, options_from, same_array, verification_arrays
from mitra_algo_gb300.backend import DeviceTimeout
from mitra_algo_gb300.mesh import prepare

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from mitra_algo_gb300 import Gb300Backend
    b = Gb300Backend(0)
    yield b
    b.close()


def tensor_call_is_correct(gpu):
    from test_gpu_tensor import from_bf16_bits, to_bf16_bits
    rng = np.random.default_rng(5)
    a1, b1 = (to_bf16_bits(rng.uniform(-1, 1, (128, 16))) for _ in range(2))
    a2 = to_bf16_bits(rng.uniform(0, 1, (128, 128)))
    b2 = to_bf16_bits(rng.uniform(-1, 1, (16, 128)))
    d, acc = gpu.tc_selftest(a1, b1, a2, b2)
    ref_d = from_bf16_bits(a1).astype(np.float64) @ from_bf16_bits(b1).astype(np.float64).T
    ref_acc = from_bf16_bits(a2).astype(np.float64) @ from_bf16_bits(b2).astype(np.float64).T
    return np.allclose(d, ref_d, rtol=1e-5, atol=1e-5) and \
        np.allclose(acc, ref_acc, rtol=1e-5, atol=1e-4)


def test_tensor_wait_runs_out_and_the_context_stays_usable(gpu):
    for _ in range(2):
        t0 = time.perf_counter()
        with pytest.raises(DeviceTimeout):
            gpu.wait_selftest("tensor", 50_000)
        assert time.perf_counter() - t0 < 1.0
        assert tensor_call_is_correct(gpu)


def test_union_find_retries_run_out_and_the_context_stays_usable(gpu):
    with pytest.raises(DeviceTimeout):
        gpu.wait_selftest("union", 0)
    assert gpu.wait_selftest("union", 1 << 20) == 1
    case = golden_cases("stage_verification")[0]
    d = case["in"]
    o = options_from(d)
    p = prepare(mesh_from(d), o)
    v = gpu.verification(p.mesh, p.topology, clusters_from(d), p.context, o)
    got = verification_arrays(v)
    for k in ("ver_side_a", "ver_side_b", "ver_patches_a_indices", "ver_patches_b_indices"):
        same_array(got[k], case["out"][k], k)
