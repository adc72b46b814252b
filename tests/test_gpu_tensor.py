"""The tensor-core path of the BF16 mean-shift: shared-memory layouts, TMA bulk
copy, tcgen05.mma into TMEM and tcgen05.ld, checked on one tile against a
plain FP32 matrix product of the same BF16 values (tolerance 1e-5 relative:
the products of BF16 values are exact in FP32; only the FP32 sums round)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def to_bf16_bits(x):
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)


def from_bf16_bits(b):
    return (b.astype(np.uint32) << 16).view(np.float32)


@pytest.fixture(scope="module")
def gpu():
    from mitra_algo_gb300 import Gb300Backend
    b = Gb300Backend(0)
    yield b
    b.close()


def test_tcgen05_tile_products(gpu):
    rng = np.random.default_rng(11)
    a1 = to_bf16_bits(rng.uniform(-1, 1, (128, 16)))
    b1 = to_bf16_bits(rng.uniform(-1, 1, (128, 16)))
    a2 = to_bf16_bits(rng.uniform(0, 1, (128, 128)))
    b2 = to_bf16_bits(rng.uniform(-1, 1, (16, 128)))
    d, acc = gpu.tc_selftest(a1, b1, a2, b2)
    ref_d = from_bf16_bits(a1).astype(np.float64) @ from_bf16_bits(b1).astype(np.float64).T
    ref_acc = from_bf16_bits(a2).astype(np.float64) @ from_bf16_bits(b2).astype(np.float64).T
    assert np.allclose(d, ref_d, rtol=1e-5, atol=1e-5), np.max(np.abs(d - ref_d))
    assert np.allclose(acc, ref_acc, rtol=1e-5, atol=1e-4), np.max(np.abs(acc - ref_acc))


def test_tcgen05_structured_operands(gpu):
    """Identity-like operands expose any row/column permutation of the
    layouts."""
    a1 = np.zeros((128, 16), np.float32)
    a1[np.arange(128), np.arange(128) % 16] = np.arange(128) + 1
    b1 = np.zeros((128, 16), np.float32)
    b1[np.arange(128), np.arange(128) % 16] = 1
    a2 = np.zeros((128, 128), np.float32)
    a2[np.arange(128), np.arange(128)] = 1
    b2 = (np.arange(16)[:, None] * 1000 + np.arange(128)[None, :]).astype(np.float32) / 4096
    bits = [to_bf16_bits(x) for x in (a1, b1, a2, b2)]
    d, acc = gpu.tc_selftest(*bits)
    vals = [from_bf16_bits(x).astype(np.float64) for x in bits]
    assert np.allclose(d, vals[0] @ vals[1].T, rtol=1e-6, atol=1e-6)
    assert np.allclose(acc, vals[2] @ vals[3].T, rtol=1e-6, atol=1e-6)
