"""The autotuner's search (mitra_algo_gb300/autotune.py) on a stand-in for
the GPU backend whose timings are a known function of the launch shapes:
coordinate descent finds the fastest shape, keeps the defaults when nothing
beats them by the margin, tries only the parameters a precision uses, and
answers from its cache the second time."""
import pytest

from mitra_algo_gb300.autotune import CANDIDATES, DEFAULTS, autotune, signature
from mitra_algo_gb300.types import Options


class FakeMesh:
    vertex_count = 54_756


class FakeGpu:
    def __init__(self, cost):
        self.cost, self.calls = cost, []

    def detect_fast(self, mesh, sample, options, precision, seeds, mode, tuning, **kw):
        self.calls.append(dict(tuning))
        return {"stage_ms": {"mean_shift": self.cost(tuning), "other": 10.0}}


def test_finds_the_fastest_shape():
    def cost(t):  # separable, best at vote_bits 7, 32 CTAs/SM, 2 tc CTAs/SM, interval 16
        return (100 + 5 * abs(t["vote_bits"] - 7) + 4 * abs(t["simt_blocks_per_sm"] - 32) / 32 +
                6 * abs(t["tc_ctas_per_sm"] - 2) + (0 if t["check_interval"] == 16 else 3))
    gpu = FakeGpu(cost)
    r = autotune(gpu, FakeMesh(), list(range(20_000)), Options(), precision="bf16")
    assert r["tuning"] == {"vote_bits": 7, "simt_blocks_per_sm": 32, "tc_ctas_per_sm": 2,
                           "check_interval": 16}
    assert r["ms"] < r["default_ms"] and not r["cached"]


def test_keeps_the_defaults_within_the_margin():
    gpu = FakeGpu(lambda t: 100 - (0.5 if t["vote_bits"] == 6 else 0))  # 0.5% better only
    r = autotune(gpu, FakeMesh(), list(range(100)), Options(), precision="bf16", margin=0.02)
    assert r["tuning"] == DEFAULTS


def test_fp32_tries_only_its_parameters():
    gpu = FakeGpu(lambda t: 100.0)
    autotune(gpu, FakeMesh(), list(range(100)), Options(), precision="fp32", repeats=1)
    for t in gpu.calls:
        assert t["tc_ctas_per_sm"] == DEFAULTS["tc_ctas_per_sm"]
        assert t["check_interval"] == DEFAULTS["check_interval"]
    tried = len(gpu.calls) - 2  # warm-up and the defaults
    assert tried == len(CANDIDATES["vote_bits"]) + len(CANDIDATES["simt_blocks_per_sm"]) - 2


def test_cache(tmp_path):
    cache = tmp_path / "tuning.json"
    gpu = FakeGpu(lambda t: 100 - t["vote_bits"])
    first = autotune(gpu, FakeMesh(), list(range(100)), Options(), cache=cache)
    n = len(gpu.calls)
    again = autotune(gpu, FakeMesh(), list(range(100)), Options(), cache=cache)
    assert len(gpu.calls) == n and again["cached"] and again["tuning"] == first["tuning"]
    # another kind of workload is tuned afresh
    autotune(gpu, FakeMesh(), list(range(100)), Options(bandwidth=0.05), cache=cache)
    assert len(gpu.calls) > n


def test_signature_rounds_counts():
    o = Options()
    assert signature(54_000, 20_000, 2048, "bf16", "rigid", o) == \
        signature(56_000, 21_000, 2048, "bf16", "rigid", o)
    assert signature(54_000, 20_000, 2048, "bf16", "rigid", o) != \
        signature(54_000, 20_000, 2048, "fp32", "rigid", o)


def test_unknown_precision():
    with pytest.raises(ValueError):
        autotune(FakeGpu(lambda t: 1.0), FakeMesh(), [], Options(), precision="fp16")
