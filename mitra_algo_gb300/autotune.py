"""Autotuner of the mean shift's launch shapes.

The throughput path has four launch-shape parameters (sym_fast_options):

* ``vote_bits`` - Morton bits per coordinate of the vote order, i.e. how
  finely the votes are sorted into 128-vote chunks (the chunks' boxes decide
  which chunks a tile of seeds reads);
* ``simt_blocks_per_sm`` - the CTAs per SM the SIMT mean-shift grid aims at
  (the FP32 approach and the FP32 polish split the chunks of each seed tile
  over that many CTAs);
* ``tc_ctas_per_sm`` - the tensor kernel's chunk-list pieces per SM, i.e. the
  number of waves the BF16 approach's lists are cut into;
* ``check_interval`` - BF16 approach iterations between the host's looks at
  the active-seed count.

None changes the method: they change the work split, the order of FP32 sums
and how long the loop runs past its last active iteration.  ``autotune``
times ``Gb300Backend.detect_fast`` on one workload with each candidate
value, one parameter at a time (coordinate descent from the defaults), by
the device time of the whole pipeline (the sum of its stage timings, best of
``repeats`` runs), and keeps a candidate only when it is faster by more than
``margin``.  Results can be cached in a JSON file keyed by the workload's
shape (vertex, sample and seed counts rounded to powers of two, precision,
mode, options), so a service tunes once per kind of mesh.
"""
from __future__ import annotations

import json
import math
from pathlib import Path

from .backend import TUNING_KEYS

DEFAULTS = {"vote_bits": 8, "simt_blocks_per_sm": 128, "tc_ctas_per_sm": 1, "check_interval": 8}
CANDIDATES = {
    "vote_bits": (6, 7, 8, 9),
    "simt_blocks_per_sm": (32, 64, 128, 256),
    "tc_ctas_per_sm": (1, 2, 3),
    "check_interval": (4, 8, 16),
}
# parameters that have no effect on a precision's run are not tried
USED_BY = {"fp32": ("vote_bits", "simt_blocks_per_sm"),
           "bf16": ("vote_bits", "simt_blocks_per_sm", "tc_ctas_per_sm", "check_interval")}


def signature(vertices: int, samples: int, seeds: int, precision: str, mode: str,
              options) -> str:
    """The cache key: counts rounded to powers of two, and what else sets the
    amount of work (options, precision, mode)."""
    bucket = lambda n: 0 if n <= 0 else int(round(math.log2(n)))  # noqa: E731
    return (f"v{bucket(vertices)}-s{bucket(samples)}-k{bucket(seeds)}-{precision}-{mode}-"
            f"t{options.pair_threshold:g}-h{options.bandwidth:g}-p{options.prune:g}")


def _load(cache):
    if cache and Path(cache).exists():
        return json.loads(Path(cache).read_text())
    return {}


def autotune(gpu, mesh, sample, options, precision="bf16", seeds=2048, mode="rigid",
             repeats=2, margin=0.02, cache=None, **kw) -> dict:
    """Tunes the launch shapes of detect_fast on (mesh, sample, options).
    Returns {"tuning": {...}, "ms": best, "default_ms": defaults' time,
    "trials": [(tuning, ms), ...], "cached": bool}.  `kw` are further
    detect_fast arguments (iterations, vote_cap ...)."""
    if precision not in USED_BY:
        raise ValueError(f"unknown precision {precision!r}")
    samples = len(sample) if sample is not None else math.ceil(mesh.vertex_count *
                                                               options.sample_ratio)
    key = signature(mesh.vertex_count, samples, seeds, precision, mode, options)
    stored = _load(cache)
    if key in stored:
        return dict(stored[key], cached=True)

    def run(t):
        best = math.inf
        for _ in range(repeats):
            r = gpu.detect_fast(mesh, sample, options, precision=precision, seeds=seeds,
                                mode=mode, tuning=t, **kw)
            best = min(best, sum(r["stage_ms"].values()))
        return best

    run(DEFAULTS)  # warm-up: the workspace reaches its size
    best = dict(DEFAULTS)
    best_ms = default_ms = run(best)
    trials = [(dict(best), best_ms)]
    for name in USED_BY[precision]:
        for value in CANDIDATES[name]:
            if value == best[name]:
                continue
            t = dict(best, **{name: value})
            ms = run(t)
            trials.append((t, ms))
            if ms < best_ms * (1 - margin):
                best, best_ms = t, ms
    out = {"tuning": best, "ms": best_ms, "default_ms": default_ms, "trials": trials}
    if cache:
        stored[key] = out
        Path(cache).write_text(json.dumps(stored, indent=1))
    return dict(out, cached=False)


assert set(DEFAULTS) == set(TUNING_KEYS) == set(CANDIDATES)
