#!/usr/bin/env python3
"""Benchmark of the symmetry hot path on GB300.

Workload (rigid mode, FP32 vs BF16-refined mean-shift): an icosphere
subdivided 6 times, radially displaced by a seeded 12-bump motif repeated in
5-fold rotation about z, plus a partial copy translated 0.4 along x, Gaussian
vertex noise 1e-3 of the bbox diagonal (54,756 vertices, 109,102 faces);
20,000 area-weighted samples, pair threshold 0.25 (~1e7 pairs), 6-D rigid
votes, 2,048 mean-shift seeds, bandwidth 0.1; mean-shift approach phase of
up to 300 iterations (BF16 tensor cores, or FP32 for the comparison form),
then up to 30 FP32 polish iterations (Newton steps near the modes) for both
forms.  Synthetic data, seeded.

One step = the whole hot path on one mesh: curvature, prune, exact pairing,
6-D votes, vote sort, mean-shift, modes, verification of the top 20 modes.

  value  - meshes/s with the mesh resident in HBM (sym_mesh_load once),
           device time from CUDA events on the library's stream, L2 flushed
           (256 MiB write) before every step;
  e2e    - meshes/s through the public C ABI from pinned host buffers: every
           step uploads the raw mesh (sym_mesh_load_raw: GPU prepare), runs
           sym_detect_fast_sampled (the area-weighted sample drawn on the
           device from the options' seed, then the whole path) and reads the
           result back.

`c1_exact` - the reference's CPU-runnable case (the mirrored 128 x 128 height
           field) through the bit-exact stage path of the C ABI against the
           oracle port of the reference's CPU path, both measured end to end,
           results compared.

`--impl reference` times the oracle port of the reference's CPU path on
bounded samples of the same workload, one sample per host core at once, and
states the per-mesh time those samples imply by the reference's own work
counts (a lower bound: the reference stops with "Too many mean-shift modes"
on this mesh).  `cpu_baseline` is one such sample on one core.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import tempfile
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "meshes/s and pair votes/s, BF16-refined vs plain FP32 on GPU at ≤1e-4 mode error"
SAMPLES = 20000
PAIR_THRESHOLD = 0.25
BANDWIDTH = 0.1
SEEDS = 2048
ITERATIONS = 300  # mean-shift approach-phase iterations (BF16, or FP32)
POLISH = 30       # FP32 polish iterations (both forms)
VOTE_CAP = 0      # votes entering the mean shift (0: all)
WORKLOAD = "motif icosphere L6, rigid mode, 6-D votes"
# DRAM bytes (read + write) per (seed tile, vote chunk) pair of ms_tile_tc,
# from the ncu capture summarised in profiles/ms_tile_tc.md
TRAFFIC_PER_CHUNK_PAIR = 8300.0
IMAGE_BYTES = 8224.0  # one chunk image: the algorithmic bytes of a (tile, chunk) pair
BATCH_SAMPLES, BATCH_SEEDS = 4000, 512  # per mesh of the uneven batch


def reflection_bench(gpu, steps=5):
    """Reflection mode on the mirrored height field of the reference's
    CPU-runnable case (128 x 128 grid, 8 bumps mirrored in x, 2,000 samples,
    5% curvature tolerance, bandwidth 0.02): meshes/s of the BF16-refined and
    FP32 forms (host wall clock around synchronous calls, after two warm-up
    runs) and the plane each finds first; then the BF16 form with 5 FP64
    refinement passes (`refine`): its rate and the top plane's distance from
    the exact mirror plane x = 0 before and after."""
    from mitra_algo_gb300.mesh import mirrored_heightfield, prepare
    from mitra_algo_gb300.types import Options, Rng
    mesh = mirrored_heightfield(size=128, bumps=8, seed=0)
    opts = Options(sample_ratio=2000 / mesh.vertex_count, pair_threshold=0.05, bandwidth=0.02,
                   max_pairs=10 ** 7, max_votes=2 * 10 ** 7, max_clusters=8)
    p = prepare(mesh, opts)
    f = gpu.curvature(p.mesh, p.topology, opts)
    sample = gpu.select(p.mesh, f, p.topology.weights, opts, Rng(opts.seed)).sample
    resident = gpu.load_mesh(p)
    out = {"workload": "mirrored height field 128 x 128, reflection mode",
           "vertices": int(mesh.vertex_count), "samples": int(len(sample))}
    for pr in ("bf16", "fp32"):
        kw = dict(precision=pr, seeds=512, max_iterations=100, polish_iterations=POLISH,
                  mode="reflection")
        for _ in range(2):
            r = gpu.detect_fast(resident, sample, opts, **kw)
        t0 = time.perf_counter()
        for _ in range(steps):
            r = gpu.detect_fast(resident, sample, opts, **kw)
        dt = (time.perf_counter() - t0) / steps
        out[pr] = {"meshes_per_s": round(1.0 / dt, 3), "pairs": int(r["pairs"]),
                   "votes": int(r["votes"]),
                   "plane": [round(x, 6) for x in r["plane_normal"][0]] +
                            [round(r["plane_offset"][0], 6)] if r["clusters"] else None,
                   "coverage": round(r["coverage"][0], 4) if r["clusters"] else None}

    def plane_error(r):  # max |n - (+-1, 0, 0)| + |offset| of the top plane
        n = np.asarray(r["plane_normal"][0])
        return float(np.abs(np.abs(n) - np.array([1.0, 0.0, 0.0])).max() + abs(r["plane_offset"][0]))

    kw = dict(precision="bf16", seeds=512, max_iterations=100, polish_iterations=POLISH,
              mode="reflection")
    plain = gpu.detect_fast(resident, sample, opts, **kw)
    for _ in range(2):
        r = gpu.detect_fast(resident, sample, opts, refine=5, **kw)
    t0 = time.perf_counter()
    for _ in range(steps):
        r = gpu.detect_fast(resident, sample, opts, refine=5, **kw)
    dt = (time.perf_counter() - t0) / steps
    if r["clusters"]:
        out["bf16_refined_transforms"] = {
            "refine_passes": 5, "meshes_per_s": round(1.0 / dt, 3),
            "plane_error_before": plane_error(plain), "plane_error_after": plane_error(r),
            "coverage": round(r["coverage"][0], 4)}
    resident.close()
    return out


def batch_bench(gpu, n, workers):
    """Meshes/s of an uneven batch (motif icospheres of 3.5k-54k vertices,
    drawn so that sizes spread over that range, 2-5 fold rotations, noise
    sigma in [0, 5e-3] of the diagonal): sym_detect_fast one mesh after the
    other on one context, against sym_detect_fast_batch with `workers`
    contexts, and the batch again with the FP32 mean shift.  Host wall clock
    around each pass (the calls are synchronous); mesh preparation,
    curvature and sampling are not timed."""
    import torch
    from mitra_algo_gb300.mesh import motif_sphere, prepare
    from mitra_algo_gb300.types import Options, Rng
    rng = np.random.default_rng(2024)
    jobs, sizes = [], []
    for i in range(n):
        u = rng.random()
        level = 4 if u < 0.37 else (5 if u < 0.77 else 6)
        mesh = motif_sphere(level=level, bumps=int(rng.integers(6, 13)),
                            folds=int(rng.integers(2, 6)), partial_shift=float(rng.uniform(0.2, 0.5)),
                            noise=float(rng.uniform(0.0, 5e-3)), seed=100 + i)
        opts = Options(sample_ratio=min(1.0, BATCH_SAMPLES / mesh.vertex_count),
                       pair_threshold=PAIR_THRESHOLD, bandwidth=BANDWIDTH, max_pairs=2 * 10 ** 7,
                       max_votes=5 * 10 ** 7, max_clusters=8)
        p = prepare(mesh, opts)
        f = gpu.curvature(p.mesh, p.topology, opts)
        sample = gpu.select(p.mesh, f, p.topology.weights, opts, Rng(opts.seed)).sample
        jobs.append((gpu.load_mesh(p), sample, opts))
        sizes.append(mesh.vertex_count)
    kw = dict(precision="bf16", seeds=BATCH_SEEDS, max_iterations=100, polish_iterations=POLISH)

    def loop():
        return [gpu.detect_fast(m, s, o, **kw) for m, s, o in jobs]

    def together():
        return gpu.detect_fast_batch(jobs, workers=workers, **kw)

    def together_fp32():
        return gpu.detect_fast_batch(jobs, workers=workers, **dict(kw, precision="fp32"))

    out = {}
    for name, fn in (("per_mesh_loop", loop), ("batched", together),
                     ("batched_fp32", together_fp32)):
        fn()  # warm-up: workspaces reach their size
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        out[name] = (time.perf_counter() - t0, r)
    for m, _, _ in jobs:
        m.close()
    (t_loop, r_loop), (t_batch, r_batch) = out["per_mesh_loop"], out["batched"]
    t_fp32 = out["batched_fp32"][0]
    same = all(a["pairs"] == b["pairs"] and a["modes"] == b["modes"] and
               a["rotation"] == b["rotation"] for a, b in zip(r_loop, r_batch))
    return {"meshes": n, "vertices": [int(min(sizes)), int(max(sizes))],
            "samples_per_mesh": BATCH_SAMPLES, "seeds": BATCH_SEEDS, "workers": workers,
            "per_mesh_loop_meshes_per_s": round(n / t_loop, 3),
            "batched_meshes_per_s": round(n / t_batch, 3),
            "batched_fp32_meshes_per_s": round(n / t_fp32, 3),
            "batched_bf16_over_fp32": round(t_fp32 / t_batch, 3),
            "pairs": int(sum(r["pairs"] for r in r_batch)),
            "results_equal": bool(same), "clock": "host wall clock, synchronous calls"}


def _wall(fn):
    """Host wall-clock seconds of fn() between two device synchronisations,
    and its result."""
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = fn()
    torch.cuda.synchronize()
    return time.perf_counter() - t0, r


def batch_cpu_reference(meshes, results, pair_samples=10 ** 9):
    """The reference's CPU path (the oracle port, bit-exact with the
    reference's CPU library) on a few meshes of a batch, each on one host
    core: reference_sample with `pair_samples` pruned samples paired (scaled
    to all of them by candidate pairs; every sample by default), the clustering's
    cost per seed-vote evaluation taken on 4,000 of the mesh's votes, and
    one verification of the mesh's reported top motion (x max_clusters).
    Returns the per-mesh lower bounds, their mean, and the implied meshes/s
    on one core and on all host cores at once (meshes are independent),
    both upper bounds; the reference stops with "Too many mean-shift modes"
    at MODE_BUDGET trajectories on meshes whose votes need more."""
    from mitra_algo_gb300.mesh import prepare
    from mitra_algo_gb300.types import ClusterOutput, Csr
    per = []
    for (mesh, o), r in zip(meshes, results):
        p = prepare(mesh, o)
        one = ClusterOutput(np.array([int(r["reflection"][0])], np.uint8),
                            np.asarray(r["rotation"][0], float).reshape(1, 9),
                            np.asarray(r["translation"][0], float).reshape(1, 3),
                            np.asarray(r["plane_normal"][0], float).reshape(1, 3),
                            np.array([r["plane_offset"][0]], float),
                            Csr(np.zeros(2, np.uint64), np.zeros(0, np.int32)))
        ref = reference_sample(p, o, pair_samples=pair_samples, cluster=one)
        per.append(ref)
    mean_s = statistics.mean(x["per_mesh_s"] for x in per)
    cores = os.cpu_count() or 1
    return {"kind": "port", "meshes_sampled": len(per), "cores_one_mesh_each": 1,
            "per_mesh_s_lower_bound": [round(x["per_mesh_s"], 2) for x in per],
            "sample_s": round(sum(x["sample_s"] for x in per), 2),
            "meshes_per_s_one_core": round(1 / mean_s, 4),
            "meshes_per_s_all_cores": round(cores / mean_s, 3), "host_cores": cores,
            "mean_shift_s_lower_bound": [round(x["model_s"]["mean_shift_lower_bound"], 2)
                                         for x in per],
            "how": "oracle port of the reference's CPU backend, one core per mesh; "
                   "per-mesh time = measured curvature, selection, pairing and votes + "
                   "MODE_BUDGET trajectories x votes x measured cost per seed-vote "
                   "evaluation + one verification x max_clusters; the mean-shift term is "
                   "the least work before the reference stops with 'Too many mean-shift "
                   "modes', which it reaches whenever its trajectories' windows hold fewer "
                   "than votes / MODE_BUDGET votes each, so the per-mesh time is a lower "
                   "bound and meshes/s an upper bound"}


def c4_leg(gpu, count=256, samples=2000, seeds=256):
    """The uneven batch (mesh.uneven_batch): `count` meshes of
    2k-60k vertices (icospheres, tori, mirrored height fields; 1-4 planted
    symmetries; noise sigma in [0, 5e-3]), each loaded raw through the GPU
    prepare and sampled on the device: meshes/s of sym_detect_fast one mesh
    after the other, against sym_detect_fast_fused (one mean shift for every
    mesh's seeds) in both mean-shift forms.  Host wall clock around each
    pass after a warm-up pass; the loads are not timed."""
    from mitra_algo_gb300.mesh import uneven_batch
    from mitra_algo_gb300.types import Options
    t_gen = time.perf_counter()
    batch = uneven_batch(count)
    jobs, modes, opts = [], [], []
    for mesh, mode, _ in batch:
        o = Options(sample_ratio=min(1.0, samples / mesh.vertex_count),
                    pair_threshold=0.25 if mode == "rigid" else 0.05, bandwidth=BANDWIDTH,
                    max_pairs=10 ** 8, max_votes=2 * 10 ** 9 - 1, max_clusters=8)
        jobs.append((gpu.load_mesh_raw(mesh, o), None, o))
        modes.append(mode)
        opts.append(o)
    t_gen = time.perf_counter() - t_gen
    kw = dict(seeds=seeds, max_iterations=ITERATIONS, polish_iterations=POLISH)

    def loop(pr):
        return [gpu.detect_fast(m, None, o, precision=pr, mode=md, **kw)
                for (m, _, o), md in zip(jobs, modes)]

    def fused(pr):
        return gpu.detect_fast_fused(jobs, precision=pr, mode=modes, **kw)

    fused("bf16")
    t_fb, (rb, stats) = _wall(lambda: fused("bf16"))
    t_ff, (rf, _) = _wall(lambda: fused("fp32"))
    loop("bf16")
    t_lb, rl = _wall(lambda: loop("bf16"))
    for m, _, _ in jobs:
        m.close()

    def found(rs):  # meshes whose top mode is supported by Newton-converged seeds and covers 30%
        return sum(1 for r in rs if r["clusters"] and r["precise"][0] and r["coverage"][0] >= 0.3)
    same = sum(1 for a, b in zip(rl, rb) if a["pairs"] == b["pairs"] and a["votes"] == b["votes"])
    picks = [i for i in (0, count // 3, 2 * count // 3, count - 1) if rl[i]["clusters"]][:4]
    cpu_ref = batch_cpu_reference([(batch[i][0], opts[i]) for i in picks], [rl[i] for i in picks])
    return {"meshes": count, "vertices": [int(min(m.vertex_count for m, _, _ in batch)),
                                          int(max(m.vertex_count for m, _, _ in batch))],
            "samples_per_mesh": samples, "seeds_per_mesh": seeds,
            "per_mesh_loop_meshes_per_s": round(count / t_lb, 2),
            "fused_meshes_per_s": round(count / t_fb, 2),
            "fused_fp32_meshes_per_s": round(count / t_ff, 2),
            "fused_over_loop": round(t_lb / t_fb, 2), "fused_bf16_over_fp32": round(t_ff / t_fb, 2),
            "votes": int(stats["votes"]), "approach_iterations": int(stats["iterations"]),
            "fused_device_ms": {k: round(stats[k], 2) for k in
                                ("votes_ms", "vote_set_ms", "bulk_ms", "polish_ms",
                                 "modes_verification_ms")},
            "same_pairs_and_votes": same, "top_mode_found": {"loop": found(rl), "fused": found(rb)},
            "generate_and_load_s": round(t_gen, 1), "cpu_reference": cpu_ref,
            "clock": "host wall clock, synchronous calls; one warm-up pass"}


def c5_leg(gpu, count=8, samples=10000, seeds=1024, refine=3, reference_seeds=64):
    """The stress batch (mesh.stress_batch): `count` meshes of
    1e5-1e6 triangles, half reflection and half rigid, 30% of each surface
    unsymmetric relief: the full pipeline with verification and `refine`
    FP64 ICP passes, meshes/s one mesh after the other and fused; then, per
    mesh (untimed), the error of every reported motion and refined motion
    against FP64 and of `reference_seeds` seeds' modes, and the outlier
    share 1 - (sum of the reported modes' supports) / votes (a lower bound
    of the share of votes outside every mode's bandwidth: supports may
    overlap)."""
    from mitra_algo_gb300.mesh import stress_batch
    from mitra_algo_gb300.types import Options
    batch = stress_batch(count)
    jobs, modes, opts = [], [], []
    for mesh, mode in batch:
        o = Options(sample_ratio=min(1.0, samples / mesh.vertex_count), pair_threshold=0.05,
                    bandwidth=BANDWIDTH, max_pairs=10 ** 8, max_votes=2 * 10 ** 9 - 1,
                    max_clusters=8)
        jobs.append((gpu.load_mesh_raw(mesh, o), None, o))
        modes.append(mode)
        opts.append(o)
    kw = dict(seeds=seeds, max_iterations=ITERATIONS, polish_iterations=POLISH, refine=refine)
    gpu.detect_fast_fused(jobs, precision="bf16", mode=modes, **kw)
    t_fused, (rf, _) = _wall(lambda: gpu.detect_fast_fused(jobs, precision="bf16", mode=modes, **kw))
    t_loop, rl = _wall(lambda: [gpu.detect_fast(m, None, o, precision="bf16", mode=md, **kw)
                                for (m, _, o), md in zip(jobs, modes)])
    err = [gpu.detect_fast(m, None, o, precision="bf16", mode=md, reference_seeds=reference_seeds,
                           **kw) for (m, _, o), md in zip(jobs, modes)]
    for m, _, _ in jobs:
        m.close()
    precise_err = [x for r in err for x, ok in zip(r["transform_error"], r["precise"]) if ok]
    picks = [i for i in (0, 1) if i < count and rl[i]["clusters"]]
    cpu_ref = batch_cpu_reference([(batch[i][0], opts[i]) for i in picks],
                                  [rl[i] for i in picks], pair_samples=2000)
    outliers = [1 - min(1.0, sum(r["support"]) / max(r["votes"], 1)) for r in rl]
    return {"meshes": count, "triangles": [int(min(m.faces.shape[1] for m, _ in batch)),
                                           int(max(m.faces.shape[1] for m, _ in batch))],
            "modes": modes, "samples_per_mesh": samples, "seeds_per_mesh": seeds,
            "refine_passes": refine,
            "per_mesh_loop_meshes_per_s": round(count / t_loop, 3),
            "fused_meshes_per_s": round(count / t_fused, 3),
            "votes": [int(r["votes"]) for r in rl],
            "outlier_share": [round(x, 3) for x in outliers],
            "error_vs_fp64": {
                "modes_converged_max": max(r["mode_error_max"] for r in err),
                "seeds_compared": int(sum(r["seeds_compared"] for r in err)),
                "seeds_converged_both": int(sum(r["modes_compared"] for r in err)),
                "transform_precise_max": max(precise_err) if precise_err else None,
                "transform_precise_within_1e-4": sum(x <= 1e-4 for x in precise_err),
                "transform_precise_count": len(precise_err),
                "transform_all_max": max(r["transform_error_max"] for r in err),
                "refined_all_max": max(r["transform_error_refined_max"] for r in err)},
            "coverage_top": [round(r["coverage"][0], 3) if r["clusters"] else None for r in rl],
            "cpu_reference": cpu_ref,
            "clock": "host wall clock, synchronous calls; one warm-up pass"}


def c3_leg(gpu, steps=3):
    """The large single mesh (workload "c3"): the torus of 1e6
    triangles with 12 rotated motif copies (2 mirrored), 200,000 samples
    drawn on the device, votes subsampled to 1e6, 4,096 seeds: device time
    per mesh (CUDA events) of both mean-shift forms, and the error of 256
    reference seeds' modes and of the reported motions against FP64."""
    import torch
    from mitra_algo_gb300.mesh import motif_torus
    from mitra_algo_gb300.types import Options
    mesh = motif_torus(R=1.0, r=0.3, nu=1000, nv=500, copies=12, mirrored=2, noise=5e-4, seed=0)
    o = Options(sample_ratio=200_000 / mesh.vertex_count, pair_threshold=0.05, bandwidth=BANDWIDTH,
                max_pairs=10 ** 9, max_votes=2 * 10 ** 9 - 1, max_clusters=20)
    resident = gpu.load_mesh_raw(mesh, o)
    stream = torch.cuda.ExternalStream(gpu.stream_handle)
    out = {"workload": "motif torus 1e6 triangles, 200,000 samples, 1e6 subsampled votes, "
                       "4,096 seeds", "vertices": int(mesh.vertex_count)}
    for pr in ("bf16", "fp32"):
        kw = dict(precision=pr, seeds=4096, max_iterations=ITERATIONS, polish_iterations=POLISH,
                  vote_cap=1_000_000)
        e = gpu.detect_fast(resident, None, o, reference_seeds=256, **kw)
        times = []
        for _ in range(steps + 1):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            r = gpu.detect_fast(resident, None, o, **kw)
            b.record(stream)
            b.synchronize()
            times.append(a.elapsed_time(b))
        ms = statistics.mean(times[1:])
        out[pr] = {"meshes_per_s": round(1000 / ms, 3), "ms_per_step": round(ms, 2),
                   "pairs": int(r["pairs"]), "votes": int(r["votes"]),
                   "stage_ms": {k: round(v, 2) for k, v in r["stage_ms"].items()},
                   "mode_error": {"converged_both": int(e["modes_compared"]),
                                  "max": e["mode_error_max"], "within_1e-4": int(e["modes_within"]),
                                  "all_seeds_within_1e-4": int(e["seeds_within"]),
                                  "reference_seeds": int(e["seeds_compared"])},
                   "transform_error_precise_max": max(
                       [x for x, ok in zip(e["transform_error"], e["precise"]) if ok], default=None)}
    out["bf16_over_fp32"] = round(out["fp32"]["ms_per_step"] / out["bf16"]["ms_per_step"], 3)
    resident.close()
    return out


def workload(small=False, name="c2"):
    """The benchmark mesh and options; `small` is a level-5, 5,000-sample,
    256-seed variant used for profiler captures.  name "c3": the large
    single mesh - a torus (R = 1, r = 0.3) of 1e6 triangles with 12 copies of
    a seeded bump motif placed by rotations about its axis, 2 of them
    mirrored, 200,000 samples, 4,096 seeds and a mean shift over 1e6
    subsampled votes."""
    global SAMPLES, SEEDS, VOTE_CAP, PAIR_THRESHOLD, WORKLOAD
    from mitra_algo_gb300.mesh import motif_sphere, motif_torus, prepare
    from mitra_algo_gb300.types import Options
    if name == "c3":
        SAMPLES, SEEDS, VOTE_CAP, PAIR_THRESHOLD = 200_000, 4096, 1_000_000, 0.05
        WORKLOAD = "motif torus 1e6 triangles, rigid mode, 6-D votes, 1e6 subsampled votes"
        nu, nv = 1000, 500
        if small:  # the same torus and noise at 9e4 triangles, for profiler captures
            SAMPLES, SEEDS, nu, nv = 20_000, 1024, 300, 150
            WORKLOAD = "motif torus 9e4 triangles, rigid mode, 6-D votes, 1e6 subsampled votes"
        mesh = motif_torus(R=1.0, r=0.3, nu=nu, nv=nv, copies=12, mirrored=2, noise=5e-4,
                           seed=0)
        opts = Options(sample_ratio=SAMPLES / mesh.vertex_count, pair_threshold=PAIR_THRESHOLD,
                       bandwidth=BANDWIDTH, max_pairs=10 ** 9, max_votes=2 * 10 ** 9 - 1,
                       max_clusters=20)
        return prepare(mesh, opts), opts
    if small:
        SAMPLES, SEEDS = 5000, 256
    mesh = motif_sphere(level=5 if small else 6, bumps=12, folds=5, partial_shift=0.4,
                        noise=1e-3, seed=0)
    opts = Options(sample_ratio=SAMPLES / mesh.vertex_count, pair_threshold=PAIR_THRESHOLD,
                   bandwidth=BANDWIDTH, max_pairs=2 * 10 ** 7, max_votes=5 * 10 ** 7,
                   max_clusters=20)
    return prepare(mesh, opts), opts


def config(prepared, r=None):
    c = {"workload": WORKLOAD,
         "vertices": prepared.mesh.vertex_count, "faces": int(prepared.mesh.faces.shape[1]),
         "samples": SAMPLES, "pair_threshold": PAIR_THRESHOLD, "bandwidth": BANDWIDTH,
         "seeds": SEEDS, "l2": "flushed (256 MiB write) before every timed step"}
    if r:
        c.update({"pruned": int(r["pruned"]), "pairs": int(r["pairs"]), "votes": int(r["votes"])})
    if VOTE_CAP:
        c["vote_cap"] = VOTE_CAP
    return c


class Clocks:
    """nvidia-smi clock/throttle sampling during the timed region."""

    def __init__(self, path):
        self.path = path
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self, device=0):
        rows = []
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9 and f[0] == str(device):
                    rows.append(f)
        except OSError:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": float(rows[0][2]) if rows[0][2].replace(".", "").isdigit() else None,
                "reasons": reasons, "samples": len(rows)}


def peaks():
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text()), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


# ------------------------------------------------------------- CPU baseline
MODE_BUDGET = 20000  # the reference's mode budget (src/cpu/clustering.cpp:90-95)


def reference_sample(prepared, opts, seed=0, pair_samples=2000, cluster_votes=4000, cluster=None):
    """One bounded sample of the reference's CPU path on this workload,
    timed on one host core with the oracle (the CPU restatement of the
    reference's backend, bit-exact with it): curvature and selection of the
    full mesh, pairing of `pair_samples` pruned samples drawn with `seed`,
    the votes of those pairs, a reference clustering of `cluster_votes` of
    those votes (its cost per seed-vote evaluation), and the verification of
    one cluster (`cluster`, a ClusterOutput of one record; by default the
    motif sphere's planted 5-fold rotation).  Returns the measured times,
    the counts, and the per-mesh time they imply by the reference's own
    work: pairing and votes scale with the candidate pairs (S (S - 1) / 2)
    and the pairs; the mean shift runs at least MODE_BUDGET trajectories of
    at least one iteration over every vote before the reference gives up
    ("Too many mean-shift modes"), a lower bound; verification scales with
    max_clusters."""
    from mitra_algo_gb300.types import Votes
    from oracle import oracle
    cpu = oracle.OracleBackend()
    p, o = prepared, opts
    t = {}
    t0 = time.perf_counter()
    f = cpu.curvature(p.mesh, p.topology, o)
    t["curvature"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    sel = cpu.select(p.mesh, f, p.topology.weights, o, oracle.rng(o.seed))
    t["select"] = time.perf_counter() - t0
    pruned = np.asarray(sel.pruned)
    S = pruned.size
    g = np.random.default_rng(seed)
    sub = np.sort(g.choice(pruned, min(pair_samples, S), replace=False)).astype(np.int32)
    t0 = time.perf_counter()
    pairs = cpu.pairing(p.mesh, f, sub, p.context, o.with_(max_pairs=10 ** 9))
    t_pair = time.perf_counter() - t0
    t0 = time.perf_counter()
    votes = cpu.transformations(p.mesh, f, pairs, p.context, o.with_(max_votes=10 ** 9))
    t_vote = time.perf_counter() - t0
    q = min(len(votes), cluster_votes)
    vs = Votes(votes.pair[:q], votes.kind[:q], votes.rotation[:, :q], votes.translation[:, :q],
               votes.plane_normal[:, :q], votes.plane_offset[:q], votes.descriptor[:, :q])
    t0 = time.perf_counter()
    cpu.clustering(vs, p.context, o, oracle.rng(o.seed))
    t_ms = time.perf_counter() - t0
    _, evals = cpu.clustering_stats()
    from mitra_algo_gb300.types import ClusterOutput, Csr
    c = np.asarray(p.context.center)
    R = np.array([[np.cos(0.4 * np.pi), -np.sin(0.4 * np.pi), 0],
                  [np.sin(0.4 * np.pi), np.cos(0.4 * np.pi), 0], [0, 0, 1]])
    one = cluster if cluster is not None else ClusterOutput(
        np.zeros(1, np.uint8), R.reshape(1, 9), (c - R @ c).reshape(1, 3), np.zeros((1, 3)),
        np.zeros(1), Csr(np.zeros(2, np.uint64), np.zeros(0, np.int32)))
    t0 = time.perf_counter()
    cpu.verification(p.mesh, p.topology, one, p.context, o)
    t_ver = time.perf_counter() - t0
    s_sub = sub.size
    cand = S * (S - 1) / 2
    scale = cand / max(s_sub * (s_sub - 1) / 2, 1)
    pairs_est = len(pairs) * scale
    votes_est = len(votes) * scale
    per_eval = t_ms / max(evals, 1)
    model = {"curvature": t["curvature"], "select": t["select"], "pairing": t_pair * scale,
             "transformations": t_vote * scale,
             "mean_shift_lower_bound": MODE_BUDGET * votes_est * per_eval,
             "verification": t_ver * o.max_clusters}
    return {"measured_s": {"curvature": t["curvature"], "select": t["select"], "pairing": t_pair,
                           "transformations": t_vote, "clustering": t_ms, "verification": t_ver},
            "counts": {"pruned": int(S), "pair_samples": int(s_sub), "pairs": int(len(pairs)),
                       "votes": int(len(votes)), "cluster_votes": int(q),
                       "evaluations": int(evals), "pairs_est": pairs_est, "votes_est": votes_est},
            "per_mesh_s": sum(model.values()), "model_s": model,
            "sample_s": sum([t["curvature"], t["select"], t_pair, t_vote, t_ms, t_ver])}


def reference_description(r):
    c = r["counts"]
    return (f"oracle port of the reference's CPU path on one core: curvature and selection of "
            f"the full mesh, pairing of {c['pair_samples']} of {c['pruned']} pruned samples "
            f"(x S(S-1)/s(s-1) for all {c['pruned']}), their {c['votes']} votes (same scale), a "
            f"{c['cluster_votes']}-vote reference clustering (cost per seed-vote evaluation) x "
            f"{MODE_BUDGET} trajectories x one iteration over the {c['votes_est']:.3g} votes "
            f"(the least the reference runs before it stops with 'Too many mean-shift modes', "
            f"src/cpu/clustering.cpp:90-95), and the verification of one cluster x max_clusters; "
            f"per-mesh time is a lower bound, so meshes/s is an upper bound")


def cpu_baseline(prepared, opts):
    """The `cpu_baseline` object: one reference_sample on one core."""
    r = reference_sample(prepared, opts)
    return {"value": round(1.0 / r["per_mesh_s"], 10), "unit": "meshes/s", "cores": 1,
            "kind": "port", "sample": reference_description(r),
            "sample_seconds": round(r["sample_s"], 2), "reference_aborts": True,
            "stage_s": {k: round(v, 4) for k, v in r["model_s"].items()}}


def c1_exact(gpu, steps=3):
    """The reference's CPU-runnable case (mirrored height field, 128 x 128
    grid, 8 bumps mirrored in x, 2,000 samples, 5% curvature tolerance,
    bandwidth 0.02, reflection votes included) through the bit-exact stage
    path: detect() with the GB300 backend (the six stage calls of the C ABI
    from host buffers) against detect() with the oracle port of the
    reference's CPU backend on the same inputs, both measured end to end
    (wall clock, synchronous calls, host prepare included on both sides),
    and their results compared."""
    from mitra_algo_gb300.backend import detect
    from mitra_algo_gb300.mesh import mirrored_heightfield, prepare
    from mitra_algo_gb300.types import Options
    from oracle import oracle
    mesh = mirrored_heightfield(size=128, bumps=8, seed=0)
    o = Options(sample_ratio=2000 / mesh.vertex_count, pair_threshold=0.05, bandwidth=0.02)
    detect(mesh, o, gpu)  # warm-up: workspaces reach their size
    t0 = time.perf_counter()
    runs = [detect(mesh, o, gpu) for _ in range(steps)]
    t_gpu = (time.perf_counter() - t0) / steps
    g = runs[-1]
    t0 = time.perf_counter()
    c = detect(mesh, o, oracle.OracleBackend())
    t_cpu = time.perf_counter() - t0

    def stages_s(result):  # the six stages, without the host prepare
        return sum(v for k, v in result.timings if k != "prepare") / 1e3
    s_gpu = statistics.mean(stages_s(x) for x in runs)
    s_cpu = stages_s(c)
    parity = c1_parity(g, c)
    # the verification alone on the same motions (the CPU run's clusters)
    p = prepare(mesh, o)
    v_same = gpu.verification(p.mesh, p.topology, c.clusters, p.context, o)
    parity["verification_on_cpu_clusters"] = bool(
        all(np.array_equal(getattr(v_same, k).indices, getattr(c.verification, k).indices)
            for k in ("side_a", "side_b", "patches_a", "patches_b"))
        and np.array_equal(v_same.coverage, c.verification.coverage)
        and np.allclose(v_same.rms, c.verification.rms, rtol=1e-12, atol=0))
    parity["verification_end_to_end_differing_vertices"] = differing_sides(g.verification,
                                                                         c.verification)
    return {"workload": "mirrored height field 128 x 128, 2,000 samples, reflection and rigid "
                        "votes, the reference's options otherwise (its CPU-runnable case)",
            "gpu_meshes_per_s": round(1.0 / t_gpu, 3), "cpu_meshes_per_s": round(1.0 / t_cpu, 4),
            "gpu_over_cpu": round(t_cpu / t_gpu, 1),
            "stages_gpu_over_cpu": round(s_cpu / s_gpu, 1), "parity": parity,
            "pairs": int(len(c.pairs)), "votes": int(len(c.votes)),
            "clusters": int(len(c.clusters.reflection)),
            "gpu_stage_ms": {k: round(v, 2) for k, v in g.timings},
            "cpu_stage_ms": {k: round(v, 1) for k, v in c.timings},
            "cpu": "oracle port of the reference's CPU backend, one core",
            "clock": "host wall clock around detect(); GPU: mean of 3 after one warm-up"}


def differing_sides(a, b):
    """Number of (cluster, side, vertex) memberships in one verification's
    side lists but not the other's."""
    n = 0
    for side in ("side_a", "side_b"):
        x, y = getattr(a, side), getattr(b, side)
        for c in range(len(x.offsets) - 1):
            r1 = set(x.indices[x.offsets[c]:x.offsets[c + 1]].tolist())
            r2 = set(y.indices[y.offsets[c]:y.offsets[c + 1]].tolist())
            n += len(r1 ^ r2)
    return n


def c1_parity(g, c):
    """How the GPU's detect() result `g` compares with the CPU port's `c`:
    every id (pairs, vote pairs and kinds, cluster memberships, supporting
    vertices, patches) must be equal; FP64 values (features, vote
    descriptors, cluster motions, coverage, rms) are within the reference's
    own CPU/GPU bound 2e-10 (1 + |cpu|) (tests/compare_cuda.py:20-21) -- the
    GPU's curvature rounds its transcendentals differently in the last
    bits, which every later FP64 value inherits."""
    def ids(*pairs):
        return all(np.array_equal(np.asarray(a), np.asarray(b)) for a, b in pairs)

    def fp_excess(*pairs):  # largest |gpu - cpu| / (2e-10 (1 + |cpu|)); <= 1 passes
        worst = 0.0
        for a, b in pairs:
            a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
            if a.shape != b.shape:
                return float("inf")
            if a.size:
                worst = max(worst, float(np.max(np.abs(a - b) / (2e-10 * (1 + np.abs(b))))))
        return worst
    gv, cv = g.verification, c.verification
    # verification's ids follow the motions it is given, which differ in the
    # last bits: exact equality is checked on identical motions (the caller)
    out = {
        "features": fp_excess((g.features.kmin, c.features.kmin), (g.features.kmax, c.features.kmax),
                              (g.features.normal, c.features.normal)) <= 1 and
        ids((g.features.valid, c.features.valid)),
        "pairs": ids((g.pairs.a, c.pairs.a), (g.pairs.b, c.pairs.b)),
        "votes": ids((g.votes.pair, c.votes.pair), (g.votes.kind, c.votes.kind)) and
        fp_excess((g.votes.descriptor, c.votes.descriptor), (g.votes.rotation, c.votes.rotation),
                  (g.votes.translation, c.votes.translation)) <= 1,
        "clusters": ids((g.clusters.votes.offsets, c.clusters.votes.offsets),
                        (g.clusters.votes.indices, c.clusters.votes.indices)) and
        fp_excess((g.clusters.rotation, c.clusters.rotation),
                  (g.clusters.translation, c.clusters.translation)) <= 1,
        "verification": ids((gv.side_a.indices, cv.side_a.indices),
                            (gv.side_b.indices, cv.side_b.indices),
                            (gv.patches_a.indices, cv.patches_a.indices),
                            (gv.patches_b.indices, cv.patches_b.indices)) and
        fp_excess((gv.coverage, cv.coverage), (gv.rms, cv.rms)) <= 1}
    out["all"] = all(out.values())
    out["rule"] = "ids equal; FP64 values within 2e-10 (1 + |cpu|)"
    return out


def stage_rooflines(prepared, opts, r, peak_gbs):
    """Each pipeline stage's device time (CUDA events) against the
    algorithmic bytes of the stage: curvature V(12+45) + 12F + 16E + s(72V +
    8E); pairing and votes 84S + 8P + 32Q (the 6-D FP32 records); vote sort
    2 x 32Q (read and write of the records); verification 2CV x 25 + 24V +
    12F + 32 N (queries, mesh, LBVH nodes)."""
    V = prepared.mesh.vertex_count
    F = int(prepared.mesh.faces.shape[1])
    E = int(np.asarray(prepared.topology.edges).reshape(-1, 6).shape[0])
    sm = opts.smoothing
    S, P, Q, C = r["pruned"], r["pairs"], r["votes"], r["clusters"]
    bytes_ = {"curvature": V * 57 + 12 * F + 16 * E + sm * (72 * V + 8 * E),
              "pairing": 84 * S + 8 * P, "votes": 32 * Q, "vote_sort": 64 * Q,
              "verification": 2 * C * V * 25 + 24 * V + 12 * F + 32 * max(F - 1, 0)}
    out = {}
    for k, b in bytes_.items():
        ms = r["stage_ms"][k]
        gbs = b / (ms * 1e-3) / 1e9 if ms > 0 else 0.0
        out[k] = {"ms": round(ms, 3), "bytes": int(b), "gbs": round(gbs, 1),
                  "frac": round(gbs / peak_gbs, 5)}
    return out


def ctypes_sizeof_result():
    import ctypes
    from mitra_algo_gb300 import abi
    return ctypes.sizeof(abi.FastResult)


# ----------------------------------------------------------- multi-rank
def max_over_ranks(values, device, world):
    """The slowest rank's value of each entry (ranks time their replica of
    the workload; the job takes as long as its slowest rank): an all-reduce
    MAX when more than one rank runs.  No data moves between ranks - every
    rank detects on its own copy of the mesh (replicas only)."""
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return t.tolist()


def job_rate(ms_per_step, world):
    """Whole-job meshes/s: every rank finishes one mesh per step."""
    return world * 1000.0 / ms_per_step


# --------------------------------------------------------------- GPU arm
def run_gpu(args):
    import torch
    from mitra_algo_gb300 import Gb300Backend
    from mitra_algo_gb300.types import Rng

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    prepared, opts = workload(args.small, args.config)
    gpu = Gb300Backend(local)
    stream = torch.cuda.ExternalStream(gpu.stream_handle, device=torch.device("cuda", local))
    # sample: the reference's host RNG sampling (the input of the path)
    feats = gpu.curvature(prepared.mesh, prepared.topology, opts)
    sel = gpu.select(prepared.mesh, feats, prepared.topology.weights, opts, Rng(opts.seed))
    sample = sel.sample
    resident = gpu.load_mesh(prepared)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    # launch shapes of both forms chosen by the autotuner on this workload
    # before anything is timed (the profiler captures use the defaults)
    tuned, tune_s = {}, 0.0
    if not args.once and not args.no_tune:
        from mitra_algo_gb300.autotune import autotune
        t0 = time.perf_counter()
        for p in ("bf16", "fp32"):
            tuned[p] = autotune(gpu, resident, sample, opts, precision=p, seeds=SEEDS,
                                max_iterations=ITERATIONS, polish_iterations=POLISH,
                                vote_cap=VOTE_CAP)
        tune_s = time.perf_counter() - t0

    def shape(precision):
        return tuned[precision]["tuning"] if precision in tuned else None

    def step(precision, reference_seeds=0, refine=0):
        return gpu.detect_fast(resident, sample, opts, precision=precision, seeds=SEEDS,
                               max_iterations=ITERATIONS, polish_iterations=POLISH,
                               reference_seeds=reference_seeds, vote_cap=VOTE_CAP,
                               tuning=shape(precision), refine=refine)

    if args.once:  # one warm-up and one measured pipeline run (profiler captures)
        def step(precision, reference_seeds=0):  # noqa: F811 - the --kernel choice applies here
            return gpu.detect_fast(resident, sample, opts, precision=precision, seeds=SEEDS,
                                   max_iterations=ITERATIONS, polish_iterations=POLISH,
                                   vote_cap=VOTE_CAP, kernel=args.kernel)
        step(args.once)
        r = step(args.once)
        print(json.dumps({"precision": args.once, "stage_ms": r["stage_ms"], "pairs": r["pairs"],
                          "votes": r["votes"], "iterations": r["iterations"],
                          "polish_iterations": r["polish_iterations"], "bulk_ms": r["bulk_ms"],
                          "polish_ms": r["polish_ms"], "evaluations": r["mean_shift_pairs"],
                          "seed_iterations": r["seed_iterations"], "launches": r["launches"],
                          "verify_undecided": r["verify_undecided"],
                          "verify_fp64_rows": r["verify_fp64_rows"], "coverage": r["coverage"],
                          "bulk_trace": list(r["bulk_trace"]),
                          "polish_trace": list(r["polish_trace"])}))
        return

    def timed(precision, steps, warmup):
        for _ in range(warmup):
            step(precision)
        total_ms, results = 0.0, []
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.random_(0, 255)
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
            results.append(step(precision))
            with torch.cuda.stream(stream):
                b.record(stream)
            b.synchronize()
            total_ms += a.elapsed_time(b)
        return total_ms / steps, results

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    # correctness / error run (untimed): FP64 re-run of 256 seeds, FP64
    # restarts of the reported modes, and the same 2 refinement passes of
    # the GPU's and the FP64 motions
    err = {p: step(p, reference_seeds=256, refine=2) for p in ("bf16", "fp32")}
    barrier()
    with Clocks(os.path.join(tempfile.gettempdir(), f"bench_clocks_{os.getpid()}.csv")) as clk:
        ms_bf16, res_bf16 = timed("bf16", args.steps, args.warmup)
        barrier()
        ms_fp32, res_fp32 = timed("fp32", args.steps, max(1, args.warmup // 2))
        barrier()
    clocks = clk.summary(local)
    # e2e: the raw mesh (vertices and faces) in pinned host buffers -> the
    # public ABI (sym_mesh_load_raw: GPU prepare + resident load, then
    # sym_detect_fast_sampled: GPU sampling + the path) -> the result read
    # back, every step
    from mitra_algo_gb300.types import Mesh
    pv = torch.from_numpy(np.ascontiguousarray(prepared.mesh.vertices)).pin_memory().numpy()
    pf = torch.from_numpy(np.ascontiguousarray(prepared.mesh.faces)).pin_memory().numpy()
    raw = Mesh(pv, pf)
    assert raw.vertices.ctypes.data == pv.ctypes.data  # still the pinned buffer
    e2e_ms = []
    h2d = d2h = 0
    for i in range(args.warmup + args.steps):
        barrier()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        mesh_i = gpu.load_mesh_raw(raw, opts)
        r = gpu.detect_fast(mesh_i, None, opts, precision="bf16", seeds=SEEDS,
                            max_iterations=ITERATIONS, polish_iterations=POLISH,
                            vote_cap=VOTE_CAP, tuning=shape("bf16"))
        b.record(stream)
        b.synchronize()
        mesh_i.close()
        assert r["sampled"] == len(sample)  # the host-drawn sample of the other legs
        if i >= args.warmup:
            e2e_ms.append(a.elapsed_time(b))
            h2d = mesh_i.bytes() + r["h2d_bytes"]
            d2h = r["d2h_bytes"] + ctypes_sizeof_result()
    barrier()
    ms_bf16, ms_fp32, ms_e2e = max_over_ranks([ms_bf16, ms_fp32, statistics.mean(e2e_ms)],
                                              f"cuda:{local}", world)
    extra = args.config == "c2"
    batch = batch_bench(gpu, args.batch, args.batch_workers) if args.batch and extra else None
    refl = reflection_bench(gpu) if extra else None

    def gaussian_leg(steps=3):
        """The same workload with the shifted Gaussian kernel (exp weights,
        MUFU BF16x2 exponentials in the tensor kernel): both forms' device
        time per mesh (CUDA events, like the main legs) and mode error."""
        out = {"kernel": "2^(-8 d^2/h^2) - 2^-8 for d < h"}
        for p in ("bf16", "fp32"):
            kw = dict(precision=p, seeds=SEEDS, max_iterations=ITERATIONS,
                      polish_iterations=POLISH, vote_cap=VOTE_CAP, tuning=shape(p),
                      kernel="gaussian")
            e = gpu.detect_fast(resident, sample, opts, reference_seeds=256, **kw)
            t = []
            for _ in range(steps):
                with torch.cuda.stream(stream):
                    flush.random_(0, 255)
                    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    a.record(stream)
                gpu.detect_fast(resident, sample, opts, **kw)
                with torch.cuda.stream(stream):
                    b.record(stream)
                b.synchronize()
                t.append(a.elapsed_time(b))
            ms = statistics.mean(t)
            out[p] = {"meshes_per_s": round(1000.0 / ms, 4), "ms_per_step": round(ms, 3),
                      "mode_error_max": e["mode_error_max"], "compared": int(e["modes_compared"]),
                      "within_1e-4": int(e["modes_within"])}
        out["bf16_over_fp32"] = round(out["fp32"]["ms_per_step"] / out["bf16"]["ms_per_step"], 3)
        return out

    gauss = gaussian_leg() if extra else None
    c1 = c1_exact(gpu) if extra else None
    c3 = c3_leg(gpu) if extra and args.c3 else None
    c4 = c4_leg(gpu, args.c4_meshes) if extra and args.c4_meshes else None
    c5 = c5_leg(gpu, args.c5_meshes) if extra and args.c5_meshes else None
    if rank != 0:
        return
    r = res_bf16[-1]
    meshes = job_rate(ms_bf16, world)
    votes_per_s = world * r["votes"] * 1000.0 / ms_bf16
    pk, pk_kind = peaks()
    evals = statistics.mean(x["mean_shift_pairs"] for x in res_bf16)
    # roofline of the dominant kernel (ms_tile_tc): its launches timed with
    # CUDA events on the library's stream inside the timed steps
    tc_launches = sum(x["tc_launches"] for x in res_bf16)
    tc_ms = sum(x["tc_kernel_ms"] for x in res_bf16)
    tc_evals = sum(x["tc_evaluations"] for x in res_bf16)
    per_launch_ms = tc_ms / max(tc_launches, 1)
    flops_per_launch = tc_evals * 64 / max(tc_launches, 1)
    achieved = flops_per_launch / (per_launch_ms * 1e-3) / 1e12 if tc_ms else 0.0
    chunk_pairs_per_launch = tc_evals / (128 * 128) / max(tc_launches, 1)
    gbs = IMAGE_BYTES * chunk_pairs_per_launch / (per_launch_ms * 1e-3) / 1e9 if tc_ms else 0.0
    line = {
        "metric": METRIC, "value": round(meshes, 4), "unit": "meshes/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_bf16, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded motif icosphere, generated in-process)",
        "config": config(prepared, r),
        "pair_votes_per_s": round(votes_per_s, 1),
        "fp32": {"meshes_per_s": round(job_rate(ms_fp32, world), 4), "ms_per_step": round(ms_fp32, 3)},
        "bf16_over_fp32": round(ms_fp32 / ms_bf16, 3),
        "mode_error": {pr: {"reference_seeds": e["seeds_compared"],
                            "all": {"max": e["mode_error_all_max"],
                                    "mean": e["mode_error_all_mean"],
                                    "within_1e-4": e["seeds_within"]},
                            "converged_both": {"seeds": e["modes_compared"],
                                               "max": e["mode_error_max"],
                                               "mean": e["mode_error_mean"],
                                               "within_1e-4": e["modes_within"]},
                            "settled_on_ridge": {"seeds": e["seeds_settled"],
                                                 "max": e["mode_error_settled_max"]},
                            "unconverged": {"seeds": e["seeds_unconverged"],
                                            "max": e["mode_error_unconverged_max"]}}
                       for pr, e in err.items()},
        "transform_error": {pr: {"max": e["transform_error_max"],
                                 "per_mode": [round(x, 9) for x in e["transform_error"]],
                                 "precise": e["precise"],
                                 "refined_max": e["transform_error_refined_max"],
                                 "refine_passes": 2,
                                 "how": "each reported mode's motion [R, t/box] against the FP64 "
                                        "mode the FP64 mean shift reaches from the same "
                                        "position; refined: 2 FP64 ICP passes of both"}
                            for pr, e in err.items()},
        "mean_shift": {pr: {"approach_iterations": x["iterations"],
                            "approach_ms": round(x["bulk_ms"], 3),
                            "polish_iterations": x["polish_iterations"],
                            "polish_ms": round(x["polish_ms"], 3),
                            "approach_trace": x["bulk_trace"][::10],
                            "polish_trace": x["polish_trace"][::3]}
                       for pr, x in (("bf16", r), ("fp32", res_fp32[-1]))},
        "modes": r["modes"], "evaluations": evals,
        "stage_ms": {k: round(statistics.mean(x["stage_ms"][k] for x in res_bf16), 3)
                     for k in r["stage_ms"]},
        "stages": stage_rooflines(prepared, opts, {**r, "stage_ms": {
            k: statistics.mean(x["stage_ms"][k] for x in res_bf16) for k in r["stage_ms"]}},
            pk["hbm_gbs"]),
        "verification_path": {"fp64_rows": r["verify_fp64_rows"],
                              "reference_order_rows": r["verify_undecided"],
                              "queries": 2 * r["clusters"] * prepared.mesh.vertex_count},
        "e2e": {"value": round(job_rate(ms_e2e, world), 4), "unit": "meshes/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "path": "raw vertices and faces in pinned host memory -> sym_mesh_load_raw "
                        "(GPU prepare, resident mesh) -> sym_detect_fast_sampled (GPU "
                        "sampling from the seed, then the whole path) -> result on the host"},
        "roofline": {"kernel": "ms_tile_tc (BF16 tcgen05 mean-shift tile)", "bound": "hbm",
                     "achieved": round(gbs, 1), "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": round(gbs / pk["hbm_gbs"], 4),
                     "traffic": round(TRAFFIC_PER_CHUNK_PAIR * chunk_pairs_per_launch),
                     "peak_source": pk_kind,
                     "launches": tc_launches, "ms_per_launch": round(per_launch_ms, 4),
                     "chunk_pairs_per_launch": round(chunk_pairs_per_launch, 1),
                     "tensor": {"achieved": round(achieved, 3), "unit": "TFLOP/s",
                                "peak": pk["bf16_tflops_sustained"],
                                "frac": round(achieved / pk["bf16_tflops_sustained"], 5)},
                     "note": "the kernel streams one 8,224-byte chunk image per (tile of 128 "
                             "seeds, chunk of 128 votes) pair and makes 64 MMA FLOPs per seed-vote "
                             "evaluation: 127 FLOP/B, below the GB300 ridge (sustained BF16 / HBM "
                             "= 255 FLOP/B), so HBM bounds it. achieved = 8,224 B x pairs per "
                             "launch / CUDA-event time per launch; tensor.achieved = 64 x "
                             "evaluations per launch / the same time; traffic = DRAM bytes per "
                             "pair from the ncu capture in profiles/ms_tile_tc.md x pairs per "
                             "launch"},
        "clocks": clocks,
        "tuning": {**{p: {"shape": t["tuning"], "ms": round(t["ms"], 2),
                          "default_ms": round(t["default_ms"], 2)} for p, t in tuned.items()},
                   "seconds": round(tune_s, 1),
                   "how": "autotuner (coordinate descent over launch shapes, whole-pipeline "
                          "device time, 2% margin) run on this workload before timing"},
        "gpu_launches": int(sum(x["launches"] for x in res_bf16)),
    }
    if batch:
        line["batch"] = batch
    if refl:
        line["reflection"] = refl
    if gauss:
        line["gaussian_kernel"] = gauss
    if extra:
        line["c1_exact"] = c1
    for name, leg in (("c3", c3), ("c4", c4), ("c5", c5)):
        if leg:
            line[name] = leg
    if not args.no_cpu and extra:
        line["cpu_baseline"] = cpu_baseline(prepared, opts)
    print(json.dumps(line))


_WORKER = {}


def _reference_init(small):
    """Worker process set-up (spawned: no GPU state): the workload, once."""
    _WORKER["w"] = workload(small, "c2")


def _reference_worker(seed):
    """One reference_sample in a worker process."""
    prepared, opts = _WORKER["w"]
    return reference_sample(prepared, opts, seed=seed)


def run_reference(args):
    """The reference arm: the reference's CPU path (the oracle port; the
    reference's own build is x86-only here) on bounded samples of this
    workload, on every host core at once (one sample per core and step, each
    core a separate process, as meshes are independent).  ms_per_step is the
    measured wall time of a step; the meshes/s value is cores / (per-mesh
    time the samples imply), an upper bound because the reference stops
    with 'Too many mean-shift modes' before it finishes this mesh."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import multiprocessing as mp
    prepared, opts = workload(args.small)
    cores = max(1, min(os.cpu_count() or 1, 16))
    ctx = mp.get_context("spawn")
    walls, samples = [], []
    with ctx.Pool(cores, initializer=_reference_init, initargs=(args.small,)) as pool:
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            got = pool.map(_reference_worker, [1000 * i + c for c in range(cores)])
            if i >= args.warmup:
                walls.append(time.perf_counter() - t0)
                samples += got
    per_mesh = statistics.mean(x["per_mesh_s"] for x in samples)
    value = cores / per_mesh
    line = {"metric": METRIC, "value": round(value, 10), "unit": "meshes/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1e3 * statistics.mean(walls), 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded motif icosphere)", "config": config(prepared),
            "impl": "reference", "reference_aborts": True,
            "cpu_baseline": {"value": round(value, 10), "unit": "meshes/s", "cores": cores,
                             "kind": "port", "sample": reference_description(samples[0]) +
                             f"; {cores} such samples per step, one per core"},
            "per_mesh_s": {k: round(statistics.mean(x["model_s"][k] for x in samples), 3)
                           for k in samples[0]["model_s"]},
            "measured_sample_s": {k: round(statistics.mean(x["measured_s"][k] for x in samples), 4)
                                  for k in samples[0]["measured_s"]},
            "e2e": {"value": round(value, 10), "unit": "meshes/s",
                    "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline estimate")
    ap.add_argument("--no-tune", action="store_true",
                    help="default launch shapes instead of the autotuner's")
    ap.add_argument("--config", choices=["c2", "c3"], default="c2",
                    help="c2: the motif icosphere (default); c3: the 1e6-triangle torus "
                         "(no batch, reflection or CPU legs)")
    ap.add_argument("--c3", type=int, default=1, help="1: include the large-torus leg (the line's c3 field)")
    ap.add_argument("--c4-meshes", type=int, default=256,
                    help="meshes of the uneven batch leg (the c4 field; 0: skip)")
    ap.add_argument("--c5-meshes", type=int, default=8,
                    help="meshes of the stress batch leg (the c5 field; full size 64; 0: skip)")
    ap.add_argument("--batch", type=int, default=48,
                    help="meshes of the uneven batch measurement (0: skip)")
    ap.add_argument("--batch-workers", type=int, default=4,
                    help="worker contexts of sym_detect_fast_batch")
    ap.add_argument("--bandwidth", type=float, default=None, help="override the bandwidth")
    ap.add_argument("--once", choices=["bf16", "fp32"], default=None,
                    help="run the pipeline once after one warm-up run and print its stages")
    ap.add_argument("--kernel", choices=["epanechnikov", "gaussian"], default="epanechnikov",
                    help="weight kernel of the --once runs (profiler captures)")
    ap.add_argument("--small", action="store_true",
                    help="level-5 mesh, 5,000 samples, 256 seeds; with --config c3 a 9e4-triangle "
                         "torus, 20,000 samples, 1,024 seeds (profiler captures)")
    args = ap.parse_args()
    if args.bandwidth:
        global BANDWIDTH
        BANDWIDTH = args.bandwidth
    args.warmup = max(args.warmup, 3) if args.impl == "gb300" else args.warmup
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
