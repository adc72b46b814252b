"""In-tree build of the CUDA library (sm_103a) with nvcc.

Each translation unit under csrc/ is compiled in parallel to an object file
and linked into mitra_algo_gb300/_lib/libmitra_gb300.so.  Units of the exact
(parity) path are compiled with --fmad=false and the host compiler without
FMA contraction, so FP64 expressions round exactly like the reference's x86
build; throughput units keep FMA contraction.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "csrc"
OUT = HERE / "_lib"
OBJ = OUT / "obj"
LIB = OUT / "libmitra_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Translation units that keep FMA contraction (throughput kernels that are
# not required to round like the reference's FP64 CPU code).
FAST_UNITS = {"resident.cu", "meanshift_fast.cu", "meanshift_tc.cu"}


def nvcc() -> str:
    for cand in [os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]:
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _flags(unit: str, verbose: bool):
    exact = unit not in FAST_UNITS
    f = ["-O3", "-std=c++17", *ARCH, "-lineinfo", "-Xcompiler",
         "-fPIC,-ffp-contract=off" if exact else "-fPIC"]
    f.append("--fmad=false" if exact else "--fmad=true")
    if verbose:
        f += ["-Xptxas", "-v"]
    return f


def _stale(src: Path, obj: Path) -> bool:
    if not obj.exists():
        return True
    deps = [src, *SRC.glob("*.cuh"), *SRC.glob("*.hpp"), HERE.parent / "include" / "mitra_gb300.h"]
    return any(d.stat().st_mtime > obj.stat().st_mtime for d in deps)


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> Path:
    OBJ.mkdir(parents=True, exist_ok=True)
    units = sorted(SRC.glob("*.cu"))
    cc = nvcc()

    def compile_one(src: Path):
        obj = OBJ / (src.stem + ".o")
        if not force and not _stale(src, obj):
            return obj, ""
        cmd = [cc, *_flags(src.name, verbose), "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stderr}")
        return obj, r.stderr

    with ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as pool:
        results = list(pool.map(compile_one, units))
    if verbose:
        for _, log in results:
            if log:
                print(log, file=sys.stderr)
    objs = [str(o) for o, _ in results]
    if force or not LIB.exists() or any(Path(o).stat().st_mtime > LIB.stat().st_mtime for o in objs):
        cmd = [cc, "-shared", *ARCH, "-o", str(LIB), *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
