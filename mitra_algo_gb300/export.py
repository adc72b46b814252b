"""Binary result tables (sym_export_tables) and their rendering as the
reference's text files.

The reference writes its results as text with 17 significant digits
(export_result, src/io/export.cpp:37-98); at 1e7 votes that writer is the
slowest part of a parity run.  ``export_tables`` writes the same tables as
binary column files (the bits of every double kept), ``read_table`` maps one
back as numpy arrays, and ``render_text`` turns a directory of tables into
features.csv, pairs.csv, votes.csv, descriptors.csv and mesh.off exactly as
the reference writes them (``%.17g`` is what ``std::setprecision(17)``
prints in the default float format), for harnesses that read the text.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import abi
from .types import ClusterOutput, Features, Mesh, Pairs, Votes

_TYPES = {1: np.int32, 2: np.float64, 3: np.uint8}
TABLES = ("features", "pairs", "votes", "descriptors", "vertices", "faces")


def export_tables(directory, mesh: Mesh, features: Features, sample, pruned, pairs: Pairs,
                  votes: Votes, clusters: ClusterOutput, lib=None) -> Path:
    """sym_export_tables into `directory` (created if missing)."""
    lib = lib or abi.library()
    d = Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    sample = np.ascontiguousarray(sample, np.int32)
    pruned = np.ascontiguousarray(pruned, np.int32)
    cv, recs = clusters.view()
    view = abi.ExportView(mesh.view(), features.view(),
                          sample.ctypes.data_as(C.POINTER(C.c_int32)), sample.size,
                          pruned.ctypes.data_as(C.POINTER(C.c_int32)), pruned.size,
                          pairs.view(), votes.view(), cv)
    status = lib.sym_export_tables(C.byref(view), os.fsencode(str(d)))
    if status != 0:
        raise RuntimeError(lib.sym_last_error().decode())
    del recs
    return d


def read_table(path) -> dict:
    """One .symt file as {column name: array} (read-only views of a memory map)."""
    raw = np.memmap(path, np.uint8, "r")
    if bytes(raw[:8]) != b"SYMTAB01":
        raise ValueError(f"{path}: not a binary table")
    rows = int(raw[8:16].view(np.uint64)[0])
    ncols = int(raw[16:20].view(np.uint32)[0])
    out, at = {}, 24 + 32 * ncols
    for k in range(ncols):
        rec = raw[24 + 32 * k: 56 + 32 * k]
        name = bytes(rec[:24]).rstrip(b"\0").decode()
        dt = np.dtype(_TYPES[int(rec[24:28].view(np.uint32)[0])])
        at = (at + 63) // 64 * 64
        out[name] = raw[at: at + rows * dt.itemsize].view(dt)
        at += rows * dt.itemsize
    return out


def read_tables(directory) -> dict:
    return {t: read_table(Path(directory) / f"{t}.symt") for t in TABLES}


def _g(x) -> str:
    return "%.17g" % x


def render_text(directory, out_directory) -> Path:
    """The reference's features.csv, pairs.csv, votes.csv, descriptors.csv and
    mesh.off (src/io/export.cpp:40-98) from a directory of tables."""
    t = read_tables(directory)
    out = Path(out_directory)
    out.mkdir(parents=True, exist_ok=True)
    f = t["features"]
    cols = ["x", "y", "z", "kmin", "kmax", "nx", "ny", "nz", "dminx", "dminy", "dminz",
            "dmaxx", "dmaxy", "dmaxz"]
    lanes = [f[c].tolist() for c in cols]
    valid, sampled, pruned = (f[c].tolist() for c in ("valid", "sampled", "pruned"))
    with open(out / "features.csv", "w", newline="\n") as s:
        s.write("vertex,x,y,z,kmin,kmax,nx,ny,nz,dminx,dminy,dminz,dmaxx,dmaxy,dmaxz,"
                "valid,sampled,pruned\n")
        for i in range(len(valid)):
            s.write(f"{i}," + ",".join(_g(lane[i]) for lane in lanes)
                    + f",{int(valid[i] != 0)},{sampled[i]},{pruned[i]}\n")
    p = t["pairs"]
    with open(out / "pairs.csv", "w", newline="\n") as s:
        s.write("pair,a,b\n")
        for i, (a, b) in enumerate(zip(p["a"].tolist(), p["b"].tolist())):
            s.write(f"{i},{a},{b}\n")
    v = t["votes"]
    names = ["r00", "r01", "r02", "r10", "r11", "r12", "r20", "r21", "r22", "tx", "ty", "tz",
             "nx", "ny", "nz", "d"]
    lanes = [v[c].tolist() for c in names]
    pair, kind, cluster = v["pair"].tolist(), v["type"].tolist(), v["cluster"].tolist()
    with open(out / "votes.csv", "w", newline="\n") as s:
        s.write("vote,pair,type,r00,r01,r02,r10,r11,r12,r20,r21,r22,tx,ty,tz,nx,ny,nz,d,"
                "cluster\n")
        for i in range(len(pair)):
            s.write(f"{i},{pair[i]},{'reflection' if kind[i] == 1 else 'rigid'},"
                    + ",".join(_g(lane[i]) for lane in lanes) + f",{cluster[i]}\n")
    d = t["descriptors"]
    dim = d["dimension"].tolist()
    comps = [d[f"component{k}"].tolist() for k in range(12)]
    with open(out / "descriptors.csv", "w", newline="\n") as s:
        s.write("vote,dimension" + "".join(f",component{k}" for k in range(12)) + "\n")
        for i in range(len(dim)):
            s.write(f"{i},{dim[i]}" + "".join("," + (_g(comps[k][i]) if k < dim[i] else "")
                                             for k in range(12)) + "\n")
    x, y, z = (t["vertices"][c].tolist() for c in ("x", "y", "z"))
    fa, fb, fc = (t["faces"][c].tolist() for c in ("a", "b", "c"))
    with open(out / "mesh.off", "w", newline="\n") as s:
        s.write(f"OFF\n{len(x)} {len(fa)} 0\n")
        for i in range(len(x)):
            s.write(f"{_g(x[i])} {_g(y[i])} {_g(z[i])}\n")
        for i in range(len(fa)):
            s.write(f"3 {fa[i]} {fb[i]} {fc[i]}\n")
    return out
