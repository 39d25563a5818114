"""Builds libsdt_gb300.so in-tree with nvcc for sm_103a.

Each translation unit compiles in parallel, then one link.  Host code is
built with -ffp-contract=off so that host-side arithmetic (synthetic inputs,
orbital energies) gives the same bits on x86-64 and aarch64 hosts.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
LIB = LIBDIR / "libsdt_gb300.so"
BUILD = PKG / "_build"

SOURCES = ["sdt_host.cpp", "sdt_mem.cu", "sdt_tile.cu", "sdt_fused.cu", "sdt_probe.cu", "sdt_noalloc.cu", "sdt_mixed.cu",
           "sdt_split.cu", "sdt_plan.cu", "sdt_serve.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA extension cannot be built")
    return cand


def _compile(src: str, verbose: bool) -> Path:
    out = BUILD / (Path(src).stem + ".o")
    cmd = [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-c", str(CSRC / src), "-o", str(out),
           "-Xcompiler", "-fPIC,-fopenmp,-ffp-contract=off,-O3", "--expt-relaxed-constexpr"]
    if src.endswith(".cu") and verbose:
        cmd += ["-Xptxas", "-v"]
    if src.endswith(".cpp"):
        cmd += ["-x", "c++"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    if verbose and res.stderr:
        sys.stderr.write(res.stderr)
    return out


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = [CSRC / s for s in SOURCES] + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh"))
    deps.append(PKG.parent / "include" / "sdt_gb300.h")
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and not _stale():
        return LIB
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [_nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs),
           "-Xcompiler", "-fopenmp", "-lgomp", "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
