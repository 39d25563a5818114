"""The reference's own CUDA path for the (T) tiles, built for GB300.

TEST INFRASTRUCTURE ONLY (checker and baseline side).  NWChem's GPU path
for these tiles is src/tce/ccsd_t/sd_t_total.cu (the 27 sd_t_*_cuda_ FP64
SIMT kernels, dev_mem_*, compute_en_), memory.cu (its device memory pool)
and header.h.  They compile with nvcc from those three files alone (with
-DTCE_CUDA, as the reference's makefile defines it); hybrid.c (device
selection through Global Arrays) is not needed by them.

  stage(tree)   copies the three files from the NWChem tree into
                oracle/_ref/cuda/ (not committed; the folder travels with the
                working tree to the GPU host, which has no NWChem tree);
  build()       compiles them for sm_103a into oracle/_ref/libref_cuda.so;
  TileRunner    drives them the way NWChem's ccsd_t_gpu.F does: per tuple the
                reference's driver logic (the oracle's hooks: block fetch and
                sort on the host) calls sd_t_{s1,d1,d2}_k_cuda_ with host
                sub-blocks, which copy them to the device and run; then
                compute_en_ reduces the tile energies.

    python oracle/ref_cuda.py [NWCHEM_SOURCE_TREE]    # stage, then build
"""
from __future__ import annotations

import ctypes as C
import shutil
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
STAGE = HERE / "_ref" / "cuda"
LIB = HERE / "_ref" / "libref_cuda.so"
SOURCES = ["src/tce/ccsd_t/sd_t_total.cu", "src/tce/ccsd_t/memory.cu", "src/tce/ccsd_t/header.h"]


def stage(tree: Path) -> Path:
    STAGE.mkdir(parents=True, exist_ok=True)
    for rel in SOURCES:
        shutil.copyfile(tree / rel, STAGE / Path(rel).name)
    return STAGE


def staged() -> bool:
    return all((STAGE / Path(rel).name).exists() for rel in SOURCES)


def build() -> Path:
    if not staged():
        raise FileNotFoundError("the reference CUDA sources are not staged in oracle/_ref/cuda/")
    srcs = [STAGE / "sd_t_total.cu", STAGE / "memory.cu"]
    if LIB.exists() and LIB.stat().st_mtime > max(s.stat().st_mtime for s in srcs):
        return LIB
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cmd = [nvcc, "-DTCE_CUDA", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-Xcompiler", "-fPIC",
           "-shared", "-I", str(STAGE), *map(str, srcs), "-o", str(LIB) + ".tmp"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on the reference CUDA sources:\n{res.stderr[-4000:]}")
    Path(str(LIB) + ".tmp").replace(LIB)
    return LIB


class TileRunner:
    """The reference's GPU tile path over tuples of an oracle Problem."""

    def __init__(self):
        self.lib = C.CDLL(str(build()))
        self.lib.initmemmodule_()

    def tuple_energy(self, problem, tup) -> np.ndarray:
        """(E[T], E(T)) of one tuple (p4b,p5b,p6b,h1b,h2b,h3b) through the
        reference's sd_t_*_cuda_ entry points and compute_en_."""
        lib, t = self.lib, problem.tiling
        refs = lambda v: [C.byref(C.c_int64(int(x))) for x in v]
        r = t.range
        td = [int(r[b - 1]) for b in (tup[3], tup[4], tup[5], tup[0], tup[1], tup[2])]   # h1..h3, p4..p6
        lib.dev_mem_s_(*refs(td))
        lib.dev_mem_d_(*refs(td))
        problem.drive(tup,
                      lambda k, d, a, b: getattr(lib, f"sd_t_s1_{k}_cuda_")(*refs(d), None, a, b),
                      lambda k, d, a, b: getattr(lib, f"sd_t_d1_{k}_cuda_")(*refs(d), None, a, b),
                      lambda k, d, a, b: getattr(lib, f"sd_t_d2_{k}_cuda_")(*refs(d), None, a, b))
        f = 1.0 / (6 if tup[0] == tup[1] == tup[2] else 2 if (tup[0] == tup[1] or tup[1] == tup[2]) else 1)
        f /= 6 if tup[3] == tup[4] == tup[5] else 2 if (tup[3] == tup[4] or tup[4] == tup[5]) else 1
        ev = [np.ascontiguousarray(t.evl[t.offset[b - 1]:t.offset[b - 1] + r[b - 1]])
              for b in (tup[3], tup[4], tup[5], tup[0], tup[1], tup[2])]
        e = np.zeros(2)
        pd = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        lib.compute_en_(C.byref(C.c_double(f)), pd(e), *[pd(x) for x in ev], *refs(td), None, None)
        lib.dev_release_()
        return e

    def close(self) -> None:
        self.lib.finalizememmodule_()


if __name__ == "__main__":
    from f77_ref import DEFAULT_TREE
    tree = Path(sys.argv[1]) if len(sys.argv) > 1 else DEFAULT_TREE
    print(stage(tree))
    print(build())
