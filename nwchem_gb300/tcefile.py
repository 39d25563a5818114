"""NWChem TCE files on disk.

The TCE keeps T1, T2 and the two-electron integrals V2 as flat arrays of
float64 blocks: in a global array, in a Fortran direct-access file with one
8-byte record per element (src/tce/get_block.F, ioalg 0) or in an EAF file
read at byte offset 8*offset (ioalg 1).  Either way the file is a raw stream
of native doubles whose block offsets come from the hash table the TCE
builds from the tiling (src/tce/tce_t1_offset.F, tce_t2_offset.F,
tce_mo2e_offset.F).  read_tce_file rebuilds that table with the same loop
order and pairs it with the data, so a job can load NWChem's own files;
V2 files written by NWChem contain every integral block, of which the
triples path reads the vvov, ovoo and vvoo ones.

Not covered: the orbital-form integral files of the "2eorb" option
(get_hash_block_i), which use a different hash.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import _capi
from .tiling import Tiling
from .triples import FILE_T1, FILE_T2, FILE_V2, TceFile


def tce_layout(tiling: Tiling, kind: int) -> tuple[np.ndarray, int]:
    """(hash table, number of doubles) of the reference layout of a file."""
    lib = _capi.lib()
    ts = tiling.struct()
    nb, nd = C.c_int64(), C.c_int64()
    _capi.check(lib.sdt_tce_layout(C.byref(ts), kind, C.byref(nb), C.byref(nd), None), "sdt_tce_layout")
    h = np.empty(2 * nb.value + 1, dtype=np.int64)
    _capi.check(lib.sdt_tce_layout(C.byref(ts), kind, C.byref(nb), C.byref(nd), h.ctypes.data_as(_capi.PI64)),
                "sdt_tce_layout")
    return h, nd.value


def read_tce_file(path: str | Path, tiling: Tiling, kind: int, mmap: bool = True) -> TceFile:
    """Reads a raw TCE file (native float64) and attaches the reference hash."""
    h, nd = tce_layout(tiling, kind)
    path = Path(path)
    size = path.stat().st_size
    if size != 8 * nd:
        raise ValueError(f"{path}: {size} bytes, the tiling's layout needs {8 * nd}")
    data = np.memmap(path, dtype=np.float64, mode="r") if mmap else np.fromfile(path, dtype=np.float64)
    return TceFile(h, np.ascontiguousarray(data))


def write_tce_file(path: str | Path, f: TceFile, tiling: Tiling, kind: int) -> None:
    """Writes f in the reference layout; blocks absent from f are written as
    zeros (f's hash may list fewer blocks than the layout, e.g. a V2 file with
    only the blocks the triples path reads)."""
    h, nd = tce_layout(tiling, kind)
    out = np.zeros(nd, dtype=np.float64)
    n = int(h[0])
    for q in range(n):
        key, off = int(h[1 + q]), int(h[1 + n + q])
        end = int(h[2 + n + q]) if q + 1 < n else nd
        src = f.lookup(key)
        if src >= 0:
            out[off:end] = f.data[src:src + (end - off)]
    out.tofile(str(path))


__all__ = ["tce_layout", "read_tce_file", "write_tce_file", "FILE_T1", "FILE_T2", "FILE_V2"]
