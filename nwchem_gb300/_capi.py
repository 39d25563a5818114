"""ctypes binding of libsdt_gb300.so (the C ABI declared in include/sdt_gb300.h).

The library is loaded from the package's _lib/ folder.  There is no CPU
fallback: if the shared object is missing or does not load, every entry point
raises.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

_LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libsdt_gb300.so"
_lock = threading.Lock()
_lib = None

I64 = C.c_int64
PI64 = C.POINTER(C.c_int64)
PD = C.POINTER(C.c_double)


class SdtTiling(C.Structure):
    _fields_ = [("noab", I64), ("nvab", I64), ("range", PI64), ("spin", PI64), ("sym", PI64),
                ("offset", PI64), ("alpha", PI64), ("evl_sorted", PD), ("restricted", I64)]


class SdtFile(C.Structure):
    _fields_ = [("hash", PI64), ("data", PD), ("ndata", I64)]


class SdtError(RuntimeError):
    """A libsdt_gb300 call returned a non-zero status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"libsdt_gb300 error {code}: {msg}")
        self.code = code


def _declare(lib):
    sig = {
        "sdt_set_error_mode": (None, [C.c_int]),
        "sdt_last_error": (C.c_int, [C.c_char_p, C.c_size_t]),
        "sdt_tasks_count": (I64, [C.POINTER(SdtTiling)]),
        "sdt_tasks_list": (C.c_int, [C.POINTER(SdtTiling), I64, PI64]),
        "sdt_tasks_flops": (C.c_double, [C.POINTER(SdtTiling), PI64, I64]),
        "sdt_synth_file": (C.c_int, [C.POINTER(SdtTiling), C.c_int, C.c_uint64, PI64, PI64, PI64, PD]),
        "sdt_synth_evl": (C.c_int, [I64, I64, C.c_uint64, PD]),
        "sdt_tce_layout": (C.c_int, [C.POINTER(SdtTiling), C.c_int, PI64, PI64, PI64]),
        "sdt_job_create": (C.c_int, [C.POINTER(SdtTiling), C.POINTER(C.c_void_p)]),
        "sdt_job_load": (C.c_int, [C.c_void_p, C.POINTER(SdtFile), C.POINTER(SdtFile),
                                   C.POINTER(SdtFile), C.c_void_p]),
        "sdt_job_run": (C.c_int, [C.c_void_p, PI64, I64, C.c_int, PD, PD, C.c_void_p]),
        "sdt_job_destroy": (C.c_int, [C.c_void_p]),
        "sdt_job_device_bytes": (I64, [C.c_void_p]),
        "sdt_ccsd_t": (C.c_int, [C.POINTER(SdtTiling), C.POINTER(SdtFile), C.POINTER(SdtFile),
                                 C.POINTER(SdtFile), PD, PD]),
        "sdt_launch_count": (I64, []),
        "sdt_job_set_timing": (C.c_int, [C.c_void_p, C.c_int]),
        "sdt_job_set_mixed_segment": (C.c_int, [C.c_void_p, C.c_int]),
        "sdt_job_set_mixed_shape": (C.c_int, [C.c_void_p, C.c_int]),
        "sdt_job_last_kernel_ms": (C.c_double, [C.c_void_p]),
        "sdt_probe_fp64_tflops": (C.c_double, [C.c_int]),
        "sdt_plan_create": (C.c_int, [C.c_void_p, PI64, C.c_int64, C.c_int, C.POINTER(C.c_int32),
                                      C.POINTER(C.c_void_p)]),
        "sdt_plan_launch": (C.c_int, [C.c_void_p, C.c_void_p]),
        "sdt_plan_capture": (C.c_int, [C.c_void_p, C.c_void_p]),
        "sdt_plan_run": (C.c_int, [C.c_void_p, C.c_void_p, PD, PD]),
        "sdt_plan_destroy": (C.c_int, [C.c_void_p]),
        "sdt_plan_items": (C.c_int64, [C.c_void_p]),
        "sdt_server_create": (C.c_int, [C.c_int64, C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
        "sdt_server_submit": (C.c_int, [C.c_void_p, C.POINTER(SdtTiling), C.POINTER(SdtFile), C.POINTER(SdtFile),
                                        C.POINTER(SdtFile), C.c_int, C.c_int, C.POINTER(C.c_int64)]),
        "sdt_server_status": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_int), PD, PD, PD, C.c_char_p,
                                        C.c_size_t]),
        "sdt_server_drain": (C.c_int, [C.c_void_p, C.c_double]),
        "sdt_server_cancel": (C.c_int, [C.c_void_p, C.c_int64]),
        "sdt_server_set_check_ctas": (C.c_int, [C.c_void_p, C.c_int]),
        "sdt_plan_item_energies": (C.c_int, [C.c_void_p, PD, C.c_int64]),
        "sdt_server_set_queue": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double]),
        "sdt_server_queue_stats": (C.c_int, [C.c_void_p, PI64]),
        "sdt_server_job_launches": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
        "sdt_job_set_sm_exclusive": (C.c_int, [C.c_void_p, C.c_int]),
        "sdt_server_peak_bytes": (C.c_int64, [C.c_void_p]),
        "sdt_server_destroy": (C.c_int, [C.c_void_p]),
        "sdt_job_bytes": (C.c_int64, [C.POINTER(SdtTiling), C.c_int]),
        "sdt_admission_simulate": (C.c_int, [C.c_int64, PD, PI64, PD, C.c_int64, C.c_int, PD, PD]),
        "sdt_serving_simulate": (C.c_int, [C.c_int64, PD, PI64, PD, PD, C.c_int64, C.c_int, PD, PD, PD]),
        "sdt_job_set_max_ctas": (C.c_int, [C.c_void_p, C.c_int]),
        "sdt_job_stream": (C.c_void_p, [C.c_void_p]),
        "sdt_tc_selftest": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
        "sdt_tc_selftest16": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                        C.c_void_p]),
        "sdt_check_division": (C.c_int, [C.c_int64, C.c_uint64, C.POINTER(C.c_double)]),
        "sdt_check_wait_timeout": (C.c_int, [C.c_double, C.POINTER(C.c_double)]),
        "compute_en_": (None, [PD, PD, PD, PD, PD, PD, PD, PD, PI64, PI64, PI64, PI64, PI64, PI64, PD, PD]),
        "dev_mem_d_": (None, [PI64] * 6),
        "dev_mem_s_": (None, [PI64] * 6),
        "dev_release_": (None, []),
        "sdt_tile_download": (C.c_int, [PD, PD]),
        "sdt_compute_en_noalloc": (C.c_int, [C.c_double, PD, PD, PD, PD, PD, PD, PD, I64, I64, I64, I64, I64,
                                             I64, C.c_void_p, C.c_void_p, C.c_void_p]),
        "initmemmodule_": (None, []),
        "finalizememmodule_": (None, []),
        "check_device_": (C.c_int, [C.POINTER(C.c_long)]),
        "device_init_": (C.c_int, [C.POINTER(C.c_long), C.POINTER(C.c_long)]),
    }
    for k in range(1, 10):
        sig[f"sd_t_s1_{k}_cuda_"] = (None, [PI64] * 6 + [PD, PD, PD])
        sig[f"sd_t_d1_{k}_cuda_"] = (None, [PI64] * 7 + [PD, PD, PD])
        sig[f"sd_t_d2_{k}_cuda_"] = (None, [PI64] * 7 + [PD, PD, PD])
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return sig


EXPORTED = None


def lib():
    """The loaded library; raises if it was not built."""
    global _lib, EXPORTED
    with _lock:
        if _lib is None:
            if not _LIB_PATH.exists():
                raise ImportError(
                    f"{_LIB_PATH} is missing: build the CUDA extension first "
                    "(python -c 'import __graft_entry__ as g; g.build()')")
            _lib = C.CDLL(str(_LIB_PATH))
            EXPORTED = tuple(_declare(_lib).keys())
        return _lib


def library_path() -> Path:
    return _LIB_PATH


def check(rc: int, what: str = "") -> None:
    if rc != 0:
        buf = C.create_string_buffer(512)
        code = lib().sdt_last_error(buf, 512)
        raise SdtError(rc, (what + ": " if what else "") + buf.value.decode(errors="replace") + f" [{code}]")


def last_error() -> tuple[int, str]:
    buf = C.create_string_buffer(512)
    code = lib().sdt_last_error(buf, 512)
    return code, buf.value.decode(errors="replace")
