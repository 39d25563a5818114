"""GB300 (sm_103a) implementation of NWChem's TCE CCSD(T) triples tile path.

The compute runs in libsdt_gb300.so (CUDA, built by nwchem_gb300.build);
this package is the host-side mirror of the reference's (T) interface.

Importing it before CUDA starts raises CUDA_DEVICE_MAX_CONNECTIONS to 32
(unless set): the serving loop keeps a stream per job in flight beside a
resident kernel and FP64 checks that run for seconds, and with the default 8
hardware queues streams share queues, so a job's short kernels could wait
behind a long kernel of an unrelated stream.
"""
import os

os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
from ._capi import SdtError, lib, library_path
from .tiling import Tiling, config_tiling, random_tiling
from .triples import (FILE_T1, FILE_T2, FILE_V2, PREC_FP64, PREC_MIXED, PREC_MIXED_BF16, PREC_MIXED_FP16,
                      PREC_MIXED_TF32, Plan, TceFile, TriplesJob, ccsd_t, flops, molecular_scale, synth_file,
                      synth_inputs, task_list)

__all__ = ["SdtError", "lib", "library_path", "Tiling", "config_tiling", "random_tiling", "TceFile",
           "TriplesJob", "Plan", "ccsd_t", "flops", "molecular_scale", "synth_file", "synth_inputs", "task_list", "FILE_T1",
           "FILE_T2", "FILE_V2", "PREC_FP64", "PREC_MIXED", "PREC_MIXED_TF32", "PREC_MIXED_BF16",
           "PREC_MIXED_FP16"]
