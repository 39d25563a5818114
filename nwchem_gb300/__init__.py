"""GB300 (sm_103a) implementation of NWChem's TCE CCSD(T) triples tile path.

The compute runs in libsdt_gb300.so (CUDA, built by nwchem_gb300.build);
this package is the host-side mirror of the reference's (T) interface.
"""
from ._capi import SdtError, lib, library_path
from .tiling import Tiling, config_tiling, random_tiling
from .triples import (FILE_T1, FILE_T2, FILE_V2, PREC_FP64, PREC_MIXED, PREC_MIXED_BF16, PREC_MIXED_FP16,
                      PREC_MIXED_TF32, Plan, TceFile, TriplesJob, ccsd_t, flops, molecular_scale, synth_file,
                      synth_inputs, task_list)

__all__ = ["SdtError", "lib", "library_path", "Tiling", "config_tiling", "random_tiling", "TceFile",
           "TriplesJob", "Plan", "ccsd_t", "flops", "molecular_scale", "synth_file", "synth_inputs", "task_list", "FILE_T1",
           "FILE_T2", "FILE_V2", "PREC_FP64", "PREC_MIXED", "PREC_MIXED_TF32", "PREC_MIXED_BF16",
           "PREC_MIXED_FP16"]
