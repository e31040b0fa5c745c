"""saigegpu -- GB300-native SAIGE step-1 hot path (dense GRM + PCG/AI-REML).

The compute lives in ``libsaigegpu.so`` (hand-written sm_103a CUDA behind the
C ABI of ``include/saigegpu.h``); this package is the host side: the ctypes
binding, the mirror of the reference's R driver, phenotype preparation, the
multi-phenotype batching/serving loop and synthetic cohorts.
"""
from .context import (Context, GRM_FP32_SIMT, GRM_BF16_TC, GRM_BF16X3_TC, MV_FP32_SIMT,
                      MV_TF32_TC, MV_FP64_PLAIN, MV_TF32X3_TC, MV_BF16X3_TC, MV_SUBSET_EXACT, MV_SUBSET_EXACT_F8, TC_SYRK_PAIR, TC_GRMV_PAIR,
                      TC_DRAIN_BYTES, TC_SYRK_GROUP, TC_GRMV_SLICE, TC_SUBSET_PAIR, TC_SUBSET_SLICE)
from ._lib import SaigeGpuError, load

__all__ = ["Context", "SaigeGpuError", "load", "GRM_FP32_SIMT", "GRM_BF16_TC", "GRM_BF16X3_TC",
           "MV_FP32_SIMT", "MV_TF32_TC", "MV_FP64_PLAIN", "MV_TF32X3_TC", "MV_BF16X3_TC", "MV_SUBSET_EXACT", "MV_SUBSET_EXACT_F8", "TC_SYRK_PAIR",
           "TC_GRMV_PAIR", "TC_DRAIN_BYTES", "TC_SYRK_GROUP", "TC_GRMV_SLICE", "TC_SUBSET_PAIR", "TC_SUBSET_SLICE"]
