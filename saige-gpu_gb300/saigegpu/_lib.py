"""ctypes binding of libsaigegpu.so (include/saigegpu.h).

The library is the product: there is no CPU fallback.  ``load()`` raises if
the shared object is missing or cannot be loaded, and every call that returns
a non-zero status raises ``SaigeGpuError`` carrying ``sg_last_error``.
"""
import ctypes as C
import os

from .build import LIB

_lib = None

c_i64 = C.c_int64
c_i32 = C.c_int32
c_u64 = C.c_uint64
P_f32 = C.POINTER(C.c_float)
P_f64 = C.POINTER(C.c_double)
P_i32 = C.POINTER(C.c_int32)
P_i64 = C.POINTER(C.c_int64)
P_u8 = C.POINTER(C.c_uint8)
P_u64 = C.POINTER(C.c_uint64)
c_ctx = C.c_void_p

STATUS = {0: "SG_OK", 1: "SG_ERR_INVALID", 2: "SG_ERR_CUDA", 3: "SG_ERR_NOMEM", 4: "SG_ERR_STATE",
          5: "SG_ERR_IO", 6: "SG_ERR_NUMERIC", 7: "SG_ERR_NOT_FOUND", 8: "SG_ERR_TIMEOUT"}

# name -> argtypes (restype int unless listed in _RESTYPE)
SIGNATURES = {
    "sg_ctx_create": [C.c_int, c_u64, C.POINTER(c_ctx)],
    "sg_ctx_destroy": [c_ctx],
    "sg_last_error": [c_ctx],
    "sg_device_bytes_in_use": [c_ctx, P_u64],
    "sg_set_matvec_mode": [c_ctx, C.c_int],
    "sg_kernel_launches": [c_ctx, P_u64],
    "sg_ctx_make_current": [c_ctx],
    "sg_set_tc_option": [c_ctx, C.c_int, C.c_int],
    "sg_set_vr_max_mac": [c_ctx, C.c_float],
    "sg_selftest_wait_timeout": [c_ctx, C.c_double],
    "sg_get_tc_option": [c_ctx, C.c_int, P_i32],
    "sg_set_grmv_plan": [c_ctx, C.c_int, P_i32, P_i32, P_i32],
    "sg_get_grmv_plan": [c_ctx, C.c_int, P_i32, P_i32, P_i32, C.POINTER(C.c_int)],
    "sg_set_subset_plan": [c_ctx, C.c_int, P_i32, P_i32, P_i32],
    "sg_get_subset_plan": [c_ctx, C.c_int, P_i32, P_i32, P_i32, C.POINTER(C.c_int)],
    "sg_setgeno": [c_ctx, P_u8, c_u64, c_i64, c_i64, P_i32, c_i64, P_u8, C.c_float, C.c_float,
                   P_i32, c_i64, C.c_float, C.c_int, C.c_int],
    "sg_setgeno_files": [c_ctx, C.c_char_p, C.c_char_p, C.c_char_p, P_i32, c_i64, P_u8, C.c_float,
                         C.c_float, P_i32, c_i64, C.c_float, C.c_int, C.c_int],
    "sg_setgeno_device": [c_ctx, C.c_void_p, c_u64, c_i64, c_i64, P_i32, c_i64, P_u8, C.c_float,
                          C.c_float, P_i32, c_i64, C.c_float, C.c_int, C.c_int],
    "sg_geno_dims": [c_ctx, P_i64, P_i64, P_i64, P_i64],
    "sg_get_allele_freq": [c_ctx, P_f32],
    "sg_get_invstd": [c_ctx, P_f32],
    "sg_get_mac": [c_ctx, P_i32],
    "sg_get_qc_marker_mask": [c_ctx, P_u8],
    "sg_get_vr_markers": [c_ctx, P_f32, P_i32, P_i32],
    "sg_get_packed_geno": [c_ctx, P_u8],
    "sg_get_onesnp_geno": [c_ctx, c_i64, P_i32],
    "sg_get_onesnp_geno_vr": [c_ctx, c_i64, P_i32],
    "sg_get_onesnp_stdgeno": [c_ctx, c_i64, P_f32],
    "sg_grm_build": [c_ctx, C.c_int],
    "sg_grm_diag": [c_ctx, P_f64],
    "sg_build_timing": [c_ctx, P_f64],
    "sg_grm_diag_f32": [c_ctx, P_f32],
    "sg_grm_get": [c_ctx, P_f32],
    "sg_grm_matmul": [c_ctx, P_f64, c_i64, P_f64],
    "sg_grm_matmul_tf32x3_noalloc": [c_ctx, C.c_void_p, c_i64, C.c_void_p, C.c_void_p],
    "sg_grm_padded_n": [c_ctx, P_i64],
    "sg_loco_set": [c_ctx, c_i64, c_i64],
    "sg_loco_set_bim": [c_ctx, c_i64, c_i64],
    "sg_loco_clear": [c_ctx],
    "sg_getCrossprodMatAndKin": [c_ctx, P_f32, P_f32],
    "sg_getDiagOfSigma": [c_ctx, P_f32, P_f32, P_f32],
    "sg_getCrossprod": [c_ctx, P_f32, P_f32, P_f32, P_f32],
    "sg_getPCG1ofSigmaAndVector": [c_ctx, P_f32, P_f32, P_f32, C.c_int, C.c_float, P_f32, P_i32],
    "sg_pcg_solve": [c_ctx, P_f64, P_f64, P_f64, c_i64, C.c_int, C.c_double, P_f64, P_i32],
    "sg_getSigma_X": [c_ctx, P_f32, P_f32, P_f32, c_i64, C.c_int, C.c_float, P_f32],
    "sg_getSigma_G": [c_ctx, P_f32, P_f32, P_f32, C.c_int, C.c_float, P_f32],
    "sg_getCoefficients": [c_ctx, P_f32, P_f32, c_i64, P_f32, P_f32, C.c_int, C.c_float, P_f32,
                           P_f32, P_f32, P_f32, P_f32],
    "sg_GetTrace": [c_ctx, P_f32, P_f32, c_i64, P_f32, P_f32, P_f32, C.c_int, C.c_int, C.c_float,
                    C.c_float, c_u64, P_f32, P_i32],
    "sg_GetTrace_q": [c_ctx, P_f32, P_f32, c_i64, P_f32, P_f32, P_f32, C.c_int, C.c_int, C.c_float,
                      C.c_float, c_u64, P_f32, P_i32],
    "sg_getAIScore": [c_ctx, P_f32, P_f32, c_i64, P_f32, P_f32, P_f32, P_f32, P_f32, C.c_int, C.c_int,
                      C.c_float, C.c_float, c_u64, P_f32, P_f32, P_f32, P_f32],
    "sg_getAIScore_q": [c_ctx, P_f32, P_f32, c_i64, P_f32, P_f32, P_f32, P_f32, P_f32, C.c_int,
                        C.c_int, C.c_float, C.c_float, c_u64, P_f32, P_f32, P_f32, P_f32, P_f32],
    "sg_fitglmmaiRPCG": [c_ctx, P_f32, P_f32, c_i64, P_f32, P_f32, P_f32, P_f32, P_f32, C.c_int,
                         C.c_int, C.c_float, C.c_float, C.c_float, c_u64],
    "sg_fitglmmaiRPCG_q": [c_ctx, P_f32, P_f32, c_i64, P_f32, P_f32, P_f32, P_f32, P_f32, C.c_int,
                           C.c_int, C.c_float, C.c_float, C.c_float, c_u64],
    "sg_engine_reserve": [c_ctx, c_i64, c_i64],
    "sg_engine_set_pheno": [c_ctx, c_i64, P_f64, P_f64, P_u8],
    "sg_engine_forget_subsets": [c_ctx],
    "sg_engine_prepare_subset": [c_ctx, c_i64, P_u8],
    "sg_engine_subset_vr_markers": [c_ctx, c_i64, P_i32, P_i32, c_i64, P_i64],
    "sg_engine_subset_geno": [c_ctx, c_i64, c_i64, P_i32],
    "sg_engine_subset_wait": [c_ctx, c_i64],
    "sg_engine_submit": [c_ctx, c_i64, C.c_int, P_f64, c_i64, C.c_int, C.c_double, P_i64],
    "sg_engine_submit_probes": [c_ctx, c_i64, C.c_int, c_u64, c_i64, c_i64, C.c_int, C.c_double,
                                P_i64],
    "sg_engine_submit_chained": [c_ctx, c_i64, P_i64, c_i64, C.c_int, C.c_double, P_i64],
    "sg_engine_run": [c_ctx, c_i64, P_i64],
    "sg_engine_launch": [c_ctx, P_i64, P_i32],
    "sg_engine_finish": [c_ctx, P_i64],
    "sg_engine_wait": [c_ctx],
    "sg_engine_step_trace": [c_ctx, P_f64, c_i64, P_i64],
    "sg_engine_fetch": [c_ctx, c_i64, P_f64, P_i32],
    "sg_engine_cancel": [c_ctx, c_i64],
    "sg_engine_stats": [c_ctx, P_i64],
    "sg_engine_poll": [c_ctx, P_i64, c_i64, P_i64],
    "sg_engine_hold_results": [c_ctx, C.c_int],
    "sg_engine_probe_cache_clear": [c_ctx, c_i64],
    "sg_engine_probe_cached": [c_ctx, c_i64, c_u64, c_i64],
    "sg_engine_probe_dots": [c_ctx, c_i64, P_i64, P_i64, c_i64, c_u64, c_i64, P_f64, c_i64, P_f64,
                             P_i32],
    "sg_engine_probe_dots_begin": [c_ctx, c_i64, P_i64, P_i64, c_i64, c_u64, c_i64, P_f64, c_i64],
    "sg_engine_probe_dots_wait": [c_ctx, c_i64],
    "sg_engine_probe_dots_end": [c_ctx, c_i64, P_f64, P_i32],
    "sg_engine_timing": [c_ctx, P_f64],
    "sg_engine_io_bytes": [c_ctx, P_u64, P_u64],
    "sg_engine_idle_ms": [c_ctx, P_f64],
    "sg_engine_reset_timing": [c_ctx],
    "sg_synth_bed": [c_ctx, c_u64, c_i64, c_i64, C.c_double, C.POINTER(C.c_void_p), P_u64],
    "sg_synth_bed_to_host": [c_ctx, P_u8, c_u64],
    "sg_synth_genetic_value": [c_ctx, c_u64, P_f64],
    "sg_fits_create": [c_ctx, c_i64, c_i64, C.c_int, C.POINTER(C.c_void_p)],
    "sg_fits_destroy": [C.c_void_p],
    "sg_fits_last_error": [C.c_void_p],
    "sg_fits_submit": [C.c_void_p, C.c_int, c_i64, P_u8, P_f64, P_f64, C.c_int, P_f64, P_f64, P_f64,
                       C.c_double, C.c_int, C.c_int, C.c_double, C.c_int, C.c_double, c_u64, P_i64],
    "sg_fits_run": [C.c_void_p, c_i64, P_i64],
    "sg_fits_set_threads": [C.c_void_p, C.c_int],
    "sg_fits_set_launch_wait": [C.c_void_p, C.c_double],
    "sg_fits_poll": [C.c_void_p, P_i64, c_i64, P_i64],
    "sg_fits_counts": [C.c_void_p, P_i64, P_i64, P_i64],
    "sg_fits_host_times": [C.c_void_p, P_f64],
    "sg_fits_step_times": [C.c_void_p, P_f64],
    "sg_fits_fit_times": [C.c_void_p, c_i64, P_f64],
    "sg_fits_result": [C.c_void_p, c_i64, P_f64, P_f64, P_f64, P_f64, P_f64, P_f64, P_i32, P_i32, P_i64],
}
_RESTYPE = {"sg_ctx_destroy": None, "sg_last_error": C.c_char_p, "sg_fits_destroy": None,
            "sg_fits_last_error": C.c_char_p}


class SaigeGpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (STATUS.get(code, code), msg))
        self.code = code


def lib_path():
    return os.environ.get("SAIGEGPU_LIB", LIB)


def load():
    """Load the CUDA library; raise when it is absent (no fallback path exists)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        raise ImportError("libsaigegpu.so not built (%s); run __graft_entry__.build()" % path)
    lib = C.CDLL(path)
    bind(lib, strict=True)
    _lib = lib
    return lib


def bind(lib, strict=False):
    """Give ``lib``'s entry points of this ABI their argument and result types (strict: every
    one must be present); returns ``lib``."""
    for name, argtypes in SIGNATURES.items():
        if not strict and not hasattr(lib, name):
            continue
        f = getattr(lib, name)
        f.argtypes = argtypes
        f.restype = _RESTYPE.get(name, C.c_int)
    return lib
