"""The allocation-free GRM.V entry point against the regular one (GPU).

``sg_grm_matmul_tf32x3_noalloc`` serves callers that cannot allocate device
memory -- host runtimes that own every byte of HBM through their own pool, or
latency-critical loops that cannot absorb the synchronisation of cudaMalloc and
cudaFree.  The caller passes device input and output; the product's scratch is
a static device array inside the library.  This file is collected last so that
a run which stops at the first failure has already run every other test; it
builds its own context and cohort, so it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from saigegpu import GRM_FP32_SIMT, MV_TF32X3_TC, synth

pytestmark = pytest.mark.gpu


def test_noalloc_grm_matvec_matches_engine_product():
    import torch
    from saigegpu import Context, _lib
    ctx = Context(0)
    try:
        n, m = 900, 2100
        bed, _ = synth.synth_bed(61, n, m, 0.01)
        ctx.setgeno(bed, n, m)
        ctx.grm_build(GRM_FP32_SIMT)
        ctx.set_matvec_mode(MV_TF32X3_TC)
        npad = ctypes.c_int64()
        ctx._call("sg_grm_padded_n", ctypes.byref(npad))
        npad = npad.value
        rng = np.random.default_rng(12)
        for call in range(2):  # two calls in a row share (and overwrite) the static scratch
            k = 32 if call == 0 else 64
            V = rng.standard_normal((n, k))
            ref = ctx.grm_matmul(V)  # the regular entry point (engine, same split-TF32 product)
            P = torch.zeros((k, npad), dtype=torch.float32, device="cuda")
            P[:, :n] = torch.from_numpy(V.T.astype(np.float32)).cuda()
            Y = torch.empty((k, npad), dtype=torch.float32, device="cuda")
            torch.cuda.synchronize()
            ctx._call("sg_grm_matmul_tf32x3_noalloc", ctypes.c_void_p(P.data_ptr()), k,
                      ctypes.c_void_p(Y.data_ptr()), None)
            torch.cuda.synchronize()
            got = Y[:, :n].double().cpu().numpy().T
            # same tolerance as the GRM.V parity tests: FP32-class split-TF32 product
            assert np.abs(got - ref).max() / np.abs(ref).max() < 5e-6, call
        with pytest.raises(_lib.SaigeGpuError):
            ctx._call("sg_grm_matmul_tf32x3_noalloc", ctypes.c_void_p(P.data_ptr()), 33,
                      ctypes.c_void_p(Y.data_ptr()), None)
        too_many = 32 * ((2 ** 21) // (32 * npad) + 1)
        with pytest.raises(_lib.SaigeGpuError):
            ctx._call("sg_grm_matmul_tf32x3_noalloc", ctypes.c_void_p(P.data_ptr()), too_many,
                      ctypes.c_void_p(Y.data_ptr()), None)
    finally:
        ctx.close()
