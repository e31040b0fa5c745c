"""Build and call oracle/cpu_ref.c: the reference's CPU GRM.x and FP32 PCG restated in C.

TEST / CPU-BASELINE INFRASTRUCTURE ONLY (the ``cpu_baseline`` and ``--impl
reference`` legs of bench.py).  Built with gcc -O3 -fopenmp into
oracle/_build/; portable C (no -march flags), so it builds on x86 and Arm.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cpu_ref.c")
OUT = os.path.join(HERE, "_build", "libcpuref.so")
_lib = None


def build(force=False):
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    if force or not os.path.exists(OUT) or os.path.getmtime(OUT) < os.path.getmtime(SRC):
        subprocess.run(["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", SRC, "-o", OUT], check=True)
    return OUT


def load():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(OUT)
        P = C.c_void_p
        _lib.cpuref_crossprod.argtypes = [P, C.c_int64, P, C.c_int64, C.c_int64, P, P, C.c_int]
        _lib.cpuref_pcg.argtypes = [P, C.c_int64, P, C.c_int64, C.c_int64, P, P, P, P, C.c_int,
                                    C.c_float, P, C.c_int]
        _lib.cpuref_pcg.restype = C.c_int
        _lib.cpuref_synth_setgeno.argtypes = [C.c_uint64, C.c_int64, C.c_int64, C.c_double, C.c_float,
                                              C.c_float, P, C.c_int64, P, C.c_int]
        _lib.cpuref_synth_setgeno.restype = C.c_int64
    return _lib


class PackedGeno:
    """Host copy of re-packed GRM genotypes + LUT (the reference's genoClass layout)."""

    def __init__(self, packed, lut4, n):
        self.packed = np.ascontiguousarray(packed, np.uint8)
        self.m, self.pitch = self.packed.shape
        self.lut = np.ascontiguousarray(lut4, np.float32).reshape(self.m, 4)
        self.n = n

    @classmethod
    def synthetic(cls, seed, n, m, miss_rate, min_maf=0.01, max_miss=0.15, nthreads=0):
        pitch = (n + 3) // 4
        packed = np.empty((m, pitch), np.uint8)
        lut = np.empty((m, 4), np.float32)
        k = load().cpuref_synth_setgeno(seed, n, m, miss_rate, min_maf, max_miss, packed.ctypes.data,
                                        pitch, lut.ctypes.data, nthreads)
        return cls(packed[:k], lut[:k], n)

    def crossprod(self, b, nthreads=0):
        b = np.ascontiguousarray(b, np.float32)
        out = np.empty(self.n, np.float32)
        load().cpuref_crossprod(self.packed.ctypes.data, self.pitch, self.lut.ctypes.data, self.m,
                                self.n, b.ctypes.data, out.ctypes.data, nthreads)
        return out


class CpuGeno:
    """Re-packed genotypes + LUT in the reference's layout, from an oracle GenoResult."""

    def __init__(self, geno):
        from . import plink
        self.n = geno.codes.shape[1]
        self.m = geno.codes.shape[0]
        self.packed = np.ascontiguousarray(plink.pack_codes(geno.codes))
        self.pitch = self.packed.shape[1]
        lut = np.zeros((self.m, 4), np.float32)
        lut[:, :3] = plink.std_lut(geno.freq, geno.invstd)
        self.lut = np.ascontiguousarray(lut)
        self.diag32 = plink.diag_std_geno_f32(geno)

    def crossprod(self, b, nthreads=0):
        b = np.ascontiguousarray(b, np.float32)
        out = np.empty(self.n, np.float32)
        load().cpuref_crossprod(self.packed.ctypes.data, self.pitch, self.lut.ctypes.data, self.m,
                                self.n, b.ctypes.data, out.ctypes.data, nthreads)
        return out

    def pcg(self, w, tau, b, maxiter=500, tol=1e-5, nthreads=0):
        w = np.ascontiguousarray(w, np.float32)
        tau = np.ascontiguousarray(tau, np.float32)
        b = np.ascontiguousarray(b, np.float32)
        x = np.empty(self.n, np.float32)
        it = load().cpuref_pcg(self.packed.ctypes.data, self.pitch, self.lut.ctypes.data, self.m,
                               self.n, self.diag32.ctypes.data, w.ctypes.data, tau.ctypes.data,
                               b.ctypes.data, maxiter, tol, x.ctypes.data, nthreads)
        return x, it
