"""Python face of the C ABI: one ``Context`` per GPU, numpy in, numpy out.

Method names follow the reference's Rcpp entry points
(src/SAIGE/R/RcppExports.R) so that host code reads like the reference's R
driver; vectors are float32 where the reference passes Armadillo ``fvec``
and float64 for the mixed-precision engine API.
"""
import ctypes as C

import numpy as np

from . import _lib as L

GRM_FP32_SIMT, GRM_BF16_TC, GRM_BF16X3_TC = 0, 1, 2
MV_FP32_SIMT, MV_TF32_TC, MV_FP64_PLAIN, MV_TF32X3_TC, MV_BF16X3_TC, MV_SUBSET_EXACT = 0, 1, 2, 3, 4, 5
MV_SUBSET_EXACT_F8 = 6
# tcgen05 GEMM shape options (enum sg_tc_option)
TC_SYRK_PAIR, TC_GRMV_PAIR, TC_DRAIN_BYTES, TC_SYRK_GROUP, TC_GRMV_SLICE = 0, 1, 2, 3, 4
TC_SUBSET_PAIR, TC_SUBSET_SLICE = 5, 6
TC_OPTIONS = {"syrk_pair": TC_SYRK_PAIR, "grmv_pair": TC_GRMV_PAIR, "drain_bytes": TC_DRAIN_BYTES,
              "syrk_group": TC_SYRK_GROUP, "grmv_slice": TC_GRMV_SLICE, "subset_pair": TC_SUBSET_PAIR,
              "subset_slice": TC_SUBSET_SLICE}


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _ptr(a, t):
    return a.ctypes.data_as(t)


def _cols(X):
    """(n, p) matrix -> column-major contiguous copy (Armadillo layout)."""
    X = np.asarray(X)
    if X.ndim == 1:
        X = X[:, None]
    return np.asfortranarray(X).ravel(order="F"), X.shape[1]


class Context:
    def __init__(self, device=0, hbm_budget_bytes=0):
        self._L = L.load()
        h = C.c_void_p()
        rc = self._L.sg_ctx_create(device, hbm_budget_bytes, C.byref(h))
        if rc != 0:
            raise L.SaigeGpuError(rc, "sg_ctx_create(device=%d) failed" % device)
        self._h = h
        self.n = None

    # ------------------------------------------------------------ plumbing
    def close(self):
        if getattr(self, "_h", None):
            self._L.sg_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _call(self, name, *args):
        rc = getattr(self._L, name)(self._h, *args)
        if rc != 0:
            msg = self._L.sg_last_error(self._h)
            raise L.SaigeGpuError(rc, (msg or b"").decode())
        return rc

    def last_error(self):
        return (self._L.sg_last_error(self._h) or b"").decode()

    def bytes_in_use(self):
        v = C.c_uint64()
        self._call("sg_device_bytes_in_use", C.byref(v))
        return v.value

    def kernel_launches(self):
        v = C.c_uint64()
        self._call("sg_kernel_launches", C.byref(v))
        return v.value

    def make_current(self):
        """Make this context's GPU current on the calling thread (worker threads of a runner)."""
        self._call("sg_ctx_make_current")

    def set_tc_option(self, option, value):
        """Shape option of the tcgen05 GEMMs (TC_* constants; process-wide)."""
        self._call("sg_set_tc_option", int(option), int(value))

    def get_tc_option(self, option):
        v = C.c_int32()
        self._call("sg_get_tc_option", int(option), C.byref(v))
        return v.value

    def tc_options(self):
        """All tcgen05 shape options as a dict name -> value."""
        return {name: self.get_tc_option(opt) for name, opt in TC_OPTIONS.items()}

    def _set_plan(self, fn, plan):
        plan = sorted(plan)
        mc = np.array([p[0] for p in plan], np.int32)
        pr = np.array([p[1] for p in plan], np.int32)
        sl = np.array([p[2] for p in plan], np.int32)
        P = C.POINTER(C.c_int32)
        self._call(fn, len(plan), _ptr(mc, P), _ptr(pr, P), _ptr(sl, P))

    def _get_plan(self, fn):
        cap = 64
        mc, pr, sl = (np.zeros(cap, np.int32) for _ in range(3))
        n = C.c_int()
        P = C.POINTER(C.c_int32)
        self._call(fn, cap, _ptr(mc, P), _ptr(pr, P), _ptr(sl, P), C.byref(n))
        return [(int(mc[i]), int(pr[i]), int(sl[i])) for i in range(n.value)]

    def set_grmv_plan(self, plan):
        """Per-width split-BF16 GRM.V choices: a list of (max_cols, pair, slice) with increasing
        max_cols ([] clears)."""
        self._set_plan("sg_set_grmv_plan", plan)

    def grmv_plan(self):
        return self._get_plan("sg_get_grmv_plan")

    def set_subset_plan(self, plan):
        """Per-width choices of the subset-exact engine's genotype GEMMs: (max_cols, pair, slice)."""
        self._set_plan("sg_set_subset_plan", plan)

    def subset_plan(self):
        return self._get_plan("sg_get_subset_plan")

    def set_tc_options(self, opts):
        """Set options from a dict name -> value (as returned by ``tc_options``)."""
        for name, v in opts.items():
            self.set_tc_option(TC_OPTIONS[name], v)

    def set_matvec_mode(self, mode):
        self._call("sg_set_matvec_mode", int(mode))
        self._mv_mode = int(mode)

    def matvec_mode(self):
        """The engine last selected through set_matvec_mode (None before the first call)."""
        return getattr(self, "_mv_mode", None)

    # ------------------------------------------------------------ genotypes (setgeno)
    @staticmethod
    def _geno_args(n_fam, sub_1based, pheno_mask, vr_random):
        sub = np.arange(1, n_fam + 1, dtype=np.int32) if sub_1based is None else np.ascontiguousarray(sub_1based, np.int32)
        mask = np.ones(n_fam, np.uint8) if pheno_mask is None else np.ascontiguousarray(pheno_mask, np.uint8)
        vr = np.zeros(1, np.int32) if vr_random is None else np.ascontiguousarray(vr_random, np.int32)
        nvr = 0 if vr_random is None else len(vr)
        return sub, mask, vr, nvr

    def set_vr_max_mac(self, max_mac):
        """Categorical variance ratios for the next setgeno (g_maxMACVarRatio; -1 = single ratio)."""
        self._call("sg_set_vr_max_mac", float(max_mac))
        self._vr_max_mac = float(max_mac)

    def setgeno(self, bed, n_fam, m_bim, sub_1based=None, pheno_mask=None, min_maf=0.01,
                max_missing=0.15, vr_random=None, min_mac_vr=20.0, is_var_ratio=False,
                is_diag_one=False):
        buf = np.frombuffer(bed, dtype=np.uint8) if isinstance(bed, (bytes, bytearray)) else np.ascontiguousarray(bed, np.uint8)
        sub, mask, vr, nvr = self._geno_args(n_fam, sub_1based, pheno_mask, vr_random)
        self._geno_src = ("setgeno", (buf, n_fam, m_bim), dict(
            min_maf=min_maf, max_missing=max_missing, vr_random=vr_random, min_mac_vr=min_mac_vr,
            is_var_ratio=is_var_ratio, is_diag_one=is_diag_one), sub, mask)
        self._call("sg_setgeno", _ptr(buf, L.P_u8), buf.size, n_fam, m_bim, _ptr(sub, L.P_i32), len(sub),
                   _ptr(mask, L.P_u8), min_maf, max_missing, _ptr(vr, L.P_i32), nvr, min_mac_vr,
                   int(is_var_ratio), int(is_diag_one))
        self.n = len(sub)

    def setgeno_files(self, bed, bim, fam, sub_1based, n_fam, pheno_mask=None, min_maf=0.01,
                      max_missing=0.15, vr_random=None, min_mac_vr=20.0, is_var_ratio=False,
                      is_diag_one=False):
        sub, mask, vr, nvr = self._geno_args(n_fam, sub_1based, pheno_mask, vr_random)
        self._geno_src = ("setgeno_files", (bed, bim, fam), dict(
            min_maf=min_maf, max_missing=max_missing, vr_random=vr_random, min_mac_vr=min_mac_vr,
            is_var_ratio=is_var_ratio, is_diag_one=is_diag_one), sub, mask, n_fam)
        self._call("sg_setgeno_files", bed.encode(), bim.encode(), fam.encode(), _ptr(sub, L.P_i32),
                   len(sub), _ptr(mask, L.P_u8), min_maf, max_missing, _ptr(vr, L.P_i32), nvr,
                   min_mac_vr, int(is_var_ratio), int(is_diag_one))
        self.n = len(sub)

    def setgeno_device(self, ptr, length, n_fam, m_bim, sub_1based=None, pheno_mask=None,
                       min_maf=0.01, max_missing=0.15, vr_random=None, min_mac_vr=20.0,
                       is_var_ratio=False, is_diag_one=False):
        sub, mask, vr, nvr = self._geno_args(n_fam, sub_1based, pheno_mask, vr_random)
        self._geno_src = ("setgeno_device", (ptr, length, n_fam, m_bim), dict(
            min_maf=min_maf, max_missing=max_missing, vr_random=vr_random, min_mac_vr=min_mac_vr,
            is_var_ratio=is_var_ratio, is_diag_one=is_diag_one), sub, mask)
        self._call("sg_setgeno_device", C.c_void_p(ptr), length, n_fam, m_bim, _ptr(sub, L.P_i32),
                   len(sub), _ptr(mask, L.P_u8), min_maf, max_missing, _ptr(vr, L.P_i32), nvr,
                   min_mac_vr, int(is_var_ratio), int(is_diag_one))
        self.n = len(sub)

    def dims(self):
        v = [C.c_int64() for _ in range(4)]
        self._call("sg_geno_dims", *[C.byref(x) for x in v])
        return dict(n=v[0].value, m_total=v[1].value, m_qc=v[2].value, m_vr=v[3].value)

    def allele_freq(self):
        out = np.empty(self.dims()["m_qc"], np.float32)
        self._call("sg_get_allele_freq", _ptr(out, L.P_f32))
        return out

    def invstd(self):
        out = np.empty(self.dims()["m_qc"], np.float32)
        self._call("sg_get_invstd", _ptr(out, L.P_f32))
        return out

    def mac(self):
        out = np.empty(self.dims()["m_qc"], np.int32)
        self._call("sg_get_mac", _ptr(out, L.P_i32))
        return out

    def qc_marker_mask(self):
        out = np.empty(self.dims()["m_total"], np.uint8)
        self._call("sg_get_qc_marker_mask", _ptr(out, L.P_u8))
        return out.astype(bool)

    def vr_markers(self):
        m = self.dims()["m_vr"]
        f, mac, idx = np.empty(m, np.float32), np.empty(m, np.int32), np.empty(m, np.int32)
        self._call("sg_get_vr_markers", _ptr(f, L.P_f32), _ptr(mac, L.P_i32), _ptr(idx, L.P_i32))
        return f, mac, idx

    def packed_geno(self):
        d = self.dims()
        out = np.empty((d["m_qc"], (d["n"] + 3) // 4), np.uint8)
        self._call("sg_get_packed_geno", _ptr(out, L.P_u8))
        return out

    def onesnp_geno(self, i, vr=False):
        out = np.empty(self.n, np.int32)
        self._call("sg_get_onesnp_geno_vr" if vr else "sg_get_onesnp_geno", i, _ptr(out, L.P_i32))
        return out

    def onesnp_stdgeno(self, i):
        out = np.empty(self.n, np.float32)
        self._call("sg_get_onesnp_stdgeno", i, _ptr(out, L.P_f32))
        return out

    # ------------------------------------------------------------ GRM
    def grm_build(self, precision=GRM_FP32_SIMT):
        self._call("sg_grm_build", int(precision))
        self._grm_prec = int(precision)

    # ------------------------------------------------------------ per-subset cohorts
    def cohort(self):
        """The current cohort (1-based .fam indices and .fam phenotype mask) and GRM settings."""
        src = getattr(self, "_geno_src", None)
        if src is None:
            raise RuntimeError("no genotypes loaded")
        return dict(sub=src[3].copy(), mask=src[4].copy(), grm=getattr(self, "_grm_prec", None),
                    mode=getattr(self, "_mv_mode", None))

    def set_cohort(self, sub_1based, pheno_mask, grm=None, mode=None):
        """Reload the same genotypes for another sample list -- allele frequencies, QC, imputation,
        standardisation and the diagonal are recomputed over it, as setgeno does for the samples
        of one phenotype (FIT.cpp:739-1024) -- then rebuild the GRM and restore the product mode."""
        src = getattr(self, "_geno_src", None)
        if src is None:
            raise RuntimeError("no genotypes loaded")
        kind, args, kw = src[0], src[1], src[2]
        if kind == "setgeno_files":
            self.setgeno_files(*args, sub_1based, src[5], pheno_mask=pheno_mask, **kw)
        else:
            getattr(self, kind)(*args, sub_1based=sub_1based, pheno_mask=pheno_mask, **kw)
        if grm is not None:
            self.grm_build(grm)
        if mode is not None:
            self.set_matvec_mode(mode)

    def subset_cohort(self, keep):
        """Restrict the cohort to the samples where ``keep`` (bool over the current cohort) is
        true and rebuild the GRM with the current settings; returns the previous cohort."""
        prev = self.cohort()
        keep = np.asarray(keep, bool)
        if keep.shape != prev["sub"].shape:
            raise ValueError("keep must cover the %d cohort samples" % len(prev["sub"]))
        sub = prev["sub"][keep]
        fam_mask = np.zeros_like(prev["mask"])
        fam_mask[sub - 1] = prev["mask"][sub - 1]
        self.set_cohort(sub, fam_mask, prev["grm"], prev["mode"])
        return prev

    def grm_padded_n(self):
        """N rounded up to the 128-row tile: the GRM's leading dimension on the device."""
        v = C.c_int64()
        self._call("sg_grm_padded_n", C.byref(v))
        return v.value

    def build_timing(self):
        t = np.zeros(5, np.float64)
        self._call("sg_build_timing", _ptr(t, L.P_f64))
        return dict(qc_ms=t[0], repack_ms=t[1], diag_ms=t[2], zbuild_ms=t[3], syrk_ms=t[4])

    def grm_diag(self):
        out = np.empty(self.n, np.float64)
        self._call("sg_grm_diag", _ptr(out, L.P_f64))
        return out

    def grm_diag_f32(self):
        out = np.empty(self.n, np.float32)
        self._call("sg_grm_diag_f32", _ptr(out, L.P_f32))
        return out

    def grm_get(self):
        out = np.empty((self.n, self.n), np.float32)
        self._call("sg_grm_get", _ptr(out, L.P_f32))
        return out

    def grm_matmul(self, V):
        """K V for V of shape (n,) or (n, k)."""
        V = np.asarray(V, np.float64)
        single = V.ndim == 1
        flat, k = _cols(V)
        flat = _f64(flat)
        out = np.empty(self.n * k, np.float64)
        self._call("sg_grm_matmul", _ptr(flat, L.P_f64), k, _ptr(out, L.P_f64))
        out = out.reshape(k, self.n).T
        return out[:, 0] if single else out

    def loco_set(self, begin, end):
        """Leave GRM markers [begin, end] out (setStartEndIndex); the engine must be idle."""
        self._call("sg_loco_set", int(begin), int(end))

    def loco_set_bim(self, begin, end):
        """Leave the GRM markers inside .bim markers [begin, end] (one chromosome) out: on a resident
        GRM at once; in the subset-exact engines per phenotype, at each slot's next set."""
        self._call("sg_loco_set_bim", int(begin), int(end))

    def loco_clear(self):
        self._call("sg_loco_clear")

    # ------------------------------------------------------------ Rcpp drop-ins
    def getCrossprodMatAndKin(self, b):
        b = _f32(b)
        out = np.empty(self.n, np.float32)
        self._call("sg_getCrossprodMatAndKin", _ptr(b, L.P_f32), _ptr(out, L.P_f32))
        return out

    def getDiagOfSigma(self, w, tau):
        w, tau = _f32(w), _f32(tau)
        out = np.empty(self.n, np.float32)
        self._call("sg_getDiagOfSigma", _ptr(w, L.P_f32), _ptr(tau, L.P_f32), _ptr(out, L.P_f32))
        return out

    def getCrossprod(self, b, w, tau):
        b, w, tau = _f32(b), _f32(w), _f32(tau)
        out = np.empty(self.n, np.float32)
        self._call("sg_getCrossprod", _ptr(b, L.P_f32), _ptr(w, L.P_f32), _ptr(tau, L.P_f32),
                   _ptr(out, L.P_f32))
        return out

    def getPCG1ofSigmaAndVector(self, w, tau, b, maxiterPCG=500, tolPCG=1e-5, return_iters=False):
        w, tau, b = _f32(w), _f32(tau), _f32(b)
        out = np.empty(self.n, np.float32)
        it = C.c_int32()
        self._call("sg_getPCG1ofSigmaAndVector", _ptr(w, L.P_f32), _ptr(tau, L.P_f32), _ptr(b, L.P_f32),
                   int(maxiterPCG), float(tolPCG), _ptr(out, L.P_f32), C.byref(it))
        return (out, it.value) if return_iters else out

    def pcg_solve(self, w, tau, B, maxiterPCG=500, tolPCG=1e-5):
        """FP64 multi-RHS solve; B (n,) or (n, k).  Returns (X, iters)."""
        B = np.asarray(B, np.float64)
        single = B.ndim == 1
        flat, k = _cols(B)
        flat, w, tau = _f64(flat), _f64(w), _f64(tau)
        X = np.empty(self.n * k, np.float64)
        it = np.empty(k, np.int32)
        self._call("sg_pcg_solve", _ptr(w, L.P_f64), _ptr(tau, L.P_f64), _ptr(flat, L.P_f64), k,
                   int(maxiterPCG), float(tolPCG), _ptr(X, L.P_f64), _ptr(it, L.P_i32))
        X = X.reshape(k, self.n).T
        return (X[:, 0], it[0]) if single else (X, it)

    def getSigma_X(self, w, tau, X, maxiterPCG=500, tolPCG=1e-5):
        flat, p = _cols(X)
        flat, w, tau = _f32(flat), _f32(w), _f32(tau)
        out = np.empty(self.n * p, np.float32)
        self._call("sg_getSigma_X", _ptr(w, L.P_f32), _ptr(tau, L.P_f32), _ptr(flat, L.P_f32), p,
                   int(maxiterPCG), float(tolPCG), _ptr(out, L.P_f32))
        return out.reshape(p, self.n).T

    def getSigma_G(self, w, tau, g, maxiterPCG=500, tolPCG=1e-5):
        w, tau, g = _f32(w), _f32(tau), _f32(g)
        out = np.empty(self.n, np.float32)
        self._call("sg_getSigma_G", _ptr(w, L.P_f32), _ptr(tau, L.P_f32), _ptr(g, L.P_f32),
                   int(maxiterPCG), float(tolPCG), _ptr(out, L.P_f32))
        return out

    def getCoefficients(self, Y, X, w, tau, maxiterPCG=500, tolPCG=1e-5):
        Xf, p = _cols(X)
        Y, Xf, w, tau = _f32(Y), _f32(Xf), _f32(w), _f32(tau)
        n = self.n
        SY, SX = np.empty(n, np.float32), np.empty(n * p, np.float32)
        cov, alpha, eta = np.empty(p * p, np.float32), np.empty(p, np.float32), np.empty(n, np.float32)
        self._call("sg_getCoefficients", _ptr(Y, L.P_f32), _ptr(Xf, L.P_f32), p, _ptr(w, L.P_f32),
                   _ptr(tau, L.P_f32), int(maxiterPCG), float(tolPCG), _ptr(SY, L.P_f32),
                   _ptr(SX, L.P_f32), _ptr(cov, L.P_f32), _ptr(alpha, L.P_f32), _ptr(eta, L.P_f32))
        return dict(Sigma_iY=SY, Sigma_iX=SX.reshape(p, n).T, cov=cov.reshape(p, p).T, alpha=alpha,
                    eta=eta)

    def _trace(self, name, Sigma_iX, X, w, tau, cov, nrun, maxiterPCG, tolPCG, cutoff, seed, nout):
        SX, p = _cols(Sigma_iX)
        Xf, _ = _cols(X)
        SX, Xf, w, tau = _f32(SX), _f32(Xf), _f32(w), _f32(tau)
        cv = _f32(np.asarray(cov).ravel(order="F"))
        tr = np.empty(nout, np.float32)
        nr = C.c_int32()
        self._call(name, _ptr(SX, L.P_f32), _ptr(Xf, L.P_f32), p, _ptr(w, L.P_f32), _ptr(tau, L.P_f32),
                   _ptr(cv, L.P_f32), int(nrun), int(maxiterPCG), float(tolPCG), float(cutoff),
                   int(seed), _ptr(tr, L.P_f32), C.byref(nr))
        return tr, nr.value

    def GetTrace(self, Sigma_iX, X, w, tau, cov, nrun=30, maxiterPCG=500, tolPCG=1e-5,
                 traceCVcutoff=0.0025, seed=200):
        tr, nr = self._trace("sg_GetTrace", Sigma_iX, X, w, tau, cov, nrun, maxiterPCG, tolPCG,
                             traceCVcutoff, seed, 1)
        return float(tr[0]), nr

    def GetTrace_q(self, Sigma_iX, X, w, tau, cov, nrun=30, maxiterPCG=500, tolPCG=1e-5,
                   traceCVcutoff=0.0025, seed=200):
        return self._trace("sg_GetTrace_q", Sigma_iX, X, w, tau, cov, nrun, maxiterPCG, tolPCG,
                           traceCVcutoff, seed, 2)

    def _ai_args(self, Y, X, w, tau, Sigma_iY, Sigma_iX, cov):
        Xf, p = _cols(X)
        SX, _ = _cols(Sigma_iX)
        cv = np.asarray(cov).ravel(order="F")
        return [_f32(Y), _f32(Xf), p, _f32(w), _f32(tau), _f32(Sigma_iY), _f32(SX), _f32(cv)]

    def getAIScore(self, Y, X, w, tau, Sigma_iY, Sigma_iX, cov, nrun=30, maxiterPCG=500,
                   tolPCG=1e-5, traceCVcutoff=0.0025, seed=200):
        Y, Xf, p, w, tau, SY, SX, cv = self._ai_args(Y, X, w, tau, Sigma_iY, Sigma_iX, cov)
        out = [C.c_float() for _ in range(3)]
        PY = np.empty(self.n, np.float32)
        self._call("sg_getAIScore", _ptr(Y, L.P_f32), _ptr(Xf, L.P_f32), p, _ptr(w, L.P_f32),
                   _ptr(tau, L.P_f32), _ptr(SY, L.P_f32), _ptr(SX, L.P_f32), _ptr(cv, L.P_f32),
                   int(nrun), int(maxiterPCG), float(tolPCG), float(traceCVcutoff), int(seed),
                   *[C.byref(o) for o in out], _ptr(PY, L.P_f32))
        return dict(YPAPY=out[0].value, Trace=out[1].value, AI=out[2].value, PY=PY)

    def getAIScore_q(self, Y, X, w, tau, Sigma_iY, Sigma_iX, cov, nrun=30, maxiterPCG=500,
                     tolPCG=1e-5, traceCVcutoff=0.0025, seed=200):
        Y, Xf, p, w, tau, SY, SX, cv = self._ai_args(Y, X, w, tau, Sigma_iY, Sigma_iX, cov)
        a, b = C.c_float(), C.c_float()
        tr, AI, PY = np.empty(2, np.float32), np.empty(4, np.float32), np.empty(self.n, np.float32)
        self._call("sg_getAIScore_q", _ptr(Y, L.P_f32), _ptr(Xf, L.P_f32), p, _ptr(w, L.P_f32),
                   _ptr(tau, L.P_f32), _ptr(SY, L.P_f32), _ptr(SX, L.P_f32), _ptr(cv, L.P_f32),
                   int(nrun), int(maxiterPCG), float(tolPCG), float(traceCVcutoff), int(seed),
                   C.byref(a), C.byref(b), _ptr(tr, L.P_f32), _ptr(AI, L.P_f32), _ptr(PY, L.P_f32))
        return dict(YPAPY=a.value, YPA0PY=b.value, Trace=tr, AI=AI.reshape(2, 2).T, PY=PY)

    def fitglmmaiRPCG(self, Y, X, w, tau, Sigma_iY, Sigma_iX, cov, nrun=30, maxiterPCG=500,
                      tolPCG=1e-5, tol=0.02, traceCVcutoff=0.0025, seed=200, quantitative=False):
        Y, Xf, p, w, t, SY, SX, cv = self._ai_args(Y, X, w, tau, Sigma_iY, Sigma_iX, cov)
        t = np.array(t, np.float32)
        self._call("sg_fitglmmaiRPCG_q" if quantitative else "sg_fitglmmaiRPCG", _ptr(Y, L.P_f32),
                   _ptr(Xf, L.P_f32), p, _ptr(w, L.P_f32), _ptr(t, L.P_f32), _ptr(SY, L.P_f32),
                   _ptr(SX, L.P_f32), _ptr(cv, L.P_f32), int(nrun), int(maxiterPCG), float(tolPCG),
                   float(tol), float(traceCVcutoff), int(seed))
        return dict(tau=t)

    # ------------------------------------------------------------ batched engine
    def engine_reserve(self, max_columns, max_phenos):
        self._call("sg_engine_reserve", int(max_columns), int(max_phenos))

    def engine_set_pheno(self, slot, w, tau, mask=None):
        w, tau = _f64(w), _f64(tau)
        m = None if mask is None else np.ascontiguousarray(mask, np.uint8)
        self._call("sg_engine_set_pheno", int(slot), _ptr(w, L.P_f64), _ptr(tau, L.P_f64),
                   None if m is None else _ptr(m, L.P_u8))

    def engine_prepare_subset(self, slot, mask=None):
        """Launch the first half of a slot's subset set-up without waiting (subset-exact engine)."""
        m = None if mask is None else np.ascontiguousarray(mask, np.uint8)
        self._call("sg_engine_prepare_subset", int(slot), None if m is None else _ptr(m, L.P_u8))

    def engine_subset_wait(self, slot):
        self._call("sg_engine_subset_wait", int(slot))

    def engine_subset_vr_markers(self, slot):
        """(bim indices, MAC over the subset) of a set-up slot's variance-ratio markers."""
        n = C.c_int64()
        self._call("sg_engine_subset_vr_markers", int(slot), None, None, 0, C.byref(n))
        idx, mac = np.empty(max(n.value, 1), np.int32), np.empty(max(n.value, 1), np.int32)
        self._call("sg_engine_subset_vr_markers", int(slot), _ptr(idx, L.P_i32), _ptr(mac, L.P_i32), n.value,
                   C.byref(n))
        return idx[:n.value], mac[:n.value]

    def engine_subset_geno(self, slot, marker):
        """Genotypes of a .bim marker for every cohort sample, missing calls at the slot's subset fill."""
        out = np.empty(self.n, np.int32)
        self._call("sg_engine_subset_geno", int(slot), int(marker), _ptr(out, L.P_i32))
        return out

    def engine_forget_subsets(self):
        """Subset-exact engine: rebuild every slot's subset state at its next engine_set_pheno."""
        self._call("sg_engine_forget_subsets")

    def engine_submit(self, slot, kind, B, maxiter=500, tol=1e-5):
        flat, k = _cols(np.asarray(B, np.float64))
        flat = _f64(flat)
        ids = np.empty(k, np.int64)
        self._call("sg_engine_submit", int(slot), int(kind), _ptr(flat, L.P_f64), k, int(maxiter),
                   float(tol), _ptr(ids, L.P_i64))
        return ids

    def engine_submit_probes(self, slot, kind, seed, run0, k, maxiter=500, tol=1e-5):
        ids = np.empty(k, np.int64)
        self._call("sg_engine_submit_probes", int(slot), int(kind), int(seed), int(run0), int(k),
                   int(maxiter), float(tol), _ptr(ids, L.P_i64))
        return ids

    def engine_submit_chained(self, slot, src_ids, maxiter=500, tol=1e-5):
        """PCG solves whose right-hand sides are the results of the requests src_ids."""
        src = np.ascontiguousarray(src_ids, np.int64)
        ids = np.empty(len(src), np.int64)
        self._call("sg_engine_submit_chained", int(slot), _ptr(src, L.P_i64), len(src), int(maxiter), float(tol),
                   _ptr(ids, L.P_i64))
        return ids

    def engine_run(self, max_steps=1 << 30):
        fin = C.c_int64()
        self._call("sg_engine_run", int(max_steps), C.byref(fin))
        return fin.value

    def engine_launch(self):
        """Start one step without waiting; returns (launched, columns retired at admission)."""
        fin = C.c_int64()
        launched = C.c_int32()
        self._call("sg_engine_launch", C.byref(fin), C.byref(launched))
        return bool(launched.value), fin.value

    def engine_finish(self):
        """Wait for the launched step (if any) and retire its columns; returns how many finished."""
        fin = C.c_int64()
        self._call("sg_engine_finish", C.byref(fin))
        return fin.value

    def engine_wait(self):
        """Block until the launched step has run on the device, without finishing it."""
        self._call("sg_engine_wait")

    def engine_fetch(self, rid, out=None):
        x = np.empty(self.n, np.float64) if out is None else out
        it = C.c_int32()
        self._call("sg_engine_fetch", int(rid), _ptr(x, L.P_f64), C.byref(it))
        return x, it.value

    def engine_try_fetch(self, rid, out=None):
        x = np.empty(self.n, np.float64) if out is None else out
        it = C.c_int32()
        rc = self._L.sg_engine_fetch(self._h, int(rid), _ptr(x, L.P_f64), C.byref(it))
        if rc == 4:
            return None
        if rc != 0:
            raise L.SaigeGpuError(rc, self.last_error())
        return x, it.value

    def engine_cancel(self, rid):
        self._call("sg_engine_cancel", int(rid))

    def engine_hold_results(self, hold=True):
        self._call("sg_engine_hold_results", int(bool(hold)))

    def engine_poll(self, max_ids=1 << 16):
        ids = np.empty(max_ids, np.int64)
        n = C.c_int64()
        self._call("sg_engine_poll", _ptr(ids, L.P_i64), int(max_ids), C.byref(n))
        return ids[:n.value]

    def engine_probe_dots(self, slot, ids_pcg, ids_prod, seed, run0, SX):
        """Device-side Hutchinson reductions; returns (dots (k, 2+2p), PCG iterations (k,))."""
        ip = np.ascontiguousarray(ids_pcg, np.int64)
        ia = np.ascontiguousarray(ids_prod, np.int64)
        k = len(ip)
        SXf, p = _cols(np.asarray(SX, np.float64))
        SXf = _f64(SXf)
        out = np.empty(k * (2 + 2 * p), np.float64)
        it = np.empty(k, np.int32)
        self._call("sg_engine_probe_dots", int(slot), _ptr(ip, L.P_i64), _ptr(ia, L.P_i64), k, int(seed),
                   int(run0), _ptr(SXf, L.P_f64), p, _ptr(out, L.P_f64), _ptr(it, L.P_i32))
        return out.reshape(k, 2 + 2 * p), it

    def engine_probe_cache_clear(self, slot=-1):
        self._call("sg_engine_probe_cache_clear", int(slot))

    def engine_probe_cached(self, slot, seed, run):
        return bool(self._L.sg_engine_probe_cached(self._h, int(slot), int(seed), int(run)))

    def engine_timing(self):
        t = np.zeros(6, np.float64)
        self._call("sg_engine_timing", _ptr(t, L.P_f64))
        return dict(step_ms=t[0], gemm_ms=t[1], gemm_launches=int(t[2]), gemm_flops=t[3],
                    gemm_cols=t[4], useful_cols=t[5])

    def engine_reset_timing(self):
        self._call("sg_engine_reset_timing")

    def engine_idle_ms(self):
        """(ms between consecutive engine steps, ms of it from launch admission to the step, host ms
        of finishes after their step drained) since the last timing reset."""
        v = np.zeros(3)
        self._call("sg_engine_idle_ms", _ptr(v, L.P_f64))
        return float(v[0]), float(v[1]), float(v[2])

    def engine_step_trace(self, max_steps=65536):
        """Per-step records since the last timing reset, shape (steps, 8): GRM.V columns, occupied
        columns, GRM.V ms, step ms, idle ms before the step (-1 for the first), host ms from the
        previous finish to this launch (-1 for the first), host ms inside the launch, slot uploads
        the admission waited for."""
        out = np.zeros((max_steps, 8))
        n = C.c_int64()
        self._call("sg_engine_step_trace", _ptr(out, L.P_f64), int(max_steps), C.byref(n))
        return out[:n.value].copy()

    def engine_io_bytes(self):
        """(host->device, device->host) bytes moved by engine calls since the last timing reset."""
        a, b = C.c_uint64(), C.c_uint64()
        self._call("sg_engine_io_bytes", C.byref(a), C.byref(b))
        return a.value, b.value

    def engine_stats(self):
        s = np.zeros(4, np.int64)
        self._call("sg_engine_stats", _ptr(s, L.P_i64))
        return dict(steps=int(s[0]), retired=int(s[1]), column_iterations=int(s[2]), grm_passes=int(s[3]))

    # ------------------------------------------------------------ synthetic cohorts
    def synth_bed(self, seed, n, m, miss_rate):
        p, ln = C.c_void_p(), C.c_uint64()
        self._call("sg_synth_bed", int(seed), int(n), int(m), float(miss_rate), C.byref(p), C.byref(ln))
        return p.value, ln.value

    def synth_bed_to_host(self, length):
        out = np.empty(length, np.uint8)
        self._call("sg_synth_bed_to_host", _ptr(out, L.P_u8), int(length))
        return out

    def synth_genetic_value(self, seed):
        out = np.empty(self.n, np.float64)
        self._call("sg_synth_genetic_value", int(seed), _ptr(out, L.P_f64))
        return out
