"""Generate the golden fixtures under tests/golden/ from the reference project's example data.

Run with the path of a (read-only) checkout of the reference project:

    python tests/golden/make_golden.py <reference checkout>

It writes (all derived from ``src/SAIGE/extdata``):

* ``plink_1000x10k.bed.gz``  -- the example PLINK genotypes
  (``input/plinkforGRM_1000samples_10kMarkers.bed``), gzip'd verbatim;
* ``plink_1000x10k_frq.npy``  -- PLINK's A1 MAF column of the matching ``.frq``
  (known-answer test for the decode);
* ``pheno_1000.npz``          -- y_binary, y_quantitative, x1, x2 of
  ``input/pheno_1000samples.txt_withdosages_withBothTraitTypes.txt`` in .fam order;
* ``golden_fits.json``        -- theta, coefficients and the first fitted
  values of ``output/example_binary_fullGRM.rda``, ``example_binary.rda`` and
  ``example_quantitative_fullGRM.rda`` plus the null variance ratios of the
  matching ``.varianceRatio.txt`` files;
* ``example_binary_includenonAutoforvarRatio.rda`` and
  ``example_binary_includenonAutoforvarRatio_FemaleOnly.rda`` -- those step-1
  model files, verbatim (R's own serialisation, for the byte-exact round trip of
  ``saigegpu.rdata``; the second holds closures, environments, a namespace,
  promises, calls and byte code);
* ``model_schema_binary_fullGRM.json`` -- the layout (``saigegpu.rdata.schema``)
  of ``example_binary_fullGRM.rda``'s model: field names, types, shapes,
  attributes and classes, with its LOCO results;
* ``binary_fullGRM_model.npz`` -- that model's y, design X (after the QR
  covariate transform) and its column names, sample IDs, covariate offset,
  fitted values and obj.noK arrays (ScoreTest_NULL_Model, FIT.R:579-591), which
  do not depend on the GRM;
* ``pheno_1000samples.txt`` and ``samples_1000.fam`` -- the example phenotype
  file and .fam, verbatim, for the phenotype preamble (prep.read_phenotypes).

The ``.rda`` files are R serialisation (XDR, version 2/3) of a list whose
first seven elements are theta, coefficients, linear.predictors,
fitted.values, Y, residuals and cov (FIT.R:220-236); ``_RReader`` below reads
just enough of the format to reach them.
"""
import gzip
import json
import os
import shutil
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "saige-gpu_gb300"))


class _RReader:
    """Minimal reader of R's XDR serialisation: enough for numeric lists."""

    def __init__(self, data):
        self.b = data
        self.o = 0
        self.refs = []

    def _int(self):
        v = struct.unpack_from(">i", self.b, self.o)[0]
        self.o += 4
        return v

    def _len(self):
        n = self._int()
        if n == -1:
            hi, lo = self._int(), self._int()
            n = (hi << 32) + lo
        return n

    def header(self):
        assert self.b[:5] in (b"RDX2\n", b"RDX3\n"), self.b[:5]
        self.o = 5
        assert self.b[self.o:self.o + 2] == b"X\n"
        self.o += 2
        version = self._int()
        self._int(); self._int()
        if version == 3:
            n = self._int()
            self.o += n

    def item(self, max_vec=None):
        flags = self._int()
        t = flags & 0xFF
        has_attr = bool(flags & (1 << 9))
        has_tag = bool(flags & (1 << 10))
        if t == 254:  # NILVALUE
            return None
        if t in (253, 252, 251, 250, 242, 241):
            return ("special", t)
        if t == 255:  # REFSXP
            idx = flags >> 8
            if idx == 0:
                idx = self._int()
            return self.refs[idx - 1]
        if t == 1:  # SYMSXP
            name = self.item()
            self.refs.append(("sym", name))
            return ("sym", name)
        if t in (2, 6, 3, 5, 17, 240, 239):  # pairlist-like
            attr = self.item() if has_attr else None
            tag = self.item() if has_tag else None
            car = self.item()
            cdr = self.item()
            return ("pair", tag, car, cdr, attr)
        if t == 4:  # ENVSXP
            self._int()
            env = ["env"]
            self.refs.append(env)
            for _ in range(4):
                env.append(self.item())
            return env
        if t == 9:  # CHARSXP
            n = self._int()
            if n == -1:
                return None
            s = self.b[self.o:self.o + n].decode("utf-8", "replace")
            self.o += n
            return s
        if t in (10, 13):
            n = self._len()
            v = np.frombuffer(self.b, dtype=">i4", count=n, offset=self.o).astype(np.int64)
            self.o += 4 * n
        elif t == 14:
            n = self._len()
            v = np.frombuffer(self.b, dtype=">f8", count=n, offset=self.o).astype(np.float64)
            self.o += 8 * n
        elif t == 16:
            n = self._len()
            v = [self.item() for _ in range(n)]
        elif t in (19, 20):
            n = self._len()
            k = n if max_vec is None else min(n, max_vec)
            v = [self.item() for _ in range(k)]
            if k < n:
                return ("vec_prefix", v)
        elif t == 24:
            n = self._len()
            v = self.b[self.o:self.o + n]
            self.o += n
        else:
            raise NotImplementedError("R type %d" % t)
        attr = self.item() if has_attr else None
        return ("val", t, v, attr)


def read_rda_prefix(path, k=7):
    data = gzip.open(path, "rb").read()
    r = _RReader(data)
    r.header()
    top = r.item(max_vec=None) if False else None
    # top-level pairlist: flags, tag, then the object
    flags = r._int()
    assert flags & 0xFF == 2
    if flags & (1 << 9):
        r.item()
    if flags & (1 << 10):
        r.item()
    obj = r.item(max_vec=k)
    assert obj[0] == "vec_prefix"
    out = []
    for it in obj[1]:
        out.append(np.asarray(it[2], np.float64))
    return out


def main(ref_root):
    ext = os.path.join(ref_root, "src", "SAIGE", "extdata")
    inp = os.path.join(ext, "input")
    outp = os.path.join(ext, "output")
    stem = os.path.join(inp, "plinkforGRM_1000samples_10kMarkers")
    bed = open(stem + ".bed", "rb").read()
    with open(os.path.join(HERE, "plink_1000x10k.bed.gz"), "wb") as raw, \
            gzip.GzipFile(fileobj=raw, mode="wb", compresslevel=9, mtime=0) as f:
        f.write(bed)
    fam = [l.split()[1] for l in open(stem + ".fam")]
    bim_n = sum(1 for _ in open(stem + ".bim"))
    frq = [l.split() for l in open(stem + ".frq")][1:]
    maf = np.array([float(r[4]) for r in frq], dtype=np.float64)
    np.save(os.path.join(HERE, "plink_1000x10k_frq.npy"), maf)

    ph = [l.split() for l in open(os.path.join(inp, "pheno_1000samples.txt_withdosages_withBothTraitTypes.txt"))]
    hdr, rows = ph[0], ph[1:]
    col = {h: i for i, h in enumerate(hdr)}
    by_iid = {r[col["IID"]]: r for r in rows}
    sel = [by_iid[i] for i in fam]
    np.savez(os.path.join(HERE, "pheno_1000.npz"),
             y_binary=np.array([float(r[col["y_binary"]]) for r in sel]),
             y_quantitative=np.array([float(r[col["y_quantitative"]]) for r in sel]),
             x1=np.array([float(r[col["x1"]]) for r in sel]),
             x2=np.array([float(r[col["x2"]]) for r in sel]),
             n_fam=len(fam), m_bim=bim_n)

    names = ["theta", "coefficients", "linear_predictors", "fitted_values", "Y", "residuals", "cov"]
    golden = {}
    for f in ["example_binary_fullGRM", "example_binary", "example_quantitative_fullGRM"]:
        vals = read_rda_prefix(os.path.join(outp, f + ".rda"))
        d = {nm: v.ravel().tolist() for nm, v in zip(names, vals) if nm in ("theta", "coefficients", "cov")}
        d["linear_predictors_head"] = vals[2].ravel()[:50].tolist()
        d["fitted_values_head"] = vals[3].ravel()[:50].tolist()
        d["linear_predictors_mean"] = float(vals[2].mean())
        golden[f] = d
    vr = {}
    for f in ["example_binary_fullGRM", "example_binary", "example_quantitative"]:
        p = os.path.join(outp, f + ".varianceRatio.txt")
        rows = [l.split() for l in open(p) if l.strip()]
        vr[f] = [float(r[0]) for r in rows if len(r) > 1 and r[1] == "null"]
    golden["variance_ratio_null"] = vr
    with open(os.path.join(HERE, "golden_fits.json"), "w") as f:
        json.dump(golden, f, indent=1)

    from saigegpu import rdata
    for f in ("example_binary_includenonAutoforvarRatio.rda", "example_binary_includenonAutoforvarRatio_FemaleOnly.rda"):
        shutil.copyfile(os.path.join(outp, f), os.path.join(HERE, f))
    _, objs = rdata.read_rda(os.path.join(outp, "example_binary_fullGRM.rda"))
    with open(os.path.join(HERE, "model_schema_binary_fullGRM.json"), "w") as f:
        json.dump(rdata.schema(dict(objs)["modglmm"]), f, separators=(",", ":"))
    from saigegpu import output
    mod = output.read_model_rda(os.path.join(outp, "example_binary_fullGRM.rda"))
    nk = mod["obj.noK"]
    xnames = dict(objs)["modglmm"]["X"].attr("dimnames").value[1].value
    np.savez_compressed(os.path.join(HERE, "binary_fullGRM_model.npz"), y=mod["y"], X=mod["X"],
                        X_names=np.array(xnames), sample_ids=np.array(mod["sampleID"]),
                        offset=np.ravel(mod["offset"]), mu=np.ravel(mod["fitted.values"]),
                        theta=mod["theta"], **{"noK_" + k: np.asarray(v) for k, v in nk.items()})
    shutil.copyfile(os.path.join(inp, "pheno_1000samples.txt_withdosages_withBothTraitTypes.txt"),
                    os.path.join(HERE, "pheno_1000samples.txt"))
    shutil.copyfile(stem + ".fam", os.path.join(HERE, "samples_1000.fam"))
    print("wrote fixtures to", HERE)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <reference checkout>")
    main(sys.argv[1])
