"""PLINK .bed decode, per-marker QC and standardisation (oracle).

Restates ``genoClass`` of FIT.cpp (src/SAIGE/src/SAIGE_fitGLMM_fast.cpp):

* bit map ``Get_OneSNP_Geno_atBeginning`` FIT.cpp:346-357 -- with b = bit0,
  a = bit1 of each 2-bit field: 00 -> 2, 01 -> missing, 10 -> 1, 11 -> 0
  (it counts the A1 allele);
* counts over samples flagged in ``indicatorGenoSamplesWithPheno`` only
  (FIT.cpp:376-385);
* first frequency over non-missing, integer fill ``int(round(2p))``,
  ``alleleCount += fill * nMissing`` and the second frequency over all
  ``Nnomissing`` samples (FIT.cpp:436-484), all in float32 like the reference;
* QC ``min(p,1-p) >= minMAF && missingRate <= maxMissing`` (FIT.cpp:490-495);
  variance-ratio markers (MAC >= minMAC and in a given random set) leave the
  GRM (FIT.cpp:521-547);
* re-pack of the GRM markers in ``subSampleInGeno`` (1-based) order with the
  missing calls replaced by the fill value (FIT.cpp:551-575);
* ``Std = sqrt(2p(1-p))``, ``invStd = 1/Std`` or 0 (FIT.cpp:916-921, float);
* 3-entry standardisation LUT ``(g - 2p) * invStd`` (FIT.cpp:152-159) and the
  GRM diagonal ``sum_m z^2`` (``Get_Diagof_StdGeno`` FIT.cpp:665-704).
"""
import numpy as np

# 2-bit PLINK field value -> reference genotype code (3 = missing)
BED_LUT = np.array([2, 3, 1, 0], dtype=np.uint8)
# genotype 0/1/2 -> 2-bit field of the re-packed GRM genotypes
# (setGenotype with HOM_ALT=3, HET=2, HOM_REF=0; FIT.cpp:40-44, 560-566)
PACK_CODE = np.array([3, 2, 0], dtype=np.uint8)


def bed_bytes_per_marker(n):
    return (n + 3) // 4


def decode_marker(raw, n):
    """Decode one marker's ceil(n/4) bytes to n codes in {0,1,2,3=missing}."""
    raw = np.asarray(raw, dtype=np.uint8)
    fields = np.stack([(raw >> (2 * j)) & 3 for j in range(4)], axis=1).reshape(-1)
    return BED_LUT[fields[:n]]


def decode_bed(bed, n, m):
    """Decode a whole .bed (bytes incl. the 3-byte magic) to an (m, n) code array."""
    buf = np.frombuffer(bed, dtype=np.uint8) if isinstance(bed, (bytes, bytearray)) else np.asarray(bed, np.uint8)
    assert buf[0] == 0x6C and buf[1] == 0x1B and buf[2] == 0x01, "not a SNP-major PLINK .bed"
    nb = bed_bytes_per_marker(n)
    body = buf[3:3 + nb * m].reshape(m, nb)
    fields = np.stack([(body >> (2 * j)) & 3 for j in range(4)], axis=2).reshape(m, nb * 4)
    return BED_LUT[fields[:, :n]]


def _round_half_away(x32):
    # std::round on a non-negative float: floor(x + 0.5) evaluated exactly
    return int(np.floor(np.float64(x32) + 0.5))


class GenoResult:
    """What ``setGenoObj`` leaves behind for the GRM markers (and VR markers)."""


def setgeno(bed, n_fam, m_bim, sub_1based, pheno_mask, min_maf=0.01, max_miss=0.15,
            vr_random_set=None, min_mac_vr=20.0, is_var_ratio=False, max_mac_vr=-1.0):
    """Restatement of ``genoClass::setGenoObj`` (FIT.cpp:739-1024).

    ``max_mac_vr`` != -1: categorical variance-ratio markers (g_maxMACVarRatio, FIT.cpp:497-518):
    every marker with min_mac_vr <= MAC < max_mac_vr, and the random set's markers from max_mac_vr up.

    Returns a ``GenoResult`` with: ``codes`` (m_qc, nn) genotype 0/1/2 of the
    GRM markers in sub-sample order (missing already filled), ``freq``,
    ``invstd`` (float32), ``mac`` (int), ``qc_mask`` (m_bim bools),
    and the same for the variance-ratio markers (``vr_*``).
    """
    codes_all = decode_bed(bed, n_fam, m_bim)  # (m, n)
    sub0 = np.asarray(sub_1based, dtype=np.int64) - 1
    nn = len(sub0)
    mask = np.asarray(pheno_mask, dtype=bool)
    vr_set = set() if vr_random_set is None else set(int(v) for v in vr_random_set)

    out_codes, freqs, invstds, macs, qc = [], [], [], [], []
    vr_codes, vr_freqs, vr_invstds, vr_macs, vr_idx = [], [], [], [], []
    f32 = np.float32
    for i in range(m_bim):
        c = codes_all[i]
        cm = c[mask]
        n_miss = int(np.count_nonzero(cm == 3))
        allele = int(cm[cm != 3].astype(np.int64).sum())
        with np.errstate(divide="ignore", invalid="ignore"):
            alt = f32(allele) / f32((nn - n_miss) * 2)
        miss_rate = f32(n_miss) / f32(nn)
        fill = _round_half_away(f32(2) * alt) if np.isfinite(alt) else 0
        if n_miss > 0:
            allele = allele + fill * n_miss
        alt = f32(allele) / f32(nn * 2)
        maf = min(alt, f32(1) - alt)
        mac = min(allele, nn * 2 - allele)
        pass_qc = bool(maf >= f32(min_maf) and miss_rate <= f32(max_miss))
        pass_vr = False
        if is_var_ratio and max_mac_vr != -1.0:
            if min_mac_vr <= mac < max_mac_vr:
                pass_vr = True
            elif mac >= max_mac_vr:
                pass_vr = i in vr_set
        elif is_var_ratio and mac >= min_mac_vr:
            pass_vr = i in vr_set
        if pass_vr:
            pass_qc = False
        qc.append(pass_qc)
        if pass_qc or pass_vr:
            g = c[sub0].copy()
            g[g == 3] = fill
            std = np.sqrt(f32(2) * alt * (f32(1) - alt))
            inv = f32(0) if std == 0 else f32(1) / std
            if pass_qc:
                out_codes.append(g.astype(np.uint8)); freqs.append(alt); invstds.append(inv); macs.append(mac)
            if pass_vr:
                vr_codes.append(g.astype(np.uint8)); vr_freqs.append(alt); vr_invstds.append(inv)
                vr_macs.append(mac); vr_idx.append(i)
    r = GenoResult()
    r.n = nn
    r.codes = np.array(out_codes, dtype=np.uint8).reshape(-1, nn)
    r.freq = np.array(freqs, dtype=np.float32)
    r.invstd = np.array(invstds, dtype=np.float32)
    r.mac = np.array(macs, dtype=np.int64)
    r.qc_mask = np.array(qc, dtype=bool)
    r.vr_codes = np.array(vr_codes, dtype=np.uint8).reshape(-1, nn)
    r.vr_freq = np.array(vr_freqs, dtype=np.float32)
    r.vr_invstd = np.array(vr_invstds, dtype=np.float32)
    r.vr_mac = np.array(vr_macs, dtype=np.int64)
    r.vr_index = np.array(vr_idx, dtype=np.int64)
    return r


def pack_codes(codes):
    """Re-pack (m, nn) genotypes 0/1/2 to the reference's 2-bit layout (m, ceil(nn/4))."""
    m, nn = codes.shape
    nb = bed_bytes_per_marker(nn)
    f = np.zeros((m, nb * 4), dtype=np.uint8)
    f[:, :nn] = PACK_CODE[codes]
    f = f.reshape(m, nb, 4)
    return (f[:, :, 0] | (f[:, :, 1] << 2) | (f[:, :, 2] << 4) | (f[:, :, 3] << 6)).astype(np.uint8)


def std_lut(freq, invstd):
    """(m, 3) float32 LUT (g - 2p) * invStd exactly as setStdGenoLookUpArr (FIT.cpp:152-159)."""
    freq = np.asarray(freq, np.float32)
    invstd = np.asarray(invstd, np.float32)
    p2 = np.float32(2) * freq
    g = np.arange(3, dtype=np.float32)[None, :]
    return ((g - p2[:, None]).astype(np.float32) * invstd[:, None]).astype(np.float32)


def std_geno(geno):
    """Standardised genotype matrix Z (m_qc, nn) float32 as Get_OneSNP_StdGeno (FIT.cpp:582-662)."""
    lut = std_lut(geno.freq, geno.invstd)
    return np.take_along_axis(lut, geno.codes.astype(np.int64), axis=1)


def diag_std_geno(geno, dtype=np.float64):
    """sum_m z_m^2 per sample (``Get_Diagof_StdGeno`` FIT.cpp:665-704)."""
    z = std_geno(geno).astype(dtype)
    return (z * z).sum(axis=0)


def diag_std_geno_f32(geno):
    """FP32 ``m_DiagStd + z % z`` accumulated marker by marker, as the reference does."""
    z = std_geno(geno)
    acc = np.zeros(z.shape[1], np.float32)
    for m in range(z.shape[0]):
        acc = (acc + (z[m] * z[m]).astype(np.float32)).astype(np.float32)
    return acc
