"""GPU genotype decode / QC / re-pack / diagonal: bit-exact against the oracle."""
import numpy as np
import pytest

from oracle import plink
from saigegpu import synth

pytestmark = pytest.mark.gpu


def _check(ctx, bed, n_fam, m, sub, mask, min_maf=0.01, max_miss=0.15, vr=None, vr_on=False):
    ctx.setgeno(bed, n_fam, m, sub, mask, min_maf, max_miss, vr, 20.0, vr_on)
    o = plink.setgeno(bed, n_fam, m, sub, mask.astype(bool), min_maf, max_miss, vr, 20.0, vr_on)
    d = ctx.dims()
    assert d["m_qc"] == o.codes.shape[0] and d["n"] == len(sub)
    np.testing.assert_array_equal(ctx.qc_marker_mask(), o.qc_mask)
    np.testing.assert_array_equal(ctx.allele_freq().view(np.uint32), o.freq.view(np.uint32))
    np.testing.assert_array_equal(ctx.invstd().view(np.uint32), o.invstd.view(np.uint32))
    np.testing.assert_array_equal(ctx.mac(), o.mac)
    np.testing.assert_array_equal(ctx.packed_geno(), plink.pack_codes(o.codes))
    np.testing.assert_array_equal(ctx.grm_diag_f32().view(np.uint32), plink.diag_std_geno_f32(o).view(np.uint32))
    np.testing.assert_allclose(ctx.grm_diag(), plink.diag_std_geno(o), rtol=1e-12)
    if o.codes.shape[0]:
        j = o.codes.shape[0] // 2
        np.testing.assert_array_equal(ctx.onesnp_geno(j), o.codes[j])
        np.testing.assert_array_equal(ctx.onesnp_stdgeno(j).view(np.uint32),
                                      plink.std_geno(o)[j].view(np.uint32))
    if vr_on:
        f, mac, idx = ctx.vr_markers()
        np.testing.assert_array_equal(idx, o.vr_index)
        np.testing.assert_array_equal(mac, o.vr_mac)
    return o


def test_golden_bed_bit_exact(gpu_ctx, golden_plink):
    bed, n, m, _ = golden_plink
    _check(gpu_ctx, bed, n, m, np.arange(1, n + 1), np.ones(n, np.uint8))


def test_subset_shuffled_order_missing_and_vr(gpu_ctx):
    n, m = 203, 301  # n % 4 != 0, n % 16 != 0
    bed, _ = synth.synth_bed(11, n, m, 0.05)
    rng = np.random.default_rng(4)
    sub = rng.permutation(np.arange(1, n + 1))[:171].astype(np.int32)
    mask = np.zeros(n, np.uint8)
    mask[sub - 1] = 1
    vr = rng.choice(m, 60, replace=False)
    _check(gpu_ctx, bed, n, m, sub, mask, 0.02, 0.1, vr, True)


def test_edge_sizes(gpu_ctx):
    for n, m in [(1, 3), (5, 17), (67, 2), (129, 64)]:
        bed, _ = synth.synth_bed(5 + n, n, m, 0.2)
        _check(gpu_ctx, bed, n, m, np.arange(1, n + 1), np.ones(n, np.uint8), 0.0, 1.0)


def test_device_synthetic_bed_matches_cpu_recipe(gpu_ctx):
    for n, m, miss in [(1001, 37, 0.02), (64, 5, 0.0), (7, 3, 0.5)]:
        ptr, ln = gpu_ctx.synth_bed(123, n, m, miss)
        dev = gpu_ctx.synth_bed_to_host(ln).tobytes()
        cpu, _ = synth.synth_bed(123, n, m, miss)
        assert dev == cpu
        gpu_ctx.setgeno_device(ptr, ln, n, m, min_maf=0.0, max_missing=1.0)
        assert gpu_ctx.dims()["m_total"] == m


def test_bad_inputs_raise(gpu_ctx):
    from saigegpu import SaigeGpuError
    with pytest.raises(SaigeGpuError):
        gpu_ctx.setgeno(b"\x00\x00\x00" + bytes(10), 4, 10)
    bed, _ = synth.synth_bed(1, 8, 4, 0.0)
    with pytest.raises(SaigeGpuError):
        gpu_ctx.setgeno(bed, 8, 4, np.array([0, 1], np.int32))
    with pytest.raises(SaigeGpuError):
        gpu_ctx.setgeno(bed[:-1], 8, 4)
