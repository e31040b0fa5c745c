"""Benchmark: null-model fits/hr at N=100k on a resident GRM (batched mixed precision).

Workload (the batching form of the metric, on the precision form's cohort):
N = 100,000 samples x M = 150,000 markers synthetic cohort (p ~ U(0.01,0.5),
HWE genotypes, 2% missing; seed 1003), GRM built once on the GPU (decode ->
BF16 standardised genotypes -> tcgen05 SYRK, FP32 K resident in HBM).  One
step = one batch of P null-model fits run to convergence through the batched
engine: P = 64 phenotypes, half binary (prevalence U(0.05,0.3)), half
quantitative (h2 U(0.1,0.6)), each with a sample mask dropping U(5%,40%) of the
cohort, 2 covariates, y + 30 Rademacher probes per trace, split-BF16 tcgen05
GRM.V (--mode) with FP64 PCG recurrences; the driver overlaps its host work with
the next engine step (--blocking-runner turns that off).

value  = fits/hr over the device-busy time of the engine steps (CUDA events on
         the engine stream), i.e. with the inputs resident in HBM;
e2e    = fits/hr by wall clock through the C ABI with host buffers (phenotype
         vectors H2D, solutions D2H every step);
roofline: the dominant kernel (the tcgen05 GRM.V) -- algorithmic bytes per
         pass over the split GRM (4 B per stored element for BF16 halves, 8 B
         for TF32 halves, + 8-12 B per RHS entry) or its tensor FLOPs (three
         products), whichever bounds it, over its event-timed duration;
reference_gpu_algorithm: the reference's K.x (two cuBLAS SGEMV over the FP32
         N x M genotype matrix, one RHS) timed on the same GPU, extrapolated;
cpu_baseline: the reference's CPU GRM.x (oracle/cpu_ref.c, OpenMP, all host
         cores) timed on a bounded sample, extrapolated to fits/hr with the
         measured PCG iterations per fit;
plain: the plain FP64 single-RHS PCG path on the same GPU, timed per iteration
         and extrapolated the same way.

``--impl reference`` times the reference's CPU path (the oracle's C
restatement) on the host cores only.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "saige-gpu_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "null-model fits/hr at N=100k (batched mixed-prec vs plain FP64 PCG); p50/p99"
# PCG column-iterations per fit of this workload (N = 100k, M = 150k, 64 phenotypes), measured by the
# GPU arm (its line reports the value of each run under per_fit); the reference arm extrapolates its
# per-product CPU time with this fixed count
PCG_COLUMN_ITERATIONS_PER_FIT = 513.9


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=100_000)
    ap.add_argument("--m", type=int, default=150_000)
    ap.add_argument("--phenos", type=int, default=64)
    ap.add_argument("--miss", type=float, default=0.02)
    ap.add_argument("--seed", type=int, default=1003)
    ap.add_argument("--mode", default="subset", choices=["subset", "subset8", "bf16x3", "tf32x3", "tf32", "fp32"],
                    help="GRM.V engine: subset = each phenotype's GRM from its own samples (the reference's "
                         "setgeno per phenotype; genotype GEMMs of BF16 halves), subset8 = the same with FP16 "
                         "high and E4M3 low halves; the others restrict the cohort GRM to the phenotype's "
                         "samples (an approximation for masked phenotypes)")
    ap.add_argument("--grm", default="bf16x3", choices=["bf16x3", "bf16"],
                    help="GRM build of the cohort-GRM engines: split-BF16 standardised genotypes (four "
                         "products) or BF16 (one)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="skip the tcgen05 shape autotuner")
    ap.add_argument("--no-ref-gpu", action="store_true",
                    help="skip timing the reference's two-SGEMV K.x algorithm on this GPU")
    ap.add_argument("--driver", default="native", choices=["native", "python"],
                    help="fit driver: C++ (sg_fits_*) or the Python generators of saigegpu.serve")
    ap.add_argument("--workers", type=int, default=None,
                    help="host threads for the fits' driver math (default: native driver half the cores, "
                         "at most 8; Python driver 1)")
    ap.add_argument("--launch-wait-ms", type=float, default=None,
                    help="native driver: how long a launch may wait for the fits the last step made ready "
                         "(default: the library's)")
    ap.add_argument("--blocking-runner", action="store_true",
                    help="step the engine synchronously instead of overlapping the driver with the next step")
    ap.add_argument("--serve-requests", type=int, default=32,
                    help="requests of the serving-form block (Poisson arrivals, 0 = skip)")
    ap.add_argument("--loco-chroms", type=int, default=0,
                    help="after the timed steps, Get_Coef_LOCO of the last batch's phenotypes with this many "
                         "chromosomes (22 blocks of the .bim markers) left out in turn, timed (0 = skip)")
    ap.add_argument("--json-out", default=None)
    return ap.parse_args()


# ------------------------------------------------------------------ distributed plumbing (replicas)
def dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allsum(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# ------------------------------------------------------------------ clocks sampler
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if len(r) > 5 + k and r[5 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


# ------------------------------------------------------------------ workload
def make_specs(ctx, args, rng_seed, batch=0):
    """P phenotypes over the cohort: half binary, half quantitative, sample masks 5-40% dropped;
    ``batch`` gives a distinct set of phenotypes (traits, masks) from the same generator."""
    from saigegpu import prep, serve, synth
    n = ctx.n
    rng = np.random.default_rng(rng_seed)
    gvs = [ctx.synth_genetic_value(args.seed * 7 + k) for k in range(2)]
    specs = []
    for k in range(args.phenos):
        trait = "binary" if k % 2 == 0 else "quantitative"
        gv = gvs[k % 2] * rng.choice([-1, 1]) + 0.3 * gvs[(k + 1) % 2]
        gv = gv / gv.std()
        drop = rng.uniform(0.05, 0.40)
        mask = rng.uniform(size=n) > drop
        S = np.nonzero(mask)[0]
        y, C = synth.simulate_pheno(gv, args.seed * 100 + 1000 * batch + k, trait, tau=0.3,
                                    prevalence=rng.uniform(0.05, 0.3), h2=rng.uniform(0.1, 0.6))
        f0 = prep.make_fit0(y[S], C[S], trait, True)
        specs.append(serve.FitSpec(f0, trait, mask=mask, name="pheno%d" % k))
    return specs


def run_batch(ctx, specs, cols, pipelined=True, workers=None, driver="native", launch_wait_ms=None,
              max_phenos=None):
    from saigegpu import MV_SUBSET_EXACT, native, serve
    if ctx.matvec_mode() == MV_SUBSET_EXACT:
        # every batch sets its phenotypes' subsets up from scratch (QC, fill, 1/sd, fill-change map
        # and diagonal over each subset), as new phenotypes would, inside the timed region
        ctx.engine_forget_subsets()
    t0 = time.perf_counter()
    if driver == "native":
        res, jobs = native.fit_batch(ctx, specs, max_columns=cols, max_phenos=max_phenos, pipelined=pipelined,
                                     threads=workers, launch_wait_ms=launch_wait_ms)
    else:
        res, jobs = serve.fit_batch(ctx, specs, max_columns=cols, max_phenos=max_phenos, pipelined=pipelined,
                                    workers=workers)
    wall = time.perf_counter() - t0
    errs = [r for r in res if isinstance(r, Exception)]
    if errs:
        raise errs[0]
    return res, jobs, wall


# DRAM traffic of the split-BF16 GRM.V over its algorithmic bytes, from ncu on a smaller case
# (dram__bytes_read.sum + dram__bytes_write.sum of two launches at N = 24,576)
GRMV_TRAFFIC_RATIO = 1.023
# the same for the subset-exact GRM.V: ncu DRAM bytes of its two genotype GEMMs at N = 30,080,
# M_g = 45,056, 192 columns (2.813 + 2.798 GB) over that launch's algorithmic bytes (5.536 GB)
SUBSET_TRAFFIC_RATIO = 1.014
SUBSET_TRAFFIC_BASIS = ("ncu DRAM bytes of both genotype GEMMs of a 192-column launch at N = 30,080, M_g = 45,056 "
                        "over its algorithmic bytes (1.014), times this launch's algorithmic bytes")
GRMV_TRAFFIC_BASIS = ("ncu DRAM bytes of two N=24576 launches (224 and 512 columns) over their algorithmic bytes "
                      "(1.008, 1.037; mean 1.023), times this launch's algorithmic bytes")


def subset_roofline(peaks, t_dev, np_, mg, f8=False):
    """Roofline of the subset-exact engine's GRM.V (two genotype GEMMs and the small kernels around
    them, timed together by the engine's CUDA events).  Algorithmic work per launch over C columns:
    bytes = the genotype matrix read by both GEMMs (2 B per sample and marker each) + the centred
    vector halves and T' halves read (4 B each per entry) + T and U written (4 B); FLOPs = two
    GEMMs of 2 N_p M_g per column (one product each, as the reference's two SGEMVs per K.x,
    gpuSymMatMult.cu:211-252).  ``executed``: two BF16 products per GEMM."""
    launches = max(1, t_dev["gemm_launches"])
    ms = t_dev["gemm_ms"] / launches
    cols = t_dev["gemm_cols"] / launches
    bytes_alg = 2.0 * 2.0 * np_ * mg + 8.0 * (np_ + mg) * cols
    flops_alg = 2.0 * 2.0 * np_ * mg * cols
    # executed tensor work in BF16-product equivalents: two BF16 products, or one FP16 product plus one
    # E4M3 product at twice the rate
    prod = 1.5 if f8 else 2.0
    hbm = peaks.get("hbm_gbs", 6800.0)
    tc_peak = peaks.get("bf16_tflops_sustained", 1700.0)
    t = ms * 1e-3
    a_bw = bytes_alg / t / 1e9
    a_tc = flops_alg / t / 1e12
    common = {"traffic": None if f8 else round(SUBSET_TRAFFIC_RATIO * bytes_alg),
              "traffic_basis": None if f8 else SUBSET_TRAFFIC_BASIS,
              "kernel": ("tc_gemm_kernel<fp16 + e4m3, kSplitB8>" if f8 else "tc_gemm_kernel<bf16, kSplitB>")
                        + " x 2 (G'V, G T') + subset kernels",
              "per_launch_ms": round(ms, 3), "columns_per_launch": round(cols, 1),
              "algorithmic_bytes_per_launch": bytes_alg, "algorithmic_flops_per_launch": flops_alg,
              "algorithmic_basis": "bytes: G read by both GEMMs + vector halves read + T and U written; "
                                   "FLOPs: 2 GEMMs x 2 N_p M_g per column",
              "executed": {"products": prod, "tensor_flops_per_launch": prod * flops_alg,
                           "tflops": round(prod * a_tc, 1), "peak": tc_peak,
                           "frac": round(prod * a_tc / tc_peak, 4),
                           "peak_source": "measured bf16_tflops_sustained (MEASURED_PEAKS.json)"}}
    if a_bw / hbm >= a_tc / tc_peak:
        return dict({"bound": "hbm", "achieved": round(a_bw, 1), "peak": hbm, "unit": "GB/s",
                     "frac": round(a_bw / hbm, 4), "peak_source": "measured hbm_gbs (MEASURED_PEAKS.json)"},
                    **common)
    return dict({"bound": "tensor", "achieved": round(a_tc, 1), "peak": tc_peak, "unit": "TFLOP/s",
                 "frac": round(a_tc / tc_peak, 4),
                 "peak_source": "measured bf16_tflops_sustained (MEASURED_PEAKS.json)"}, **common)


def grm_roofline(ctx, peaks, t_dev, n, np_, mode="bf16x3", traffic=None):
    """Roofline of the dominant kernel (the GRM.V) from the engine's own CUDA-event timing.

    Algorithmic work per launch, whatever the precision form executes: bytes = the stored K (4 B
    per entry for the two BF16 halves, 8 B for TF32 halves, 4 B for one FP32 K) + the P halves
    read and Y written per column; FLOPs = 2 N_p^2 per column (one product).  The binding roof is
    the one on which this work takes longer; frac = achieved / peak on it.  The tensor peak is the
    measured sustained BF16 rate (the kernel runs inside seconds-long steps; TF32 at half of it).
    ``executed`` adds the tensor work the kernel issues (three products for the split forms)."""
    launches = max(1, t_dev["gemm_launches"])
    ms = t_dev["gemm_ms"] / launches
    cols = t_dev["gemm_cols"] / launches
    bf16 = mode == "bf16x3"
    split = mode in ("tf32x3", "bf16x3")
    kb = 4.0 if bf16 else (8.0 if split else 4.0)
    pb = 4.0 if bf16 else (8.0 if split else 4.0)
    bytes_alg = kb * np_ * np_ + (pb + 4.0) * np_ * cols
    flops_alg = 2.0 * np_ * np_ * cols
    products = 3.0 if split else 1.0
    hbm = peaks.get("hbm_gbs", 6800.0)
    tc_peak = peaks.get("bf16_tflops_sustained", 1700.0) / (1.0 if bf16 else 2.0)
    kname = "tc_gemm_kernel<%s,split>" % ("bf16" if bf16 else "tf32")
    t = ms * 1e-3
    a_bw = bytes_alg / t / 1e9
    a_tc = flops_alg / t / 1e12
    common = {"traffic": None if traffic is None else round(traffic * bytes_alg),
              "traffic_basis": None if traffic is None else GRMV_TRAFFIC_BASIS,
              "kernel": kname, "per_launch_ms": round(ms, 3),
              "columns_per_launch": round(cols, 1), "algorithmic_bytes_per_launch": bytes_alg,
              "algorithmic_flops_per_launch": flops_alg,
              "algorithmic_basis": "bytes: stored K + P read + Y written; FLOPs: 2 N_p^2 per column",
              "executed": {"products": products, "tensor_flops_per_launch": products * flops_alg,
                           "tflops": round(products * a_tc, 1), "peak": tc_peak,
                           "frac": round(products * a_tc / tc_peak, 4),
                           "peak_source": "measured bf16_tflops_sustained (MEASURED_PEAKS.json)"
                                          + ("" if bf16 else ", TF32 at half of it")}}
    if a_bw / hbm >= a_tc / tc_peak:
        return dict({"bound": "hbm", "achieved": round(a_bw, 1), "peak": hbm, "unit": "GB/s",
                     "frac": round(a_bw / hbm, 4),
                     "peak_source": "measured hbm_gbs (MEASURED_PEAKS.json)"}, **common)
    return dict({"bound": "tensor", "achieved": round(a_tc, 1), "peak": tc_peak, "unit": "TFLOP/s",
                 "frac": round(a_tc / tc_peak, 4),
                 "peak_source": ("measured bf16_tflops_sustained (MEASURED_PEAKS.json)" if bf16 else
                                 "TF32 = half the measured bf16_tflops_sustained (MEASURED_PEAKS.json)")},
                **common)


def step_width_summary(trace):
    """How wide the engine steps were (GRM.V columns per launch) and where the GRM.V time went."""
    if len(trace) == 0:
        return None
    cols, occ, gemm, idle = trace[:, 0], trace[:, 1], trace[:, 2], trace[:, 4]
    narrow = cols <= 128  # K-streaming bound: the K halves' read sets the time
    idle = idle[idle >= 0]  # the first step of a run has no predecessor (-1)
    out = {"steps": int(len(trace)),
           "columns_p10_p50_p90": [float(np.percentile(cols, q)) for q in (10, 50, 90)],
           "occupied_mean": round(float(occ.mean()), 1),
           "grmv_ms_share_steps_le_128_columns": round(float(gemm[narrow].sum() / max(gemm.sum(), 1e-9)), 3),
           "steps_le_128_columns": int(narrow.sum())}
    if len(idle):
        # device gap before each step (admission included): typical, tail and the largest
        out["idle_ms_p50_p90_p99_max"] = [round(float(np.percentile(idle, q)), 3) for q in (50, 90, 99)] + [
            round(float(idle.max()), 3)]
    if trace.shape[1] >= 8 and len(trace) > 1:
        # the five largest gaps with their host side: ms from the previous finish to the launch,
        # ms inside the launch, slot uploads the admission waited for
        top = np.argsort(-trace[:, 4])[:5]
        out["largest_gaps"] = [[round(float(trace[i, 4]), 2), round(float(trace[i, 5]), 2),
                                round(float(trace[i, 6]), 2), int(trace[i, 7])] for i in top]
        gaps = trace[trace[:, 5] >= 0, 5]
        out["host_gap_ms_p50_p99"] = [round(float(np.percentile(gaps, q)), 3) for q in (50, 99)] if len(gaps) else None
    return out


def serving_block(ctx, args, cols):
    """Serving form: Poisson arrivals (mean 2/s) of fits on sample subsets of 20k..N, admitted as
    slots and columns free up; reports fits/hr over the run and p50/p99 latency from arrival."""
    from saigegpu import prep, serve, synth
    n = ctx.n
    rng = np.random.default_rng(args.seed + 99)
    gv = ctx.synth_genetic_value(args.seed * 13)
    gv = gv / gv.std()
    arrivals, t = [], 0.0
    for k in range(args.serve_requests):
        t += rng.exponential(0.5)
        trait = "binary" if k % 2 == 0 else "quantitative"
        keep = rng.uniform(min(1.0, 20000 / n), 1.0)
        mask = rng.uniform(size=n) < keep
        S = np.nonzero(mask)[0]
        y, C = synth.simulate_pheno(gv, args.seed * 1000 + k, trait, tau=0.3,
                                    prevalence=rng.uniform(0.05, 0.3), h2=rng.uniform(0.1, 0.6))
        f0 = prep.make_fit0(y[S], C[S], trait, True)
        arrivals.append((t, serve.FitSpec(f0, trait, mask=mask)))
    t0 = time.perf_counter()
    if args.driver == "native":
        from saigegpu import native
        done = native.serve(ctx, arrivals, max_columns=cols, max_phenos=max(4, args.phenos),
                            pipelined=not args.blocking_runner, threads=args.workers)
    else:
        done = serve.serve(ctx, arrivals, max_columns=cols, max_phenos=max(4, args.phenos),
                           pipelined=not args.blocking_runner, workers=args.workers)
    wall = time.perf_counter() - t0
    lat = sorted(j.t_done - j.t_arrive for j in done)
    ok = sum(1 for j in done if j.error is None)
    return {"requests": len(arrivals), "completed": ok, "arrival_rate_per_s": 2.0,
            "fits_per_hr": round(ok / wall * 3600.0, 1), "wall_s": round(wall, 1),
            "latency_s": {"p50": round(float(np.percentile(lat, 50)), 3),
                          "p99": round(float(np.percentile(lat, 99)), 3)},
            "subsets": "20k..N samples", "max_concurrent_fits": max(4, args.phenos)}


def load_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "fallback": True}


def cpu_baseline(ctx, iters_per_fit, budget_s=25.0):
    """Reference CPU GRM.x (oracle C restatement, all host cores) on the resident cohort."""
    from oracle import cpu_ref
    d = ctx.dims()
    packed = ctx.packed_geno()
    freq, inv = ctx.allele_freq(), ctx.invstd()
    p2 = (np.float32(2) * freq).astype(np.float32)
    lut = np.zeros((len(freq), 4), np.float32)
    for g in range(3):
        lut[:, g] = ((np.float32(g) - p2).astype(np.float32) * inv).astype(np.float32)
    pg = cpu_ref.PackedGeno(packed, lut, d["n"])
    b = np.random.default_rng(0).standard_normal(d["n"]).astype(np.float32)
    times = []
    t_start = time.perf_counter()
    while not times or (time.perf_counter() - t_start < budget_s and len(times) < 3):
        t = time.perf_counter()
        pg.crossprod(b)
        times.append(time.perf_counter() - t)
    tm = min(times)
    return {"value": round(3600.0 / (tm * iters_per_fit), 6), "unit": "fits/hr", "cores": os.cpu_count(),
            "kind": "port",
            "sample": "%d GRM.x products (parallelCrossProdOpenMP restated in C, N=%d, M=%d), %.2f s each; "
                      "fits/hr extrapolated with %.0f GRM.x per fit measured on the GPU path" %
                      (len(times), d["n"], d["m_qc"], tm, iters_per_fit)}


def plain_fp64(ctx, iters_per_fit):
    """Plain FP64 single-RHS PCG on the same GPU: event-timed per-iteration cost, extrapolated."""
    from saigegpu import MV_FP64_PLAIN
    n = ctx.n
    ctx.set_matvec_mode(MV_FP64_PLAIN)
    rng = np.random.default_rng(1)
    w = rng.uniform(0.05, 0.25, n)
    b = rng.standard_normal(n)
    ctx.pcg_solve(w, np.array([1.0, 0.3]), b, 2, 1e-30)  # warm-up
    ctx.engine_reset_timing()
    t0 = time.perf_counter()
    _, it = ctx.pcg_solve(w, np.array([1.0, 0.3]), b, 8, 1e-30)
    wall = time.perf_counter() - t0
    t = ctx.engine_timing()
    per_iter = t["step_ms"] / max(1, it) / 1e3
    return {"fits_per_hr": round(3600.0 / (per_iter * iters_per_fit), 3), "ms_per_iteration": round(per_iter * 1e3, 3),
            "wall_ms_per_iteration": round(wall / max(1, it) * 1e3, 3),
            "basis": "FP64 GEMV over the FP32 GRM, one RHS per solve; %.0f PCG iterations per fit" % iters_per_fit}


def reference_gpu_matvec(n, m_qc, iters_per_fit, reps=5):
    """The reference's own GPU algorithm for K.x, restated with cuBLAS through torch on this GPU:
    two FP32 SGEMV over the N x M standardised genotype matrix Z per product (y = Z'x, z = Z y),
    one right-hand side, as gpuSymMatMult::sym_sgemv (gpuSymMatMult.cu:211-252) on a single rank.
    Z holds seeded random values (SGEMV time does not depend on them).  Extrapolated to fits/hr
    with the measured PCG iterations per fit; the host PCG vector work is not included."""
    import torch
    try:
        Z = torch.empty((m_qc, n), dtype=torch.float32, device="cuda")  # column-major N x M
    except RuntimeError as ex:
        return {"unavailable": "could not hold Z (%d x %d FP32): %s" % (n, m_qc, str(ex).splitlines()[0])}
    g = torch.Generator(device="cuda")
    g.manual_seed(7)
    for i in range(0, m_qc, 8192):
        Z[i:i + 8192].normal_(generator=g)
    x = torch.randn(n, device="cuda", generator=g)
    s = torch.cuda.current_stream()
    for _ in range(2):
        z = torch.mv(Z.t(), torch.mv(Z, x))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(reps):
        z = torch.mv(Z.t(), torch.mv(Z, x))
    e1.record(s)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    del Z, z, x
    torch.cuda.empty_cache()
    z_bytes = 4.0 * n * m_qc
    return {"fits_per_hr": round(3600.0 / (ms * 1e-3 * iters_per_fit), 3), "ms_per_matvec": round(ms, 3),
            "GBps": round(2 * z_bytes / (ms * 1e-3) / 1e9, 1), "z_gb": round(z_bytes / 1e9, 1),
            "basis": "2 cuBLAS SGEMV over FP32 Z per K.x, single RHS; %.0f PCG iterations per fit; "
                     "matvec only (reference's host vector work and MPI allreduce excluded)" % iters_per_fit}


def run_ours(args, rank, world, local):
    import torch
    from saigegpu import (Context, GRM_BF16_TC, GRM_BF16X3_TC, MV_BF16X3_TC, MV_TF32X3_TC, MV_TF32_TC,
                          MV_FP32_SIMT, MV_SUBSET_EXACT, MV_SUBSET_EXACT_F8)
    exact = args.mode in ("subset", "subset8")
    peaks = load_peaks()
    ctx = Context(local)
    t_setup = time.perf_counter()
    ptr, ln = ctx.synth_bed(args.seed + rank, args.n, args.m, args.miss)
    ctx.setgeno_device(ptr, ln, args.n, args.m)
    decode_t = ctx.build_timing()
    torch.cuda.synchronize()
    tune_report = None
    d = ctx.dims()
    syrk_flops = float(d["n"]) * (d["n"] + 1) * d["m_qc"]
    syrk1_ms = None  # the single-product BF16 SYRK (the tuner's chosen shape)
    if not args.no_tune and args.mode in ("subset", "subset8", "bf16x3"):
        # SYRK shape (and for the cohort-GRM engine the per-width GRM.V plan) from measured times;
        # leaves the single-product BF16 GRM built
        from saigegpu import tune
        tune_report = tune.tune(ctx, mode=MV_BF16X3_TC, grmv=not exact)
        syrk1_ms = tune_report["syrk"]["times_ms"][tune_report["syrk"]["chosen"]]
    # the cohort GRM: split-BF16 standardised genotypes (16 significant bits, four products) for the
    # cohort-GRM engines, so that tau lands within 1e-4 of FP64 arithmetic; the subset-exact engine
    # needs none (the plain FP64 comparator keeps the tuner's BF16 GRM, or builds one)
    grm_prec = GRM_BF16X3_TC if args.grm == "bf16x3" else GRM_BF16_TC
    if exact:
        grm_prec = GRM_BF16_TC
    t0 = time.perf_counter()
    if not (exact and tune_report is not None):
        ctx.grm_build(grm_prec)
    grm_s = time.perf_counter() - t0
    bt = ctx.build_timing()
    if syrk1_ms is None and grm_prec == GRM_BF16_TC:
        syrk1_ms = bt["syrk_ms"]
    build_products = 4 if grm_prec == GRM_BF16X3_TC else 1
    specs = make_specs(ctx, args, args.seed + 17 * rank)
    # the timed steps: K batches of new phenotypes (their own traits and sample subsets), streamed
    # through P phenotype slots -- a fit enters as soon as one finishes, as a serving process runs
    timed_specs = [sp for b in range(args.steps) for sp in make_specs(ctx, args, args.seed + 17 * rank + 1 + b, b + 1)]
    mode = {"subset": MV_SUBSET_EXACT, "subset8": MV_SUBSET_EXACT_F8, "bf16x3": MV_BF16X3_TC,
            "tf32x3": MV_TF32X3_TC, "tf32": MV_TF32_TC, "fp32": MV_FP32_SIMT}[args.mode]
    ctx.set_matvec_mode(mode)
    g_ms = ctx.build_timing()["zbuild_ms"] if exact else None  # the genotype matrix build
    if exact and tune_report is not None:
        # CTA pairs and K slices of the genotype GEMMs per launch width, from measured times
        from saigegpu import tune
        tune_report["subset"] = tune.tune_subset(ctx, mode=mode)
        tune_report["subset_plan"] = ctx.subset_plan()
    from saigegpu import serve as _serve
    cols = _serve.columns_for(specs)
    setup_s = time.perf_counter() - t_setup
    for _ in range(args.warmup):
        run_batch(ctx, specs, cols, not args.blocking_runner, args.workers, args.driver, args.launch_wait_ms)
    L0 = ctx.kernel_launches()
    ctx.engine_reset_timing()
    barrier(world)
    torch.cuda.synchronize()
    walls, jobs_all, res_all, host_t = [], [], [], {}
    with Clocks(local) as clk:
        res, jobs, wall = run_batch(ctx, timed_specs, cols, not args.blocking_runner, args.workers, args.driver,
                                    args.launch_wait_ms, max_phenos=args.phenos)
        walls.append(wall)
        jobs_all += jobs
        res_all += res
        for k, v in getattr(jobs[0], "host_times", {}).items():
            host_t[k] = host_t.get(k, 0.0) + v
    torch.cuda.synchronize()
    barrier(world)
    launches = ctx.kernel_launches() - L0
    io_h2d, io_d2h = ctx.engine_io_bytes()
    idle_ms, admit_ms, finish_ms = ctx.engine_idle_ms()
    trace = ctx.engine_step_trace()
    tdev = ctx.engine_timing()
    dev_s = tdev["step_ms"] / 1e3
    total_wall = sum(walls)
    fits = args.phenos * args.steps
    wall_max = allmax(total_wall, world)
    dev_max = allmax(dev_s, world)
    fits_all = allsum(fits, world)
    value = fits_all / dev_max * 3600.0
    e2e = fits_all / wall_max * 3600.0
    # per-fit latency from its admission to a phenotype slot (native driver), else from submission
    lat = sorted((j.service_s if getattr(j, "service_s", None) is not None else j.t_done - j.t_start)
                 for j in jobs_all)
    col_iters = float(np.mean([j.column_iterations for j in jobs_all]))
    cols_per_fit = float(np.mean([j.columns for j in jobs_all]))
    # bytes the engine API copied per step (counted by the library): right-hand sides, weights,
    # probe tables, column states, fetched results and probe reductions
    h2d = int(io_h2d // max(1, args.steps))
    d2h = int(io_d2h // max(1, args.steps))
    # DRAM bytes per launch scaled from an ncu capture of a smaller case
    traffic = GRMV_TRAFFIC_RATIO if args.mode == "bf16x3" else None
    npad_n = ctx.grm_padded_n()
    mg = (args.m + 127) // 128 * 128
    if exact:
        roof = subset_roofline(peaks, tdev, npad_n, mg, f8=args.mode == "subset8")
    else:
        roof = grm_roofline(ctx, peaks, tdev, d["n"], npad_n, args.mode, traffic)
    out = {
        "metric": METRIC, "value": round(value, 2), "unit": "fits/hr", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total_wall / args.steps * 1e3, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"subset": "bf16x2-tc/fp64", "subset8": "fp16+e4m3-tc/fp64", "bf16x3": "bf16x3-tc/fp64",
                  "tf32x3": "tf32x3-tc/fp64",
                  "tf32": "tf32-tc/fp64", "fp32": "fp32/fp64"}[args.mode],
        "data": "synthetic (seeded cohort generator; the reference's 150k x 100k synthetic AFR set is external)",
        "config": {"workload": "batched null-model fits on a resident GRM", "n_samples": d["n"],
                   "m_markers_qc": d["m_qc"], "m_markers": args.m, "missing": args.miss,
                   "phenotypes_per_step": args.phenos,
                   "timed_region": ("%d steps x %d new phenotypes (own traits and sample subsets, each set up "
                                    "inside the timed region), streamed through %d phenotype slots in one "
                                    "batched call" % (args.steps, args.phenos, args.phenos)),
                   "traits": "half binary / half quantitative",
                   "sample_masks": "drop U(5%,40%)", "probes": 30,
                   "semantics": ("exact per phenotype: each phenotype's GRM from its own samples' allele "
                                 "frequencies, fill, QC and 1/sd (setgeno per phenotype, FIT.cpp:376-385, 436-495)"
                                 if exact else
                                 "masked approximation: the cohort GRM restricted to each phenotype's samples"),
                   "grm": ("genotype matrix (0/1/2, %s) in both layouts, K_S applied as G'V then G T' with "
                           "per-phenotype weights; no K" % ("FP16 and E4M3" if args.mode == "subset8" else "BF16")
                           if exact else
                           "split-BF16 tcgen05 SYRK (four products), FP32 K" if args.grm == "bf16x3"
                           else "BF16 tcgen05 SYRK, FP32 K"),
                   "grm_v": args.mode,
                   "l2": ("inputs larger than L2 (genotype matrix %.0f GB per GEMM)" % (2.0 * npad_n * mg / 1e9)
                          if exact else "inputs larger than L2 (GRM %.0f GB)" % (4.0 * ctx.n ** 2 / 1e9)),
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "value_basis": ("device-busy time of engine steps (CUDA events); the phenotypes' subset "
                                   "set-ups run on low-priority streams beside and between the steps and count "
                                   "only where they lengthen a step (all of their time is in e2e)"
                                   if exact else "device-busy time of engine steps (CUDA events)"),
                   "runner": "blocking" if args.blocking_runner else "pipelined",
                   "driver": args.driver,
                   "driver_threads": args.workers if args.workers is not None else (
                       "half the cores, at most 8" if args.driver == "native" else 1),
                   "launch_wait_ms": args.launch_wait_ms if args.launch_wait_ms is not None else "library default"},
        "e2e": {"value": round(e2e, 2), "unit": "fits/hr", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "latency_s": {"p50": round(float(np.percentile(lat, 50)), 3), "p99": round(float(np.percentile(lat, 99)), 3),
                      "basis": "per fit, from its admission to a phenotype slot to its result"},
        "gpu_launches": int(launches),
        "roofline": roof,
        "grm_build": {"grm": "bf16 (plain FP64 comparator only)" if exact else args.grm,
                      "seconds": round(grm_s, 3), "syrk_products": build_products,
                      "syrk_algorithmic_flops": syrk_flops,
                      "syrk_executed_flops": build_products * syrk_flops,
                      "syrk_ms": round(bt["syrk_ms"], 2),
                      "syrk_algorithmic_tflops": round(syrk_flops / (bt["syrk_ms"] * 1e-3) / 1e12, 1),
                      "syrk_algorithmic_frac_of_bf16_sustained": round(
                          syrk_flops / (bt["syrk_ms"] * 1e-3) / 1e12 / peaks.get("bf16_tflops_sustained", 1700.0), 4),
                      "syrk_executed_tflops": round(build_products * syrk_flops / (bt["syrk_ms"] * 1e-3) / 1e12, 1),
                      "syrk_executed_frac_of_bf16_sustained": round(
                          build_products * syrk_flops / (bt["syrk_ms"] * 1e-3) / 1e12
                          / peaks.get("bf16_tflops_sustained", 1700.0), 4),
                      "zbuild_ms": round(bt["zbuild_ms"], 2),
                      # packed genotypes read + Z written (BF16, both halves for the split build)
                      "zbuild_GBps": round((d["m_qc"] * ((d["n"] + 3) // 4)
                                            + (4.0 if build_products == 4 else 2.0) * ctx.n * d["m_qc"])
                                           / (bt["zbuild_ms"] * 1e-3) / 1e9, 1)},
        "decode": {"qc_ms": round(decode_t["qc_ms"], 2), "repack_ms": round(decode_t["repack_ms"], 2),
                   "diag_ms": round(decode_t["diag_ms"], 2),
                   "qc_GBps": round(args.m * ((args.n + 3) // 4) / (decode_t["qc_ms"] * 1e-3) / 1e9, 1),
                   "repack_GBps": round(2.0 * d["m_qc"] * ((d["n"] + 3) // 4) / (decode_t["repack_ms"] * 1e-3) / 1e9, 1),
                   "peak_GBps": peaks.get("hbm_gbs")},
        "per_fit": {"pcg_column_iterations": round(col_iters, 1), "columns": round(cols_per_fit, 1),
                    "converged": int(sum(1 for r in res_all if r["converged"])), "fits": len(res_all)},
        "setup_s": round(setup_s, 1),
        # engine: the stepping thread's seconds (waits for the device included); driver: the fits'
        # host arithmetic, summed over the driver's worker threads; the rest are engine calls within it
        "wall_breakdown_s_per_step": {k: round(v / args.steps, 3) for k, v in host_t.items()},
        "between_steps_s_per_step": {"total": round(idle_ms / 1e3 / args.steps, 3),
                                     "launch_admission": round(admit_ms / 1e3 / args.steps, 3),
                                     "finish_host": round(finish_ms / 1e3 / args.steps, 3)},
        "step_widths": step_width_summary(trace),
    }
    if exact:
        gb = 2.0 * 2.0 * npad_n * mg + mg * ((args.n + 3) // 4)  # both layouts written + codes read
        out["genotype_matrix_build"] = {"ms": round(g_ms, 2), "GB": round(gb / 1e9, 2),
                                        "GBps": round(gb / (g_ms * 1e-3) / 1e9, 1)}
    if syrk1_ms is not None:  # the single-product BF16 SYRK (N(N+1)M FLOP), timed by the library's events
        tf = syrk_flops / (syrk1_ms * 1e-3) / 1e12
        out["syrk_bf16"] = {"syrk_ms": round(syrk1_ms, 2), "flops": syrk_flops, "tflops": round(tf, 1),
                            "frac_of_bf16_peak": round(tf / peaks.get("bf16_tflops", 1900.0), 4),
                            "frac_of_bf16_sustained": round(tf / peaks.get("bf16_tflops_sustained", 1700.0), 4)}
    if tune_report is not None:
        from saigegpu import tune
        out["tuning"] = tune.report_json(tune_report)
    out["clocks"] = clk.summary()
    if rank == 0 and args.serve_requests > 0:
        out["serving"] = serving_block(ctx, args, cols)
    if rank == 0 and exact and args.loco_chroms > 0:
        out["loco"] = loco_block(ctx, timed_specs[-args.phenos:], res_all[-args.phenos:], args.loco_chroms, cols)
    if rank == 0:
        out["plain_fp64_single_rhs"] = plain_fp64(ctx, col_iters)
        out["speedup_vs_plain_fp64"] = round(value / out["plain_fp64_single_rhs"]["fits_per_hr"], 1)
        if not args.no_ref_gpu:
            rg = reference_gpu_matvec(d["n"], d["m_qc"], col_iters)
            out["reference_gpu_algorithm"] = rg
            if "fits_per_hr" in rg:
                out["speedup_vs_reference_gpu_algorithm"] = round(value / rg["fits_per_hr"], 1)
        if not args.no_cpu_baseline:
            out["cpu_baseline"] = cpu_baseline(ctx, col_iters)
    ctx.close()
    return out


def loco_block(ctx, specs, fits, chroms, cols):
    """Step 1's LOCO pass (FIT.R:251-295, 504-540) for fitted phenotypes in the subset-exact engine:
    Get_Coef_LOCO of every phenotype with each of the first ``chroms`` of 22 chromosomes (contiguous
    blocks of the .bim markers) left out of its own GRM (``sg_loco_set_bim``), through the Python
    generator driver (``serve.fit_loco``); wall time of the whole pass, subset set-ups included."""
    from saigegpu import serve
    m = ctx.dims()["m_total"]
    ranges = serve.loco_ranges(1 + (np.arange(m) * 22) // m)
    sel = {c: ranges[c] for c in range(1, 1 + min(chroms, 22))}
    t0 = time.perf_counter()
    got = serve.fit_loco(ctx, specs, fits, sel, max_columns=cols, bim=True)
    wall = time.perf_counter() - t0
    bad = sum(1 for c in sel for r in got[c] if isinstance(r, Exception))
    done = len(sel) * len(specs) - bad
    return {"chromosomes": len(sel), "phenotypes": len(specs), "failed": bad, "wall_s": round(wall, 2),
            "chromosome_fits_per_hr": round(done / wall * 3600.0, 1),
            "basis": "Get_Coef_LOCO per phenotype and chromosome, each phenotype's own GRM markers of the "
                     "chromosome left out; wall time through serve.fit_loco (Python generators)"}


def c1_full_fit(seed=1001, n=2000, m=5000, miss=0.01):
    """One full binary null-model fit at N = 2,000, M = 5,000 on the host cores: the oracle's AI-REML
    driver over the C restatement of the reference's CPU GRM.x (parallelCrossProdOpenMP,
    FIT.cpp:1576-1598; OpenMP over all cores).  Returns the measured fit time and what the
    per-product extrapolation used at N = 100k predicts for the same fit."""
    from oracle import aireml, cpu_ref, plink
    from saigegpu import prep, synth
    bed, codes = synth.synth_bed(seed, n, m, miss)
    g = plink.setgeno(bed, n, m, np.arange(1, n + 1), np.ones(n, bool), 0.01, 0.15)
    cg = cpu_ref.CpuGeno(g)

    class CpuRefGRM:
        """GRM.x through the reference's CPU algorithm, one column at a time."""
        def __init__(self):
            self.n, self.m_qc, self.is_diag_one = n, g.freq.shape[0], False
            self.diag_sum = plink.diag_std_geno(g)
            self.products = 0

        def matvec(self, B):
            B = np.asarray(B)
            if B.ndim == 1:
                self.products += 1
                return cg.crossprod(B).astype(np.float64)
            self.products += B.shape[1]
            return np.column_stack([cg.crossprod(B[:, j]).astype(np.float64) for j in range(B.shape[1])])

    grm = CpuRefGRM()
    gv = synth.genetic_value_from_codes(g.codes, 3)
    y, C = synth.simulate_pheno(gv, seed, "binary", tau=0.3, prevalence=0.2)
    f0 = prep.make_fit0(y, C, "binary", True)
    t0 = time.perf_counter()
    fit = aireml.glmmkin_binary(grm, f0)
    fit_s = time.perf_counter() - t0
    b = np.random.default_rng(0).standard_normal(n).astype(np.float32)
    cg.crossprod(b)
    reps = 20
    t0 = time.perf_counter()
    for _ in range(reps):
        cg.crossprod(b)
    per = (time.perf_counter() - t0) / reps
    return {"n": n, "m_qc": int(grm.m_qc), "seconds": round(fit_s, 3), "fits_per_hr": round(3600.0 / fit_s, 2),
            "grm_products": int(grm.products), "product_ms": round(per * 1e3, 3),
            "products_share_of_fit": round(grm.products * per / fit_s, 3),
            "tau": [float(x) for x in fit["theta"]],
            "basis": "oracle AI-REML driver (numpy) over the C restatement of the reference's CPU GRM.x; "
                     "products_share_of_fit = the part of the fit the per-product extrapolation counts"}


def run_reference(args, rank, world):
    """The reference's CPU path (oracle C restatement of parallelCrossProdOpenMP) on the host cores:
    each step times one GRM.x product at the workload's N and M, extrapolated to fits/hr with the
    workload's PCG column-iterations per fit; one full fit at N = 2,000 is timed beside it."""
    if rank != 0:
        return None
    from oracle import cpu_ref
    iters = PCG_COLUMN_ITERATIONS_PER_FIT
    basis = "%.1f PCG column-iterations per fit (measured by the GPU arm on this workload)" % iters
    t0 = time.perf_counter()
    pg = cpu_ref.PackedGeno.synthetic(args.seed, args.n, args.m, args.miss)
    setup = time.perf_counter() - t0
    b = np.random.default_rng(0).standard_normal(args.n).astype(np.float32)
    for _ in range(args.warmup):
        pg.crossprod(b)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        pg.crossprod(b)
        times.append(time.perf_counter() - t)
    per = float(np.mean(times))
    value = 3600.0 / (per * iters)
    c1 = None
    try:
        c1 = c1_full_fit()
    except Exception as ex:  # the C1 fit is a companion figure; the line stands without it
        c1 = {"unavailable": str(ex).splitlines()[0][:200]}
    return {
        "metric": METRIC, "value": round(value, 6), "unit": "fits/hr", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(per * 1e3, 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32", "data": "synthetic (same cohort recipe, generated on the host)",
        "config": {"workload": "batched null-model fits on a resident GRM", "n_samples": args.n,
                   "m_markers_qc": pg.m, "step": "one GRM.x product of the reference's CPU path"},
        "impl": "reference",
        "cpu_baseline": {"value": round(value, 6), "unit": "fits/hr", "cores": os.cpu_count(), "kind": "port",
                         "sample": "one GRM.x per step (oracle/cpu_ref.c restating FIT.cpp:1576-1598), "
                                   "%.2f s each; extrapolated with %s; setup %.0f s" % (per, basis, setup)},
        "c1_full_fit": c1,
        "e2e": {"value": round(value, 6), "unit": "fits/hr", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    args = parse()
    rank, world, local = dist_init(args)
    if args.impl == "reference":
        out = run_reference(args, rank, world)
    else:
        out = run_ours(args, rank, world, local)
    if rank == 0 and out is not None:
        line = json.dumps(out)
        print(line, flush=True)
        if args.json_out:
            with open(args.json_out, "w") as f:
                f.write(line + "\n")


if __name__ == "__main__":
    main()
