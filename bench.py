"""Benchmark: seconds to the top-k PCs of a PLINK genotype matrix on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload c3] [--precision fp8|bf16|fp32|fp64]

One step = the whole hot path on one synthetic workload: packed genotypes ->
counts and allele frequencies -> window-based RSVD (winSVD, 7 epochs for the
64-window schedule) -> U, S, V.  The default form is the FP8 one (E4M3
tensor-core products in the range-finding epochs, the exact 27-bit BF16 form
in the final ones); --precision bf16 measures the exact form alone.

* ``value``: steps timed with CUDA events (synchronised on both sides), the
  packed matrix already resident in HBM (device-to-device load into the
  operator, then run_halko).  The packed matrix (50 GB for c3) is far larger
  than L2, so no flush is needed between steps.
* ``e2e``: the same through the C-ABI with host buffers: pinned host .bed body
  -> pcaone_gpu_load_bed (H2D inside the timed region) -> run_halko -> U, S, V
  back to the host.
* ``roofline``: the dominant kernel (the window H or G product), algorithmic
  flops 2*N*SNPs*L per launch over its CUDA-event time on the library's
  stream; ``executed_tflops`` counts the MMA work actually issued (three
  integer BF16 slices of the sketch, padded to a multiple of 16 columns).
  ``traffic`` is the DRAM bytes per launch of that kernel from an ncu capture
  of a window of the same shape, where one exists.
* ``accuracy`` (PLINK workloads): after the timed steps, the same workload
  runs once in the FP64-grade form (six 9-bit slices: 54-bit operands, exact
  integer accumulation; the GPU oracle) and once in the plain FP32 CUDA-core
  form; the line reports each form's largest principal angle (sin) and
  relative eigenvalue error against the oracle on the well-separated leading
  PCs, and the FP32 form's time over ``value``.
* EM workloads (``c4``: ``--emu``) report the EM iterations and, with
  ``--warm-start``, the learned start's statistics.
* ``cpu_baseline`` / ``--impl reference``: the reference's own CPU path (its
  sources compiled for this host into oracle/_ref/ref_driver, OpenMP on every
  host core) on two bounded samples of the same population model (REF_SAMPLES),
  extrapolated to the whole workload linearly in N*M and labelled so; the
  numpy/LAPACK restatement (oracle/) stands in when the reference cannot be
  built on the host.

Multi-GPU: the path is not sharded (replicas only); under torchrun each rank
runs its own replica and the slowest rank's time is reported.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

import numpy as np  # noqa: E402

PEAKS_FALLBACK = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}

# cpu sample: first N' samples x M' SNPs of the same population model
CPU_SAMPLE = {"nsamples": 6000, "nsnps": 30000}


def load_peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return d, "measured"
    return PEAKS_FALLBACK, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.path = tempfile.mktemp(suffix=".csv")
        self.proc = None

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        smax = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        loaded = [x for x in sm if x is not None]
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(rows)}


# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the
# tensor-core window products, from one ncu capture of a window of the
# workload's shape, keyed by (workload, product class of kernel_stats)
NCU_TRAFFIC = {
    # one capture of a window of the 1M-SNP workload (15,625 SNPs x 200,064
    # samples); the E4M3 G and H products both run k_tc_g<2> (H on the
    # sample-major copy)
    ("c3", "g_product_e4m3"): 821.3e6 + 118.8e6,
    ("c3", "h_product_e4m3"): 841.3e6 + 182.0e6,
}


def workload_params(name: str, precision: str):
    from pcaone_gb300 import capi, synthetic
    wl = synthetic.WORKLOADS[name]
    prec = {"fp32": capi.PREC_FP32, "bf16": capi.PREC_BF16, "bf16x3": capi.PREC_BF16X3,
            "fp8": capi.PREC_FP8, "fp64": capi.PREC_FP64}[precision]
    p = capi.default_params(svd=wl.get("svd", 2), k=wl["k"], oversamples=wl["p"], maxp=wl["maxp"],
                            bands=wl["bands"], perm=wl.get("perm", 1), standardize=0 if wl.get("dense") else 1,
                            precision=prec)
    if wl.get("emu"):
        p.emu = 1
        p.tolem = wl.get("tolem", 1e-5)
        p.maxiter = wl.get("maxiter", 100)
    return wl, p


def workload_desc(name: str, wl: dict, model, bps: int) -> str:
    N, M = model.nsamples, model.nsnps
    kind = (f"FP16 dosages ({M * N * 2 / 1e9:.1f} GB)" if wl.get("dense") else
            f"PLINK ({M * bps / 1e9:.1f} GB packed)")
    d = (f"{name}: N={N} x M={M} {kind}, {model.npop} populations, k={wl['k']}, "
         f"p={wl['p']}, {'winSVD ' + str(wl['bands']) + ' windows' if wl.get('svd', 2) == 2 else 'sSVD'}, "
         f"{wl['maxp'] + 1} epochs")
    if wl.get("emu"):
        d += f", EM to tol {wl.get('tolem', 1e-5):g} (at most {wl.get('maxiter', 100)} iterations)"
    return d


_cpu_sample_cache = {}


def cpu_sample_run(name: str):
    """Time the oracle (numpy restatement of the reference's path) on a bounded
    sample; returns (seconds for the sample, seconds scaled to the workload,
    description, cores).  The sample is drawn once per process."""
    from oracle import halko as H
    from pcaone_gb300 import synthetic
    wl = synthetic.WORKLOADS[name]
    n, m = CPU_SAMPLE["nsamples"], CPU_SAMPLE["nsnps"]
    if name not in _cpu_sample_cache:
        model = synthetic.model_for(name, seed=1, nsamples=n, nsnps=m)
        _cpu_sample_cache[name] = synthetic.sample_packed_bed(model)
        H.build_rng_lib()
    packed = _cpu_sample_cache[name]
    t0 = time.perf_counter()
    d = H.OracleData(packed, n, perm=bool(wl.get("perm", 1)), bands=wl["bands"])
    H.run_pca_with_halko(d, wl["k"], wl["p"], maxp=wl["maxp"])
    t = time.perf_counter() - t0
    scale = (wl["nsamples"] * wl["nsnps"]) / (n * m)
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    desc = (f"numpy/LAPACK restatement of the reference's in-core path (decode, AF, standardise, shuffle, "
            f"winSVD {wl['maxp'] + 1} epochs, k={wl['k']}, p={wl['p']}, {wl['bands']} windows) on the first {n} "
            f"samples x {m} SNPs of the same population model; {t:.2f} s measured, scaled by N*M x{scale:.1f}")
    if wl.get("emu"):
        desc += "; one RSVD pass (EM iterations not included)"
    return t, t * scale, desc, cores


# ---------------------------------------------------------------------------
# The reference's own CPU path (oracle/_ref/ref_driver: the reference's sources
# compiled for this host, driven like src/Halko.cpp:271-320) on bounded samples
# of the workload's population model, with every host core.
# ---------------------------------------------------------------------------
# a half-size and a full-size sample: their times per genotype show the N*M
# scaling that the extrapolation to the whole workload uses
REF_SAMPLES = ({"nsamples": 8000, "nsnps": 25000}, {"nsamples": 8000, "nsnps": 50000})
REF_DRIVER = os.path.join(REPO, "oracle", "_ref", "ref_driver")


def host_cores() -> int:
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()


def cpu_model() -> str:
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for line in out.splitlines():
            if line.startswith("Model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


_gen_model = None


def _gen_init(model):
    global _gen_model
    _gen_model = model


def _gen_chunk(span):
    from pcaone_gb300 import synthetic
    lo, hi = span
    return lo, synthetic.pack_codes(synthetic.sample_codes(_gen_model, lo, hi), False, _gen_model.seed + lo)


def write_sample_plink(name: str, nsamples: int, nsnps: int, prefix: str) -> None:
    """The workload's population model at nsamples x nsnps, drawn by the numpy
    generator in a pool of host processes (chunks of 4096 SNPs, the same bytes
    as synthetic.sample_packed_bed), written as a PLINK fileset."""
    import multiprocessing as mp
    from pcaone_gb300 import synthetic
    model = synthetic.model_for(name, seed=1, nsamples=nsamples, nsnps=nsnps)
    packed = np.empty((nsnps, synthetic.bytes_per_snp(nsamples)), dtype=np.uint8)
    spans = [(lo, min(nsnps, lo + 4096)) for lo in range(0, nsnps, 4096)]
    with mp.get_context("spawn").Pool(max(1, min(host_cores(), len(spans))), _gen_init, (model,)) as pool:
        for lo, block in pool.imap_unordered(_gen_chunk, spans):
            packed[lo:lo + block.shape[0]] = block
    synthetic.write_plink(prefix, packed, nsamples)


def ref_driver():
    """oracle/_ref/ref_driver, built from the reference tree (PCAONE_REF_TREE) or
    the staged copy in oracle/_ref/tree when missing; None if neither builds."""
    if not os.path.exists(REF_DRIVER):
        subprocess.run(["make", "-C", os.path.join(REPO, "oracle"), "ref", f"-j{host_cores()}"],
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    return REF_DRIVER if os.path.exists(REF_DRIVER) else None


def ref_options(wl: dict) -> list:
    """PCAone options of the workload (the driver keeps p as given)."""
    opts = ["-d", str(wl.get("svd", 2)), "-k", str(wl["k"]), "--maxp", str(wl["maxp"]), "-w", str(wl["bands"]),
            "--seed", "112", "--force-oversamples", str(wl["p"])]
    if not wl.get("perm", 1):
        opts.append("-S")
    if wl.get("emu"):
        opts += ["--emu", "--tol-em", str(wl.get("tolem", 1e-5)), "--maxiter", str(wl.get("maxiter", 100))]
    return opts


def ref_run(drv: str, prefix: str, outdir: str, wl: dict, threads: int) -> dict:
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    cmd = [drv, outdir, "--timing", "-b", prefix] + ref_options(wl)
    t0 = time.perf_counter()
    r = subprocess.run(cmd, capture_output=True, text=True, env=env)
    wall = time.perf_counter() - t0
    if r.returncode != 0:
        raise RuntimeError(f"reference driver failed ({r.returncode}): {r.stderr[-400:]}")
    out = json.loads(r.stdout.strip().splitlines()[-1])
    out["wall_s"] = wall
    return out


class RefSamples:
    """The two PLINK samples of one workload in a temporary directory."""

    def __init__(self, name: str):
        self.dir = tempfile.mkdtemp(prefix="pcaone_ref_")
        self.prefixes = []
        for q, smp in enumerate(REF_SAMPLES):
            prefix = os.path.join(self.dir, f"s{q}")
            write_sample_plink(name, smp["nsamples"], smp["nsnps"], prefix)
            self.prefixes.append(prefix)

    def close(self):
        import shutil
        shutil.rmtree(self.dir, ignore_errors=True)


def ref_extrapolate(wl: dict, small: dict, large: list) -> dict:
    """Per-genotype time of the two sample sizes and the whole-workload
    seconds extrapolated linearly in N*M from the larger sample."""
    full = wl["nsamples"] * wl["nsnps"]
    n_large = large[0]["nsamples"] * large[0]["nsnps"]
    s_e = small["total_s"] / (small["nsamples"] * small["nsnps"])
    t_large = statistics.median(r["total_s"] for r in large)
    return {"value": t_large * full / n_large, "t_large": t_large,
            "ns_per_genotype": {"half_sample": s_e * 1e9, "sample": t_large / n_large * 1e9},
            "factor": full / n_large}


def ref_sample_desc(wl: dict, ex: dict, small: dict, large: list, threads: int) -> str:
    L = large[0]
    return (f"the reference's own CPU path (its sources compiled on this host, -O3, OpenMP, Eigen GEMM) through "
            f"oracle/_ref/ref_driver: read .bed, allele frequencies, decode, standardise, shuffle, winSVD "
            f"{wl['maxp'] + 1} epochs, k={wl['k']}, p={wl['p']}, {wl['bands']} windows; samples of the same "
            f"population model: {L['nsamples']} x {L['nsnps']} ({ex['t_large']:.2f} s, of which prepare "
            f"{L['prepare_s']:.2f} s) and {small['nsamples']} x {small['nsnps']} ({small['total_s']:.2f} s); "
            f"{ex['ns_per_genotype']['sample']:.2f} vs {ex['ns_per_genotype']['half_sample']:.2f} ns per genotype; "
            f"EXTRAPOLATED linearly in N*M (x{ex['factor']:.0f}) to the whole workload; {threads} threads "
            f"({cpu_model()})")


def reference_cpu_baseline(name: str, wl: dict):
    """One timing of the reference at each sample size (the repo arm's
    cpu_baseline); None when the reference cannot be built on this host."""
    drv = None if wl.get("dense") else ref_driver()
    if drv is None:
        return None
    smp = RefSamples(name)
    try:
        threads = host_cores()
        small = ref_run(drv, smp.prefixes[0], smp.dir, wl, threads)
        large = [ref_run(drv, smp.prefixes[1], smp.dir, wl, threads)]
    finally:
        smp.close()
    ex = ref_extrapolate(wl, small, large)
    return {"value": ex["value"], "unit": "s", "cores": threads, "kind": "reference",
            "sample": ref_sample_desc(wl, ex, small, large, threads), "measured_s": ex["t_large"]}


def timed_call(fn):
    """(seconds by CUDA events, result) of one call, synchronised on both sides."""
    import torch
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    out = fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1e3, out


def accuracy_block(args, params, step_with, outputs, t_dev):
    """The measured form's errors, and the FP32 form's, against one run of the
    FP64-grade form on the same resident matrix (same seed, same Omega, same
    schedule); the FP32 form's time over the measured one."""
    from pcaone_gb300 import accuracy as A
    from pcaone_gb300 import capi
    p64 = capi.Params.from_buffer_copy(params)
    p64.precision = capi.PREC_FP64
    t64, (Uo, So, Vo, _) = timed_call(lambda: step_with(p64))
    U, S, V = outputs
    errors = {args.precision: A.compare_pcs(U, S, V, Uo, So, Vo)}
    out = {"oracle": "FP64-grade form: six 9-bit integer slices of the test matrix and of G (54 bits per column), "
                     "exact integer accumulation in TMEM, FP64 slice combination and epilogues; same Omega and "
                     "schedule", "oracle_s": t64,
           "bars": {"sin_angle": 1e-6, "eig_relerr": 1e-8}, "errors": errors,
           "S_oracle_top": [float(x) for x in So[:8]]}
    if args.precision == "fp8":
        pb = capi.Params.from_buffer_copy(params)
        pb.precision = capi.PREC_BF16
        tb, (Ub, Sb, Vb, _) = timed_call(lambda: step_with(pb))
        errors["bf16"] = A.compare_pcs(Ub, Sb, Vb, Uo, So, Vo)
        out["bf16_form_s"] = tb
    if args.precision != "fp32":
        p32 = capi.Params.from_buffer_copy(params)
        p32.precision = capi.PREC_FP32
        t32, (U32, S32, V32, _) = timed_call(lambda: step_with(p32))
        errors["fp32"] = A.compare_pcs(U32, S32, V32, Uo, So, Vo)
        out["fp32_form_s"] = t32
        out["speedup_vs_fp32_form"] = t32 / t_dev
    return out


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, int(os.environ.get("LOCAL_RANK", "0"))
    import torch.distributed as dist
    dist.init_process_group("gloo")
    return dist.get_rank(), ws, int(os.environ.get("LOCAL_RANK", "0"))


def reduce_max(x: float, ws: int) -> float:
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws: int):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def run_reference(args):
    """The reference arm: the reference's own CPU path on bounded samples of the
    workload (REF_SAMPLES), all host threads; rank 0 only.  Falls back to the
    numpy/LAPACK restatement (kind "port") when the reference cannot be built
    on this host."""
    rank, ws, _ = dist_init()
    if rank != 0:
        return
    wl_name = args.workload
    from pcaone_gb300 import synthetic
    wl = synthetic.WORKLOADS[wl_name]
    config = {"workload": f"{wl_name}: N={wl['nsamples']} x M={wl['nsnps']} "
                          f"{'FP16 dosages' if wl.get('dense') else 'PLINK'}, k={wl['k']}, p={wl['p']}, winSVD "
                          f"{wl['bands']} windows, {wl['maxp'] + 1} epochs"}
    drv = None if wl.get("dense") else ref_driver()
    line = {"impl": "reference", "metric": "sec_to_topk_pcs", "unit": "s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config}
    if drv is not None:
        threads = host_cores()
        smp = RefSamples(wl_name)
        try:
            small = ref_run(drv, smp.prefixes[0], smp.dir, wl, threads)
            for _ in range(max(0, args.warmup - 1)):
                ref_run(drv, smp.prefixes[1], smp.dir, wl, threads)
            large = [ref_run(drv, smp.prefixes[1], smp.dir, wl, threads) for _ in range(args.steps)]
        finally:
            smp.close()
        ex = ref_extrapolate(wl, small, large)
        v = ex["value"]
        line.update({"value": v, "value_kind": "extrapolated from the measured sample (cpu_baseline.sample)",
                     "ms_per_step": statistics.median(r["wall_s"] for r in large) * 1e3,
                     "ms_per_step_note": "measured wall time of one step (one run of the sample)",
                     "cpu_baseline": {"value": v, "unit": "s", "cores": threads, "kind": "reference",
                                      "sample": ref_sample_desc(wl, ex, small, large, threads),
                                      "measured_s": ex["t_large"]},
                     "extrapolation": ex})
    else:
        times, walls = [], []
        desc, cores = "", 1
        for it in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            _, scaled, desc, cores = cpu_sample_run(wl_name)
            if it >= args.warmup:
                times.append(scaled)
                walls.append(time.perf_counter() - t0)
        v = statistics.median(times)
        line.update({"value": v, "value_kind": "extrapolated from the measured sample (cpu_baseline.sample)",
                     "ms_per_step": statistics.median(walls) * 1e3,
                     "cpu_baseline": {"value": v, "unit": "s", "cores": cores, "kind": "port", "sample": desc}})
    line["e2e"] = {"value": line["value"], "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    print(json.dumps(line), flush=True)


def run_dense(args, wl, params, model, peaks, peak_kind, rank, ws, local):
    """Dense (FileBinary, FP16) workloads: generated once on the device, each
    step runs the RSVD on the resident matrix."""
    import torch
    from pcaone_gb300 import capi
    N, M = model.nsamples, model.nsnps
    L = wl["k"] + wl["p"]
    ctx = capi.Context(local)
    ctx.load_synthetic_dense(model, wl.get("sd", 0.1))
    for _ in range(args.warmup):
        ctx.run_halko(params)
    torch.cuda.synchronize()
    ctx.set_profiling(True)
    launches0 = ctx.launch_count()
    times = []
    with ClockSampler(local) as clocks:
        barrier(ws)
        for _ in range(args.steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            U, S, V, _ = ctx.run_halko(params)
            e1.record()
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
        barrier(ws)
    launches = ctx.launch_count() - launches0
    kstats = ctx.kernel_stats()
    ctx.set_profiling(False)
    t_dev = reduce_max(sum(times) / len(times), ws)
    dom = max(kstats, key=lambda k: kstats[k]["ms"])
    ks = kstats[dom]
    # algorithmic bytes: the FP16 values the product reads, 2 bytes per entry = flops / L
    gbs = (ks["flops"] / L) / (ks["ms"] / 1e3) / 1e9 if ks["ms"] > 0 else 0.0
    peak = peaks.get("hbm_gbs", PEAKS_FALLBACK["hbm_gbs"])
    tflops = ks["flops"] / (ks["ms"] / 1e3) / 1e12 if ks["ms"] > 0 else 0.0
    roof = {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak, "traffic": None,
            "kernel": f"k_tc_{dom[0]}<dense>", "algorithmic_tflops": tflops,
            "note": (f"dense FP16 input: {2 * L} flop per 2-byte value, below the ridge, so HBM-bound; achieved = "
                     f"FP16 bytes read per launch / event time; peak = {peak_kind} copy bandwidth")}
    if rank == 0:
        line = {
            "metric": "sec_to_topk_pcs", "value": t_dev, "unit": "s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_dev * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f16", "data": "synthetic",
            "config": {"workload": workload_desc(args.workload, wl, model, 0), "precision": args.precision,
                       "l2": "inputs larger than L2 (FP16 matrix resident in HBM)", "replicas": ws},
            "clocks": clocks.summary(),
            "e2e": None,
            "e2e_note": "dense workloads are generated on the device; the host float32 image is not built",
            "gpu_launches": int(launches), "roofline": roof, "cpu_baseline": None, "kernels": kstats,
            "pcs": {"S_top": [float(x) for x in S[:5]]},
        }
        print(json.dumps(line), flush=True)
    ctx.close()


def host_mem_available():
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) * 1024
    except OSError:
        pass
    return None


def out_of_core_block(args, capi, local, pinned, M, N, params, in_core, in_core_perm):
    """The out-of-core form (pcaone_gpu_load_bed_stream) on the same matrix:
    the library's pinned host copy of the rows, two device slots of one window
    each within a 4 GiB device budget; seconds per run with the rows in host
    memory (CUDA events) and bytes streamed per run.  The window method's
    shuffle follows the reference's out-of-core order (permute_plink), so the
    PCs are compared with the in-core run's (its std::shuffle order) on the
    well-separated components, loadings back in file order."""
    from pcaone_gb300.accuracy import compare_pcs
    import torch
    stride = (N + 127) // 128 * 32
    avail = host_mem_available()
    if avail is not None and avail < 1.5 * M * stride:
        return {"skipped": f"{avail / 1e9:.0f} GB of host memory available, the pinned copy needs "
                           f"{M * stride / 1e9:.0f} GB"}
    budget = 4 << 30
    ctx = capi.Context(local)
    try:
        t0 = time.perf_counter()
        ctx.load_bed_stream(pinned.data_ptr(), N, budget, nsnps=M)
        load_s = time.perf_counter() - t0
        ctx.run_halko(params)  # warm-up
        ctx.stream_info()
        times, fetched = [], []
        for _ in range(max(1, min(args.steps, 3))):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            U, S, V, _ = ctx.run_halko(params)
            e1.record()
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
            fetched.append(ctx.stream_info()[1])
        t = sum(times) / len(times)
        Vf = np.empty_like(V)
        Vf[ctx.perm()] = V
        Vi = np.empty_like(in_core[2])
        Vi[in_core_perm] = in_core[2]
        agree = compare_pcs(U, S, Vf, in_core[0], in_core[1], Vi)
        svd = "window" if params.svd == capi.SVD_WINDOW else "single"
        blk, nblk = capi.stream_plan(M, N, params.svd, params.bands, budget)
        return {"value": t, "unit": "s", "device_budget_bytes": budget, "block_snps": blk, "blocks": nblk,
                "method": svd, "load_s": load_s, "bytes_streamed_per_run": sum(fetched) / len(fetched),
                "stream_gbs": sum(fetched) / len(fetched) / t / 1e9, "vs_in_core": agree,
                "note": "rows in the library's pinned host copy (device row layout), windows in the reference's "
                        "out-of-core order (permute_plink, --buffer 2); each window copied to a device slot by "
                        "pitched copies on a second stream while the previous window's products run; load_s "
                        "includes pinning the host copy"}
    finally:
        ctx.close()


def run_ours(args):
    rank, ws, local = dist_init()
    import torch
    from pcaone_gb300 import capi, synthetic
    torch.cuda.set_device(local)
    wl, params = workload_params(args.workload, args.precision)
    if args.maxiter is not None:
        params.maxiter = args.maxiter
        wl = dict(wl, maxiter=args.maxiter)
    model = synthetic.model_for(args.workload, seed=1)
    if wl.get("dense"):
        peaks, peak_kind = load_peaks()
        return run_dense(args, wl, params, model, peaks, peak_kind, rank, ws, local)
    N, M = model.nsamples, model.nsnps
    bps = (N + 3) // 4
    L = wl["k"] + wl["p"]
    peaks, peak_kind = load_peaks()

    ctx = capi.Context(local)
    if args.warm_start:
        ctx.set_warm_start(capi.mlp_default_params())
    # the resident source matrix (value path) and a pinned host copy (e2e path)
    src = capi.Context(local)
    src.load_synthetic(model)
    dev_src = torch.empty((M, bps), dtype=torch.uint8, device=f"cuda:{local}")
    pinned = torch.empty((M, bps), dtype=torch.uint8, pin_memory=True)
    src.get_bed(out_ptr=pinned.data_ptr())
    dev_src.copy_(pinned)
    src.close()
    torch.cuda.synchronize()

    em_iters = []

    def step_device_with(p):
        ctx.load_bed_device(dev_src.data_ptr(), bps, M, N)
        return ctx.run_halko(p)

    def step_device():
        out = step_device_with(params)
        em_iters.append(out[3])
        return out

    load_s = []

    def step_e2e():
        t0 = time.perf_counter()
        ctx.load_bed_ptr(pinned.data_ptr(), M, N)
        load_s.append(time.perf_counter() - t0)
        return ctx.run_halko(params)

    for _ in range(args.warmup):
        step_device()
    torch.cuda.synchronize()

    # ---- value: resident inputs, CUDA events around each step ----
    ctx.set_profiling(True)
    launches0 = ctx.launch_count()
    times = []
    with ClockSampler(local) as clocks:
        barrier(ws)
        torch.cuda.synchronize()
        for _ in range(args.steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            U, S, V, _ = step_device()
            e1.record()
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
        barrier(ws)
    launches = ctx.launch_count() - launches0
    kstats = ctx.kernel_stats()
    host_phases = ctx.timings()  # host-clock phases of the last timed run_halko call
    ctx.set_profiling(False)
    t_dev = reduce_max(sum(times) / len(times), ws)

    # ---- e2e: host buffers through the C-ABI ----
    step_e2e()
    torch.cuda.synchronize()
    etimes = []
    for _ in range(args.steps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        step_e2e()
        e1.record()
        torch.cuda.synchronize()
        etimes.append(e0.elapsed_time(e1) / 1e3)
    t_e2e = reduce_max(sum(etimes) / len(etimes), ws)
    h2d = M * bps + N * L * 8

    # ---- out-of-core: the rows stay in pinned host memory, SNP blocks streamed ----
    ooc = None
    if rank == 0 and not args.no_out_of_core:
        ooc = out_of_core_block(args, capi, local, pinned, M, N, params, (U, S, V), ctx.perm())
    d2h = (N + M) * wl["k"] * 8 + wl["k"] * 8

    # ---- roofline of the dominant kernel (and of every product class) ----
    bf16_peak = peaks.get("bf16_tflops", PEAKS_FALLBACK["bf16_tflops"])
    tc = args.precision != "fp32"
    LPtc = (L + 15) // 16 * 16

    def roofline_of(cls):
        ks = kstats[cls]
        e4m3 = cls.endswith("_e4m3")
        achieved = ks["flops"] / (ks["ms"] / 1e3) / 1e12 if ks["ms"] > 0 else 0.0
        # the dense E4M3 rate is twice the BF16 one on this tensor core (4.5 vs
        # 2.25 PFLOP/s nominal); no FP8 GEMM is measured, so its peak is 2x the
        # measured BF16
        peak = 2.0 * bf16_peak if e4m3 else bf16_peak
        nslices = 2 if e4m3 else 6 if args.precision == "fp64" else 3
        executed = achieved * (nslices * LPtc / L) if tc else achieved
        per_launch_s = ks["ms"] / 1e3 / max(1, ks["launches"])
        # both tensor-core products run k_tc_g (mode 2: E4M3, 0: BF16 digits); H
        # reads the sample-major copy of the rows
        kname = (f"k_tc_g<{2 if e4m3 else 0}> ({cls[0].upper()} product)") if tc else f"k_window_{cls[0]}"
        traffic = NCU_TRAFFIC.get((args.workload, cls)) if tc else None
        r = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
             "frac": achieved / peak, "traffic": traffic, "kernel": kname,
             "executed_tflops": executed, "executed_frac": executed / peak,
             "hbm_gbs": (traffic / per_launch_s / 1e9) if traffic else None,
             "note": (f"{args.precision} form; {ks['launches']} launches, {ks['ms']:.1f} ms of "
                      f"{sum(times) * 1e3:.1f} ms; achieved = algorithmic 2*N*SNPs*L per launch / event time; "
                      f"peak = {'2x ' if e4m3 else ''}{peak_kind} bf16 dense"
                      f"{' (E4M3 dense rate)' if e4m3 else ''}; executed counts {nslices} integer slices of "
                      f"{LPtc} columns; traffic per launch from ncu of the same window shape (null: not captured)")}
        if not tc:
            r["note"] += "; the FP32 form runs on CUDA cores, not the tensor pipe"
        return r

    dom = max(kstats, key=lambda k: kstats[k]["ms"])
    roof = roofline_of(dom)
    roof_by_class = {cls: roofline_of(cls) for cls in kstats if kstats[cls]["launches"] > 0}

    # ---- accuracy against the FP64-grade form; the FP32 CUDA-core form ----
    accuracy = None
    if rank == 0 and not args.no_accuracy and not wl.get("emu"):
        accuracy = accuracy_block(args, params, step_device_with, (U, S, V), t_dev)

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        cpu = reference_cpu_baseline(args.workload, wl)
        if cpu is None:
            t_s, t_full, desc, cores = cpu_sample_run(args.workload)
            if wl.get("emu"):
                t_full *= (em_iters[-1] + 2) if em_iters else 1
                desc += f"; scaled by {em_iters[-1] + 2 if em_iters else 1} RSVD passes (EM iterations + 2)"
            cpu = {"value": t_full, "unit": "s", "cores": cores, "kind": "port", "sample": desc}

    if rank == 0:
        line = {
            "metric": "sec_to_topk_pcs", "value": t_dev, "unit": "s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_dev * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": args.precision, "data": "synthetic",
            "config": {"workload": workload_desc(args.workload, wl, model, bps),
                       "precision": args.precision, "l2": "inputs larger than L2 (packed matrix resident in HBM)",
                       "replicas": ws},
            "clocks": clocks.summary(),
            "e2e": {"value": t_e2e, "unit": "s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "load_s": statistics.median(load_s[1:]) if len(load_s) > 1 else None,
                    "load_gbs": M * bps / statistics.median(load_s[1:]) / 1e9 if len(load_s) > 1 else None},
            "gpu_launches": int(launches),
            "roofline": roof,
            "roofline_by_class": roof_by_class,
            "cpu_baseline": cpu,
            "kernels": kstats,
            "host_s": host_phases,
            "pcs": {"S_top": [float(x) for x in S[:5]]},
            "accuracy": accuracy,
            "out_of_core": ooc,
        }
        if wl.get("emu"):
            line["em"] = {"iterations": em_iters[-1] if em_iters else None, "tolem": params.tolem,
                          "warm_start": bool(args.warm_start)}
            if args.warm_start:
                line["em"]["mlp"] = ctx.mlp_stats()
        print(json.dumps(line), flush=True)
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c3")
    ap.add_argument("--precision", default="fp8", choices=["fp32", "bf16", "bf16x3", "fp8", "fp64"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the FP64-grade and FP32 reference runs")
    ap.add_argument("--no-out-of-core", action="store_true", help="skip the streamed (out-of-core) runs")
    ap.add_argument("--warm-start", action="store_true", help="learned EM warm start (EM workloads)")
    ap.add_argument("--maxiter", type=int, default=None, help="EM iteration cap (EM workloads)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
