"""Headline benchmark: ALS_SPD time to relative residual 1e-8 on one GB300.

Workload (the reference's CPU-runnable ALS configuration, at the smallest rank
that reaches 1e-8): d=8, n=4 Laplacian-sum TT operator (rank 2), random rank-4
right-hand side, random normalised rank-32 start, seeded 0xBAADF00D; one step =
one full ALS_SPD solve from the start until the FP64 residual ||Ax-b||/||b|| at
the end of a half-sweep is <= 1e-8 (cap 20 half-sweeps).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

The gb300 arm times both the mixed form (FP32 CG with FP64 refinement; the
line's `value`) and the plain FP64 form. `e2e` repeats the mixed solve through
the C ABI from pinned host buffers with the uploads and the download inside the
timed region. The reference arm times the CPU restatement of the reference's
algorithm (dense LAPACK local solves) on this host's cores.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(workload="ALS_SPD d=8 n=4 Laplacian, rhs rank 4, x rank 32, to rel. residual 1e-8", d=8, n=4,
                rhs_rank=4, x_rank=32, target=1e-8, max_half_sweeps=20, seed="0xBAADF00D")
METRIC = "ALS/DMRG time to rel. residual 1e-8"
SEED = 0xBAADF00D


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--workloads", default="all", choices=["all", "headline"],
                   help="all: also time TT round/dot (d=32 r=64), ADF (d=10, 200k samples) and the 4096-instance batch")
    p.add_argument("--batch-count", type=int, default=4096)
    p.add_argument("--only", choices=["round", "adf", "batch", "dmrg", "tc"],
                   help="run one secondary workload alone and print its JSON (for profiling)")
    p.add_argument("--adf-iterations", type=int, default=50, help="ADF iterations per timed run")
    return p.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


class ClockSampler:
    """nvidia-smi clock / throttle samples while the timed region runs."""

    def __init__(self, gpu=0):
        self.gpu, self.samples, self.proc = gpu, [], None

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([v.strip() for v in line.split(",")])

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.3)
        self.proc.terminate()
        self.proc.wait(timeout=5)
        sm = [float(s[1]) for s in self.samples if len(s) > 8 and s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if len(s) > 8 and s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples if len(s) > 8 for i in range(4) if s[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def make_inputs(xg, ctx):
    """Operator, rhs and start on the device, drawn with the library's engine."""
    xg.seed(SEED)
    A = xg.TTOperator.from_cores(xg.laplacian_cores(WORKLOAD["d"], WORKLOAD["n"]), ctx=ctx)
    b = xg.TTTensor.random([WORKLOAD["n"]] * WORKLOAD["d"], WORKLOAD["rhs_rank"], ctx=ctx)
    x0 = xg.TTTensor.random([WORKLOAD["n"]] * WORKLOAD["d"], WORKLOAD["x_rank"], ctx=ctx)
    x0 /= x0.frob_norm()
    return A, b, x0


def als_variant(xg, precision):
    v = xg.ALS_SPD.copy()
    v.convergenceEpsilon = 0.0
    v.residual_target = WORKLOAD["target"]
    v.precision = precision
    return v


def matvec_cost(ranks, opranks, dims, w):
    """Per 1-site local matvec at each position k: flops 2 n r r' (r R + n R R' + R' r')
    and minimal operand bytes w (r^2 R + r n r' + R n^2 R' + r'^2 R')."""
    out = {}
    for k in range(len(dims)):
        r, rp, R, Rp, n = ranks[k], ranks[k + 1], opranks[k], opranks[k + 1], dims[k]
        out[k] = (2 * n * r * rp * (r * R + n * R * Rp + Rp * rp), w * (r * r * R + r * n * rp + R * n * n * Rp + rp * rp * Rp))
    return out


def read_profile_traffic(name):
    """dram bytes per launch of a kernel class from its committed ncu summary (None if absent)."""
    path = os.path.join(ROOT, "profiles", f"{name}.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.strip().startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


def read_profile_field(name, field):
    """A `field: value` line of a committed ncu summary (None if absent)."""
    path = os.path.join(ROOT, "profiles", f"{name}.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.strip().startswith(field + ":"):
            try:
                return float(line.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


def reference_cpu_times():
    """The compiled xerus reference timed on the build host by oracle/ref/time_reference.py
    (the GPU host has no copy of the reference sources to build it): None if absent."""
    path = os.path.join(ROOT, "oracle", "ref_cpu_times.json")
    return json.load(open(path)) if os.path.exists(path) else None


def ref_leg(key, threads_key, fields):
    """One configuration's compiled-reference timings, labelled with the host they come from."""
    t = reference_cpu_times()
    if not t or key not in t or threads_key not in t[key]:
        return None
    out = {f: t[key][threads_key][f] for f in fields if f in t[key][threads_key]}
    out["kind"] = "reference"
    out["threads"] = int(threads_key.split("_")[1])
    out["host"] = f"{t['host']['cpu']} ({t['host']['cores']} cores, {t['host']['machine']}, {t['host']['openblas']}): " \
                  "the build host, not the GPU host"
    return out


def bench_qr_shape(xg, ctx, reps=20):
    """The headline's move_core factorisation on its own: Householder QR with Q of a
    128 x 32 core (rank-32 cores of mode size 4), timed by the context's CUDA events over
    `reps` launches. Algorithmic bytes: read A, write Q and R (8 (2 m n + n^2))."""
    m, n = 128, 32
    xg.seed(1)
    x = xg.TTTensor.random([m, n], n, ctx=ctx)
    flat, r = x.get_flat(), x.all_ranks()
    for _ in range(3):
        x.set_flat(flat, ranks=r)
        x.assume_core_position(0)
        x.move_core(1, True)
    ctx.profile(True)
    for _ in range(reps):
        x.set_flat(flat, ranks=r)
        x.assume_core_position(0)
        x.move_core(1, True)
    nl, ms = ctx.profile_get("qr")
    ctx.profile(False)
    per = ms / max(nl, 1)
    alg = 8.0 * (2 * m * n + n * n)
    return {"shape": f"{m} x {n} with Q", "launches": nl, "avg_launch_ms": per, "us_per_factorisation": 1e3 * per,
            "algorithmic_bytes_per_launch": alg, "algorithmic_flops_per_launch": 4.0 * m * n * n - 4.0 * n ** 3 / 3}


def bench_cfg1_rank8(xg, ctx, torch, stream, steps):
    """Configuration 1 as stated: ALS_SPD on the d=8, n=4 Laplacian, x rank 8, 20
    half-sweeps with convergenceEpsilon 0 (stops at residual ~1.2e-3: rank 8 cannot reach
    1e-8), FP64 and mixed, with the compiled reference's time beside it."""
    xg.seed(SEED)
    A = xg.TTOperator.from_cores(xg.laplacian_cores(8, 4), ctx=ctx)
    b = xg.TTTensor.random([4] * 8, 4, ctx=ctx)
    x0 = xg.TTTensor.random([4] * 8, 8, ctx=ctx)
    x0 /= x0.frob_norm()
    out = {"workload": "ALS_SPD d=8 n=4 Laplacian, rhs rank 4, x rank 8, 20 half-sweeps, convergenceEpsilon 0"}
    for name, prec in (("fp64", xg.FP64), ("mixed", xg.MIXED)):
        v = xg.ALS_SPD.copy()
        v.convergenceEpsilon = 0.0
        v.precision = prec
        times = []
        for i in range(steps + 2):
            x = x0.copy()
            torch.cuda.synchronize()
            e0, e1 = _events(torch, stream)
            e0.record(stream)
            v(A, x, b, 20)
            e1.record(stream)
            torch.cuda.synchronize()
            if i >= 2:
                times.append(e0.elapsed_time(e1))
        out[name] = {"ms": statistics.mean(times), "residual": xg.residual(A, x, b), "energy": v.last_report.energy}
    out["cpu_reference_build_host"] = ref_leg("cfg1", "threads_8", ["r8_hs20_seconds", "r8_hs20_residual"])
    return out


def _events(torch, stream):
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def bench_round_dot(xg, ctx, torch, stream, steps, cpu):
    """TT rounding and dot product: d=32, n=4, rank 64, cores N(0, 1/8); move_core(d-1)
    (pivoted QC sweep), round to rank 32, dot with an independent second tensor (FP64)."""
    d, n = 32, 4
    xg.seed(SEED)
    x0 = xg.TTTensor.random([n] * d, 64, 0.0, 1.0 / 8, ctx=ctx)
    y = xg.TTTensor.random([n] * d, 64, 0.0, 1.0 / 8, ctx=ctx)
    t = {"move_core": [], "round": [], "dot": []}
    for i in range(steps + 1):
        x = x0.copy()
        torch.cuda.synchronize()
        for name, fn in (("move_core", lambda: x.move_core(d - 1)), ("round", lambda: x.round(32)),
                         ("dot", lambda: xg.dot(x0, y))):
            e0, e1 = _events(torch, stream)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            if i > 0:
                t[name].append(e0.elapsed_time(e1))
    out = {"workload": "TT move_core + round(32) + dot, d=32 n=4 rank 64, FP64", "ranks_after_round": x.ranks()[:4],
           "ms": {k: statistics.mean(v) for k, v in t.items()}}
    # precision forms: the contractions on the tensor cores (QR and SVD stay FP64);
    # singular-value, norm and dot-product errors against the FP64 form
    x = x0.copy()
    sp64 = np.array(x.round(32, spectra=True))
    nrm64, dot64 = x.frob_norm(), xg.dot(x0, y)
    forms = {}
    try:
        for form in ("tf32x3", "bf16x3", "tf32"):
            ctx.set_contraction_precision(form)
            tf = {"move_core": [], "round": [], "dot": []}
            for i in range(steps + 1):
                x = x0.copy()
                torch.cuda.synchronize()
                for name, fn in (("move_core", lambda: x.move_core(d - 1)), ("round", lambda: x.round(32)),
                                 ("dot", lambda: xg.dot(x0, y))):
                    e0, e1 = _events(torch, stream)
                    e0.record(stream)
                    fn()
                    e1.record(stream)
                    torch.cuda.synchronize()
                    if i > 0:
                        tf[name].append(e0.elapsed_time(e1))
            x = x0.copy()
            sp = np.array(x.round(32, spectra=True))
            forms[form] = {"ms": {k: statistics.mean(v) for k, v in tf.items()},
                           "singular_value_rel_err_max": float(np.max(np.abs(sp - sp64) / np.abs(sp64))),
                           "norm_rel_err": abs(x.frob_norm() / nrm64 - 1), "dot_rel_err": abs(xg.dot(x0, y) / dot64 - 1),
                           "dot_err_over_norms": abs(xg.dot(x0, y) - dot64) / (x0.frob_norm() * y.frob_norm())}
    finally:
        ctx.set_contraction_precision("fp64")
    out["precision_forms"] = forms
    if cpu:
        from oracle import xtt_oracle as o
        xh = o.TT(x0.get_cores(), x0.canonicalized, x0.corePosition)
        yh = o.TT(y.get_cores(), y.canonicalized, y.corePosition)
        c = {}
        t0 = time.perf_counter()
        o.move_core(xh, d - 1)
        c["move_core"] = 1e3 * (time.perf_counter() - t0)
        t0 = time.perf_counter()
        o.tt_round(xh, [32] * (d - 1))
        c["round"] = 1e3 * (time.perf_counter() - t0)
        t0 = time.perf_counter()
        o.tt_dot(o.TT(x0.get_cores(), x0.canonicalized, x0.corePosition), yh)
        c["dot"] = 1e3 * (time.perf_counter() - t0)
        out["cpu_ms"] = c
        out["cpu_kind"] = "port (numpy/LAPACK, all BLAS threads)"
    return out


def bench_adf(xg, ctx, torch, stream, iters, peak, cpu):
    """ADF completion: d=10, n=8, rank-6 target, 200000 samples (+N(0,1e-6) noise),
    rank-6 model, `iters` iterations of ADFVariant(iters, 0, 1)."""
    d, n, r, N = 10, 8, 6, 200000
    xg.seed(SEED)
    target = xg.TTTensor.random([n] * d, r, ctx=ctx)
    m = xg.SinglePointMeasurementSet.random(N, [n] * d)
    m.measure(target)
    noise = np.zeros(N)
    xg._lib.load().xtt_random_normal(0.0, 1e-6, N, noise.ctypes.data_as(xg._lib.c_double_p))
    m.measuredValues = m.measuredValues + noise
    x0 = xg.TTTensor.random([n] * d, r, ctx=ctx)
    out = {"workload": "ADF d=10 n=8 rank 6, 200000 samples", "iterations": iters}
    for name, prec, w in (("fp64", xg.FP64, 8), ("fp32", xg.MIXED, 4)):
        xg.ADFVariant(2, 0.0, 1.0, precision=prec)(x0.copy(), m)  # warm-up
        x = x0.copy()
        torch.cuda.synchronize()
        e0, e1 = _events(torch, stream)
        e0.record(stream)
        res = xg.ADFVariant(iters, 0.0, 1.0, precision=prec)(x, m)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / iters
        # per iteration: stack updates, residuals, gradient scatter and slice norms over all
        # positions, N d w (5 r + 4) bytes (w = 8 in FP64, 4 with FP32 stacks)
        alg = N * d * w * (5 * r + 4)
        out[name] = {"ms_per_iteration": ms, "samples_per_s": N / (ms / 1e3), "final_residual_fp64_checked": res,
                     "roofline": {"bound": "hbm", "achieved": alg / (ms / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                                  "frac": alg / (ms / 1e3) / 1e9 / peak, "algorithmic_bytes_per_iteration": alg}}
        # where an iteration's time goes: a separate run with per-class CUDA-event timing
        ctx.profile(True)
        xg.ADFVariant(iters, 0.0, 1.0, precision=prec)(x0.copy(), m)
        ctx.profile(False)
        out[name]["kernel_ms_per_iteration"] = {k: ctx.profile_get(k)[1] / iters for k in
                                                ("adf_res_grad", "adf_slicenorm", "adf_stack", "qr", "gemm")}
    out["fp32_speedup_vs_fp64"] = out["fp64"]["ms_per_iteration"] / out["fp32"]["ms_per_iteration"]
    if cpu:
        from oracle import xtt_oracle as o
        xh = o.TT(x0.get_cores(), x0.canonicalized, x0.corePosition)
        t0 = time.perf_counter()
        o.adf(xh, m.positions, m.measuredValues, 1, 0.0, 1.0)
        out["cpu_ms_per_iteration"] = 1e3 * (time.perf_counter() - t0)
        out["cpu_sample"] = "1 iteration of the same problem (numpy port, all BLAS threads)"
    return out


FP64_NOMINAL_GFLOPS = 1250.0  # GB300 dense FP64, nominal
FP32_NOMINAL_GFLOPS = 152 * 128 * 2 * 2.07  # 152 SMs x 128 FP32 FMA per clock x 2.07 GHz


def config4_params(count, seed=SEED):
    """Shapes of the config-4 batch, instance by instance: (d, n, shift, rhs rank, start
    rank) with d ~ U{4..16}, n ~ U{2..8}, shift ~ U[0.1, 1], rhs rank ~ U{2..8}, start
    rank ~ U{4..32} (maximal-reduced when drawn)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        d, n = int(rng.integers(4, 17)), int(rng.integers(2, 9))
        shift = float(rng.uniform(0.1, 1.0))
        out.append((d, n, shift, int(rng.integers(2, 9)), int(rng.integers(4, 33))))
    return out


def config4_instance(xg, ctx, i, params, seed=SEED):
    """Instance i of the config-4 batch on the device: its own random state (seed + i),
    the Laplacian sum plus its shift, a random rhs and a random normalised start."""
    d, n, shift, rb, rx = params
    xg.seed(seed + i)
    A = xg.TTOperator.from_cores(xg.laplacian_cores(d, n, shift=shift), ctx=ctx)
    b = xg.TTTensor.random([n] * d, rb, ctx=ctx)
    x = xg.TTTensor.random([n] * d, rx, ctx=ctx)
    x /= x.frob_norm()
    return A, x, b


def bench_batch(xg, ctx, count, steps):
    """Config-4 batch: `count` independent SPD problems, d ~ U{4..16}, n ~ U{2..8},
    Laplacian sum + shift U[0.1, 1], rhs rank ~ U{2..8}, start rank ~ U{4..32}
    (maximal-reduced), 4 ALS sweeps each, in one persistent launch (CUDA graph)."""
    As, xs, bs = [], [], []
    for i, prm in enumerate(config4_params(count)):
        A, x, b = config4_instance(xg, ctx, i, prm)
        As.append(A)
        xs.append(x)
        bs.append(b)
    saved = [(x.get_flat(), x.all_ranks()) for x in xs]

    def restore():
        for x, (f, r) in zip(xs, saved):
            x.set_flat(f, ranks=r)
            x.assume_core_position(0)

    out = {"workload": f"{count} independent ALS_SPD problems (config 4), 4 sweeps each", "count": count}
    for name, prec in (("fp64", xg.FP64), ("mixed", xg.MIXED)):
        v = xg.ALS_SPD.copy()
        v.convergenceEpsilon = 0.0
        v.precision = prec
        restore()
        _, _, rep = xg.als_batch(As, xs, bs, variant=v, numHalfSweeps=8, autotune=True)
        ms, its = [], None
        for _ in range(steps):
            restore()
            en, its, rep = xg.als_batch(As, xs, bs, variant=v, numHalfSweeps=8)
            ms.append(rep["milliseconds"])
        t = statistics.mean(ms)
        # algorithmic flops: per instance, its CG iterations times its mean 1-site local matvec,
        # plus one operator-environment push (the same contraction) per micro-step
        flops = 0.0
        for prm, (_, rk), it in zip(config4_params(count), saved, its):
            d, n = prm[0], prm[1]
            mv = matvec_cost(rk, [1] + [2] * (d - 1) + [1], [n] * d, 8)
            mean_mv = statistics.mean(mv[k][0] for k in range(d))
            flops += float(it) * mean_mv + 8 * (d - 1) * mean_mv
        gfs = flops / (t / 1e3) / 1e9
        # the FP64 form against the FP64 peak; the mixed form's CG runs in FP32 on the CUDA cores
        peak, pname = (FP64_NOMINAL_GFLOPS, "FP64") if name == "fp64" else (FP32_NOMINAL_GFLOPS, "FP32 CUDA-core")
        out[name] = {"ms": t, "instances_per_s": count / (t / 1e3), "launch": {k: rep[k] for k in ("threads", "ctas_per_sm", "ctas", "tile")},
                     "cg_iterations": int(its.sum()), "energy_sum": float(en.sum()),
                     "algorithmic_gflop": flops / 1e9, "gflop_per_s": gfs, "peak_frac": gfs / peak,
                     "peak": f"{peak:.0f} GFLOP/s {pname}, of nominal (MEASURED_PEAKS.json has neither figure)"}
    out["mixed_speedup_vs_fp64"] = out["fp64"]["ms"] / out["mixed"]["ms"]
    return out


def run_gpu(args):
    import torch
    import xerus_gb300 as xg
    from xerus_gb300 import build
    rank, local_rank, world = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    torch.cuda.set_device(local_rank)
    build.build()
    ctx = xg.Context(local_rank)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    A, b, x0 = make_inputs(xg, ctx)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")  # > 129 MB L2

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def solve(precision):
        x = x0.copy()
        v = als_variant(xg, precision)
        v(A, x, b, WORKLOAD["max_half_sweeps"])
        return x, v.last_report

    work = {}

    def timed(precision, steps, warmup, profile=False):
        for _ in range(warmup):
            solve(precision)
        if profile:
            ctx.profile(True)
        times, reports = [], []
        launches0 = ctx.kernel_launches()
        for _ in range(steps):
            flush.zero_()
            barrier()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            x, rep = solve(precision)
            e1.record(stream)
            barrier()
            times.append(e0.elapsed_time(e1) / 1e3)
            reports.append(rep)
        launches = ctx.kernel_launches() - launches0
        prof = {}
        if profile:
            for name in ("cg_fp64", "cg_mixed", "gemm", "qr", "svd"):
                prof[name] = ctx.profile_get(name)
                work[name] = ctx.profile_work(name)
            ctx.profile(False)
        return times, reports, launches, prof, x

    clocks = ClockSampler(local_rank)
    clocks.start()
    t_mix, rep_mix, launches_mix, _, x_mix = timed(xg.MIXED, args.steps, args.warmup)
    t_64, rep_64, launches_64, _, x_64 = timed(xg.FP64, args.steps, args.warmup)
    clk = clocks.stop()
    # per-kernel-class event timing in separate (untimed) passes: events add host work
    nprof = max(1, min(3, args.steps))
    _, _, _, prof_mix, _ = timed(xg.MIXED, nprof, 0, profile=True)
    prof_work = dict(work)
    _, _, _, prof_64, _ = timed(xg.FP64, nprof, 0, profile=True)
    prof_steps = nprof
    res_mix = xg.residual(A, x_mix, b)
    res_64 = xg.residual(A, x_64, b)

    # end to end through the C ABI: host buffers in, result out, every step
    import ctypes
    hA = [np.ascontiguousarray(c) for c in A.get_cores()]
    hb, hx0 = b.get_flat(), x0.get_flat()
    pin = lambda a: torch.from_numpy(a).pin_memory().numpy()
    hA_flat, hb, hx0 = pin(np.concatenate([c.ravel() for c in hA])), pin(hb), pin(hx0)
    A_ranks, b_ranks, x_ranks = A.all_ranks(), b.all_ranks(), x0.all_ranks()
    Ad = xg.TTOperator([WORKLOAD["n"]] * WORKLOAD["d"], A_ranks, ctx=ctx)
    bd = xg.TTTensor([WORKLOAD["n"]] * WORKLOAD["d"], b_ranks, ctx=ctx)
    xd = xg.TTTensor([WORKLOAD["n"]] * WORKLOAD["d"], x_ranks, ctx=ctx)
    hout = pin(np.zeros(x0.size()))
    e2e_times = []
    v = als_variant(xg, xg.MIXED)
    for i in range(args.warmup + args.steps):
        flush.zero_()
        barrier()
        t0 = time.perf_counter()
        Ad.set_flat(hA_flat)
        bd.set_flat(hb)
        bd.assume_core_position(0)
        xd.set_flat(hx0, ranks=x_ranks)
        xd.assume_core_position(0)
        v(Ad, xd, bd, WORKLOAD["max_half_sweeps"])
        out = xd.get_flat()
        resid = v.last_report.residual
        torch.cuda.synchronize()
        if i >= args.warmup:
            e2e_times.append(time.perf_counter() - t0)
    h2d = 8 * (hA_flat.size + hb.size + hx0.size)
    d2h = 8 * (out.size + 1)

    # roofline of the dominant kernel class (the persistent CG) over the timed mixed solves
    ranks, opr, dims = x0.all_ranks(), A.all_ranks(), x0.dimensions
    iters = sum(r.local_iterations for r in rep_mix) / len(rep_mix)
    refs = sum(r.refinements for r in rep_mix) / len(rep_mix)
    steps_per = rep_mix[0].micro_steps
    cost32, cost64 = matvec_cost(ranks, opr, dims, 4), matvec_cost(ranks, opr, dims, 8)
    # sweep visits the optimised positions (rank < full) evenly; use their mean per-matvec cost
    opt = [k for k in range(1, len(dims) - 1)]
    f_avg = sum(cost32[k][0] for k in opt) / len(opt)
    b32 = sum(cost32[k][1] for k in opt) / len(opt)
    b64 = sum(cost64[k][1] for k in opt) / len(opt)
    # per solve: FP32 matvecs = CG iterations; FP64 matvecs = one per refinement pass + 1 per step
    cg_launches, cg_ms = prof_mix.get("cg_mixed", (0, 0.0))
    per_launch_ms = cg_ms / max(cg_launches, 1)
    mv32 = iters / max(steps_per, 1)
    mv64 = (refs + steps_per) / max(steps_per, 1)
    alg_bytes = mv32 * b32 + mv64 * b64
    alg_flops = (mv32 + mv64) * f_avg
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {"hbm_gbs": 6800.0}
    achieved = alg_bytes / (per_launch_ms / 1e3) / 1e9 if per_launch_ms > 0 else 0.0
    traffic = read_profile_traffic("cg_cluster_mixed_als_d8_r32")
    top = max(prof_mix.items(), key=lambda kv: kv[1][1])[0] if prof_mix else None

    value = statistics.mean(t_mix)
    vmax = value
    if world > 1:
        t = torch.tensor([value], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        vmax = float(t.item())
    if rank != 0:
        return None
    line = {
        "metric": METRIC, "value": vmax, "unit": "s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * vmax, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64+f32 (mixed: FP32 CG, FP64 refinement and residual)", "data": "synthetic, seeded 0xBAADF00D",
        "config": dict(WORKLOAD, precision="mixed", parallelism="replicas" if world > 1 else "single GPU",
                       l2="flushed (256 MB write) between timed steps"),
        "fp64": {"ms_per_step": 1e3 * statistics.mean(t_64), "half_sweeps": rep_64[0].half_sweeps,
                 "residual": res_64, "cg_iterations": rep_64[0].local_iterations, "gpu_launches": launches_64 // args.steps,
                 "cg_kernel_ms": prof_64.get("cg_fp64", (0, 0.0))[1] / prof_steps},
        "mixed": {"ms_per_step": 1e3 * value, "half_sweeps": rep_mix[0].half_sweeps, "residual": res_mix,
                  "cg_iterations": rep_mix[0].local_iterations, "refinements": rep_mix[0].refinements},
        "mixed_speedup_vs_fp64": statistics.mean(t_64) / value,
        "e2e": {"value": statistics.mean(e2e_times), "unit": "s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "residual": resid},
        "gpu_launches": launches_mix // args.steps,
        "roofline": {"kernel": "k_cg_mixed (persistent CG)", "bound": "hbm", "achieved": achieved,
                     "peak": peaks.get("hbm_gbs", 6800.0), "unit": "GB/s",
                     "frac": achieved / peaks.get("hbm_gbs", 6800.0), "traffic": traffic,
                     "peak_source": "of measured" if "hbm_gbs" in peaks else "of fallback",
                     "algorithmic_bytes_per_launch": alg_bytes, "algorithmic_flops_per_launch": alg_flops,
                     "avg_launch_ms": per_launch_ms, "launches": cg_launches,
                     "tflops_achieved": alg_flops / (per_launch_ms / 1e3) / 1e12 if per_launch_ms > 0 else 0.0,
                     "top_kernel_class_by_time": top,
                     "kernel_ms_per_step": {k: v[1] / prof_steps for k, v in prof_mix.items()}},
        "clocks": clk,
    }
    # per-class kernel time and declared algorithmic work (profiled mixed passes)
    classes = {}
    for name in ("cg_mixed", "qr", "gemm"):
        nl, ms = prof_mix.get(name, (0, 0.0))
        by, fl = prof_work.get(name, (0.0, 0.0))
        if nl:
            classes[name] = {"ms_per_step": ms / prof_steps, "launches_per_step": nl / prof_steps,
                             "bytes_per_step": by / prof_steps, "flops_per_step": fl / prof_steps,
                             "GB_per_s": by / (ms / 1e3) / 1e9 if ms > 0 and by else None,
                             "GFLOP_per_s": fl / (ms / 1e3) / 1e9 if ms > 0 and fl else None}
    line["kernel_classes"] = classes
    if top == "qr":
        # the dominant class's most frequent launch (the move_core factorisation of a 128 x 32
        # core with Q) timed on its own, so achieved bytes, duration and the ncu traffic all
        # describe the same launch
        q = bench_qr_shape(xg, ctx)
        ach = q["algorithmic_bytes_per_launch"] / (q["avg_launch_ms"] / 1e3) / 1e9
        traffic = read_profile_traffic("qr_cl1_als_d8_r32")
        line["roofline"] = {"kernel": "k_qr_cl1 (FP64 Householder QR with Q, 128 x 32, 8-CTA cluster)",
                            "bound": "hbm", "achieved": ach, "peak": peaks.get("hbm_gbs", 6800.0), "unit": "GB/s",
                            "frac": ach / peaks.get("hbm_gbs", 6800.0), "traffic": traffic,
                            "traffic_over_algorithmic": traffic / q["algorithmic_bytes_per_launch"] if traffic else None,
                            "peak_source": "of measured" if "hbm_gbs" in peaks else "of fallback",
                            "algorithmic_bytes_per_launch": q["algorithmic_bytes_per_launch"],
                            "algorithmic_flops_per_launch": q["algorithmic_flops_per_launch"],
                            "avg_launch_ms": q["avg_launch_ms"], "launches": q["launches"],
                            "us_per_factorisation": q["us_per_factorisation"],
                            "fp64_pipe_pct": read_profile_field("qr_cl1_als_d8_r32", "fp64_pipe_pct_128x32"),
                            "top_kernel_class_by_time": top,
                            "class_launches_per_step": classes["qr"]["launches_per_step"] if "qr" in classes else None,
                            "note": "latency-bound: one cluster barrier and a dependent FP64 reflector chain per "
                                    "column; operands in L2 / shared memory, so the HBM fraction is not the limit",
                            "kernel_ms_per_step": {k: v[1] / prof_steps for k, v in prof_mix.items()},
                            "cg_mixed": line["roofline"]}
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(A, b, x0, samples=1)
    line["cpu_reference_build_host"] = ref_leg("cfg1", "threads_8", ["r32_hs2_seconds", "r32_hs2_residual"])
    if args.workloads == "all":
        peak = peaks.get("hbm_gbs", 6800.0)
        cpu = not args.no_cpu_baseline
        wl = {}
        wl["als_cfg1_rank8_hs20"] = bench_cfg1_rank8(xg, ctx, torch, stream, 5)
        wl["round_dot_d32_r64"] = bench_round_dot(xg, ctx, torch, stream, 3, cpu)
        wl["round_dot_d32_r64"]["cpu_reference_build_host"] = {
            t: ref_leg("cfg2", t, ["move_core_seconds", "round_seconds", "dot_seconds"]) for t in ("threads_1", "threads_8")}
        wl["adf_d10_n8_r6_200k"] = bench_adf(xg, ctx, torch, stream, args.adf_iterations, peak, cpu)
        r5 = ref_leg("cfg5", "threads_8", ["adf50_seconds", "adf50_residual"])
        if r5:
            r5["ms_per_iteration"] = r5["adf50_seconds"] * 1e3 / 50
        wl["adf_d10_n8_r6_200k"]["cpu_reference_build_host"] = r5
        wl["batch_als_cfg4"] = bench_batch(xg, ctx, args.batch_count, 2)
        wl["batch_als_cfg4"]["cpu_reference_build_host"] = ref_leg(
            "cfg4", "threads_8", ["instances_per_s", "sample_seconds", "sample_instances", "sample"])
        wl["als_tc_d20_n8_r128"] = bench_tc_als(xg, ctx, torch, stream, peaks)
        wl["dmrg_cfg3_d20_n8"] = bench_dmrg(xg, ctx, torch, stream, 16)
        line["workloads"] = wl
    return line


def cpu_baseline(A, b, x0, samples=1):
    """The CPU restatement of the reference's ALS (dense LAPACK local solves) on this
    host, on the same inputs, timed for `samples` full solves."""
    from oracle import xtt_oracle as o
    Ah = o.TTOp(A.get_cores())
    bh = o.TT(b.get_cores(), True, 0)
    ts = []
    for _ in range(samples):
        x = o.TT(x0.get_cores(), True, 0)
        t0 = time.perf_counter()
        o.als_spd(Ah, x, bh, 1, WORKLOAD["max_half_sweeps"], 0.0, residual_target=WORKLOAD["target"])
        ts.append(time.perf_counter() - t0)
    return {"value": statistics.mean(ts), "unit": "s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"{samples} full solve(s) of the same workload (numpy/LAPACK dense local solves, all BLAS threads)"}


def run_reference(args):
    rank, _, world = dist_env()
    if rank != 0:
        return None
    from oracle import xtt_oracle as o
    d, n = WORKLOAD["d"], WORKLOAD["n"]
    rs = o.RandomEngine(SEED)
    Ah = o.laplace_operator(d, n)
    bh = o.tt_random([n] * d, WORKLOAD["rhs_rank"], rs)
    x0 = o.tt_random([n] * d, WORKLOAD["x_rank"], rs)
    x0 = o.tt_scale(x0, 1.0 / o.frob_norm(x0))
    ts = []
    for i in range(args.warmup + args.steps):
        x = x0.copy()
        t0 = time.perf_counter()
        o.als_spd(Ah, x, bh, 1, WORKLOAD["max_half_sweeps"], 0.0, residual_target=WORKLOAD["target"])
        if i >= args.warmup:
            ts.append(time.perf_counter() - t0)
    v = statistics.mean(ts)
    return {"metric": METRIC, "value": v, "unit": "s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * v, "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic, seeded 0xBAADF00D", "config": WORKLOAD, "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "s", "cores": os.cpu_count(), "kind": "port",
                             "sample": "each step one full solve (dense LAPACK local solves, all BLAS threads)"},
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def bench_dmrg(xg, ctx, torch, stream, half_sweeps):
    """Two-site DMRG_SPD on the d=20, n=8 Laplacian sum plus a
    diagonal potential U[0,1] per mode (operator rank 3), random rank-16 start,
    ranks free to grow to 128 with SVD cutoff 1e-10, run until the FP64 residual
    reaches 1e-8 (checked after every half-sweep) or `half_sweeps` half-sweeps;
    FP64 and mixed forms, exact (orthonormal) environments."""
    d, n = 20, 8
    rng = np.random.default_rng(SEED)
    V = [rng.uniform(0.0, 1.0, n) for _ in range(d)]
    xg.seed(SEED)
    A = xg.TTOperator.from_cores(xg.laplacian_cores(d, n, potentials=V, rank3=True), ctx=ctx)
    b = xg.TTTensor.random([n] * d, 4, ctx=ctx)
    x0 = xg.TTTensor.random([n] * d, 16, ctx=ctx)
    x0 /= x0.frob_norm()
    out = {"workload": "DMRG_SPD d=20 n=8, operator rank 3, rank-16 start, max rank 128, SVD eps 1e-10, "
                       f"to residual 1e-8 (at most {half_sweeps} half-sweeps), exact environments"}
    for name, prec in (("fp64", xg.FP64), ("mixed", xg.MIXED)):
        v = xg.DMRG_SPD.copy()
        v.convergenceEpsilon = 0.0
        v.precision = prec
        v.exact_environment = True
        v.max_rank = 128
        v.svd_epsilon = 1e-10
        v.residual_target = 1e-8
        v(A, x0.copy(), b, 1)  # warm-up
        x = x0.copy()
        torch.cuda.synchronize()
        e0, e1 = _events(torch, stream)
        e0.record(stream)
        en = v(A, x, b, half_sweeps)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        out[name] = {"ms": ms, "half_sweeps": v.last_report.half_sweeps, "energy": en, "max_rank": max(x.ranks()),
                     "cg_iterations": v.last_report.local_iterations, "residual": xg.residual(A, x, b)}
    v = xg.DMRG_SPD.copy()
    v.convergenceEpsilon = 0.0
    v.precision = xg.MIXED
    v.exact_environment = True
    v.max_rank = 128
    v.svd_epsilon = 1e-10
    v.residual_target = 1e-8
    ctx.profile(True)
    v(A, x0.copy(), b, half_sweeps)
    ctx.profile(False)
    out["mixed_classes_ms"] = {k: ctx.profile_get(k)[1] for k in ("cg_mixed", "cg_fp64", "cg_tc", "gemm", "qr", "svd")}
    out["mixed_speedup_vs_fp64"] = out["fp64"]["ms"] / out["mixed"]["ms"]
    return out


def bench_tc_als(xg, ctx, torch, stream, peaks, rank=128, half_sweeps=2, reps=2):
    """Ranks >= 64: one-site ALS_SPD on the DMRG workload's operator (d=20, n=8,
    Laplacian sum plus a diagonal potential, operator rank 3; rhs rank 4), random
    rank-`rank` start, `half_sweeps` half-sweeps. FP64 form vs the mixed form, whose
    local solves there run on the tensor cores (FP64 refinement of FP32 CG with
    split-TF32 tcgen05 operator stages). CUDA events on the context's stream, no
    profiling in the timed runs; one profiled mixed run for the tensor-core GEMM's
    class figures."""
    d, n = 20, 8
    rng = np.random.default_rng(SEED)
    V = [rng.uniform(0.0, 1.0, n) for _ in range(d)]
    xg.seed(SEED)
    A = xg.TTOperator.from_cores(xg.laplacian_cores(d, n, potentials=V, rank3=True), ctx=ctx)
    b = xg.TTTensor.random([n] * d, 4, ctx=ctx)
    x0 = xg.TTTensor.random([n] * d, rank, ctx=ctx)
    x0 /= x0.frob_norm()
    out = {"workload": f"ALS_SPD d=20 n=8 (Laplacian sum + diagonal potential, operator rank 3), rhs rank 4, x rank {rank}, "
                       f"{half_sweeps} half-sweeps", "local_unknowns": rank * n * rank}
    for name, prec in (("fp64", xg.FP64), ("mixed", xg.MIXED)):
        v = xg.ALS_SPD.copy()
        v.convergenceEpsilon = 0.0
        v.precision = prec
        v(A, x0.copy(), b, 1)  # warm-up
        ts = []
        for _ in range(reps):
            x = x0.copy()
            torch.cuda.synchronize()
            e0, e1 = _events(torch, stream)
            e0.record(stream)
            en = v(A, x, b, half_sweeps)
            e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        out[name] = {"ms": statistics.mean(ts), "energy": en, "residual": xg.residual(A, x, b),
                     "cg_iterations": v.last_report.local_iterations, "refinements": v.last_report.refinements}
    out["mixed_speedup_vs_fp64"] = out["fp64"]["ms"] / out["mixed"]["ms"]
    v = xg.ALS_SPD.copy()
    v.convergenceEpsilon = 0.0
    v.precision = xg.MIXED
    ctx.profile(True)
    v(A, x0.copy(), b, half_sweeps)
    ctx.profile(False)
    nl, ms = ctx.profile_get("cg_tc")
    # algorithmic work of the FP32 CG on the tensor cores: per iteration one local
    # matvec, 2 n r r' (r R + n R R' + R' r') flops at an interior site, times 3 MMAs
    # per K step (split TF32); the launch also holds the FP64 refinement residuals
    r_, R_ = rank, 3
    mv = 2 * n * r_ * r_ * (r_ * R_ + n * R_ * R_ + R_ * r_)
    its = v.last_report.local_iterations
    fl = 3.0 * mv * its
    tf32_peak = 0.5 * peaks.get("bf16_tflops", 1900.0)
    ach = fl / (ms / 1e3) / 1e12 if ms > 0 else 0.0
    out["classes_ms"] = {k: ctx.profile_get(k)[1] for k in ("cg_tc", "cg_fp64", "gemm", "gemm_df", "qr")}
    out["roofline_cg_tc"] = {"kernel": "k_cg_mixed_tc (persistent: tcgen05 kind::tf32 operator stages, FP64 refinement)",
                             "bound": "tensor", "launches": nl, "avg_launch_ms": ms / max(nl, 1),
                             "cg_iterations": its, "algorithmic_flops_per_launch": fl / max(nl, 1), "achieved": ach,
                             "peak": tf32_peak, "unit": "TFLOP/s", "frac": ach / tf32_peak,
                             "peak_source": "half of measured bf16 (dense TF32 runs at half the BF16 rate)",
                             "note": "latency-bound: grid barriers between the 3 operator stages and the CG "
                                     "reductions; 16-192 work items per stage"}
    return out


def run_only(args):
    import torch
    import xerus_gb300 as xg
    from xerus_gb300 import build
    build.build()
    ctx = xg.Context(0)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {"hbm_gbs": 6800.0}
    cpu = not args.no_cpu_baseline
    if args.only == "round":
        return bench_round_dot(xg, ctx, torch, stream, args.steps, cpu)
    if args.only == "adf":
        return bench_adf(xg, ctx, torch, stream, args.adf_iterations, peaks.get("hbm_gbs", 6800.0), cpu)
    if args.only == "batch":
        return bench_batch(xg, ctx, args.batch_count, args.steps)
    if args.only == "tc":
        return bench_tc_als(xg, ctx, torch, stream, peaks)
    return bench_dmrg(xg, ctx, torch, stream, 16)


def main():
    args = parse()
    if args.only:
        print(json.dumps(run_only(args)))
        return
    line = run_reference(args) if args.impl == "reference" else run_gpu(args)
    if line is not None:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
