#!/usr/bin/env python
"""Benchmark of the GB300 permanent path; prints ONE JSON line (rank 0).

Workload (default): the plain Glynn/BBFG permanent of the top-left n x n block
of a seeded Haar-random 2n x 2n unitary, n = 36, complex128 (the single large
permanent configuration, n in {30, 34, 36, 40}).  One step = one permanent.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--n 36] [--mode fast|fp64]
  python bench.py --impl reference ...   # the reference algorithm on host cores
  python bench.py --workload repeated|batched|grad|pmf|mesh   # the other hot-path entry points

value   permanents/s with the matrix already resident in HBM (device-pointer
        entry point, CUDA events on the launching stream; L2 flushed between
        steps by writing a 256 MiB buffer);
e2e     the same metric through the public host-buffer entry point
        (gbperm_perm): pinned host matrix -> device copy, compute, result copied
        back, every step;
roofline  the permanent kernel: algorithmic FP64-equivalent flops
        (8 n 2^(n-1) per permanent) / kernel time against the FP64 FMA peak
        measured live by the library's probe, and for the double-float path
        the FP32 pipe peak too;
cpu_baseline  the C oracle (a restatement of the reference's BBFG double
        calculator with its 4 x threads segmentation) on all host cores, on a
        bounded sample of the same permanent's Gray range, scaled to perm/s.
"""
from __future__ import annotations

import argparse
import ctypes
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

METRIC = "complex perm/s at n=30/36/40 & batched k=8-28 vs plain GPU, rel err <=1e-10"
UNIT = "perm/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="plain",
                    choices=["plain", "repeated", "batched", "grad", "pmf", "mesh", "sampler"],
                    help="plain: single n x n Haar block (default); repeated: 60-mode / 30-photon "
                         "multiplicity permanent; batched: 4096 uneven k=8..28 permanents in one launch "
                         "(--batch-count, --batch-kmax); "
                         "grad: permanent + full gradient; pmf: one 60-mode / 30-photon boson-sampling "
                         "probability layer; mesh: 512-term Clements-mesh log-likelihood, forward + backward; "
                         "sampler: seeded boson samples, 40 modes / 20 photons")
    ap.add_argument("--n", type=int, default=36)
    ap.add_argument("--mode", default=None, choices=["fx", "fast", "fp64"],
                    help="arithmetic of the product: fx (integer mantissas, at least FP64 accuracy; the "
                         "plain default), fp64 (FP64 pipe; the default of the other workloads), fast "
                         "(double-float on the FP32 pipe, recomputed in FP64 above its error bar)")
    ap.add_argument("--check-steps", type=int, default=3,
                    help="plain: timed matrices recomputed by the other two products for the accuracy "
                         "check and their own rates")
    ap.add_argument("--seed", type=int, default=36)
    ap.add_argument("--batch-count", type=int, default=4096, help="batched: permanents per batch")
    ap.add_argument("--batch-kmax", type=int, default=28, help="batched: largest k (k uniform 8..kmax)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="length of the CPU baseline sample, seconds")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.batch_count < 1 or not 8 <= args.batch_kmax <= 32:
        ap.error("--batch-count must be >= 1 and --batch-kmax in 8..32")
    if args.mode is None:
        args.mode = {"plain": "fx", "repeated": "fx", "batched": "fx", "grad": "fast", "pmf": "fx",
                     "sampler": "fx"}.get(args.workload, "fp64")
    if args.mode == "fx" and args.workload not in ("plain", "repeated", "batched", "grad", "pmf", "sampler"):
        ap.error("--mode fx: the integer-mantissa product serves the plain, repeated, batched, grad, pmf and "
                 "sampler workloads")
    if args.workload == "grad" and args.mode == "fp64":
        ap.error("--workload grad: the gradient sweep runs the 'fast' or the 'fx' product")
    return args


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def flops_plain(n: int) -> float:
    return 8.0 * n * 2.0 ** (n - 1)


# ------------------------------------------------------------ CPU baseline
def workload_desc(args) -> str:
    """The workload line of `config`, the same for both arms."""
    n = args.n
    if args.workload == "repeated":
        return ("repeated permanent: 60-mode Haar, one photon in modes 0-29, output occupation "
                "from a seeded multinomial (multiplicities <= 4)")
    if args.workload == "batched":
        return (f"{args.batch_count} uneven k x k permanents, k uniform 8..{args.batch_kmax}, rows/cols drawn "
                "with repetition from a seeded 100-mode Haar unitary; one persistent launch per step")
    if args.workload == "grad":
        n = min(n, 32)
        return (f"permanent and full {n}x{n} complex gradient of the top-left block of a seeded "
                f"Haar {2 * n}x{2 * n} unitary, one sweep")
    if args.workload == "pmf":
        return ("boson-sampling pmf layer: 60-mode Haar, one input photon in modes 0-29, a seeded "
                "uniform-multinomial sample of 29 photons; 30 leave-one-out permanents per layer")
    if args.workload == "sampler":
        return ("boson samples: 40-mode Haar, one photon in each of modes 0-19, generalised Clifford & Clifford B "
                "sampler with the reference's mt19937 stream (seeded); one sample per step")
    if args.workload == "mesh":
        return ("512 terms log|perm(U_S)|^2, 12 photons in a 40-mode Clements mesh (seeded uniform "
                "phases, seeded mode sets), forward + backward to the 1560 phases")
    return f"plain permanent, top-left {n}x{n} block of a seeded Haar {2 * n}x{2 * n} unitary"


def cpu_sample_rate(A: np.ndarray, seconds: float, threads: int = 0, prec: int = 0):
    """Gray steps/s of the oracle on all host cores, on a bounded contiguous
    sample of the permanent's Gray range (calibrated to ~`seconds`).
    prec 0: double (the reference's lib 7); 1: binary128 (its lib 8 on
    AArch64, where long double is binary128)."""
    from tests import oracle_bind as orc

    lib = orc.lib()
    P = ctypes.c_void_p
    fn = lib.orc_bbfg_range_prec
    fn.argtypes = [P, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                   ctypes.c_uint64, ctypes.c_uint64, P]
    a = np.ascontiguousarray(A, dtype=np.complex128)
    n = a.shape[0]
    total = 1 << (n - 1)
    out = np.zeros(4)
    # calibrate on a small sample, then run the measured sample
    span = min(total, 1 << (22 if prec == 0 else 16))
    t0 = time.perf_counter()
    rc = fn(a.ctypes.data_as(P), n, n, n, prec, threads, 0, span, out.ctypes.data_as(P))
    dt = time.perf_counter() - t0
    rate = span / max(dt, 1e-9)
    span = int(min(total, max(1 << (20 if prec == 0 else 14), rate * seconds)))
    start = (total - span) // 2
    t0 = time.perf_counter()
    rc |= fn(a.ctypes.data_as(P), n, n, n, prec, threads, start, start + span, out.ctypes.data_as(P))
    dt = time.perf_counter() - t0
    if rc != 0:
        raise RuntimeError("orc_bbfg_range_prec failed")
    return span / dt, span, dt


def host_threads() -> int:
    return os.cpu_count() or 1


# committed ncu summaries holding the DRAM bytes of one launch of each
# product's plain kernel; the traffic is the fixed-point tables and the
# per-block partial sums, so it does not grow with the Gray steps
_TRAFFIC_PROFILES = {"fx": "plain_fx_kernel_n28.md", "fast": "plain_df_kernel_n36_launches.md",
                     "fp64": "plain_group_kernel_fp64_n28.md"}


def traffic_from_profile(n: int, mode: str):
    """DRAM bytes per launch of the plain kernel of `mode`, read from the
    committed ncu summary of that kernel (profiles/), or None."""
    name = _TRAFFIC_PROFILES.get(mode)
    if name is None:
        return None
    try:
        text = open(os.path.join(ROOT, "profiles", name)).read()
    except OSError:
        return None
    import re
    rd = re.search(r"dram__bytes_read\.sum \| ([0-9,]+) B", text)
    wr = re.search(r"dram__bytes_write\.sum \| ([0-9,]+) B", text)
    if not rd or not wr:
        return None
    return int(rd.group(1).replace(",", "")) + int(wr.group(1).replace(",", ""))


# --------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region.

    start() returns once the first sample has arrived; stop() waits for the
    first sample after the region.  The report covers the samples inside the
    region plus the last one before it and the first one after it, so a
    region shorter than the 100 ms sampling interval is still bracketed."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[tuple[float, str]] = []
        self.thread = None
        self.t0 = self.t1 = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()
        deadline = time.perf_counter() + 5.0
        while not self.lines and time.perf_counter() < deadline and self.proc.poll() is None:
            time.sleep(0.005)
        self.t0 = time.perf_counter()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.t1 = time.perf_counter()
        deadline = self.t1 + 1.0
        while (not self.lines or self.lines[-1][0] <= self.t1) and time.perf_counter() < deadline \
                and self.proc.poll() is None:
            time.sleep(0.005)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        lines = list(self.lines)
        before = [ln for ln in lines if ln[0] <= self.t0]
        inside = [ln for ln in lines if self.t0 < ln[0] <= self.t1]
        after = [ln for ln in lines if ln[0] > self.t1]
        window = before[-1:] + inside + after[:1]
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for _, ln in window:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm), "samples_inside": len(inside)}


# ------------------------------------------------------------ reference arm
def run_reference(args, rank, world):
    if rank != 0:
        return 0
    from piquassoboost_gb300.workloads import haar_block

    n = args.n
    A = haar_block(n, seed=args.seed)
    thr = host_threads()
    per_step = max(2.0, args.cpu_seconds / 3.0)
    for _ in range(args.warmup):
        cpu_sample_rate(A, min(1.0, per_step / 4), thr)
    rates, spans, times = [], [], []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r, span, dt = cpu_sample_rate(A, per_step, thr)
        rates.append(r)
        spans.append(span)
        times.append(dt)
    wall = time.perf_counter() - t0
    steps_per_s = sum(spans) / sum(times)
    perm_s = steps_per_s / 2.0 ** (n - 1)
    line = {
        "impl": "reference",
        "metric": METRIC, "value": perm_s, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * wall / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_desc(args), "n": n, "seed": args.seed},
        "cpu_baseline": {"value": perm_s, "unit": UNIT, "cores": thr, "kind": "port",
                         "sample": f"per step a contiguous sample of ~{int(statistics.mean(spans))} of the "
                                   f"2^{n - 1} Gray steps (reference BBFG double algorithm, C restatement, "
                                   f"{thr} threads, 4 x threads segments); perm/s = steps/s / 2^{n - 1}"},
        "e2e": {"value": perm_s, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------- our arm
def _imad_ops_plain(n: int) -> float:
    """Algorithmic 32x32->64 multiply-adds of one plain permanent on the
    integer-mantissa product: 12 per complex multiply, n - 1 multiplies per
    Gray step, 2^(n-1) steps."""
    return 12.0 * (n - 1) * 2.0 ** (n - 1)


def run_ours(args, rank, world, local):
    import torch

    from piquassoboost_gb300 import _native as nat
    from piquassoboost_gb300.workloads import haar_block

    if not torch.cuda.is_available():
        print(json.dumps({"error": "no CUDA device"}))
        return 1
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    lib = nat.load()
    n = args.n
    arith = nat.arith_of(args.mode)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    sptr = ctypes.c_void_p(stream.cuda_stream)
    # per-rank, per-step seeded inputs (weak scaling: every rank does its own permanents)
    nsteps = args.warmup + args.steps
    from piquassoboost_gb300.replicas import shard_seeds

    mats = [haar_block(n, seed=sd) for sd in shard_seeds(args.seed, rank, nsteps)]
    d_mats = [torch.from_numpy(m).to(dev) for m in mats]
    ws_bytes = int(lib.gbperm_perm_workspace_size(n, n))
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    d_out = torch.zeros(2, dtype=torch.float64, device=dev)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    # prepare + permanent kernel; the double-float kernel also queues its
    # integer-mantissa twin (it returns at once unless the range check or
    # the error estimate hands it the permanent); above 36 rows the fast
    # mode runs the integer-mantissa kernel alone
    launches_per_step = 3 if args.mode == "fast" and n <= nat.get_option("df.max_rows") else 2

    def step(i, a=arith):
        rc = lib.gbperm_perm_dev(ctypes.c_void_p(d_mats[i].data_ptr()), n, n, n, a,
                                 ctypes.c_void_p(d_out.data_ptr()), None, ctypes.c_void_p(ws.data_ptr()),
                                 ws_bytes, sptr)
        nat.check(rc)

    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize()
    peaks = {k: nat.probe_peak(k) for k in ("fp64", "fp32", "imad_wide")}

    clocks = ClockSampler(local)
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    results = []
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(args.steps):
        flush.zero_()
        ev[k][0].record(stream)
        step(args.warmup + k)
        ev[k][1].record(stream)
        results.append(d_out.clone())
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    kern_ms = [a.elapsed_time(b) for a, b in ev]
    got = [complex(r[0].item(), r[1].item()) for r in results]
    from piquassoboost_gb300.replicas import replica_throughput

    # replicas: every rank computed its own `steps` permanents
    value, t_max = replica_throughput(args.steps, wall, device=dev)

    # e2e through the public host-buffer entry point, pinned input, every step
    pinned = [torch.from_numpy(m).pin_memory() for m in mats[args.warmup:]]
    out = np.zeros(2)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for k in range(args.steps):
        rc = lib.gbperm_perm(ctypes.c_void_p(pinned[k].data_ptr()), n, n, n, arith,
                             out.ctypes.data_as(ctypes.c_void_p), None, None)
        nat.check(rc)
    torch.cuda.synchronize()
    e2e, _ = replica_throughput(args.steps, time.perf_counter() - t1, device=dev)

    # the same first `check_steps` timed matrices through the other products:
    # each one's own rate and roofline, and the headline results checked
    # against the FP64 kernel (relative to |perm| and to the product of the
    # row 2-norms); the double-float path runs as users get it, with its
    # on-device recomputation in FP64 when its error estimate is above 1e-10
    nchk = max(0, min(args.check_steps, args.steps))
    idx = [args.warmup + k for k in range(nchk)]
    flops = flops_plain(n)
    products = {}
    ref64 = {}
    for mode in ("fp64", "fx", "fast"):
        if mode == args.mode and mode != "fp64":
            continue
        st = nat.Stats()
        ms, vals, esc, ests = [], [], 0, []
        # the fast mode's size rule (df.max_rows) sends larger square
        # matrices straight to the integer-mantissa product
        by_rule = mode == "fast" and n > nat.get_option("df.max_rows")
        for i in idx:
            v = nat.perm(mats[i], mode=mode, stats=st)
            ms.append(st.kernel_ms)
            vals.append(v)
            if mode == "fast":
                ests.append(st.err_est)
                esc += int(not by_rule and st.arith != nat.ARITH_DF32)
        if mode == "fp64":
            ref64 = dict(zip(idx, vals))
            if args.mode == "fp64":
                continue
        if not ms:
            continue
        d = {"kernel_ms": ms, "perm_per_s": len(ms) / (sum(ms) * 1e-3),
             "fp64_equivalent_tflops": flops / (statistics.mean(ms) * 1e-3) / 1e12}
        if mode == "fp64":
            d.update({"dtype": "f64", "kernel": "plain_group_kernel" if n > 8 else "plain_kernel",
                      "frac_of_fp64_peak": d["fp64_equivalent_tflops"] / peaks["fp64"]})
        elif mode == "fx":
            d.update({"dtype": "int64 mantissas (>= f64 accuracy)", "kernel": "plain_fx_kernel"})
        elif by_rule:
            d.update({"dtype": "int64 mantissas", "kernel": "plain_fx_kernel",
                      "note": f"n > df.max_rows ({nat.get_option('df.max_rows')}): the fast mode runs the "
                              "integer-mantissa product alone"})
        else:
            d.update({"dtype": "f32 pairs (double-float product)", "kernel": "plain_df_kernel",
                      "escalated_steps": esc, "err_est": ests,
                      "note": "an escalated step reruns the permanent on the integer-mantissa kernel: "
                              "kernel_ms includes the double-float pass it discards"})
        products[mode] = d
        if mode != "fp64":
            products[mode]["rel_err_vs_fp64_kernel"] = [abs(v - ref64[i]) / abs(ref64[i]) for i, v in zip(idx, vals)]

    check = {}
    if ref64 and args.mode != "fp64":
        rel = [abs(got[k] - ref64[i]) / abs(ref64[i]) for k, i in enumerate(idx)]
        rown = [abs(got[k] - ref64[i]) / float(np.prod(np.linalg.norm(mats[i], axis=1))) for k, i in enumerate(idx)]
        check = {"timed_results_checked": nchk, "rel_err_vs_fp64_kernel": rel, "max_rel_err": max(rel),
                 "err_by_row_norm_product": rown}

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return 0

    avg_ms = statistics.mean(kern_ms)
    ach_flops = flops / (avg_ms * 1e-3) / 1e12
    if args.mode == "fx":
        ach = _imad_ops_plain(n) / (avg_ms * 1e-3) / 1e12
        roof = {"bound": "int", "achieved": ach, "peak": peaks["imad_wide"], "unit": "Tops/s",
                "frac": ach / peaks["imad_wide"], "traffic": traffic_from_profile(n, args.mode),
                "kernel": "plain_fx_kernel",
                "work_per_launch": f"12 (n-1) 2^(n-1) = {_imad_ops_plain(n):.4g} 32x32->64 multiply-adds "
                                   f"(12 per complex multiply of 31-bit limbs)",
                "peak_source": "mad.wide.s32 probe (gbperm_probe_peak kind 3), measured in this run",
                "fp64_equivalent_tflops": ach_flops, "fp64_peak_tflops": peaks["fp64"],
                "x_fp64_peak": ach_flops / peaks["fp64"]}
    else:
        roof = {"bound": "fp64", "achieved": ach_flops, "peak": peaks["fp64"], "unit": "TFLOP/s",
                "frac": ach_flops / peaks["fp64"], "traffic": traffic_from_profile(n, args.mode),
                "kernel": ("plain_df_kernel" if args.mode == "fast" else
                           ("plain_group_kernel" if n > 8 else "plain_kernel")),
                "work_per_launch": f"8 n 2^(n-1) = {flops:.4g} algorithmic FP64-equivalent flops",
                "peak_source": "DFMA probe (gbperm_probe_peak kind 0), measured in this run"}
        if args.mode == "fast":
            roof["note"] = ("double-float product on the FP32 pipe: frac is FP64-equivalent flops against "
                            f"the FP64 FMA peak; the FP32 FMA peak measured in this run is {peaks['fp32']:.1f} TFLOP/s")

    cpu = None
    if not args.no_cpu_baseline and world == 1:
        thr = host_threads()
        rate, span, dt = cpu_sample_rate(mats[args.warmup], args.cpu_seconds, thr)
        cpu = {"value": rate / 2.0 ** (n - 1), "unit": UNIT, "cores": thr, "kind": "port",
               "sample": f"{span} contiguous Gray steps of the same {n}x{n} permanent ({dt:.1f} s, "
                         f"{thr} threads, reference BBFG double algorithm as the C oracle); "
                         f"perm/s = steps/s / 2^{n - 1}"}
        # the reference's lib 8 ("long double", binary128 on this Arm host), a short sample
        try:
            rate8, span8, dt8 = cpu_sample_rate(mats[args.warmup], min(3.0, args.cpu_seconds / 4), thr, prec=1)
            cpu["lib8_long_double"] = {"value": rate8 / 2.0 ** (n - 1), "unit": UNIT,
                                       "sample": f"{span8} Gray steps in binary128 ({dt8:.1f} s, {thr} threads)"}
        except Exception as exc:  # the lib 7 baseline above stands on its own
            cpu["lib8_long_double"] = {"value": None, "error": str(exc)[:200]}

    dtype = {"fx": "int64", "fp64": "f64", "fast": "f32x2"}[args.mode]
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": dtype, "data": "synthetic",
        "config": {"workload": workload_desc(args), "n": n, "arith": args.mode, "seed": args.seed,
                   "l2": "flushed (256 MiB write) between steps", "parallelism": f"replicas x{world}"},
        "roofline": roof,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": n * n * 16, "d2h_bytes_per_step": 16},
        "clocks": clk,
        "gpu_launches": launches_per_step * args.steps,
        "kernel_ms": kern_ms,
        "accuracy": check,
        "products": products,
        "peaks": peaks,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


# ------------------------------------------------------- secondary workloads
# repeated, batched, grad and pmf: same contract as the plain workload (W
# untimed warm-up steps, K timed steps, e2e through the host-buffer entry
# point, a roofline object against the FP64 FMA peak measured live, clocks
# sampled during the timed region and, at N = 1, a CPU baseline from the C
# oracle on all host cores).

_P = ctypes.c_void_p


def _line(args, world, value, unit, ms_per_step, config, roofline, cpu, e2e, launches, extra=None, clocks=None,
          dtype="f64"):
    d = {"metric": METRIC, "value": value, "unit": unit, "n_gpus": world, "steps": args.steps,
         "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
         "vs_baseline": None, "dtype": dtype, "data": "synthetic", "config": config, "roofline": roofline,
         "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches}
    if clocks is not None:
        d["clocks"] = clocks
    if args.impl == "reference":
        d["impl"] = "reference"
    if extra:
        d.update(extra)
    print(json.dumps(d), flush=True)


def _roof(flops, ms, peak, kernel):
    ach = flops / (ms * 1e-3) / 1e12
    return {"bound": "fp64", "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": ach / peak,
            "traffic": None, "kernel": kernel, "peak_source": "gbperm_probe_peak (DFMA probe), this run"}


def _oracle():
    # the CPU baseline legs only
    from tests import oracle_bind as orc
    return orc


def run_secondary(args, rank, world, local):
    import torch

    if args.impl == "reference":
        if rank != 0:
            return 0
        return _reference_secondary(args, world)
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    fn = {"repeated": _repeated, "batched": _batched, "grad": _grad, "pmf": _pmf, "mesh": _mesh,
          "sampler": _sampler}[args.workload]
    rc = fn(args, rank, world, torch)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return rc


def _max_over_ranks(torch, world, t):
    if world == 1:
        return t
    import torch.distributed as dist
    tt = torch.tensor([t], device="cuda", dtype=torch.float64)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


# --------------------------------------------------------------- repeated
def _repeated(args, rank, world, torch):
    """One 60-mode / 30-photon repeated permanent per step through the
    host-buffer entry point (the public call); each timed instance is then
    run through the other products for their rates and the check against
    the FP64 kernel."""
    from piquassoboost_gb300 import _native as nat
    from piquassoboost_gb300.workloads import repeated_instance

    mode = args.mode
    cases = [repeated_instance(seed=1000 * rank + s, modes=60, photons=30, max_mult=4)
             for s in range(args.warmup + args.steps)]
    peaks = {k: nat.probe_peak(k) for k in ("fp64", "imad_wide")}
    st = nat.Stats()
    for U, i, o in cases[:args.warmup]:
        nat.perm_repeated(U, i, o, mode=mode)
    kms, flops, imad, got, launches = [], 0.0, 0.0, [], 0
    clk = ClockSampler(torch.cuda.current_device())
    clk.start()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for U, i, o in cases[args.warmup:]:
        got.append(nat.perm_repeated(U, i, o, mode=mode, stats=st))
        kms.append(st.kernel_ms)
        flops += st.flops
        # 12 32x32->64 multiply-adds per complex multiply, photons - 1
        # multiplies per Gray step
        imad += 12.0 * (int(np.sum(o)) - 1) * st.steps
        launches += st.launches
    wall = _max_over_ranks(torch, world, time.perf_counter() - t0)
    clocks = clk.stop()
    # the host-buffer call is the public API: e2e == the timed loop itself
    value = world * args.steps / (sum(kms) * 1e-3)
    e2e = world * args.steps / wall
    products, ref64 = {}, []
    for other in ("fp64", "fx", "fast"):
        if other == mode:
            continue
        ms, vals, esc = [], [], 0
        for U, i, o in cases[args.warmup:]:
            s2 = nat.Stats()
            vals.append(nat.perm_repeated(U, i, o, mode=other, stats=s2))
            ms.append(s2.kernel_ms)
            esc += int(other == "fast" and s2.arith != nat.ARITH_DF32)
        products[other] = {"kernel_ms": ms, "perm_per_s": len(ms) / (sum(ms) * 1e-3)}
        if other == "fast":
            products[other]["escalated_or_skipped"] = esc
        if other == "fp64":
            ref64 = vals
            products[other]["frac_of_fp64_peak"] = flops / (sum(ms) * 1e-3) / 1e12 / peaks["fp64"]
    rel = [abs(a - b) / abs(b) for a, b in zip(got, ref64)] if ref64 else []
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        orc = _oracle()
        U, i, o = cases[args.warmup]
        t = time.perf_counter()
        n = 0
        while time.perf_counter() - t < args.cpu_seconds and n < 20:
            orc.bbfg_repeated(U, i, o, prec=0)
            n += 1
        dt = time.perf_counter() - t
        cpu = {"value": n / dt, "unit": "perm/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"{n} full permanents of the first timed instance (reference repeated BBFG double "
                         f"algorithm as the C oracle, {os.cpu_count()} threads)"}
    avg = statistics.mean(kms)
    if mode == "fx":
        ach = imad / args.steps / (avg * 1e-3) / 1e12
        roof = {"bound": "int", "achieved": ach, "peak": peaks["imad_wide"], "unit": "Tops/s",
                "frac": ach / peaks["imad_wide"], "traffic": None, "kernel": "repeated_fx_kernel",
                "work_per_launch": "12 (photons - 1) multiply-adds per Gray step of the multiplicity form",
                "peak_source": "mad.wide.s32 probe (gbperm_probe_peak kind 3), measured in this run",
                "fp64_equivalent_tflops": flops / args.steps / (avg * 1e-3) / 1e12}
    else:
        roof = _roof(flops / args.steps, avg, peaks["fp64"],
                     "repeated_df_kernel" if mode == "fast" else "repeated_kernel")
    if rank == 0:
        _line(args, world, value, "perm/s", 1000 * wall / args.steps,
              {"workload": workload_desc(args), "arith": mode,
               "l2": "inputs < 100 KB; compute-bound, no flush"},
              roof, cpu, {"value": e2e, "unit": "perm/s", "h2d_bytes_per_step": 60 * 60 * 16 + 2 * 60 * 8,
                          "d2h_bytes_per_step": 48}, launches,
              {"kernel_ms": kms, "products": products, "rel_err_vs_fp64_kernel": rel,
               "max_rel_err": max(rel) if rel else None}, clocks=clocks,
              dtype={"fx": "int64", "fp64": "f64", "fast": "f32x2"}[mode])
    return 0


# ---------------------------------------------------------------- batched
def _batched_multiplicity(args, rank, world, torch):
    """The batched configuration through the multiplicity plan
    (gbperm_rep_batch_*): the instances' row and column draws as (input,
    output) state pairs of the 100-mode unitary, the form the reference's
    batched calculator takes, each walked as a repeated permanent in one
    persistent launch; against sequential plain-GPU launches of the same
    k x k submatrices in the same (integer-mantissa) arithmetic."""
    from piquassoboost_gb300 import _native as nat
    from piquassoboost_gb300.workloads import batched_index_sets, index_sets_to_states

    count, kmax, modes = args.batch_count, args.batch_kmax, 100
    U, rows, cols = batched_index_sets(count, seed=4 + 1000 * rank, modes=modes, kmin=8, kmax=kmax)
    pairs = index_sets_to_states(rows, cols, modes)
    mats = [np.ascontiguousarray(U[np.ix_(r, c)]) for r, c in zip(rows, cols)]
    ks = np.array([len(r) for r in rows])
    flops_plain = float(np.sum(8.0 * ks * 2.0 ** (ks - 1)))
    peaks = {k: nat.probe_peak(k) for k in ("fp64", "imad_wide")}
    lib = nat.load()
    t_plan = time.perf_counter()
    plan = nat.RepBatchPlan(U, pairs)
    t_plan = time.perf_counter() - t_plan
    info = plan.info()
    stream = torch.cuda.current_stream()
    d_out = torch.zeros(2 * count, dtype=torch.float64, device="cuda")
    for _ in range(args.warmup):
        plan.run_dev(d_out.data_ptr(), stream.cuda_stream)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clk = ClockSampler(torch.cuda.current_device())
    clk.start()
    t0 = time.perf_counter()
    for k in range(args.steps):
        ev[k][0].record(stream)
        plan.run_dev(d_out.data_ptr(), stream.cuda_stream)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    wall = _max_over_ranks(torch, world, time.perf_counter() - t0)
    clocks = clk.stop()
    kms = [a.elapsed_time(b) for a, b in ev]
    value = world * count * args.steps / wall
    got = d_out.cpu().numpy().reshape(-1, 2)
    got = got[:, 0] + 1j * got[:, 1]
    # e2e: the public host call a user makes for a list of state pairs
    # (planning, upload, the persistent launch and the copy back), every step
    t1 = time.perf_counter()
    for _ in range(args.steps):
        nat.perm_repeated_many(U, pairs, mode="fx")
    e2e = world * count * args.steps / _max_over_ranks(torch, world, time.perf_counter() - t1)
    # sequential plain-GPU launches of the k x k submatrices, same arithmetic
    dm = [torch.from_numpy(m).to("cuda") for m in mats]
    ws_b = int(lib.gbperm_perm_workspace_size(kmax, kmax))
    ws = torch.empty(ws_b, dtype=torch.uint8, device="cuda")
    sout = torch.zeros(2 * count, dtype=torch.float64, device="cuda")
    sp = _P(stream.cuda_stream)
    for i in range(min(8, count)):  # warm the plain path
        k = dm[i].shape[0]
        nat.check(lib.gbperm_perm_dev(_P(dm[i].data_ptr()), k, k, k, nat.ARITH_FX64, _P(sout.data_ptr() + 16 * i),
                                      None, _P(ws.data_ptr()), ws_b, sp))
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i, m in enumerate(dm):
        k = m.shape[0]
        nat.check(lib.gbperm_perm_dev(_P(m.data_ptr()), k, k, k, nat.ARITH_FX64, _P(sout.data_ptr() + 16 * i),
                                      None, _P(ws.data_ptr()), ws_b, sp))
    e1.record(stream)
    torch.cuda.synchronize()
    seq_ms = e0.elapsed_time(e1)
    b = sout.cpu().numpy().reshape(-1, 2)
    b = b[:, 0] + 1j * b[:, 1]
    diff = float(np.max(np.abs(got - b) / np.abs(b)))
    avg = statistics.mean(kms)
    # roofline: the integer multiply-adds of the walked steps (12 per
    # complex multiply, photons - 1 multiplies per step)
    ach = info["mul_ops"] / (avg * 1e-3) / 1e12
    roof = {"bound": "int", "achieved": ach, "peak": peaks["imad_wide"], "unit": "Tops/s",
            "frac": ach / peaks["imad_wide"], "traffic": None, "kernel": "rep_batched_kernel",
            "work_per_launch": f"{info['steps']:.4g} Gray steps of the instances' multiplicity forms "
                               f"(the expanded k x k sums: {float(np.sum(2.0 ** (ks - 1))):.4g} steps)",
            "peak_source": "mad.wide.s32 probe (gbperm_probe_peak kind 3), measured in this run",
            "fp64_equivalent_tflops_of_expanded_work": flops_plain / (avg * 1e-3) / 1e12}
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        orc = _oracle()
        order = np.argsort(-ks)[::64]
        t = time.perf_counter()
        done_flops, nd = 0.0, 0
        for i in order:
            if time.perf_counter() - t > args.cpu_seconds:
                break
            orc.bbfg_repeated(U, pairs[i][0], pairs[i][1], prec=0)
            done_flops += 8.0 * ks[i] * 2.0 ** (ks[i] - 1)
            nd += 1
        dt = time.perf_counter() - t
        cpu = {"value": count / (dt * flops_plain / done_flops), "unit": "perm/s", "cores": os.cpu_count(),
               "kind": "port",
               "sample": f"{nd} size-stratified instances as repeated permanents (the reference's batched "
                         f"calculator's form; C oracle, {os.cpu_count()} threads), scaled to the batch by their "
                         f"expanded flops"}
    if rank == 0:
        _line(args, world, value, "perm/s", 1000 * wall / args.steps,
              {"workload": workload_desc(args) + "; the draws as state pairs of the unitary (multiplicity form)",
               "arith": "fx", "plan_build_s": t_plan, "items": info["items"],
               "l2": "tables resident (< 50 MB); compute-bound"},
              roof, cpu, {"value": e2e, "unit": "perm/s", "h2d_bytes_per_step": 16 * modes * modes + 16 * modes * count,
                          "d2h_bytes_per_step": 16 * count},
              # prepare, persistent worker, finalize, slot-order scatter
              4 * args.steps,
              {"sequential_plain_gpu": {"ms": seq_ms, "perm_per_s": count / (seq_ms * 1e-3),
                                        "arith": "fx", "batched_speedup": seq_ms / avg,
                                        "max_rel_diff_vs_batched": diff},
               "steps_walked_over_expanded": info["steps"] / float(np.sum(2.0 ** (ks - 1))),
               "kernel_ms": kms}, clocks=clocks, dtype="int64")
    plan.close()
    return 0


def _batched(args, rank, world, torch):
    if args.mode == "fx":
        return _batched_multiplicity(args, rank, world, torch)
    from piquassoboost_gb300 import _native as nat
    from piquassoboost_gb300.workloads import batched_instances, haar_block, repeated_instance

    mode = args.mode
    count, kmax = args.batch_count, args.batch_kmax
    mats = batched_instances(count, seed=4 + 1000 * rank, modes=100, kmin=8, kmax=kmax)
    ks = np.array([m.shape[0] for m in mats])
    flops = float(np.sum(8.0 * ks * 2.0 ** (ks - 1)))
    peak = nat.probe_peak("fp64")
    lib = nat.load()
    plan = nat.BatchPlan([m.shape for m in mats], mode=mode)
    packed = plan.pack(mats)
    # autotune the plan's shape on this batch (outside the timed region)
    default_shape, default_item = plan.shape(), plan.item_log2()
    t_tune = time.perf_counter()
    tuned_ms = plan.autotune(packed=packed, reps=1)
    t_tune = time.perf_counter() - t_tune
    dpk = torch.from_numpy(packed).to("cuda")
    dout = torch.zeros(2 * count, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    sp = _P(stream.cuda_stream)

    def step_dev():
        nat.check(lib.gbperm_batch_plan_run_dev(plan._h, _P(dpk.data_ptr()), _P(dout.data_ptr()), sp))

    for _ in range(args.warmup):
        step_dev()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clk = ClockSampler(torch.cuda.current_device())
    clk.start()
    t0 = time.perf_counter()
    for k in range(args.steps):
        ev[k][0].record(stream)
        step_dev()
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    wall = _max_over_ranks(torch, world, time.perf_counter() - t0)
    clocks = clk.stop()
    kms = [a.elapsed_time(b) for a, b in ev]
    value = world * count * args.steps / wall
    # e2e: host buffers through the plan's captured graph (H2D, kernels, D2H)
    t1 = time.perf_counter()
    for _ in range(args.steps):
        plan.run(packed=packed)
    e2e = world * count * args.steps / _max_over_ranks(torch, world, time.perf_counter() - t1)
    # sequential plain-GPU launches on the same device-resident inputs
    dm = [torch.from_numpy(m).to("cuda") for m in mats]
    ws_b = int(lib.gbperm_perm_workspace_size(kmax, kmax))
    ws = torch.empty(ws_b, dtype=torch.uint8, device="cuda")
    sout = torch.zeros(2 * count, dtype=torch.float64, device="cuda")
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i, m in enumerate(dm):
        k = m.shape[0]
        nat.check(lib.gbperm_perm_dev(_P(m.data_ptr()), k, k, k, nat.arith_of(mode), _P(sout.data_ptr() + 16 * i),
                                      None, _P(ws.data_ptr()), ws_b, sp))
    e1.record(stream)
    torch.cuda.synchronize()
    seq_ms = e0.elapsed_time(e1)
    a = dout.cpu().numpy().reshape(-1, 2)
    b = sout.cpu().numpy().reshape(-1, 2)
    diff = float(np.max(np.abs((a[:, 0] + 1j * a[:, 1]) - (b[:, 0] + 1j * b[:, 1])) /
                        np.abs(b[:, 0] + 1j * b[:, 1])))
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        orc = _oracle()
        order = np.argsort(-ks)[::64]   # every 64th instance by size: a size-stratified sample
        t = time.perf_counter()
        done_flops = 0.0
        nd = 0
        for i in order:
            if time.perf_counter() - t > args.cpu_seconds:
                break
            orc.bbfg(mats[i], prec=0)
            done_flops += 8.0 * ks[i] * 2.0 ** (ks[i] - 1)
            nd += 1
        dt = time.perf_counter() - t
        cpu = {"value": count / (dt * flops / done_flops), "unit": "perm/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"{nd} size-stratified instances ({done_flops:.3g} of {flops:.3g} flops), reference BBFG "
                         f"double algorithm as the C oracle, scaled to the whole batch"}
    if rank == 0:
        _line(args, world, value, "perm/s", 1000 * wall / args.steps,
              {"workload": workload_desc(args), "arith": mode,
               "item_log2": plan.item_log2(), "lanes_per_segment": plan.shape()[0],
               "autotune": {"default_shape": list(default_shape), "default_item_log2": default_item,
                            "chosen_shape": list(plan.shape()), "chosen_item_log2": plan.item_log2(),
                            "best_ms": tuned_ms, "tuning_s": t_tune},
               "l2": f"inputs {packed.nbytes / 1e6:.3g} MB stay resident; compute-bound"},
              _roof(flops, statistics.mean(kms), peak, "batched_kernel"),
              cpu, {"value": e2e, "unit": "perm/s", "h2d_bytes_per_step": int(packed.nbytes),
                    "d2h_bytes_per_step": 16 * count},
              # per step: prepare, worker, finalize, the FP64 redo worker and its
              # finalize (double-float plans), the slot-order scatter
              (6 if mode == "fast" else 4) * args.steps,
              {"sequential_plain_gpu": {"ms": seq_ms, "perm_per_s": count / (seq_ms * 1e-3),
                                        "batched_speedup": seq_ms / statistics.mean(kms),
                                        "max_rel_diff_vs_batched": diff}}, clocks=clocks)
    plan.close()
    return 0


# ------------------------------------------------------------------- grad
def _grad(args, rank, world, torch):
    """Permanent + full gradient per step (n <= 32). mode "fast": the
    double-float sweep, recomputed on the device by the integer-mantissa
    sweep when its range check fails or its estimate is above 1e-10 (the
    library's default); "fx": the integer-mantissa sweep alone. The forward
    it is compared with is the same product's plain permanent, as users get
    it (escalation on)."""
    from piquassoboost_gb300 import _native as nat
    from piquassoboost_gb300.workloads import haar_block

    from piquassoboost_gb300.torch_perm import permanent_and_grad, permanent_fwd

    mode = args.mode
    n = args.n if args.n <= 32 else 32
    host = [haar_block(n, seed=args.seed + 1000 * rank + s) for s in range(args.warmup + args.steps)]
    mats = [torch.tensor(h, device="cuda") for h in host]
    peak = nat.probe_peak("fp64")
    stream = torch.cuda.current_stream()
    with nat.grad_arithmetic(mode):
        for k in range(args.warmup):
            permanent_and_grad(mats[k])
            permanent_fwd(mats[k], mode=mode)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        clk = ClockSampler(torch.cuda.current_device())
        clk.start()
        t0 = time.perf_counter()
        for k in range(args.steps):
            ev[k][0].record(stream)
            permanent_and_grad(mats[args.warmup + k])
            ev[k][1].record(stream)
        torch.cuda.synchronize()
        wall = _max_over_ranks(torch, world, time.perf_counter() - t0)
        clocks = clk.stop()
        gms = [a.elapsed_time(b) for a, b in ev]
        fev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        for k in range(args.steps):
            fev[k][0].record(stream)
            permanent_fwd(mats[args.warmup + k], mode=mode)
            fev[k][1].record(stream)
        torch.cuda.synchronize()
        fms = [a.elapsed_time(b) for a, b in fev]
        # e2e through the host-buffer entry point; its stats say which steps
        # the integer-mantissa sweep recomputed
        esc, ests = 0, []
        t1 = time.perf_counter()
        for k in range(args.steps):
            st = nat.Stats()
            nat.perm_grad(host[args.warmup + k], stats=st)
            ests.append(st.err_est)
            esc += int(mode == "fast" and st.arith == nat.ARITH_FX64)
        e2e = world * args.steps / _max_over_ranks(torch, world, time.perf_counter() - t1)
    flops = 8.0 * n * 2.0 ** (n - 1)
    roof = _roof(flops, statistics.mean(gms), peak, "grad_kernel" if mode == "fast" else "grad_fx_kernel")
    roof["note"] = ("achieved counts the forward sum's FP64-equivalent flops (8 n 2^(n-1)) per forward+gradient "
                    "step; the sweep computes in " + ("float pairs on the FP32 pipe" if mode == "fast" else
                                                      "integer mantissas on the integer pipe") +
                    ", so frac is not an FP64-pipe fraction")
    if rank == 0:
        _line(args, world, world * args.steps / wall, "(perm+grad)/s", 1000 * wall / args.steps,
              {"workload": workload_desc(args), "n": n, "arith": mode},
              roof, None, {"value": e2e, "unit": "(perm+grad)/s", "h2d_bytes_per_step": n * n * 16,
                           "d2h_bytes_per_step": n * n * 16 + 16},
              # double-float chain (prepare, sweep, partial, finalize, perm)
              # and its gated integer-mantissa twin chain; fx alone: 5
              (9 if mode == "fast" else 5) * args.steps,
              {"forward_only_ms": statistics.mean(fms), "grad_ms": statistics.mean(gms),
               "grad_over_forward": statistics.mean(gms) / statistics.mean(fms),
               "escalated_steps": esc, "err_est": ests}, clocks=clocks,
              dtype="f32x2" if mode == "fast" else "int64")
    return 0


# -------------------------------------------------------------------- pmf
def _pmf(args, rank, world, torch):
    """One probability layer of the Clifford & Clifford sampler per step
    (compute_pmf of samplingHelperFunctions.cpp:78-342): 60 modes, 30 input
    photons, a 29-photon sample."""
    from piquassoboost_gb300 import _native as nat
    from piquassoboost_gb300.workloads import pmf_layer_instance

    layers = [pmf_layer_instance(seed=args.seed + 1000 * rank + s, modes=60, photons=30)
              for s in range(args.warmup + args.steps)]
    peak = nat.probe_peak("fp64")
    st = nat.Stats()
    for U, smp, cin in layers[:args.warmup]:
        nat.compute_pmf(U, smp, cin, mode=args.mode)
    # the FP64 layer on the first timed instance, for the products' ratio
    ref = {}
    if args.mode != "fp64":
        U, smp, cin = layers[args.warmup]
        s64 = nat.Stats()
        a64, x64 = nat.compute_pmf(U, smp, cin, mode="fp64", stats=s64)
        ref = {"ms": s64.kernel_ms, "pmf": a64, "addends": x64}
    kms, flops, nperm = [], 0.0, 0
    clk = ClockSampler(torch.cuda.current_device())
    clk.start()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    first = None
    for U, smp, cin in layers[args.warmup:]:
        res = nat.compute_pmf(U, smp, cin, mode=args.mode, stats=st)
        if first is None:
            first = res
        kms.append(st.kernel_ms)
        flops += st.flops
        nperm += int(np.count_nonzero(cin))
    wall = _max_over_ranks(torch, world, time.perf_counter() - t0)
    clocks = clk.stop()
    # the host-buffer call is the public API: e2e is the timed loop itself
    value = world * args.steps / (sum(kms) * 1e-3)
    e2e = world * args.steps / wall
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        orc = _oracle()
        U, smp, cin = layers[args.warmup]
        t = time.perf_counter()
        nl = 0
        while nl < 1 or (time.perf_counter() - t < args.cpu_seconds and nl < 4):
            orc.compute_pmf(U, smp, cin, prec=0)
            nl += 1
        dt = time.perf_counter() - t
        cpu = {"value": nl / dt, "unit": "layers/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"{nl} full layer(s) of the first timed instance: one repeated BBFG double permanent "
                         f"per occupied input mode as in the reference, C oracle, {os.cpu_count()} threads"}
    if rank == 0:
        _line(args, world, value, "layers/s", 1000 * wall / args.steps,
              {"workload": workload_desc(args), "arith": args.mode, "l2": "inputs < 100 KB; compute-bound, no flush"},
              _roof(flops / args.steps, statistics.mean(kms), peak,
                    {"fast": "pmf_df_kernel (FP64-equivalent flops of the FP64 form)",
                     "fx": "pmf_fx_kernel (FP64-equivalent flops of the FP64 form; computes on the integer pipes)"}
                    .get(args.mode, "pmf_kernel (executed FP64 flops)")),
              cpu, {"value": e2e, "unit": "layers/s", "h2d_bytes_per_step": 60 * 60 * 16 + 2 * 60 * 8,
                    "d2h_bytes_per_step": 60 * 8 + 60 * 16}, st.launches * args.steps,
              {"permanents_per_s": value * nperm / args.steps, "kernel_ms": kms,
               "fp64_layer": ({"ms": ref["ms"], "speedup": ref["ms"] / kms[0],
                               "max_rel_diff_addends": float(np.max(np.abs(first[1] - ref["addends"])) /
                                                             np.max(np.abs(ref["addends"]))),
                               "max_abs_diff_pmf": float(np.max(np.abs(first[0] - ref["pmf"])))}
                              if ref else None)},
              clocks=clocks, dtype={"fx": "int64", "fp64": "f64", "fast": "f32x2"}[args.mode])
    return 0


# ------------------------------------------------------------------- mesh
def _mesh(args, rank, world, torch):
    """Differentiable permanents in a photonic circuit: 512 terms
    log|perm(U_S)|^2 of 12 photons in a 40-mode Clements mesh with seeded
    uniform phases, backpropagated to the 1560 phases.  A step is the whole
    forward and backward pass: mesh unitary, the 512 12 x 12 submatrices, their
    permanents and full gradients (one batched sweep), the loss and the phase
    gradient, written as ordinary torch autograd code and replayed as one
    CUDA graph (captured once; the eager step is timed beside it)."""
    from piquassoboost_gb300.torch_perm import clements_unitary, permanent
    from piquassoboost_gb300.workloads import mesh_instance, mesh_unitary

    m, k, terms = 40, 12, 512
    insts = [mesh_instance(seed=args.seed + 1000 * rank + s, modes=m, photons=k, terms=terms)
             for s in range(args.warmup + args.steps)]
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream()
    from piquassoboost_gb300.torch_perm import capture_graph

    # the step over static input buffers: phases and the two index sets
    s_ph = torch.zeros(m * (m - 1), dtype=torch.float64, device=dev)
    s_o = torch.zeros((terms, k), dtype=torch.long, device=dev)
    s_i = torch.zeros((terms, k), dtype=torch.long, device=dev)

    def step():
        ph = s_ph.detach().requires_grad_(True)
        U = clements_unitary(ph, m)
        p = permanent(U[s_o[:, :, None], s_i[:, None, :]])
        loss = torch.log((p * p.conj()).real).sum()
        (g,) = torch.autograd.grad(loss, ph)
        return loss.detach(), g

    def load(ph, o, i, non_blocking=False):
        s_ph.copy_(ph, non_blocking=non_blocking)
        s_o.copy_(o, non_blocking=non_blocking)
        s_i.copy_(i, non_blocking=non_blocking)

    dev_in = [(torch.tensor(ph, device=dev), torch.tensor(outs, device=dev), torch.tensor(ins, device=dev))
              for ph, ins, outs in insts]
    load(*dev_in[0])
    for q in range(args.warmup):
        load(*dev_in[q])
        step()
    torch.cuda.synchronize()
    # eager (one launch per op, host-side autograd between launches)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for q in range(args.steps):
        ev[q][0].record(stream)
        load(*dev_in[args.warmup + q])
        step()
        ev[q][1].record(stream)
    torch.cuda.synchronize()
    eager_ms = [a.elapsed_time(b) for a, b in ev]
    # the same step captured once as a CUDA graph; its replay must reproduce
    # the eager result of the same inputs
    graph, (g_loss, g_grad) = capture_graph(step, warmup=3)
    load(*dev_in[args.warmup])
    e_loss, e_grad = step()
    graph.replay()
    torch.cuda.synchronize()
    if abs(e_loss.item() - g_loss.item()) > 1e-12 * abs(e_loss.item()) or \
            (e_grad - g_grad).abs().max().item() > 1e-12 * max(1.0, e_grad.abs().max().item()):
        raise RuntimeError("mesh step: CUDA-graph replay differs from the eager step")
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clk = ClockSampler(torch.cuda.current_device())
    clk.start()
    t0 = time.perf_counter()
    for q in range(args.steps):
        ev[q][0].record(stream)
        load(*dev_in[args.warmup + q])
        graph.replay()
        ev[q][1].record(stream)
    torch.cuda.synchronize()
    wall = _max_over_ranks(torch, world, time.perf_counter() - t0)
    clocks = clk.stop()
    ms = [a.elapsed_time(b) for a, b in ev]
    value = world * args.steps / (sum(ms) * 1e-3)
    # e2e: phases and index sets from pinned host memory, loss and phase
    # gradient back to the host, every step
    pinned = [(torch.tensor(ph).pin_memory(), torch.tensor(outs).pin_memory(), torch.tensor(ins).pin_memory())
              for ph, ins, outs in insts[args.warmup:]]
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for q in range(args.steps):
        load(*pinned[q], non_blocking=True)
        graph.replay()
        g_loss.item()
        g_grad.cpu()
    e2e = world * args.steps / _max_over_ranks(torch, world, time.perf_counter() - t1)
    h2d = (m * (m - 1) + 2 * terms * k) * 8
    # the permanent kernels alone on the same 512 submatrices
    from piquassoboost_gb300.torch_perm import permanents_and_grads
    ph, o, i = dev_in[args.warmup]
    with torch.no_grad():
        U = clements_unitary(ph, m)
        subs = U[o[:, :, None], i[:, None, :]]
    permanents_and_grads(subs)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    permanents_and_grads(subs)
    e1.record(stream)
    torch.cuda.synchronize()
    perm_ms = e0.elapsed_time(e1)
    flops = terms * 8.0 * k * 2.0 ** (k - 1)
    from piquassoboost_gb300 import _native as nat
    peak = nat.probe_peak("fp64")
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from concurrent.futures import ThreadPoolExecutor

        orc = _oracle()
        Uc = mesh_unitary(insts[args.warmup][0], m)
        _, ins, outs = insts[args.warmup]

        def one_term(q):
            A = Uc[np.ix_(outs[q], ins[q])]
            orc.bbfg(A, prec=0, threads=1)
            for r in range(k):
                for c in range(k):
                    orc.bbfg(np.delete(np.delete(A, r, 0), c, 1), prec=0, threads=1)

        sample = 32
        t = time.perf_counter()
        with ThreadPoolExecutor(max_workers=os.cpu_count()) as ex:
            list(ex.map(one_term, range(sample)))
        dt = time.perf_counter() - t
        cpu = {"value": 1.0 / (dt * terms / sample), "unit": "(loss+grad)/s", "cores": os.cpu_count(),
               "kind": "port",
               "sample": f"{sample} of the {terms} terms: each term's 12x12 permanent and its 144 11x11 minors "
                         f"(the gradient through the reference's BBFG double algorithm, C oracle, one thread per "
                         f"term on {os.cpu_count()} threads), scaled to the whole batch; the mesh itself not counted"}
    if rank == 0:
        _line(args, world, value, "(loss+grad)/s", 1000 * wall / args.steps,
              {"workload": workload_desc(args), "arith": "fast",
               "launch": "forward + backward captured once as a CUDA graph, one replay per step (checked equal "
                         "to the eager step); eager timing in eager_step_ms",
               "l2": "inputs < 1 MB; launch- and compute-bound, no flush"},
              _roof(flops, perm_ms, peak, "grad_kernel (batched; forward flops only)"),
              cpu, {"value": e2e, "unit": "(loss+grad)/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": 1560 * 8 + 8}, 9 * args.steps,
              {"step_ms": ms, "eager_step_ms": eager_ms, "eager_steps_per_s": world * args.steps / (sum(eager_ms) * 1e-3),
               "permanent_kernels_ms": perm_ms}, clocks=clocks)
    return 0


# ---------------------------------------------------------------- sampler
_SAMPLER_MODES, _SAMPLER_PHOTONS = 40, 20


def _sampler_instance(seed):
    from piquassoboost_gb300.workloads import haar_unitary
    U = haar_unitary(_SAMPLER_MODES, seed)
    inp = np.zeros(_SAMPLER_MODES, dtype=np.int64)
    inp[:_SAMPLER_PHOTONS] = 1
    return U, inp


def _sampler(args, rank, world, torch):
    """Seeded boson samples through the native sampler (gbperm_sampler_*):
    one sample (20 probability layers, each one GPU Gray sweep) per step."""
    from piquassoboost_gb300 import _native as nat

    U, inp = _sampler_instance(args.seed + 1000 * rank)
    peak = nat.probe_peak("fp64")
    smp = nat.Sampler(U, seed=args.seed + rank, mode=args.mode)
    first = smp.simulate(inp, 1)                 # the oracle's first sample is checked below
    for _ in range(max(0, args.warmup - 1)):
        smp.simulate(inp, 1)
    st = nat.Stats()
    clk = ClockSampler(torch.cuda.current_device())
    clk.start()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    smp.simulate(inp, args.steps, stats=st)
    wall = _max_over_ranks(torch, world, time.perf_counter() - t0)
    clocks = clk.stop()
    value = world * args.steps / wall
    cpu, match = None, None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        orc = _oracle()
        t = time.perf_counter()
        ref = orc.sample_b(U, inp, 1, args.seed + rank, threads=0)
        dt = time.perf_counter() - t
        match = bool(np.array_equal(ref[0], first[0]))
        cpu = {"value": 1.0 / dt, "unit": "samples/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"one seeded sample (the oracle's C restatement of the reference sampler, pmf layers on "
                         f"{os.cpu_count()} threads)"}
    if rank == 0:
        _line(args, world, value, "samples/s", 1000 * wall / args.steps,
              {"workload": workload_desc(args), "arith": args.mode,
               "l2": "inputs < 30 KB; compute- and launch-bound"},
              _roof(st.flops, st.kernel_ms, peak, {"fx": "pmf_fx_kernel", "fast": "pmf_df_kernel"}.get(
                  args.mode, "pmf_kernel") + " (all layers of the timed samples; FP64-equivalent flops)"),
              cpu, {"value": value, "unit": "samples/s",
                    "h2d_bytes_per_step": _SAMPLER_PHOTONS * (_SAMPLER_MODES * _SAMPLER_MODES * 16 + 32 * _SAMPLER_MODES),
                    "d2h_bytes_per_step": _SAMPLER_PHOTONS * _SAMPLER_MODES * 24},
              st.launches, {"gpu_kernel_ms": st.kernel_ms, "first_sample_matches_oracle": match}, clocks=clocks,
              dtype={"fx": "int64", "fp64": "f64", "fast": "f32x2"}[args.mode])
    smp.close()
    return 0


def _reference_secondary(args, world):
    from piquassoboost_gb300.workloads import batched_instances, haar_block, repeated_instance

    orc = _oracle()
    if args.workload == "repeated":
        U, i, o = repeated_instance(seed=0, modes=60, photons=30, max_mult=4)
        ts = []
        for _ in range(args.warmup):
            orc.bbfg_repeated(U, i, o, prec=0)
        for _ in range(args.steps):
            t = time.perf_counter()
            orc.bbfg_repeated(U, i, o, prec=0)
            ts.append(time.perf_counter() - t)
        v = args.steps / sum(ts)
        unit, sample = "perm/s", "full permanents of one 60-mode / 30-photon instance"
    elif args.workload == "batched":
        count = args.batch_count
        mats = batched_instances(count, seed=4, modes=100, kmin=8, kmax=args.batch_kmax)
        ks = np.array([m.shape[0] for m in mats])
        flops = float(np.sum(8.0 * ks * 2.0 ** (ks - 1)))
        order = np.argsort(-ks)[::max(1, count // 16)]
        ts, fl = [], []
        for _ in range(args.steps):
            t = time.perf_counter()
            f = 0.0
            for i in order:
                orc.bbfg(mats[i], prec=0)
                f += 8.0 * ks[i] * 2.0 ** (ks[i] - 1)
            ts.append(time.perf_counter() - t)
            fl.append(f)
        v = count / (sum(ts) / len(ts) * flops / fl[0])
        unit, sample = "perm/s", (f"{len(order)} size-stratified instances per step, scaled to the "
                                  f"{count}-instance batch")
    elif args.workload == "mesh":
        from concurrent.futures import ThreadPoolExecutor

        from piquassoboost_gb300.workloads import mesh_instance, mesh_unitary

        ph, ins, outs = mesh_instance(seed=args.seed, modes=40, photons=12, terms=512)
        Uc = mesh_unitary(ph, 40)

        def one_term(q):
            A = Uc[np.ix_(outs[q], ins[q])]
            orc.bbfg(A, prec=0, threads=1)
            for r in range(12):
                for c in range(12):
                    orc.bbfg(np.delete(np.delete(A, r, 0), c, 1), prec=0, threads=1)

        sample = 32
        ts = []
        with ThreadPoolExecutor(max_workers=os.cpu_count()) as ex:
            for _ in range(args.steps):
                t = time.perf_counter()
                list(ex.map(one_term, range(sample)))
                ts.append((time.perf_counter() - t) * 512 / sample)
        v = args.steps / sum(ts)
        unit, sample = "(loss+grad)/s", ("32 of the 512 terms per step (permanent + 144 minors each, one thread per "
                                         "term), scaled to the batch")
    elif args.workload == "sampler":
        U, inp = _sampler_instance(args.seed)
        ts = []
        for q in range(args.steps):
            t = time.perf_counter()
            orc.sample_b(U, inp, 1, args.seed + q, threads=0)
            ts.append(time.perf_counter() - t)
        v = args.steps / sum(ts)
        unit, sample = "samples/s", "one seeded sample per step (C restatement of the reference sampler)"
    elif args.workload == "pmf":
        from piquassoboost_gb300.workloads import pmf_layer_instance

        U, smp, cin = pmf_layer_instance(seed=args.seed, modes=60, photons=30)
        for _ in range(min(args.warmup, 1)):
            orc.compute_pmf(U, smp, cin, prec=0)
        ts = []
        for _ in range(args.steps):
            t = time.perf_counter()
            orc.compute_pmf(U, smp, cin, prec=0)
            ts.append(time.perf_counter() - t)
        v = args.steps / sum(ts)
        unit, sample = "layers/s", "full 60-mode / 30-photon pmf layers (one permanent per occupied input mode)"
    else:
        A = haar_block(min(args.n, 32), seed=args.seed)
        n = A.shape[0]
        ts = []
        for _ in range(args.steps):
            t = time.perf_counter()
            orc.bbfg(A[:24, :24], prec=0)   # the oracle has no gradient; time a 24x24 forward
            ts.append(time.perf_counter() - t)
        v = args.steps / sum(ts) / 2.0 ** (n - 24) / n
        unit, sample = "(perm+grad)/s", "forward-only 24x24 oracle time scaled by 2^(n-24) and n minors"
    _line(args, world, v, unit, 1000.0 / v if v else None, {"workload": workload_desc(args)}, None,
          {"value": v, "unit": unit, "cores": os.cpu_count(), "kind": "port", "sample": sample},
          {"value": v, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}, 0)
    return 0


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.workload != "plain":
        return run_secondary(args, rank, world, local)
    if args.impl == "reference":
        return run_reference(args, rank, world)
    return run_ours(args, rank, world, local)


if __name__ == "__main__":
    sys.exit(main())
