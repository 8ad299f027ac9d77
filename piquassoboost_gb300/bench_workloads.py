"""Secondary bench.py workloads (repeated, batched, grad), one JSON line each.

Same contract as the default plain workload: W untimed warm-up steps, K timed
steps with CUDA events on the launching stream, `e2e` through the host-buffer
entry point, a roofline object against the FP64 FMA peak measured live, and
(N = 1) a CPU baseline from the C oracle on all host cores.
"""
from __future__ import annotations

import ctypes
import json
import os
import statistics
import time

import numpy as np

from . import _native as nat
from .workloads import batched_instances, haar_block, repeated_instance

METRIC = "complex perm/s at n=30/36/40 & batched k=8-28 vs plain GPU, rel err <=1e-10"
_P = ctypes.c_void_p


def _line(args, world, value, unit, ms_per_step, config, roofline, cpu, e2e, launches, extra=None):
    d = {"metric": METRIC, "value": value, "unit": unit, "n_gpus": world, "steps": args.steps,
         "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
         "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config, "roofline": roofline,
         "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches}
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
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    if root not in sys.path:
        sys.path.insert(0, root)
    from tests import oracle_bind as orc
    return orc


def run(args, rank, world, local):
    import torch

    if args.impl == "reference":
        if rank != 0:
            return 0
        return _reference(args, world)
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    fn = {"repeated": _repeated, "batched": _batched, "grad": _grad}[args.workload]
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
    mode = args.mode
    cases = [repeated_instance(seed=1000 * rank + s, modes=60, photons=30, max_mult=4)
             for s in range(args.warmup + args.steps)]
    peak = nat.probe_peak("fp64")
    st = nat.Stats()
    for U, i, o in cases[:args.warmup]:
        nat.perm_repeated(U, i, o, mode=mode)
    kms, flops = [], 0.0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for U, i, o in cases[args.warmup:]:
        nat.perm_repeated(U, i, o, mode=mode, stats=st)
        kms.append(st.kernel_ms)
        flops += st.flops
    wall = _max_over_ranks(torch, world, time.perf_counter() - t0)
    # the host-buffer call is the public API: e2e == the timed loop itself
    value = world * args.steps / (sum(kms) * 1e-3)
    e2e = world * args.steps / wall
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
    if rank == 0:
        _line(args, world, value, "perm/s", 1000 * wall / args.steps,
              {"workload": "repeated permanent: 60-mode Haar, one photon in modes 0-29, output occupation "
                           "from a seeded multinomial (multiplicities <= 4)", "arith": mode,
               "l2": "inputs < 100 KB; compute-bound, no flush"},
              _roof(flops / args.steps, statistics.mean(kms), peak,
                    "repeated_df_kernel" if mode == "fast" else "repeated_kernel"),
              cpu, {"value": e2e, "unit": "perm/s", "h2d_bytes_per_step": 60 * 60 * 16 + 2 * 60 * 8,
                    "d2h_bytes_per_step": 48}, (3 if mode == "fast" else 2) * args.steps)
    return 0


# ---------------------------------------------------------------- batched
def _batched(args, rank, world, torch):
    mode = args.mode
    count = 4096
    mats = batched_instances(count, seed=4 + 1000 * rank, modes=100, kmin=8, kmax=28)
    ks = np.array([m.shape[0] for m in mats])
    flops = float(np.sum(8.0 * ks * 2.0 ** (ks - 1)))
    peak = nat.probe_peak("fp64")
    lib = nat.load()
    plan = nat.BatchPlan([m.shape for m in mats], mode=mode)
    packed = plan.pack(mats)
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
    t0 = time.perf_counter()
    for k in range(args.steps):
        ev[k][0].record(stream)
        step_dev()
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    wall = _max_over_ranks(torch, world, time.perf_counter() - t0)
    kms = [a.elapsed_time(b) for a, b in ev]
    value = world * count * args.steps / wall
    # e2e: host buffers through the plan's captured graph (H2D, kernels, D2H)
    t1 = time.perf_counter()
    for _ in range(args.steps):
        plan.run(packed=packed)
    e2e = world * count * args.steps / _max_over_ranks(torch, world, time.perf_counter() - t1)
    # sequential plain-GPU launches on the same device-resident inputs
    dm = [torch.from_numpy(m).to("cuda") for m in mats]
    ws_b = int(lib.gbperm_perm_workspace_size(28, 28))
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
              {"workload": "4096 uneven k x k permanents, k uniform 8..28, rows/cols drawn with repetition "
                           "from a seeded 100-mode Haar unitary; one persistent launch per step", "arith": mode,
               "item_log2": plan.item_log2(), "l2": "inputs 26 MB stay resident; compute-bound"},
              _roof(flops, statistics.mean(kms), peak, "batched_kernel"),
              cpu, {"value": e2e, "unit": "perm/s", "h2d_bytes_per_step": int(packed.nbytes),
                    "d2h_bytes_per_step": 16 * count},
              3 * args.steps,
              {"sequential_plain_gpu": {"ms": seq_ms, "perm_per_s": count / (seq_ms * 1e-3),
                                        "batched_speedup": seq_ms / statistics.mean(kms),
                                        "max_rel_diff_vs_batched": diff}})
    plan.close()
    return 0


# ------------------------------------------------------------------- grad
def _grad(args, rank, world, torch):
    from .torch_perm import permanent_and_grad, permanent_fwd

    n = args.n if args.n <= 32 else 32
    mats = [torch.tensor(haar_block(n, seed=args.seed + 1000 * rank + s), device="cuda")
            for s in range(args.warmup + args.steps)]
    peak = nat.probe_peak("fp64")
    for k in range(args.warmup):
        permanent_and_grad(mats[k])
        permanent_fwd(mats[k], mode="fast")
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    t0 = time.perf_counter()
    for k in range(args.steps):
        ev[k][0].record(stream)
        permanent_and_grad(mats[args.warmup + k])
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    wall = _max_over_ranks(torch, world, time.perf_counter() - t0)
    gms = [a.elapsed_time(b) for a, b in ev]
    fev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for k in range(args.steps):
        fev[k][0].record(stream)
        permanent_fwd(mats[args.warmup + k], mode="fast")
        fev[k][1].record(stream)
    torch.cuda.synchronize()
    fms = [a.elapsed_time(b) for a, b in fev]
    flops = 8.0 * n * 2.0 ** (n - 1)
    t1 = time.perf_counter()
    for k in range(args.steps):
        nat.perm_grad(mats[args.warmup + k].cpu().numpy())
    e2e = world * args.steps / _max_over_ranks(torch, world, time.perf_counter() - t1)
    if rank == 0:
        _line(args, world, world * args.steps / wall, "(perm+grad)/s", 1000 * wall / args.steps,
              {"workload": f"permanent and full {n}x{n} complex gradient of the top-left block of a seeded "
                           f"Haar {2 * n}x{2 * n} unitary, one sweep", "n": n, "arith": "fast"},
              _roof(flops, statistics.mean(gms), peak, "grad_kernel (forward flops only)"),
              None, {"value": e2e, "unit": "(perm+grad)/s", "h2d_bytes_per_step": n * n * 16,
                     "d2h_bytes_per_step": n * n * 16 + 16}, 4 * args.steps,
              {"forward_only_ms": statistics.mean(fms), "grad_ms": statistics.mean(gms),
               "grad_over_forward": statistics.mean(gms) / statistics.mean(fms)})
    return 0


def _reference(args, world):
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
        mats = batched_instances(4096, seed=4, modes=100, kmin=8, kmax=28)
        ks = np.array([m.shape[0] for m in mats])
        flops = float(np.sum(8.0 * ks * 2.0 ** (ks - 1)))
        order = np.argsort(-ks)[::256]
        ts, fl = [], []
        for _ in range(args.steps):
            t = time.perf_counter()
            f = 0.0
            for i in order:
                orc.bbfg(mats[i], prec=0)
                f += 8.0 * ks[i] * 2.0 ** (ks[i] - 1)
            ts.append(time.perf_counter() - t)
            fl.append(f)
        v = 4096 / (sum(ts) / len(ts) * flops / fl[0])
        unit, sample = "perm/s", "16 size-stratified instances per step, scaled to the 4096-instance batch"
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
    _line(args, world, v, unit, 1000.0 / v if v else None, {"workload": args.workload}, None,
          {"value": v, "unit": unit, "cores": os.cpu_count(), "kind": "port", "sample": sample},
          {"value": v, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}, 0)
    return 0
