"""Benchmark of the GMM EM iteration on GB300 (frames x components per second).

Workload (default): UBM EM at scale -- N = 10,000,000 frames, D = 39, fitted with M = 2048
diagonal components (features drawn from a seeded 512-component generator GMM; random-frame
initialisation). One step = one full EM iteration over all N frames: E-step (log-likelihood,
log-sum-exp posteriors, n/F/S statistics reduced in FP64) and the M-step update, with the
features resident in HBM. The features (1.56 GB) are larger than L2 (129 MB).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--precision tc|fp32]
    python bench.py --impl reference ...   # the reference CPU path on the host cores

Under torchrun each rank runs an independent replica on its own GPU (the E-step shards by
frames only through a sum of statistics; one GPU per process, no collective on the data path);
`value` is the sum over ranks of the frames x components processed divided by the slowest
rank's time. Rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "frames·components/s per EM iter"
UNIT = "frame·comp/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default=os.environ.get("GMM_BENCH_PRECISION", "tc"),
                    choices=["tc", "fp32"])
    ap.add_argument("--frames", type=int, default=10_000_000)
    ap.add_argument("--mix", type=int, default=2048)
    ap.add_argument("--dim", type=int, default=39)
    ap.add_argument("--gen-mix", type=int, default=512)
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_{os.getpid()}.csv")

    def __enter__(self):
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines()]
        except Exception:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except ValueError:
                continue
            for k, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(k)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d["hbm_gbs"], d["bf16_tflops"], d.get("bf16_tflops_sustained"), "measured"
    return 6800.0, 1900.0, 1700.0, "fallback"


def cpu_reference(args, X, w, mu, var, seconds, threads):
    """The reference CPU algorithm (the oracle port of the reference estimator, all host
    threads) on a bounded sample of the workload. Returns (fc/s, sample description)."""
    import oracle
    oracle.build(ref=False)
    n0 = min(len(X), 20000)
    t = time.perf_counter()
    st = oracle.accumulate32(X[:n0], w, mu, var, threads=threads)
    oracle.em_update(w, mu, var, st)
    dt = time.perf_counter() - t
    n = int(min(len(X), max(n0, n0 * seconds / max(dt, 1e-3))))
    t = time.perf_counter()
    st = oracle.accumulate32(X[:n], w, mu, var, threads=threads)
    oracle.em_update(w, mu, var, st)
    dt = time.perf_counter() - t
    return n * len(w) / dt, n, dt


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from gmm_gb300 import synth
    threads = os.cpu_count() or 1
    X, w, mu, var = synth.config_em(args.seed, min(args.frames, 400_000), args.dim,
                                    args.gen_mix, args.mix)
    per_step = max(1.0, 60.0 / max(1, args.steps + args.warmup))
    rates = []
    for i in range(args.warmup + args.steps):
        r, n, dt = cpu_reference(args, X, w, mu, var, per_step, threads)
        if i >= args.warmup:
            rates.append((r, n, dt))
    value = statistics.median([r for r, _, _ in rates])
    n = rates[-1][1]
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * args.frames * args.mix / value, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"UBM EM, N={args.frames} frames, M={args.mix}, D={args.dim}",
                   "frames": args.frames, "components": args.mix, "dim": args.dim,
                   "timed_sample_frames": n},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{n} frames x {args.mix} components per step (E-step + EM "
                                   "update), reference CPU algorithm (oracle port), all host threads"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    rank, world, local = dist_env()
    import torch
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    from gmm_gb300 import _lib, synth
    _lib.load()

    N, M, D = args.frames, args.mix, args.dim
    X, w, mu, var = synth.config_em(args.seed + rank, N, D, args.gen_mix, M)
    dev = _lib.Handle(local if world > 1 else 0)
    prec = _lib.PREC_TC if args.precision == "tc" else _lib.PREC_FP32
    dev.set_precision(prec)
    Xpin = torch.from_numpy(X).pin_memory()
    dX = Xpin.to(f"cuda:{local if world > 1 else 0}", non_blocking=False)
    dev.upload_model(w, mu, var)
    dev.upload_features_device(dX.data_ptr(), N, D)
    stream = torch.cuda.ExternalStream(dev.stream())

    def step():
        dev.accumulate_device(_lib.ACC_MEAN | _lib.ACC_VAR)
        dev.em_update(True, True, True)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        step()
    # kernel timing (CUDA events on the engine's stream) over the timed region
    dev.profile(True)
    dev.profile_reset()
    launches0 = dev.launch_count()
    barrier()
    with ClockSampler(local if world > 1 else 0) as clk:
        with torch.cuda.stream(stream):
            t0 = torch.cuda.Event(enable_timing=True)
            t1 = torch.cuda.Event(enable_timing=True)
            t0.record(stream)
            for _ in range(args.steps):
                step()
            t1.record(stream)
        barrier()
    ms = t0.elapsed_time(t1) / args.steps
    launches = dev.launch_count() - launches0
    prof = dev.profile_read()
    dev.profile(False)
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = world * N * M / (ms / 1e3)

    # end-to-end through the public API: host (pinned) features -> device, EM iteration,
    # updated model back to the host, every step
    e2e = None
    if not args.no_e2e:
        Xhost = Xpin.numpy()
        wb, mub, varb = np.empty(M, np.float32), np.empty((M, D), np.float32), np.empty((M, D), np.float32)

        def e2e_step():
            dev.upload_features(Xhost)
            dev.accumulate_device(_lib.ACC_MEAN | _lib.ACC_VAR)
            dev.em_update(True, True, True)
            dev.lib.gmm_read_model(dev.h, wb.ctypes.data, mub.ctypes.data, varb.ctypes.data)

        dev.upload_model(w, mu, var)
        for _ in range(2):
            e2e_step()
        barrier()
        te = time.perf_counter()
        ke = max(2, args.steps // 2)
        for _ in range(ke):
            e2e_step()
        barrier()
        e2e_ms = (time.perf_counter() - te) * 1e3 / ke
        if world > 1:
            t = torch.tensor([e2e_ms], device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            e2e_ms = float(t.item())
        e2e = {"value": world * N * M / (e2e_ms / 1e3), "unit": UNIT,
               "h2d_bytes_per_step": int(X.nbytes), "d2h_bytes_per_step": int(wb.nbytes + mub.nbytes + varb.nbytes),
               "ms_per_step": e2e_ms}

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    hbm, bf16, bf16s, peak_kind = measured_peaks()
    # dominant kernel: largest share of device time in the timed region
    top = max(prof.items(), key=lambda kv: kv[1][0]) if prof else ("none", (0.0, 1))
    name, (kms, kcnt) = top
    fc_per_launch = N * M / max(1, kcnt // args.steps) if kcnt else 0
    if name.startswith("tc_"):
        flop_fc = 2 * (2 * D + 1) * (2 if "acc" in name else 1)
    else:
        flop_fc = 2 * (2 * D + 1) if "ll" in name else 2 * (2 * D + 1)
    per_launch_ms = kms / max(1, kcnt)
    achieved = flop_fc * fc_per_launch / (per_launch_ms / 1e3) / 1e12 if kcnt else 0.0
    peak = bf16s if bf16s else bf16
    roofline = {"bound": "tensor", "kernel": name, "achieved": achieved, "peak": peak,
                "unit": "TFLOP/s", "frac": achieved / peak, "traffic": None,
                "algorithmic_flop_per_fc": flop_fc, "peak_source": f"{peak_kind} (bf16 sustained)",
                "kernel_ms_per_launch": per_launch_ms,
                "kernel_share": kms / max(1e-9, sum(v[0] for v in prof.values()))}

    cpu = None
    if world == 1 or rank == 0:
        threads = os.cpu_count() or 1
        r, n, dt = cpu_reference(args, X[:400_000], w, mu, var, args.cpu_seconds, threads)
        cpu = {"value": r, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{n} frames x {M} components (E-step + EM update) of the same workload, "
                         f"{dt:.1f} s, reference CPU algorithm (oracle port)"}

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if prec == _lib.PREC_FP32 else "bf16x3 split (tcgen05), f32 accumulate, f64 reduce",
        "data": "synthetic",
        "config": {"workload": f"UBM EM iteration, N={N} frames, M={M}, D={D} (seeded {args.gen_mix}-component generator)",
                   "frames": N, "components": M, "dim": D, "precision": args.precision,
                   "l2": "inputs larger than L2 (features 1.56 GB)", "parallelism": f"replicas x{world}"},
        "clocks": clk.summary(), "e2e": e2e, "gpu_launches": launches, "roofline": roofline,
        "cpu_baseline": cpu, "kernels": {k: {"ms": v[0], "launches": v[1]} for k, v in prof.items()},
    }
    print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
