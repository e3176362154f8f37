"""Benchmark of the all-pairs kNN-RMSD hot path (knn_rms) on GB300.

Workload (one step): all-pairs kNN-RMSD of a synthetic trajectory of
N=20,000 frames x A=1,000 atoms (8 metastable basins, OU drift 0.08 nm,
quantised to 0.001 nm, uniform masses), k=100: 4e8 ordered pairs through the
candidate screen, fused top-k, exact recheck and output.

  value  pairs/s with the frames already resident in HBM (MDS_DEVICE_IO)
  e2e    pairs/s through the C ABI with pinned host buffers: the host->device
         copy of the frames and the device->host copy of the k-NN lists are
         inside the timed region
  roofline  the screen kernel: 18*A algorithmic flops per pair (nine A-long
         contractions) / its CUDA-event time, against the measured dense
         bf16 tensor peak
  cpu_baseline  the reference's per-pair procedure and OpenMP row loop
         restated in C++ (oracle/mds_oracle.cpp, orc_knn_rms_port) on a bounded
         sample of fit rows against all reference frames, all host cores

`--impl reference` times that CPU restatement alone (the reference itself
needs GROMACS, Boost and Berkeley DB and cannot be built here).
Inputs (240 MB of frames) are larger than L2 (129 MB) in every step.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_FRAMES = 20_000
N_ATOMS = 1_000
K = 100
SEED = 2024
METRIC = "kNN-RMSD pairs/s"
UNIT = "pairs/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--precision", default=os.environ.get("MDS_BENCH_PRECISION", "bf16x3"))
    p.add_argument("--frames", type=int, default=N_FRAMES)
    p.add_argument("--atoms", type=int, default=N_ATOMS)
    p.add_argument("--k", type=int, default=K)
    p.add_argument("--cpu-rows", type=int, default=0, help="fit rows of the CPU sample (0 = auto)")
    p.add_argument("--no-cpu", action="store_true")
    return p.parse_args()


def workload(frames, atoms):
    from mdsctk_gb300 import synth

    return synth.trajectory(frames, atoms, seed=SEED, drift_sigma=0.08, basins=8, dwell=500.0)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def cpu_sample(x, rows, k, threads):
    """Time the restated reference loop on `rows` fit rows vs all frames."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import oracle as O

    O.build()
    m = np.ones(x.shape[1], np.float32)
    t0 = time.perf_counter()
    O.knn_rms_port(x, x[:rows], m, k, threads=threads)
    dt = time.perf_counter() - t0
    return rows * x.shape[0] / dt, dt


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    x = workload(args.frames, args.atoms)
    threads = os.cpu_count() or 1
    rows = args.cpu_rows or 2 * threads
    vals = []
    for _ in range(args.warmup):
        cpu_sample(x, threads, args.k, threads)
    for _ in range(args.steps):
        v, dt = cpu_sample(x, rows, args.k, threads)
        vals.append(v)
    v = sorted(vals)[len(vals) // 2]
    sample = f"{rows} fit rows x {args.frames} reference frames x {args.atoms} atoms per step"
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "fp32/fp64", "data": "synthetic",
           "config": {"workload": f"knn_rms all-pairs N={args.frames} A={args.atoms} k={args.k}",
                      "frames": args.frames, "atoms": args.atoms, "k": args.k},
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                            "sample": sample},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import numpy as np
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from mdsctk_gb300 import Context

    x = workload(args.frames, args.atoms)
    n, a, k = x.shape[0], x.shape[1], args.k
    # rows of this rank (weak scaling: every rank runs the whole workload's
    # row count against all reference frames; units = its own pairs)
    ctx = Context(local)
    dev = torch.device("cuda", local)
    xd = torch.from_numpy(x).to(dev)
    md = torch.ones(a, dtype=torch.float32, device=dev)
    kk = min(k, n - 1)
    out = (torch.empty((n, kk), dtype=torch.float64, device=dev),
           torch.empty((n, kk), dtype=torch.int32, device=dev))
    # host side for e2e: pinned frames in, pinned k-NN lists out
    xh = torch.from_numpy(x).pin_memory()
    dh = torch.empty((n, kk), dtype=torch.float64).pin_memory()
    ih = torch.empty((n, kk), dtype=torch.int32).pin_memory()
    mh = np.ones(a, np.float32)

    def step_dev():
        ctx.knn_rms(xd, None, md, k, precision=args.precision, out=out)

    def step_e2e():
        ctx.knn_rms(xh.numpy(), None, mh, k, precision=args.precision, out=(dh.numpy(), ih.numpy()))

    for _ in range(max(args.warmup, 3)):
        step_dev()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    screen_ms, recheck_ms, prep_ms, total_ms, launches, flagged = [], [], [], [], 0, 0
    for _ in range(args.steps):
        step_dev()
        st = ctx.stats()
        screen_ms.append(st["screen_ms"])
        recheck_ms.append(st["recheck_ms"])
        prep_ms.append(st["prep_ms"])
        total_ms.append(st["total_ms"])
        launches += st["launches"]
        flagged = max(flagged, st["rows_flagged"])
    ev1.record()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / args.steps
    if world > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        torch.distributed.barrier()
        ms = float(t.item())
    clocks = sampler.stop()
    # end to end through the C ABI with host buffers
    for _ in range(1):
        step_e2e()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step_e2e()
    e2e_ms = (time.perf_counter() - t0) * 1000.0 / args.steps
    pairs = float(n) * n
    value = pairs * world / (ms / 1000.0)
    e2e = pairs * world / (e2e_ms / 1000.0)
    peaks, pk_kind = measured_peaks()
    scr = sorted(screen_ms)[len(screen_ms) // 2]
    flops = 18.0 * a * pairs
    achieved = flops / (scr / 1000.0) / 1e12
    peak = float(peaks.get("bf16_tflops", 1900.0))
    # correctness spot check of the last device run: a few rows vs the oracle
    res = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None,
           "dtype": {"fp32": "fp32", "bf16x3": "bf16x3+fp32", "fp16x3": "fp16x3+fp32"}[args.precision],
           "data": "synthetic",
           "config": {"workload": f"knn_rms all-pairs N={n} A={a} k={k}", "frames": n, "atoms": a,
                      "k": k, "precision": args.precision, "basins": 8, "drift_nm": 0.08,
                      "l2": "inputs (240 MB of frames) larger than L2 every step",
                      "parallelism": f"replicas x{world}"},
           "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                        "frac": achieved / peak, "traffic": None,
                        "kernel": "screen", "kernel_ms": scr, "flops_per_launch": flops,
                        "peak_kind": f"{pk_kind} bf16 burst"},
           "stages_ms": {"prep": sorted(prep_ms)[len(prep_ms) // 2], "screen": scr,
                         "recheck": sorted(recheck_ms)[len(recheck_ms) // 2],
                         "call": sorted(total_ms)[len(total_ms) // 2]},
           "rows_flagged": flagged,
           "clocks": clocks,
           "gpu_launches": launches,
           "e2e": {"value": e2e, "unit": UNIT, "ms_per_step": e2e_ms,
                   "h2d_bytes_per_step": int(x.nbytes + a * 4),
                   "d2h_bytes_per_step": int(n * kk * 12)}}
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        rows = args.cpu_rows or 16 * threads
        v, dt = cpu_sample(x, rows, k, threads)
        res["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                               "sample": f"{rows} fit rows x {n} reference frames ({dt:.1f} s)"}
    if rank == 0:
        print(json.dumps(res))
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
