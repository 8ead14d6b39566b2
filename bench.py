"""Benchmark of the particle-to-volume path (density + AO) on GB300.

Default workload: the LJ-liquid frame (4,000,000 particles on a jittered FCC lattice, radii U[0.4,0.6],
256^3 grid), seeded synthetic data. One step = one full frame through the pipeline (binning + sort +
density gather + statistics/normalisation [+ mip + AO]).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

Prints ONE JSON line (rank 0). `value` is whole-job particles/s with inputs resident in HBM; `e2e` is the
same metric through the public C-ABI call with host input and output buffers (host<->device copies in the
timed region). Multi-GPU runs are independent replicas, one frame per rank per step (weak scaling).
"""
from __future__ import annotations

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

L2_BYTES = 126 * 2 ** 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="lj_liquid_4M")
    return ap.parse_args()


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def make_workload(name: str, rank: int = 0):
    from megamol_gb300 import synth

    if name == "lj_liquid_4M":
        f = synth.lj_liquid(seed=2 + rank)
        desc = dict(workload="lj_liquid_4M", particles=f.n, grid=list(f.res), lattice="fcc 100^3 cells, a=1.12",
                    jitter=0.08, radii="U[0.4,0.6]", kernel="bump sigma=1 (reference rbf)", cyclic=True)
        return f, desc
    if name == "uniform_100k":
        f = synth.uniform(n=100_000, seed=1 + rank)
        desc = dict(workload="uniform_100k", particles=f.n, grid=list(f.res), radius=0.5, kernel="bump sigma=1")
        return f, desc
    raise SystemExit(f"unknown workload {name}")


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.rows.append([x.strip() for x in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 5 + i and r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic(name: str):
    """Per-launch DRAM traffic of the dominant kernel from the committed ncu summary, if present."""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def cpu_reference_density(f, nthreads: int):
    """Time the reference's CPU density (the compiled ParticlesToDensity module when present, else the
    FP32 restatement with the same OpenMP structure) on one frame; returns (seconds, kind)."""
    import oracle

    os.environ["OMP_NUM_THREADS"] = str(nthreads)
    if oracle.reference_available():
        xyzr = np.ascontiguousarray(f.xyzr)
        L = [dict(type=2, data=xyzr, stride=0, radius=0.0, count=f.n)]
        t0 = time.perf_counter()
        oracle.reference_density(L, f.bbox, f.res, (1, 1, 1), False, 1.0)
        return time.perf_counter() - t0, "reference"
    t0 = time.perf_counter()
    oracle.density_f32(f.xyzr, f.bbox, f.res, (1, 1, 1), 1.0, oracle.BUMP, nthreads)
    return time.perf_counter() - t0, "port"


def run_reference(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return
    f, desc = make_workload(args.workload)
    nthreads = os.cpu_count() or 1
    for _ in range(max(0, args.warmup)):
        cpu_reference_density(f, nthreads)
    times = []
    kind = "port"
    for _ in range(args.steps):
        dt, kind = cpu_reference_density(f, nthreads)
        times.append(dt)
    tot = sum(times)
    value = f.n * args.steps / tot
    line = {"metric": "particles/s density+AO", "value": value, "unit": "particles/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference", "config": desc,
            "cpu_baseline": {"value": value, "unit": "particles/s", "cores": nthreads, "kind": kind,
                             "sample": f"full frame ({f.n} particles, density only) per step"},
            "e2e": {"value": value, "unit": "particles/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch

    from megamol_gb300 import p2v

    ws, rank, local = dist_info()
    if ws > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.cuda.current_device()
    f, desc = make_workload(args.workload, rank)
    ctx = p2v.Context(dev)
    ctx.set_params(sizex=f.res[0], sizey=f.res[1], sizez=f.res[2], cyclX=1, cyclY=1, cyclZ=1, normalize=0, sigma=1.0,
                   kernel=p2v.KERNEL_BUMP)
    V = f.res[0] * f.res[1] * f.res[2]
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    d_in = torch.from_numpy(f.xyzr).to(dev)
    d_out = torch.empty(V, dtype=torch.float32, device=dev)
    dev_lists = [p2v.ParticleList(d_in, p2v.VERTDATA_FLOAT_XYZR, count=f.n)]

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    # ---- device-resident throughput ----
    for _ in range(args.warmup):
        ctx.run_frame(dev_lists, f.bbox, d_out, stream=sp)
    stage = {"ms_binning": 0.0, "ms_density": 0.0, "ms_normalize": 0.0, "ms_ao": 0.0}
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    gi, _, _ = dist_info()
    sampler = ClockSampler(int(os.environ.get("CUDA_VISIBLE_DEVICES", str(dev)).split(",")[0]) if os.environ.get(
        "CUDA_VISIBLE_DEVICES", "").replace(",", "").isdigit() else dev)
    barrier()
    torch.cuda.synchronize()
    with sampler:
        ev0.record(stream)
        for _ in range(args.steps):
            ctx.run_frame(dev_lists, f.bbox, d_out, stream=sp)
            st = ctx.stats()
            for k in stage:
                stage[k] += st[k]
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1) / args.steps
    if ws > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = ws * f.n / (ms * 1e-3)
    clocks = sampler.summary()

    # ---- end to end through the public API, host buffers ----
    h_in = torch.from_numpy(f.xyzr).pin_memory()
    h_out = torch.empty(V, dtype=torch.float32).pin_memory()
    host_lists = [p2v.ParticleList(h_in, p2v.VERTDATA_FLOAT_XYZR, count=f.n)]
    for _ in range(2):
        ctx.run_frame(host_lists, f.bbox, h_out, stream=sp)
    e2e_steps = max(3, args.steps // 2)
    barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(e2e_steps):
        ctx.run_frame(host_lists, f.bbox, h_out, stream=sp)
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / e2e_steps
    if ws > 1:
        import torch.distributed as dist
        t = torch.tensor([e2e_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())
    e2e = {"value": ws * f.n / (e2e_ms * 1e-3), "unit": "particles/s", "h2d_bytes_per_step": int(f.n * 16),
           "d2h_bytes_per_step": int(V * 4), "ms_per_step": e2e_ms}

    # ---- roofline of the dominant kernel (density gather) ----
    peak, peak_kind = peaks()
    nb = (f.res[0] + 2) * (f.res[1] + 2) * (f.res[2] + 2)
    gather_bytes = f.n * 16 + V * 4 + nb * 4
    gather_ms = stage["ms_density"] / args.steps
    bin_ms = stage["ms_binning"] / args.steps
    achieved = gather_bytes / (gather_ms * 1e-3) / 1e9
    traffic = profile_traffic("density_gather_lj_liquid_4M.md") if args.workload == "lj_liquid_4M" else None
    roofline = {"bound": "hbm", "kernel": "p2v::gather_kernel", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                "algorithmic_bytes": gather_bytes, "ms_per_launch": gather_ms,
                "stages_ms": {"binning": bin_ms, "density": gather_ms,
                              "normalize": stage["ms_normalize"] / args.steps}}

    # ---- CPU baseline (rank 0, N=1 only) ----
    cpu = None
    if rank == 0 and ws == 1:
        nthreads = os.cpu_count() or 1
        dt, kind = cpu_reference_density(f, nthreads)
        cpu = {"value": f.n / dt, "unit": "particles/s", "cores": nthreads, "kind": kind,
               "sample": f"one full frame ({f.n} particles, density only)"}

    passes = 4
    launches_per_step = 1 + 2 + passes + 3 + 2
    if rank == 0:
        line = {"metric": "particles/s density+AO", "value": value, "unit": "particles/s", "n_gpus": ws,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": dict(desc, l2="per-step working set ~0.5 GB > 126 MB L2 (no flush)",
                               stage="density only (AO not yet in the pipeline)"),
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
                "gpu_launches": launches_per_step * args.steps, "clocks": clocks}
        print(json.dumps(line), flush=True)
    ctx.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
