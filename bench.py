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
        # the small plain-method case: Gaussian sigma = radius cut at 3 sigma
        f = synth.uniform(n=100_000, seed=1 + rank)
        desc = dict(workload="uniform_100k", particles=f.n, grid=list(f.res), radius=0.5,
                    kernel="gauss3 sigma=r (cut at 3 sigma)", cyclic=True)
        return f, desc
    if name == "uniform_16M":
        # the learned-AO inference set: 16M particles of the small case's structure, box scaled to keep the
        # number density and the voxel size
        n = 16_000_000
        scale = (n / 100_000) ** (1.0 / 3.0)
        f = synth.uniform(n=n, edge=100.0 * scale, res=int(round(128 * scale)), seed=1 + rank)
        desc = dict(workload="uniform_16M", particles=f.n, grid=list(f.res), radius=0.5,
                    kernel="bump sigma=1 (reference rbf)", cyclic=True)
        return f, desc
    if name == "mixed_phase_64M":
        f = synth.mixed_phase(seed=5 + rank)
        desc = dict(workload="mixed_phase_64M", particles=f.n, grid=list(f.res),
                    phases="FCC slab (a=1.12, jitter 0.05) + uniform gas at 1/20 density",
                    radii="0.5/0.8/1.2 in 6:3:1", kernel="bump sigma=1 (reference rbf)", cyclic=True)
        return f, desc
    raise SystemExit(f"unknown workload {name}")


def density_params(desc: dict) -> dict:
    from megamol_gb300 import p2v

    gauss = desc["kernel"].startswith("gauss3")
    return dict(kernel=p2v.KERNEL_GAUSS3 if gauss else p2v.KERNEL_BUMP, sigma=1.0)


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


AO_PARAMS = dict(ao_mode=1, ao_volume=0, ao_volume_scale=1.0, ao_cones=8, ao_steps=32, ao_levels=3, ao_apex_deg=50.0,
                 ao_offset=0.01, ao_strength=1.0, ao_cone_length=0.8, ao_early_exit=1)
AO_SAMPLE = 50_000  # particles in the CPU AO sample


def setup_frame(ctx, f, dparams=None):
    """Density once (untimed) to derive the workload's normals: unit vectors down the density gradient."""
    from megamol_gb300 import p2v, synth

    dp = dparams or dict(kernel=p2v.KERNEL_BUMP, sigma=1.0)
    ctx.set_params(sizex=f.res[0], sizey=f.res[1], sizez=f.res[2], cyclX=1, cyclY=1, cyclZ=1, normalize=1,
                   ao_mode=p2v.AO_NONE, **dp)
    V = f.res[0] * f.res[1] * f.res[2]
    vol = np.empty(V, np.float32)
    ctx.run_frame([p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR)], f.bbox, vol)
    nrm = synth.gradient_normals(f.xyzr, vol.reshape(f.res[2], f.res[1], f.res[0]), f.bbox)
    ctx.set_params(**AO_PARAMS)
    return vol.reshape(f.res[2], f.res[1], f.res[0]), nrm


def cpu_reference_density(f, nthreads: int, kernel: int = 0):
    """Time the reference's CPU density (the compiled ParticlesToDensity module when present, else the
    FP32 restatement with the same OpenMP structure) on one frame; returns (seconds, kind, grid). The
    reference has only its bump rbf: the 3-sigma Gaussian is timed with the restatement."""
    import oracle

    os.environ["OMP_NUM_THREADS"] = str(nthreads)
    if oracle.reference_available() and kernel == oracle.BUMP:
        xyzr = np.ascontiguousarray(f.xyzr)
        L = [dict(type=2, data=xyzr, stride=0, radius=0.0, count=f.n)]
        t0 = time.perf_counter()
        vol, _ = oracle.reference_density(L, f.bbox, f.res, (1, 1, 1), True, 1.0)
        return time.perf_counter() - t0, "reference", vol
    t0 = time.perf_counter()
    vol = oracle.density_f32(f.xyzr, f.bbox, f.res, (1, 1, 1), 1.0, kernel, nthreads)
    vol, _, _ = oracle.normalize_minmax_f32(vol)
    return time.perf_counter() - t0, "port", vol


def ao_sample(f) -> int:
    return AO_SAMPLE if f.res[0] * f.res[1] * f.res[2] <= 256 ** 3 else AO_SAMPLE // 10


def cpu_cone_ao(f, grid, nrm, sample: int):
    """Time the CPU cone march (restatement of the MDAO shader, OpenMP) on `sample` particles; returns
    seconds for the sample."""
    import oracle

    h = oracle.spacing_f64(f.bbox, f.res)
    bmin = [f.bbox[a] - 0.5 * h[a] for a in range(3)]
    bsize = [f.res[a] * h[a] for a in range(3)]
    lv = oracle.mip_chain_f64(grid, AO_PARAMS["ao_levels"], AO_PARAMS["ao_volume_scale"])
    dirs = oracle.cone_dirs(AO_PARAMS["ao_cones"], np.deg2rad(np.float32(AO_PARAMS["ao_apex_deg"])))
    idx = np.linspace(0, f.n - 1, sample).astype(np.int64)
    t0 = time.perf_counter()
    oracle.cone_ao_f64(lv, dirs, f.xyzr[idx], nrm[idx], bmin, bsize, offset=AO_PARAMS["ao_offset"],
                       strength=AO_PARAMS["ao_strength"], cone_length=AO_PARAMS["ao_cone_length"],
                       shortest_edge=float(min(f.res)), max_lod=float(AO_PARAMS["ao_levels"] - 1),
                       steps=AO_PARAMS["ao_steps"], early_exit=1, border=0, sat_scale=AO_PARAMS["ao_volume_scale"])
    return time.perf_counter() - t0


def cpu_pipeline(f, nthreads, grid=None, nrm=None, kernel: int = 0):
    """CPU particles/s of density + plain cone AO: the density stage on the full frame, the AO stage on a
    sample of particles scaled to the frame (AO_SAMPLE, a tenth of that above 256^3 voxels, so the CPU leg
    stays within about half a minute)."""
    from megamol_gb300 import synth

    dt_d, kind, vol = cpu_reference_density(f, nthreads, kernel)
    if nrm is None:
        nrm = synth.gradient_normals(f.xyzr, vol, f.bbox)
    sample = ao_sample(f)
    dt_ao = cpu_cone_ao(f, vol, nrm, sample) * (f.n / sample)
    return f.n / (dt_d + dt_ao), kind, dt_d, dt_ao


def run_reference(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return
    if args.workload == "trajectory_64":
        print(json.dumps({"impl": "reference", "unavailable": "the CPU reference arm times single frames; "
                          "run it on the default workload"}), flush=True)
        return
    f, desc = make_workload(args.workload)
    kern = density_params(desc)["kernel"]
    nthreads = os.cpu_count() or 1
    from megamol_gb300 import synth

    _, _, vol = cpu_reference_density(f, nthreads, kern)
    nrm = synth.gradient_normals(f.xyzr, vol, f.bbox)
    for _ in range(max(0, args.warmup)):
        cpu_pipeline(f, nthreads, nrm=nrm, kernel=kern)
    vals, kind = [], "port"
    tot = 0.0
    for _ in range(args.steps):
        v, kind, dt_d, dt_ao = cpu_pipeline(f, nthreads, nrm=nrm, kernel=kern)
        vals.append(v)
        tot += dt_d + dt_ao
    value = f.n * args.steps / tot
    line = {"metric": "particles/s density+AO", "value": value, "unit": "particles/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference", "config": dict(desc, ao="plain cone march 8 cones x 32 steps, 3-level mip"),
            "cpu_baseline": {"value": value, "unit": "particles/s", "cores": nthreads, "kind": kind,
                             "sample": f"density on the full frame ({f.n} particles) + cone AO on {ao_sample(f)} "
                                       "particles scaled to the frame, per step"},
            "e2e": {"value": value, "unit": "particles/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def train_learned_ao(ctx, f_main, dparams=None, workload: str = "lj_liquid_4M"):
    """Train the learned AO on cone-march pairs of other frames. LJ liquid: two other LJ frames (seeds 3
    and 4, 500,000 pairs each) and ten uniform 100k-particle frames of the small plain-method workload.
    Other workloads: other seeds of the same workload (the cone length is a fraction of the volume, so the
    network must see the box geometry it infers on): two frames of 1,000,000 pairs, one for the 64M frame."""
    from megamol_gb300 import p2v, synth

    ctx.mlp_clear()
    total = 0
    if workload == "lj_liquid_4M":
        frames = [(synth.lj_liquid(seed=s), 500_000) for s in (3, 4)]
        frames += [(synth.uniform(n=100_000, seed=10 + k), 100_000) for k in range(10)]
    elif workload == "uniform_100k":
        frames = [(make_workload(workload, rank=100 + k)[0], 100_000) for k in range(12)]
    else:
        kk = (100,) if workload == "mixed_phase_64M" else (100, 101)
        frames = [(make_workload(workload, rank=k)[0], 1_000_000) for k in kk]
    for k, (f, npairs) in enumerate(frames):
        ctx.set_params(sizex=f.res[0], sizey=f.res[1], sizez=f.res[2], ao_mode=p2v.AO_NONE, normalize=1,
                       **(dparams or {}))
        vol = np.empty(f.res[0] * f.res[1] * f.res[2], np.float32)
        ctx.run_frame([p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR)], f.bbox, vol)
        nrm = synth.gradient_normals(f.xyzr, vol.reshape(f.res[2], f.res[1], f.res[0]), f.bbox)
        ctx.set_params(**AO_PARAMS)
        total = ctx.mlp_collect([p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR, normals=nrm)], f.bbox, npairs,
                                seed=100 + k)
    rep = ctx.mlp_train(seed=7)
    ctx.set_params(sizex=f_main.res[0], sizey=f_main.res[1], sizez=f_main.res[2], normalize=1, **AO_PARAMS)
    return total, rep


def time_pipeline(ctx, lists, bbox, out, steps, warmup, stream, torch, barrier, sampler=None, tag="timed"):
    """Device time per step (CUDA events on the launching stream) and per-stage times from the library.
    The timed steps run inside an NVTX range named `tag` (profilers can restrict themselves to it)."""
    for _ in range(warmup):
        ctx.run_frame(lists, bbox, out, stream=stream.cuda_stream)
    stage = {"ms_binning": 0.0, "ms_density": 0.0, "ms_normalize": 0.0, "ms_ao": 0.0, "ao_fallback": 0}
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    if sampler:
        sampler.__enter__()
    torch.cuda.nvtx.range_push(tag)
    ev0.record(stream)
    for _ in range(steps):
        ctx.run_frame(lists, bbox, out, stream=stream.cuda_stream)
        st = ctx.stats()
        for k in stage:
            stage[k] += st[k]
    ev1.record(stream)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    if sampler:
        sampler.__exit__()
    barrier()
    return ev0.elapsed_time(ev1) / steps, {k: v / steps for k, v in stage.items()}


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
    dparams = density_params(desc)
    pairs, train_rep = train_learned_ao(ctx, f, dparams, args.workload)
    grid0, nrm = setup_frame(ctx, f, dparams)
    V = f.res[0] * f.res[1] * f.res[2]
    stream = torch.cuda.Stream()
    d_in = torch.from_numpy(f.xyzr).to(dev)
    d_nrm = torch.from_numpy(nrm).to(dev)
    d_ao = torch.empty(f.n, dtype=torch.float32, device=dev)
    d_out = torch.empty(V, dtype=torch.float32, device=dev)
    dev_lists = [p2v.ParticleList(d_in, p2v.VERTDATA_FLOAT_XYZR, count=f.n, normals=d_nrm, ao_out=d_ao)]

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    def max_over_ranks(x):
        if ws > 1:
            import torch.distributed as dist
            t = torch.tensor([x], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            return float(t.item())
        return x

    # ---- the density tile for this frame: the autotuner times the compiled tiles on it (density only);
    # both pipelines below use the winner ----
    ctx.set_params(ao_mode=p2v.AO_NONE, tile_x=0, tile_y=0, tile_z=0)
    tune = ctx.autotune_batch([dict(lists=dev_lists, bbox=f.bbox, out=d_out, size=f.res)])
    # ---- plain cone-march pipeline ----
    ctx.set_params(ao_mode=p2v.AO_CONE)
    ms_plain, st_plain = time_pipeline(ctx, dev_lists, f.bbox, d_out, args.steps, args.warmup, stream, torch, barrier,
                                       tag="plain")
    ms_plain = max_over_ranks(ms_plain)
    ao_plain = d_ao.cpu().numpy().copy()
    # ---- learned-AO pipeline (MLP, cone-march fallback) ----
    ctx.set_params(ao_mode=p2v.AO_LEARNED)
    sampler = ClockSampler(dev)
    ms_learn, st_learn = time_pipeline(ctx, dev_lists, f.bbox, d_out, args.steps, args.warmup, stream, torch, barrier,
                                       sampler, tag="learned")
    ms_learn = max_over_ranks(ms_learn)
    ao_learn = d_ao.cpu().numpy()
    rmse = float(np.sqrt(np.mean((ao_learn.astype(np.float64) - ao_plain) ** 2)))
    clocks = sampler.summary()
    use_learned = rmse <= 0.02
    mode = p2v.AO_LEARNED if use_learned else p2v.AO_CONE
    ms, st = (ms_learn, st_learn) if use_learned else (ms_plain, st_plain)
    ctx.set_params(ao_mode=mode)
    value = ws * f.n / (ms * 1e-3)

    # ---- end to end through the public API, host buffers ----
    h_in = torch.from_numpy(f.xyzr).pin_memory()
    h_nrm = torch.from_numpy(nrm).pin_memory()
    h_ao = torch.empty(f.n, dtype=torch.float32).pin_memory()
    h_out = torch.empty(V, dtype=torch.float32).pin_memory()
    host_lists = [p2v.ParticleList(h_in, p2v.VERTDATA_FLOAT_XYZR, count=f.n, normals=h_nrm, ao_out=h_ao)]
    e2e_steps = max(3, args.steps // 2)
    e2e_ms, _ = time_pipeline(ctx, host_lists, f.bbox, h_out, e2e_steps, 2, stream, torch, barrier, tag="e2e")
    e2e_ms = max_over_ranks(e2e_ms)
    e2e = {"value": ws * f.n / (e2e_ms * 1e-3), "unit": "particles/s", "h2d_bytes_per_step": int(f.n * (16 + 12)),
           "d2h_bytes_per_step": int(V * 4 + f.n * 4), "ms_per_step": e2e_ms}

    # ---- roofline of the dominant kernel of the measured pipeline ----
    peak, peak_kind = peaks()
    nb = (f.res[0] + 2) * (f.res[1] + 2) * (f.res[2] + 2)
    gather_bytes = f.n * 16 + V * 4 + nb * 4
    lv_bytes, d = 0, list(f.res)
    for _ in range(AO_PARAMS["ao_levels"]):
        lv_bytes += d[0] * d[1] * d[2] * 4
        d = [max(1, x // 2) for x in d]
    ao_bytes = f.n * (16 + 12 + 4) + lv_bytes
    ao_name = "p2v::mlp_infer_tc_kernel (+ mip levels, stencil textures, fallback cone march)" if use_learned else \
        "p2v::cone_ao_kernel (+ mip levels)"
    if st["ms_ao"] >= st["ms_density"]:
        dom = (ao_name, ao_bytes, st["ms_ao"], "learned_ao_lj_liquid_4M.md" if use_learned else "cone_ao_lj_liquid_4M.md")
    else:
        dom = ("p2v::gather_fixed_kernel", gather_bytes, st["ms_density"], "density_gather_lj_liquid_4M.md")
    achieved = dom[1] / (dom[2] * 1e-3) / 1e9
    roofline = {"bound": "hbm", "kernel": dom[0], "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_kind": peak_kind,
                "traffic": profile_traffic(dom[3]) if args.workload == "lj_liquid_4M" else None,
                "algorithmic_bytes": dom[1], "ms_per_launch": dom[2],
                "stages_ms": {k: st[k] for k in ("ms_binning", "ms_density", "ms_normalize", "ms_ao")},
                "density_gather": {"algorithmic_bytes": gather_bytes, "ms": st["ms_density"],
                                   "frac": gather_bytes / (st["ms_density"] * 1e-3) / 1e9 / peak}}

    # ---- CPU baseline (rank 0, N=1 only) ----
    cpu = None
    if rank == 0 and ws == 1:
        nthreads = os.cpu_count() or 1
        v, kind, dt_d, dt_ao = cpu_pipeline(f, nthreads, nrm=nrm, kernel=dparams["kernel"])
        cpu = {"value": v, "unit": "particles/s", "cores": nthreads, "kind": kind,
               "sample": f"density on the full frame ({f.n} particles, {dt_d:.2f} s) + plain cone AO on "
                         f"{ao_sample(f)} particles scaled to the frame ({dt_ao:.2f} s)"}

    # kernels per frame: scalar init, pack, [the counting sort by cell: histogram, tile sums, tile scan, cell
    # starts, scatter, in-cell order], digit histogram + scan, the radix passes (9/8-bit digits over the bin
    # keys; an odd count and launched gated after a counting sort), cell starts (3), gather, finalize +
    # normalise; AO: normals, mips, sorted copies, then the cone march or stencil textures (2) + tensor-core
    # inference + fallback cone march, and the AO back to input order
    key_bits = int(nb).bit_length()
    passes = (key_bits + 8) // 9
    counting = nb + 1 <= 64 * f.n
    if counting and passes % 2 == 0:
        passes += 1
    launches_density = 1 + 1 + (6 if counting else 0) + 2 + passes + 3 + 1 + 2
    launches_ao = 1 + (AO_PARAMS["ao_levels"] - 1) + 1 + (5 if use_learned else 2)
    if rank == 0:
        line = {"metric": "particles/s density+AO", "value": value, "unit": "particles/s", "n_gpus": ws,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32 (MLP: bf16 x bf16 -> f32)", "data": "synthetic",
                "config": dict(desc, ao=("learned AO (MLP 60-64-64-1, BF16 tensor cores) with cone-march fallback"
                                         if use_learned else "plain cone march") +
                                        ", 8 cones x 32 steps, 3-level mip, gradient normals",
                               l2="per-step working set ~0.6 GB > 126 MB L2 (no flush)"),
                "learned_vs_plain": {"plain_particles_per_s": ws * f.n / (ms_plain * 1e-3), "plain_ms": ms_plain,
                                     "learned_particles_per_s": ws * f.n / (ms_learn * 1e-3), "learned_ms": ms_learn,
                                     "speedup": ms_plain / ms_learn, "ao_rmse_learned_vs_plain": rmse,
                                     "ao_max_err": float(np.abs(ao_learn - ao_plain).max()),
                                     "fallback_particles": int(st_learn["ao_fallback"]),
                                     "plain_ao_ms": st_plain["ms_ao"], "learned_ao_ms": st_learn["ms_ao"],
                                     "training": {"pairs": pairs, "val_rmse": train_rep["val_rmse"],
                                                  "steps": train_rep["steps"], "ms": train_rep["ms"]}},
                "density_tile": {"tile": tune["tile"], "candidates_ms": {"x".join(map(str, c["tile"])): c["ms"]
                                                                         for c in tune["candidates"] if c["lanes"] == 1}},
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
                "gpu_launches": (launches_density + launches_ao) * args.steps, "clocks": clocks}
        print(json.dumps(line), flush=True)
    ctx.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_batch_bench(args):
    """Batched-trajectory workload: 64 frames of 1-8 Gaussian blobs, particle counts log-uniform in
    [50k, 2M], grids 64^3-256^3 matched to extent, density + plain cone AO (8 cones x 32 steps, 3 levels,
    gradient normals). One step = the whole batch through p2v_run_batch (one CUDA-graph launch); the
    autotuner picks the density tile and the lane count first. Also reported: the same frames one
    p2v_run_frame call after another, and the batch without its graph."""
    import torch

    from megamol_gb300 import p2v, synth

    ws, rank, local = dist_info()
    if ws > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.cuda.current_device()
    traj = synth.trajectory(frames=64, seed=3 + 1000 * rank)
    ctx = p2v.Context(dev)
    # setup (untimed): gradient normals from each frame's own density
    frames_dev, frames_host, total = [], [], 0
    for f in traj:
        ctx.set_params(sizex=f.res[0], sizey=f.res[1], sizez=f.res[2], ao_mode=p2v.AO_NONE, normalize=1,
                       kernel=p2v.KERNEL_BUMP, sigma=1.0)
        vol = np.empty(f.res[0] * f.res[1] * f.res[2], np.float32)
        ctx.run_frame([p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR)], f.bbox, vol)
        nrm = synth.gradient_normals(f.xyzr, vol.reshape(f.res[2], f.res[1], f.res[0]), f.bbox)
        V = f.res[0] * f.res[1] * f.res[2]
        d_in = torch.from_numpy(f.xyzr).to(dev)
        d_n = torch.from_numpy(nrm).to(dev)
        d_ao = torch.empty(f.n, dtype=torch.float32, device=dev)
        d_out = torch.empty(V, dtype=torch.float32, device=dev)
        frames_dev.append(dict(lists=[p2v.ParticleList(d_in, p2v.VERTDATA_FLOAT_XYZR, count=f.n, normals=d_n,
                                                       ao_out=d_ao)], bbox=f.bbox, out=d_out, size=f.res))
        h_in = torch.from_numpy(f.xyzr).pin_memory()
        h_n = torch.from_numpy(nrm).pin_memory()
        h_ao = torch.empty(f.n, dtype=torch.float32).pin_memory()
        h_out = torch.empty(V, dtype=torch.float32).pin_memory()
        frames_host.append(dict(lists=[p2v.ParticleList(h_in, p2v.VERTDATA_FLOAT_XYZR, count=f.n, normals=h_n,
                                                        ao_out=h_ao)], bbox=f.bbox, out=h_out, size=f.res))
        total += f.n
    ctx.set_params(normalize=1, batch_graph=1, tile_x=0, tile_y=0, tile_z=0, batch_lanes=0, **AO_PARAMS)
    tune = ctx.autotune_batch(frames_dev)

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    def timed(frames, steps, warmup, graph=True):
        ctx.set_params(batch_graph=1 if graph else 0)
        for _ in range(warmup):
            ctx.run_batch(frames)
        barrier()
        torch.cuda.synchronize()
        t = []
        for _ in range(steps):
            ctx.run_batch(frames)
            t.append(ctx.stats()["ms_total"])
        torch.cuda.synchronize()
        barrier()
        return sum(t) / len(t)

    sampler = ClockSampler(dev)
    sampler.__enter__()
    ms = timed(frames_dev, args.steps, max(args.warmup, 3))
    sampler.__exit__()
    ms_eager = timed(frames_dev, max(3, args.steps // 4), 2, graph=False)
    ms_e2e = timed(frames_host, max(3, args.steps // 2), 3)
    # the same frames one p2v_run_frame after another (stream-synchronous per frame)
    seq = []
    for _ in range(2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for fd in frames_dev:
            ctx.set_params(sizex=fd["size"][0], sizey=fd["size"][1], sizez=fd["size"][2])
            ctx.run_frame(fd["lists"], fd["bbox"], fd["out"])
        torch.cuda.synchronize()
        seq.append((time.perf_counter() - t0) * 1e3)
    ms_seq = min(seq)
    if ws > 1:
        import torch.distributed as dist
        t = torch.tensor([ms, ms_e2e], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms, ms_e2e = float(t[0]), float(t[1])
    h2d = sum(f.n * (16 + 12) for f in traj)
    d2h = sum(f.n * 4 + f.res[0] * f.res[1] * f.res[2] * 4 for f in traj)
    if rank == 0:
        line = {"metric": "particles/s density+AO (batched trajectory)", "value": ws * total / (ms * 1e-3),
                "unit": "particles/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": "trajectory_64", "frames": len(traj), "particles": total,
                           "particles_per_frame": "log-uniform [50k, 2M]", "grids": sorted({f.res[0] for f in traj}),
                           "ao": "plain cone march, 8 cones x 32 steps, 3-level mip, gradient normals",
                           "l2": "per-step working set several GB > 126 MB L2 (no flush)"},
                "batch": {"autotuned_tile": tune["tile"], "autotuned_lanes": tune["lanes"],
                          "ms_graph": ms, "ms_eager": ms_eager, "ms_frame_by_frame": ms_seq,
                          "speedup_vs_frame_by_frame": ms_seq / ms},
                "e2e": {"value": ws * total / (ms_e2e * 1e-3), "unit": "particles/s", "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h, "ms_per_step": ms_e2e},
                "gpu_launches": None, "clocks": sampler.summary()}
        print(json.dumps(line), flush=True)
    ctx.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "trajectory_64":
        run_batch_bench(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
