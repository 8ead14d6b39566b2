"""Multi-GPU sharding of the particle-to-volume path (one process per GPU, torch.distributed).

Three forms, all with the reference's semantics kept bit for bit where the reference defines them:

* Frames of a trajectory are independent units: `shard_frames` deals them to ranks (largest first onto the
  least-loaded rank) and each rank computes its frames with no collective on the data path (weak scaling).
* One large frame splits into z-slabs of grid nodes (`slab_ranges`). A rank keeps the particles whose
  footprint reaches its slab (`slab_particle_mask`: the reference's node window [c - f, c + f] with
  f = ceil(r / h) and the cyclic wrap, ParticlesToDensity.cpp:562-603), computes only its slab from them (the
  library's slab_z0 / slab_z1: tiles of the slab's planes only), and the global statistics travel in three
  scalar all-reduces (FP64 sum, min, max) before the min-max normalisation of ParticlesToDensity.cpp:676-682 is
  applied with the global values (`normalize_slab`).
* AO of one large frame across slabs (`run_slab_ao`): the cones reach a large fraction of the box (0.8 of it by
  default), far beyond any halo, so the normalised slabs are all-gathered into the whole grid on every rank (the
  replicated pyramid base: every rank builds the same mip levels from it), and each rank marches the cones of the
  particles it owns (those whose node plane falls in its slab) against that grid (`p2v_run_ao_on_grid`).
* `aggregate_volume` is the MPIVolumeAggregator equivalent (MPIVolumeAggregator.cpp:60-170): an all-reduce of
  the whole volume with MAX, MIN, SUM or PROD, then the global min / max of the first component computed the
  way the module does (per-rank chunks, `max` starting at 0).

The compute step is a callable, so the same host logic runs with the GPU library on GPU ranks and with the
CPU oracle in the gloo tests."""
from __future__ import annotations

import math
from typing import Callable, Sequence

import numpy as np


def shard_frames(weights: Sequence[float], world_size: int, rank: int) -> list[int]:
    """Indices of the frames rank `rank` computes: frames sorted by weight (particle count plus grid
    work), each dealt to the currently least-loaded rank; ties go to the lower rank and the lower index, so
    every rank derives the same assignment without communication. Returned in ascending frame order."""
    order = sorted(range(len(weights)), key=lambda i: (-float(weights[i]), i))
    load = [0.0] * world_size
    mine = []
    for i in order:
        r = min(range(world_size), key=lambda k: (load[k], k))
        load[r] += float(weights[i])
        if r == rank:
            mine.append(i)
    return sorted(mine)


def slab_ranges(nz: int, world_size: int) -> list[tuple[int, int]]:
    """Contiguous node ranges [z0, z1) along z, as equal as possible (the first nz % world_size slabs one
    node thicker)."""
    base, extra = divmod(nz, world_size)
    out, z = [], 0
    for r in range(world_size):
        t = base + (1 if r < extra else 0)
        out.append((z, z + t))
        z += t
    return out


def slab_particle_mask(xyzr: np.ndarray, bbox, res, cyclic_z: bool, z0: int, z1: int,
                       support_scale: float = 1.0) -> np.ndarray:
    """Particles whose node window along z reaches nodes [z0, z1). The window is the reference's
    [c - f, c + f] with c = trunc((z - min) / h) and f = ceil(support_scale * r / h) in float
    (ParticlesToDensity.cpp:562-575; support_scale = 1 for the reference's bump rbf, 3 * sigma for the 3-sigma
    Gaussian), wrapped modulo the node count on a cyclic axis. A particle kept by a slab it does not reach
    only costs work; a particle dropped from a slab it reaches would change the result, so the test is
    conservative: one extra node on each side."""
    x = np.asarray(xyzr, np.float32).reshape(-1, 4)
    nz = int(res[2])
    lo, hi = np.float32(bbox[2]), np.float32(bbox[5])
    h = np.float32(abs(hi - lo)) / np.float32(nz - 1)
    with np.errstate(invalid="ignore", over="ignore"):
        q = (x[:, 2] - lo) / h
        c = np.trunc(np.where(np.isfinite(q), q, 0.0)).astype(np.int64)
        f = np.ceil(np.float32(support_scale) * x[:, 3] / h)
        f = np.where(np.isfinite(f), f, 0).astype(np.int64) + 1
    a, b = c - f, c + f  # inclusive node window
    if not cyclic_z:
        return (b >= z0) & (a < z1)
    # cyclic: the window covers (b - a + 1) consecutive nodes modulo nz
    width = b - a + 1
    full = width >= nz
    s = np.mod(a, nz)
    e = s + width  # exclusive end in unwrapped coordinates, s in [0, nz)
    hit = ((s < z1) & (e > z0)) | ((s < z1 + nz) & (e > z0 + nz))
    return full | hit


def normalize_slab(slab, vmin: float, vmax: float):
    """ParticlesToDensity.cpp:676-682 with global extrema: (v - min) * (1 / (max - min)) in float32."""
    rcp = np.float32(1.0) / (np.float32(vmax) - np.float32(vmin))
    if isinstance(slab, np.ndarray):
        return ((slab.astype(np.float32) - np.float32(vmin)) * rcp).astype(np.float32)
    import torch

    return (slab - torch.tensor(np.float32(vmin), device=slab.device)) * torch.tensor(rcp, device=slab.device)


def _allreduce_scalar(value: float, op: str, dtype, group=None) -> float:
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.tensor([value], dtype=dtype, device=dev)
    dist.all_reduce(t, op={"sum": dist.ReduceOp.SUM, "min": dist.ReduceOp.MIN, "max": dist.ReduceOp.MAX}[op],
                    group=group)
    return float(t.item())


def run_slab(compute: Callable[[np.ndarray, int, int], np.ndarray], xyzr: np.ndarray, bbox, res, cyclic_z: bool,
             rank: int, world_size: int, normalize: bool = True, support_scale: float = 1.0, group=None):
    """This rank's slab of one large frame. `compute(particles, z0, z1)` returns grid planes [z0, z1) (z, y, x; not
    normalised) computed from a particle subset; the slab's nodes receive exactly the contributions they receive
    from the whole frame. Returns (slab, (z0, z1), global min, global max, global FP64 sum)."""
    import torch  # noqa: F401  (the collectives below)

    z0, z1 = slab_ranges(int(res[2]), world_size)[rank]
    keep = slab_particle_mask(xyzr, bbox, res, cyclic_z, z0, z1, support_scale)
    slab = np.ascontiguousarray(compute(np.ascontiguousarray(np.asarray(xyzr, np.float32).reshape(-1, 4)[keep]), z0, z1))
    lmin = float(slab.min()) if slab.size else math.inf
    lmax = float(slab.max()) if slab.size else -math.inf
    lsum = float(slab.astype(np.float64).sum())
    import torch as _t

    gmin = _allreduce_scalar(lmin, "min", _t.float32, group)
    gmax = _allreduce_scalar(lmax, "max", _t.float32, group)
    gsum = _allreduce_scalar(lsum, "sum", _t.float64, group)
    if normalize:
        slab = normalize_slab(slab, gmin, gmax)
    return slab, (z0, z1), gmin, gmax, gsum


def owned_particles(xyzr: np.ndarray, bbox, res, z0: int, z1: int) -> np.ndarray:
    """Mask of the particles a slab rank owns for AO: those whose nearest node plane round((z - min) / h), clamped
    into the grid, lies in [z0, z1). Every particle has exactly one owner."""
    x = np.asarray(xyzr, np.float32).reshape(-1, 4)
    nz = int(res[2])
    lo, hi = np.float32(bbox[2]), np.float32(bbox[5])
    h = np.float32(abs(hi - lo)) / np.float32(nz - 1)
    with np.errstate(invalid="ignore", over="ignore"):
        q = np.floor((x[:, 2] - lo) / h + np.float32(0.5))
    k = np.clip(np.where(np.isfinite(q), q, 0), 0, nz - 1).astype(np.int64)
    return (k >= z0) & (k < z1)


def run_slab_ao(compute: Callable[[np.ndarray, int, int], np.ndarray],
                ao_on_grid: Callable[[np.ndarray, np.ndarray], np.ndarray], xyzr: np.ndarray, bbox, res,
                cyclic_z: bool, rank: int, world_size: int, support_scale: float = 1.0, group=None):
    """Density and AO of one large frame across z-slab ranks. The density slabs come from `run_slab` (normalised
    with the global extrema); an all-gather assembles the whole normalised grid on every rank; then
    `ao_on_grid(particles, grid)` returns the AO of this rank's owned particles (`owned_particles`) against the
    whole grid. Returns (slab, (z0, z1), AO of the owned particles, owned mask)."""
    import torch
    import torch.distributed as dist

    slab, (z0, z1), _, _, _ = run_slab(compute, xyzr, bbox, res, cyclic_z, rank, world_size, True, support_scale,
                                       group)
    ranges = slab_ranges(int(res[2]), world_size)
    plane = int(res[0]) * int(res[1])
    thick = max(b - a for a, b in ranges)
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    mine = torch.zeros(thick * plane, dtype=torch.float32, device=dev)
    mine[: slab.size] = torch.from_numpy(np.ascontiguousarray(slab, np.float32).reshape(-1)).to(dev)
    parts = [torch.empty_like(mine) for _ in range(world_size)]
    dist.all_gather(parts, mine, group=group)
    grid = np.concatenate([parts[r][: (b - a) * plane].cpu().numpy() for r, (a, b) in enumerate(ranges)])
    grid = grid.reshape(int(res[2]), int(res[1]), int(res[0]))
    own = owned_particles(xyzr, bbox, res, z0, z1)
    ao = ao_on_grid(np.ascontiguousarray(np.asarray(xyzr, np.float32).reshape(-1, 4)[own]), grid)
    return slab, (z0, z1), np.asarray(ao, np.float32), own


def p2v_slab_compute(ctx, bbox, res, **params):
    """A `compute` for run_slab on a GPU rank: the library's density of planes [z0, z1) (slab_z0 / slab_z1) from
    the given particles, not normalised (the slab ranks normalise with the global extrema)."""
    from megamol_gb300 import p2v

    def compute(particles, z0, z1):
        ctx.set_params(sizex=int(res[0]), sizey=int(res[1]), sizez=int(res[2]), normalize=0, ao_mode=p2v.AO_NONE,
                       slab_z0=int(z0), slab_z1=int(z1), **params)
        out = np.empty(int(res[0]) * int(res[1]) * (int(z1) - int(z0)), np.float32)
        ctx.run_frame([p2v.ParticleList(particles, p2v.VERTDATA_FLOAT_XYZR)], bbox, out)
        ctx.set_params(slab_z0=0, slab_z1=0)
        return out.reshape(int(z1) - int(z0), int(res[1]), int(res[0]))

    return compute


def p2v_ao_on_grid(ctx, bbox, **ao_params):
    """An `ao_on_grid` for run_slab_ao on a GPU rank: the library's AO of the given particles against the
    gathered whole grid (p2v_run_ao_on_grid), normals down that grid's gradient unless ao_params say otherwise."""
    from megamol_gb300 import p2v

    def ao_on_grid(particles, grid):
        ctx.set_params(sizex=grid.shape[2], sizey=grid.shape[1], sizez=grid.shape[0], normalize=1,
                       **dict(dict(ao_normals=p2v.NORMALS_GRADIENT), **ao_params))
        ao = np.full(particles.shape[0], np.nan, np.float32)
        ctx.run_ao_on_grid([p2v.ParticleList(particles, p2v.VERTDATA_FLOAT_XYZR, ao_out=ao)], bbox,
                           np.ascontiguousarray(grid, np.float32).reshape(-1))
        return ao

    return ao_on_grid


def aggregate_volume(volume, components: int = 1, op: str = "sum", group=None):
    """MPIVolumeAggregator on torch.distributed: all-reduce the volume with op in {max, min, sum, prod}
    (MPIVolumeAggregator.cpp:97-124), then the global min / max of the first component: each rank scans its
    chunk of numFloats / size + 1 values with stride `components`, starting from min = FLT_MAX and max = 0
    (:133-150), and the two extrema are all-reduced. `volume` is a float32 torch tensor (CPU for gloo, CUDA
    for NCCL); returns (aggregated volume, global min, global max)."""
    import torch
    import torch.distributed as dist

    ops = {"max": dist.ReduceOp.MAX, "min": dist.ReduceOp.MIN, "sum": dist.ReduceOp.SUM,
           "prod": dist.ReduceOp.PRODUCT}
    if op not in ops:
        raise ValueError(f"unknown operation {op}")
    out = volume.detach().clone().contiguous().view(-1)
    dist.all_reduce(out, op=ops[op], group=group)
    size, rank = dist.get_world_size(group), dist.get_rank(group)
    n = out.numel()
    chunk = n // size + 1
    beg, end = rank * chunk, min((rank + 1) * chunk, n)
    part = out[beg:end:components] if beg < end else out[:0]
    lmin = float(part.min().item()) if part.numel() else float(np.finfo(np.float32).max)
    lmax = max(float(part.max().item()), 0.0) if part.numel() else 0.0
    lmin = min(lmin, float(np.finfo(np.float32).max))
    gmin = _allreduce_scalar(lmin, "min", torch.float32, group)
    gmax = _allreduce_scalar(lmax, "max", torch.float32, group)
    return out.view_as(volume), gmin, gmax
