"""Multi-rank sharding on CPU: world_size-2 gloo process groups (spawned processes, 127.0.0.1) with the CPU
oracle as each rank's compute step. Frame sharding must reproduce every frame exactly once; the z-slab
decomposition of one frame must reproduce the single-process grid bit for bit (FP32 restatement, one
thread, particle order kept); the volume aggregation must match numpy's reductions and the reference's
min / max rule."""
import os
import socket
import tempfile

import numpy as np
import pytest

import oracle
from megamol_gb300 import sharding, synth


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def spawn(fn, nprocs, *args):
    import torch.multiprocessing as mp

    port = free_port()
    with tempfile.TemporaryDirectory() as d:
        mp.spawn(_entry, args=(nprocs, port, d, fn) + args, nprocs=nprocs, join=True)
        return [dict(np.load(os.path.join(d, f"rank{r}.npz"), allow_pickle=True)) for r in range(nprocs)]


def _entry(rank, world, port, outdir, fn, *args):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        res = fn(rank, world, *args)
        np.savez(os.path.join(outdir, f"rank{rank}.npz"), **res)
    finally:
        dist.destroy_process_group()


# ---- workers (module level: spawned processes import them) ----
def small_frames(k=6, seed=11):
    out = []
    for i, f in enumerate(synth.trajectory(frames=k, nmin=1_000, nmax=8_000, seed=seed)):
        res = (24 + 4 * i, 24 + 2 * i, 20 + 3 * i)
        out.append((f, res))
    return out


def frame_worker(rank, world):
    frames = small_frames()
    weights = [f.n + 0.25 * np.prod(res) for f, res in frames]
    mine = sharding.shard_frames(weights, world, rank)
    out = {"mine": np.array(mine, np.int64)}
    for i in mine:
        f, res = frames[i]
        out[f"grid{i}"] = oracle.density_f32(f.xyzr, f.bbox, res, nthreads=1)
    return out


def slab_worker(rank, world, cyclic, kernel, sigma):
    rng = np.random.default_rng(21)
    n = 6000
    x = np.empty((n, 4), np.float32)
    x[:, :3] = rng.uniform(0.0, 30.0, (n, 3))
    x[:, 3] = rng.uniform(0.5, 1.6, n)
    x[::50, 2] = rng.uniform(-3.0, 0.5, x[::50].shape[0])   # near and beyond the lower z face
    bbox, res = (0.0, 0.0, 0.0, 30.0, 30.0, 30.0), (28, 26, 31)
    cyc = (1, 1, 1) if cyclic else (0, 0, 0)
    compute = lambda p, z0, z1: oracle.density_f32(p, bbox, res, cyclic=cyc, sigma=sigma, kernel=kernel,
                                                   nthreads=1)[z0:z1]
    scale = 1.0 if kernel == oracle.BUMP else 3.0 * sigma
    slab, (z0, z1), gmin, gmax, gsum = sharding.run_slab(compute, x, bbox, res, bool(cyclic), rank, world,
                                                         normalize=True, support_scale=scale)
    return {"slab": slab, "z": np.array([z0, z1]), "stats": np.array([gmin, gmax, gsum])}


AO_KW = dict(offset=0.01, strength=1.0, cone_length=0.8, steps=32, early_exit=1, border=0, sat_scale=1.0)


def _ao_frame():
    rng = np.random.default_rng(31)
    n = 5000
    x = np.empty((n, 4), np.float32)
    x[:, :3] = rng.uniform(0.0, 30.0, (n, 3))
    x[:, 3] = rng.uniform(0.5, 1.2, n)
    return x, (0.0, 0.0, 0.0, 30.0, 30.0, 30.0), (24, 22, 26)


def _oracle_ao_on_grid(bbox, res):
    def ao_on_grid(particles, grid):
        h = oracle.spacing_f64(bbox, res)
        bmin = [bbox[a] - 0.5 * h[a] for a in range(3)]
        bsize = [res[a] * h[a] for a in range(3)]
        nrm = oracle.gradient_normals_f32(grid, bbox, res, particles)
        lv = oracle.mip_chain_f64(grid, 3, 1.0)
        dirs = oracle.cone_dirs(8, np.deg2rad(np.float32(50.0)))
        return oracle.cone_ao_f64(lv, dirs, particles, nrm, bmin, bsize, shortest_edge=float(min(res)), max_lod=2.0,
                                  **AO_KW)
    return ao_on_grid


def slab_ao_worker(rank, world):
    x, bbox, res = _ao_frame()
    compute = lambda p, z0, z1: oracle.density_f32(p, bbox, res, nthreads=1)[z0:z1]
    slab, (z0, z1), ao, own = sharding.run_slab_ao(compute, _oracle_ao_on_grid(bbox, res), x, bbox, res, True, rank,
                                                   world)
    return {"slab": slab, "ao": ao, "own": own}


def aggregate_worker(rank, world, op, comp):
    import torch

    rng = np.random.default_rng(100 + rank)
    v = rng.uniform(-0.5, 2.0, 7 * 5 * 3 * comp).astype(np.float32)
    out, gmin, gmax = sharding.aggregate_volume(torch.from_numpy(v), components=comp, op=op)
    return {"out": out.numpy(), "mm": np.array([gmin, gmax], np.float64)}


# ---- tests ----
def test_shard_frames_is_a_partition_and_balanced():
    w = [5.0, 1.0, 9.0, 3.0, 3.0, 7.0, 2.0]
    parts = [sharding.shard_frames(w, 3, r) for r in range(3)]
    assert sorted(sum(parts, [])) == list(range(len(w)))
    loads = [sum(w[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(w)
    assert parts == [sharding.shard_frames(w, 3, r) for r in range(3)]  # deterministic


def test_slab_ranges_cover_the_grid():
    for nz, ws in [(31, 2), (256, 8), (7, 3), (3, 4)]:
        r = sharding.slab_ranges(nz, ws)
        assert r[0][0] == 0 and r[-1][1] == nz
        assert all(a[1] == b[0] for a, b in zip(r, r[1:]))
        assert max(b - a for a, b in r) - min(b - a for a, b in r) <= 1


def test_frame_sharding_gloo():
    frames = small_frames()
    res = spawn(frame_worker, 2)
    seen = sorted(list(res[0]["mine"]) + list(res[1]["mine"]))
    assert seen == list(range(len(frames)))
    for r in res:
        for i in r["mine"]:
            f, rs = frames[int(i)]
            ref = oracle.density_f32(f.xyzr, f.bbox, rs, nthreads=1)
            assert np.array_equal(r[f"grid{int(i)}"], ref)


@pytest.mark.parametrize("cyclic,kernel,sigma", [(True, oracle.BUMP, 1.0), (False, oracle.BUMP, 1.0),
                                                  (True, oracle.GAUSS3, 0.7)])
def test_slab_decomposition_gloo(cyclic, kernel, sigma):
    res = spawn(slab_worker, 2, cyclic, kernel, sigma)
    # single-process reference with the same inputs
    rng = np.random.default_rng(21)
    n = 6000
    x = np.empty((n, 4), np.float32)
    x[:, :3] = rng.uniform(0.0, 30.0, (n, 3))
    x[:, 3] = rng.uniform(0.5, 1.6, n)
    x[::50, 2] = rng.uniform(-3.0, 0.5, x[::50].shape[0])
    cyc = (1, 1, 1) if cyclic else (0, 0, 0)
    full = oracle.density_f32(x, (0.0, 0.0, 0.0, 30.0, 30.0, 30.0), (28, 26, 31), cyclic=cyc, sigma=sigma,
                              kernel=kernel, nthreads=1)
    norm, mn, mx = oracle.normalize_minmax_f32(full)
    got = np.concatenate([r["slab"] for r in res], axis=0)
    assert [tuple(r["z"]) for r in res] == sharding.slab_ranges(31, 2)
    assert np.array_equal(got, norm.reshape(full.shape))
    for r in res:
        assert r["stats"][0] == mn and r["stats"][1] == mx
        assert abs(r["stats"][2] - full.astype(np.float64).sum()) <= 1e-9 * abs(full.astype(np.float64).sum())


def test_slab_ao_gloo():
    """AO across z-slab ranks: the gathered grid equals the single-process normalised grid, every particle has one
    owner, and the owners' AO (cone march over the gathered grid, normals down its gradient) equals the
    single-process AO of every particle bit for bit."""
    res_ranks = spawn(slab_ao_worker, 2)
    x, bbox, res = _ao_frame()
    full = oracle.density_f32(x, bbox, res, nthreads=1)
    norm, _, _ = oracle.normalize_minmax_f32(full)
    grid = norm.reshape(full.shape)
    ref = _oracle_ao_on_grid(bbox, res)(x, grid)
    owners = np.stack([r["own"] for r in res_ranks])
    assert np.all(owners.sum(0) == 1)
    assert np.array_equal(np.concatenate([r["slab"] for r in res_ranks], 0), grid)
    got = np.full(x.shape[0], np.nan)
    for r in res_ranks:
        got[r["own"]] = r["ao"]
    assert np.array_equal(got, ref.astype(np.float32))


@pytest.mark.parametrize("op,comp", [("sum", 1), ("max", 1), ("min", 3), ("prod", 1)])
def test_aggregate_volume_gloo(op, comp):
    res = spawn(aggregate_worker, 2, op, comp)
    vs = [np.random.default_rng(100 + r).uniform(-0.5, 2.0, 7 * 5 * 3 * comp).astype(np.float32) for r in range(2)]
    ref = {"sum": vs[0] + vs[1], "max": np.maximum(vs[0], vs[1]), "min": np.minimum(vs[0], vs[1]),
           "prod": vs[0] * vs[1]}[op]
    for r in res:
        assert np.array_equal(r["out"], ref)
    # MPIVolumeAggregator.cpp:133-150: chunks of n / size + 1 values, stride = components, max starts at 0
    n = ref.size
    chunk = n // 2 + 1
    mins, maxs = [], []
    for rank in range(2):
        part = ref[rank * chunk:min((rank + 1) * chunk, n):comp]
        mins.append(part.min())
        maxs.append(max(part.max(), 0.0))
    assert res[0]["mm"][0] == np.float32(min(mins)) and res[0]["mm"][1] == np.float32(max(maxs))
