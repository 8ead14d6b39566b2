"""GPU tests of batched frames (p2v_run_batch, p2v_autotune_batch) through the C ABI.

A batch must give every frame exactly the results p2v_run_frame gives it (the exact accumulation is
order-independent), whether the frames run on one lane or several, eagerly or as a replayed CUDA graph,
and whatever lane count the autotuner picks (with the tile it picks)."""
import numpy as np
import pytest

from megamol_gb300 import build as nbuild
from megamol_gb300 import p2v, synth

pytestmark = pytest.mark.gpu

AO = dict(ao_mode=p2v.AO_CONE, ao_volume=p2v.AOVOL_DENSITY, ao_volume_scale=1.0, ao_cones=3, ao_steps=0,
          ao_levels=3, ao_early_exit=1)


@pytest.fixture(scope="module")
def ctx():
    nbuild.build()
    c = p2v.Context(0)
    yield c
    c.close()


def small_trajectory(k=6, seed=40):
    frames = synth.trajectory(frames=k, nmin=5_000, nmax=60_000, seed=seed)
    out = []
    for i, f in enumerate(frames):
        size = tuple(min(r, 48 + 8 * i) for r in f.res)  # uneven grids
        nrm = synth.random_normals(f.n, seed + i)
        out.append((f, size, nrm))
    return out


def reference(ctx, traj, with_ao):
    refs = []
    for f, size, nrm in traj:
        ctx.set_params(sizex=size[0], sizey=size[1], sizez=size[2], **(AO if with_ao else dict(ao_mode=p2v.AO_NONE)))
        vol = np.empty(size[0] * size[1] * size[2], np.float32)
        ao = np.full(f.n, np.nan, np.float32)
        L = p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR, normals=nrm if with_ao else None,
                             ao_out=ao if with_ao else None)
        meta = ctx.run_frame([L], f.bbox, vol)
        refs.append((vol, ao, meta))
    return refs


def batch_frames(traj, with_ao):
    frames, outs = [], []
    for f, size, nrm in traj:
        vol = np.full(size[0] * size[1] * size[2], np.nan, np.float32)
        ao = np.full(f.n, np.nan, np.float32)
        L = p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR, normals=nrm if with_ao else None,
                             ao_out=ao if with_ao else None)
        frames.append(dict(lists=[L], bbox=f.bbox, out=vol, size=size))
        outs.append((vol, ao))
    return frames, outs


@pytest.mark.parametrize("lanes,with_ao", [(1, False), (3, False), (4, True)])
def test_batch_equals_run_frame(ctx, lanes, with_ao):
    traj = small_trajectory()
    refs = reference(ctx, traj, with_ao)
    ctx.set_params(batch_lanes=lanes, batch_graph=1, **(AO if with_ao else dict(ao_mode=p2v.AO_NONE)))
    frames, outs = batch_frames(traj, with_ao)
    meta, stats = ctx.run_batch(frames)
    for k, ((vol, ao), (rvol, rao, rmeta)) in enumerate(zip(outs, refs)):
        assert np.array_equal(vol, rvol), k
        assert meta[k]["resolution"] == rmeta["resolution"]
        assert meta[k]["min_value"] == rmeta["min_value"] and meta[k]["max_value"] == rmeta["max_value"]
        assert stats[k]["particles_in"] == traj[k][0].n
        if with_ao:
            assert np.array_equal(ao, rao), k
    assert ctx.stats()["ms_total"] > 0.0


def test_graph_replay_follows_new_data(ctx):
    torch = pytest.importorskip("torch")
    traj = small_trajectory(k=5, seed=50)
    ctx.set_params(batch_lanes=2, batch_graph=1, ao_mode=p2v.AO_NONE)
    dev_in = [torch.from_numpy(f.xyzr.copy()).cuda() for f, _, _ in traj]
    dev_out = [torch.empty(s[0] * s[1] * s[2], dtype=torch.float32, device="cuda") for _, s, _ in traj]
    frames = [dict(lists=[p2v.ParticleList(x, p2v.VERTDATA_FLOAT_XYZR, count=f.n)], bbox=f.bbox, out=o, size=s)
              for x, o, (f, s, _) in zip(dev_in, dev_out, traj)]
    results = []
    for rep in range(3):  # eager (sizes the buffers), captured, replayed
        ctx.run_batch(frames)
        torch.cuda.synchronize()
        results.append([o.cpu().numpy().copy() for o in dev_out])
    for r in results[1:]:
        for a, b in zip(results[0], r):
            assert np.array_equal(a, b)
    # new particle data in the same buffers: the replayed graph computes the new frames
    for x in dev_in:
        x[:, :3] += 0.37
    ctx.run_batch(frames)
    torch.cuda.synchronize()
    for k, (f, size, _) in enumerate(traj):
        ctx.set_params(sizex=size[0], sizey=size[1], sizez=size[2])
        moved = f.xyzr.copy()
        moved[:, :3] += np.float32(0.37)
        vol = np.empty(size[0] * size[1] * size[2], np.float32)
        ctx.run_frame([p2v.ParticleList(moved, p2v.VERTDATA_FLOAT_XYZR)], f.bbox, vol)
        assert np.array_equal(dev_out[k].cpu().numpy(), vol), k


def test_autotune_picks_a_measured_configuration(ctx):
    traj = small_trajectory(k=4, seed=60)
    ctx.set_params(batch_lanes=0, tile_x=0, tile_y=0, tile_z=0, ao_mode=p2v.AO_NONE)
    frames, outs = batch_frames(traj, False)
    rep = ctx.autotune_batch(frames)
    # the eager frames use the tuned tile as well (a tile boundary that cuts a footprint moves the node
    # offsets' rounding, so other tiles may differ in the last bits)
    refs = reference(ctx, traj, False)
    assert len(rep["candidates"]) == 12
    assert rep["lanes"] in (1, 2, 4, 8)
    assert any(c["tile"] == rep["tile"] and c["lanes"] == rep["lanes"] for c in rep["candidates"])
    assert rep["ms_best"] == min(c["ms"] for c in rep["candidates"])
    ctx.run_batch(frames)
    for (vol, _), (rvol, _, _) in zip(outs, refs):
        assert np.array_equal(vol, rvol)


def test_autotune_chooses_the_batch_ao_form(ctx):
    """With the cone march on the density the autotuner also times both batch AO forms (the persistent launch
    and the lanes' own kernels): 24 candidates; batch_persistent = -1 then follows its choice, and either form
    gives the bits of p2v_run_frame."""
    traj = small_trajectory(k=5, seed=61)
    params = dict(AO, ao_normals=p2v.NORMALS_GRADIENT)
    ctx.set_params(batch_lanes=0, tile_x=0, tile_y=0, tile_z=0, batch_persistent=-1, **params)
    frames, outs = batch_frames(traj, True)
    rep = ctx.autotune_batch(frames)
    assert len(rep["candidates"]) == 24
    assert {c["persistent"] for c in rep["candidates"]} == {0, 1}
    assert rep["persistent"] in (0, 1)
    assert rep["ms_best"] == min(c["ms"] for c in rep["candidates"])
    refs = reference_with(ctx, traj, params)
    ctx.set_params(batch_lanes=0, tile_x=0, tile_y=0, tile_z=0, batch_persistent=-1, **params)
    ctx.run_batch(frames)
    for k, ((vol, ao), (rvol, rao)) in enumerate(zip(outs, refs)):
        assert np.array_equal(vol, rvol), k
        assert np.array_equal(ao, rao), k
    ctx.set_params(ao_normals=p2v.NORMALS_LIST, ao_mode=p2v.AO_NONE)


def test_empty_and_single_frame_batches(ctx):
    ctx.set_params(batch_lanes=4, ao_mode=p2v.AO_NONE)
    meta, stats = ctx.run_batch([])
    assert meta == []
    traj = small_trajectory(k=1, seed=70)
    refs = reference(ctx, traj, False)
    frames, outs = batch_frames(traj, False)
    ctx.run_batch(frames)
    assert np.array_equal(outs[0][0], refs[0][0])


def reference_with(ctx, traj, params):
    refs = []
    for f, size, nrm in traj:
        ctx.set_params(sizex=size[0], sizey=size[1], sizez=size[2], **params)
        vol = np.empty(size[0] * size[1] * size[2], np.float32)
        ao = np.full(f.n, np.nan, np.float32)
        ctx.run_frame([p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR, normals=nrm, ao_out=ao)], f.bbox, vol)
        refs.append((vol, ao))
    return refs


@pytest.mark.parametrize("normals", [p2v.NORMALS_LIST, p2v.NORMALS_GRADIENT])
@pytest.mark.parametrize("graph", [0, 1])
def test_persistent_batch_ao_equals_run_frame(ctx, normals, graph):
    """The persistent batch AO launch (every frame's mip levels and cone march taken from one device-side work
    queue after the lanes) gives every frame the grid and AO bits of p2v_run_frame, with list normals and with
    normals down the density gradient, eagerly and (graph) captured and replayed. ao_levels = 0: the whole
    pyramid, so every frame's march waits on a chain of five to seven levels."""
    traj = small_trajectory(k=7, seed=45)
    params = dict(AO, ao_levels=0, ao_normals=normals)
    refs = reference_with(ctx, traj, params)
    ctx.set_params(batch_lanes=3, batch_graph=graph, batch_persistent=1, **params)
    frames, outs = batch_frames(traj, True)
    for rep in range(3):  # eager; then (graph) captured; replayed
        for vol, ao in outs:
            vol.fill(np.nan)
            ao.fill(np.nan)
        ctx.run_batch(frames)
        for k, ((vol, ao), (rvol, rao)) in enumerate(zip(outs, refs)):
            assert np.array_equal(vol, rvol), (rep, k)
            assert np.array_equal(ao, rao), (rep, k)
    ctx.set_params(ao_normals=p2v.NORMALS_LIST, ao_levels=3)


def test_persistent_and_lane_batches_agree_with_device_buffers(ctx):
    """Device-resident lists and volumes (the volume doubles as the AO stage's level 0): the persistent launch
    and the lanes' own AO kernels give the same bits."""
    torch = pytest.importorskip("torch")
    traj = small_trajectory(k=5, seed=46)
    params = dict(AO, ao_normals=p2v.NORMALS_GRADIENT)
    res = {}
    for pers in (0, 1):
        ctx.set_params(batch_lanes=2, batch_graph=1, batch_persistent=pers, **params)
        frames, outs = [], []
        for f, size, _ in traj:
            d_in = torch.from_numpy(f.xyzr).cuda()
            d_ao = torch.full((f.n,), float("nan"), device="cuda")
            d_vol = torch.full((size[0] * size[1] * size[2],), float("nan"), device="cuda")
            frames.append(dict(lists=[p2v.ParticleList(d_in, p2v.VERTDATA_FLOAT_XYZR, count=f.n, ao_out=d_ao)],
                               bbox=f.bbox, out=d_vol, size=size))
            outs.append((d_vol, d_ao))
        for _ in range(3):
            ctx.run_batch(frames)
        torch.cuda.synchronize()
        res[pers] = [(v.cpu().numpy(), a.cpu().numpy()) for v, a in outs]
    for k, ((v0, a0), (v1, a1)) in enumerate(zip(res[0], res[1])):
        assert np.array_equal(v0, v1), k
        assert np.array_equal(a0, a1), k
        assert not np.isnan(a1).any(), k
    ctx.set_params(ao_normals=p2v.NORMALS_LIST)


def test_queue_wait_runs_out_and_the_context_survives(ctx):
    """The batch AO queue's bounded dependency wait: with the test hook the first mip level never reports its
    completion, so the items that need it poll queue_wait_polls times, record the timeout and stop the queue.
    p2v_run_batch reports P2V_ETIMEOUT; the next batch on the same context runs normally and gives the bits of
    p2v_run_frame."""
    traj = small_trajectory(k=4, seed=47)
    params = dict(AO, ao_levels=0)
    ctx.set_params(batch_lanes=2, batch_graph=0, batch_persistent=1, queue_wait_polls=2000, test_hold_queue=1,
                   **params)
    frames, _ = batch_frames(traj, True)
    with pytest.raises(p2v.P2VError) as err:
        ctx.run_batch(frames)
    assert err.value.status == p2v.ETIMEOUT
    ctx.set_params(queue_wait_polls=0, test_hold_queue=0)
    refs = reference_with(ctx, traj, params)
    ctx.set_params(batch_lanes=2, batch_graph=0, batch_persistent=1, **params)
    frames, outs = batch_frames(traj, True)
    ctx.run_batch(frames)
    for k, ((vol, ao), (rvol, rao)) in enumerate(zip(outs, refs)):
        assert np.array_equal(vol, rvol), k
        assert np.array_equal(ao, rao), k
    ctx.set_params(ao_levels=3)
