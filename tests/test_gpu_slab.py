"""The library's z-slab output and its AO against a supplied grid on the GPU, the two pieces the multi-rank
sharding of one large frame runs on every rank:

* slab_z0 / slab_z1: the planes [z0, z1) of a frame's grid, computed by tiles of those planes only, equal the
  same planes of the whole grid bit for bit (both accumulation modes), with the slab's metadata;
* p2v_run_ao_on_grid: the AO of a frame's particles against a supplied grid equals the AO p2v_run_frame computes
  from the frame's own grid, and the AO of a particle subset against the whole grid equals the whole frame's AO
  of those particles (the cone march and the gradient normals read only the grid);
* sharding.run_slab_ao with the GPU compute steps (one rank, gloo): the same grid and AO as one p2v_run_frame."""
import os
import socket

import numpy as np
import pytest

from megamol_gb300 import build as nbuild
from megamol_gb300 import p2v, sharding, synth

pytestmark = pytest.mark.gpu

AO = dict(ao_mode=p2v.AO_CONE, ao_volume=p2v.AOVOL_DENSITY, ao_volume_scale=1.0, ao_cones=8, ao_steps=32,
          ao_levels=3, ao_apex_deg=50.0, ao_offset=0.01, ao_strength=1.0, ao_cone_length=0.8, ao_early_exit=1,
          ao_normals=p2v.NORMALS_GRADIENT)


@pytest.fixture(scope="module")
def ctx():
    nbuild.build()
    c = p2v.Context(0)
    yield c
    c.close()


def grid_of(ctx, f, **params):
    ctx.set_params(**{"sizex": f.res[0], "sizey": f.res[1], "sizez": f.res[2], "normalize": 0,
                      "ao_mode": p2v.AO_NONE, "slab_z0": 0, "slab_z1": 0, **params})
    out = np.empty(f.res[0] * f.res[1] * f.res[2], np.float32)
    meta = ctx.run_frame([p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR)], f.bbox, out)
    return out.reshape(f.res[2], f.res[1], f.res[0]), meta


@pytest.mark.parametrize("accumulate", [p2v.ACCUM_EXACT, p2v.ACCUM_KAHAN])
def test_slab_planes_equal_the_whole_grid(ctx, accumulate):
    f = synth.lj_liquid(cells=20, res=50, seed=61)
    full, meta = grid_of(ctx, f, accumulate=accumulate)
    for z0, z1 in ((0, 13), (13, 37), (37, 50), (5, 6)):
        ctx.set_params(slab_z0=z0, slab_z1=z1)
        out = np.empty(f.res[0] * f.res[1] * (z1 - z0), np.float32)
        m = ctx.run_frame([p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR)], f.bbox, out)
        assert np.array_equal(out.reshape(z1 - z0, f.res[1], f.res[0]), full[z0:z1]), (z0, z1)
        assert m["resolution"] == [f.res[0], f.res[1], z1 - z0]
        assert m["origin"][2] == np.float32(f.bbox[2]) + np.float32(z0) * np.float32(meta["slice_dists"][2])
        assert m["max_value"] == full[z0:z1].max()
    ctx.set_params(slab_z0=0, slab_z1=0, accumulate=p2v.ACCUM_EXACT)


def test_ao_on_a_supplied_grid(ctx):
    f = synth.lj_liquid(cells=20, res=48, seed=62)
    grid, _ = grid_of(ctx, f, normalize=1)
    ctx.set_params(normalize=1, **AO)
    own = np.full(f.n, np.nan, np.float32)
    ctx.run_frame([p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR, ao_out=own)], f.bbox)
    sup = np.full(f.n, np.nan, np.float32)
    ctx.run_ao_on_grid([p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR, ao_out=sup)], f.bbox, grid.reshape(-1))
    assert np.array_equal(own, sup)
    sub = np.arange(0, f.n, 3)
    part = np.full(sub.size, np.nan, np.float32)
    ctx.run_ao_on_grid([p2v.ParticleList(np.ascontiguousarray(f.xyzr[sub]), p2v.VERTDATA_FLOAT_XYZR, ao_out=part)],
                       f.bbox, grid.reshape(-1))
    assert np.array_equal(part, own[sub])
    ctx.set_params(ao_mode=p2v.AO_NONE)


def test_run_slab_ao_one_rank_gloo(ctx):
    import torch.distributed as dist

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=0, world_size=1)
    try:
        f = synth.lj_liquid(cells=20, res=48, seed=63)
        compute = sharding.p2v_slab_compute(ctx, f.bbox, f.res, kernel=p2v.KERNEL_BUMP, sigma=1.0)
        ao_fn = sharding.p2v_ao_on_grid(ctx, f.bbox, **{k: v for k, v in AO.items()})
        slab, (z0, z1), ao, own = sharding.run_slab_ao(compute, ao_fn, f.xyzr, f.bbox, f.res, True, 0, 1)
    finally:
        dist.destroy_process_group()
    assert (z0, z1) == (0, f.res[2]) and own.all()
    grid, _ = grid_of(ctx, f, normalize=1)
    assert np.array_equal(slab, grid)
    ctx.set_params(normalize=1, **AO)
    ref = np.full(f.n, np.nan, np.float32)
    ctx.run_frame([p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR, ao_out=ref)], f.bbox)
    assert np.array_equal(ao, ref)
    ctx.set_params(ao_mode=p2v.AO_NONE)
