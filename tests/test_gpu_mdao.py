"""GPU tests of the MDAO occupancy volume and of the cone march over it, through the C ABI.

The voxeliser evaluates the fragment shader's FP32 arithmetic with explicitly rounded operations and sums
integer blend contributions, so its volume must equal the oracle's FP32 restatement bit for bit, in both
storage modes. The R8 mip chain is integer arithmetic and must match exactly too. The cone march over the
MDAO pyramid is compared with the FP64 cone march of the oracle on the same pyramid, with the bars of the
density-volume cone tests (RMS <= 1e-5, max <= 2e-3)."""
import numpy as np
import pytest

import oracle
from megamol_gb300 import build as nbuild
from megamol_gb300 import p2v, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    nbuild.build()
    c = p2v.Context(0)
    yield c
    c.close()


def frame(n=20_000, edge=40.0, seed=31):
    f = synth.uniform(n=n, edge=edge, res=48, seed=seed)
    f.xyzr[:, 3] = np.random.default_rng(seed).uniform(0.3, 1.6, f.n).astype(np.float32)
    return f


def run(ctx, f, nrm, clip=None, **params):
    base = dict(sizex=f.res[0], sizey=f.res[1], sizez=f.res[2], normalize=1, sigma=1.0, cyclX=1, cyclY=1, cyclZ=1,
                accumulate=p2v.ACCUM_EXACT, forSurfaceReconstruction=0, mass_normalize=0, kernel=p2v.KERNEL_BUMP,
                ao_mode=p2v.AO_CONE, ao_volume=p2v.AOVOL_MDAO, ao_volume_scale=1.0, ao_cones=3, ao_steps=0,
                ao_levels=0, ao_apex_deg=50.0, ao_offset=0.01, ao_strength=1.0, ao_cone_length=0.8,
                ao_early_exit=1, mdao_volume_size=64, mdao_unorm8=1)
    base.update(params)
    ctx.set_params(**base)
    ao = np.full(f.n, np.nan, np.float32)
    vol = np.empty(f.res[0] * f.res[1] * f.res[2], np.float32)
    L = p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR, normals=np.ascontiguousarray(nrm), ao_out=ao)
    ctx.run_frame([L], f.bbox, vol, clipbox=clip)
    return ao


@pytest.mark.parametrize("unorm8", [1, 0])
@pytest.mark.parametrize("vs,clip", [(64, None), (50, (3.0, -2.0, 5.0, 33.0, 38.0, 22.0))])
def test_mdao_volume_bit_exact(ctx, unorm8, vs, clip):
    f = frame()
    nrm = synth.random_normals(f.n, 3)
    run(ctx, f, nrm, clip=clip, mdao_volume_size=vs, mdao_unorm8=unorm8)
    cb = f.bbox if clip is None else clip
    dims, _, _ = oracle.mdao_dims(cb, vs)
    got = ctx.ao_volume(0)
    assert got.shape == (dims[2], dims[1], dims[0])
    ref = oracle.mdao_volume_f32(f.xyzr, cb, dims, unorm8=bool(unorm8))
    assert ref.any()
    mism = np.flatnonzero(got.ravel() != ref.ravel())
    assert mism.size == 0, (mism.size, mism[:5], got.ravel()[mism[:5]], ref.ravel()[mism[:5]])


def test_mdao_mips_r8_exact(ctx):
    f = frame(seed=32)
    nrm = synth.random_normals(f.n, 4)
    run(ctx, f, nrm, mdao_volume_size=60, mdao_unorm8=1, ao_levels=4)
    lv = ctx.ao_volume(0)
    for level in range(1, 4):
        lv = oracle.mdao_mip_u8(lv)
        got = ctx.ao_volume(level)
        assert got.shape == lv.shape and np.array_equal(got, lv), level


@pytest.mark.parametrize("unorm8,cones,steps", [(1, 3, 0), (0, 8, 32)])
def test_cone_ao_over_mdao_vs_fp64(ctx, unorm8, cones, steps):
    f = frame(seed=33)
    nrm = synth.random_normals(f.n, 5)
    ao = run(ctx, f, nrm, mdao_volume_size=64, mdao_unorm8=unorm8, ao_cones=cones, ao_steps=steps)
    dims, shortest, max_lod = oracle.mdao_dims(f.bbox, 64)
    L = int(max_lod) + 1
    levels = [ctx.ao_volume(level).astype(np.float64) for level in range(L)]
    size = [f.bbox[a + 3] - f.bbox[a] for a in range(3)]
    dirs = oracle.cone_dirs(cones, np.deg2rad(np.float32(50.0)))
    ref = oracle.cone_ao_f64(levels, dirs, f.xyzr, nrm, f.bbox[:3], size, offset=0.01, strength=1.0,
                             cone_length=0.8, shortest_edge=shortest, max_lod=max_lod, steps=steps, early_exit=1,
                             border=0, sat_scale=0.0)
    d = np.abs(ao.astype(np.float64) - ref)
    assert np.isfinite(ao).all() and 0.0 <= ao.min() and ao.max() <= 1.0
    assert np.sqrt(np.mean(d ** 2)) <= 1e-5, np.sqrt(np.mean(d ** 2))
    assert d.max() <= 2e-3, d.max()
    assert ao.min() < 0.9  # the volume occludes something


def test_mdao_empty_frame(ctx):
    f = frame(n=0, seed=34)
    ao = run(ctx, f, np.zeros((0, 3), np.float32))
    assert ao.size == 0
    assert not ctx.ao_volume(0).any()
