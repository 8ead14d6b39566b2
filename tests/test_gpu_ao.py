"""GPU tests of the AO stage through the C ABI, against the FP64 oracle restatement of the reference's
GLSL (MDAO cone march, AOSphereRenderer taps). The density grid the GPU produced is handed to the oracle,
so these tests isolate the AO arithmetic.

Bars: cone march RMS error <= 1e-5 and max error <= 2e-3 (the reference's early exit at 0.99 is a
discontinuity: a sample that sits on the threshold in one precision and not the other changes the cone's
occlusion by at most (1 - 0.99) times one sample); AOSphere max error <= 1e-5."""
import os

import numpy as np
import pytest

import oracle
from megamol_gb300 import build as nbuild
from megamol_gb300 import p2v, synth

pytestmark = pytest.mark.gpu
NT = os.cpu_count() or 1


@pytest.fixture(scope="module")
def ctx():
    nbuild.build()
    c = p2v.Context(0)
    yield c
    c.close()


def frame(n=30_000, edge=30.0, res=40, seed=21):
    f = synth.uniform(n=n, edge=edge, res=res, seed=seed)
    f.xyzr[:, 3] = np.random.default_rng(seed).uniform(0.4, 0.8, f.n).astype(np.float32)
    return f


def run_ao(ctx, f, normals, **params):
    # every parameter is set on each call: the context is shared by the tests of this module
    base = dict(sizex=f.res[0], sizey=f.res[1], sizez=f.res[2], normalize=1, sigma=1.0, cyclX=1, cyclY=1, cyclZ=1,
                accumulate=p2v.ACCUM_EXACT, forSurfaceReconstruction=0, mass_normalize=0, kernel=p2v.KERNEL_BUMP,
                ao_volume=p2v.AOVOL_DENSITY, ao_volume_scale=1.0, ao_cones=3, ao_steps=0, ao_levels=0,
                ao_apex_deg=50.0, ao_offset=0.01, ao_strength=1.0, ao_cone_length=0.8, ao_early_exit=1,
                aos_deposit=p2v.AOS_DEPOSIT_CPU, aos_clip=0, aos_clip_plane=[0.0] * 4, ao_normals=p2v.NORMALS_LIST,
                ao_march=p2v.AO_MARCH_THREAD, ao_brick_order=0)
    base.update(params)
    ctx.set_params(**base)
    ao = np.full(f.n, np.nan, np.float32)
    vol = np.empty(f.res[0] * f.res[1] * f.res[2], np.float32)
    L = p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR, normals=np.ascontiguousarray(normals), ao_out=ao)
    meta = ctx.run_frame([L], f.bbox, vol)
    return ao, vol.reshape(f.res[2], f.res[1], f.res[0]), meta


def cone_oracle(f, vol, normals, cones, steps, levels, apex=50.0, offset=0.01, strength=1.0, cone_length=0.8,
                scale=1.0, early_exit=1):
    h = oracle.spacing_f64(f.bbox, f.res)
    bmin = [f.bbox[a] - 0.5 * h[a] for a in range(3)]
    bsize = [f.res[a] * h[a] for a in range(3)]
    lv = oracle.mip_chain_f64(vol, levels, scale)
    dirs = oracle.cone_dirs(cones, np.deg2rad(np.float32(apex)))
    return oracle.cone_ao_f64(lv, dirs, f.xyzr, normals, bmin, bsize, offset=offset, strength=strength,
                              cone_length=cone_length, shortest_edge=float(min(f.res)), max_lod=float(levels - 1),
                              steps=steps, early_exit=early_exit, border=0, sat_scale=scale)


@pytest.mark.parametrize("cones,steps,levels", [(3, 0, 6), (8, 32, 3), (8, 16, 4)])
def test_cone_ao_vs_fp64(ctx, cones, steps, levels):
    f = frame()
    nrm = synth.random_normals(f.n, 5)
    ao, vol, _ = run_ao(ctx, f, nrm, ao_mode=p2v.AO_CONE, ao_cones=cones, ao_steps=steps, ao_levels=levels)
    ref = cone_oracle(f, vol, nrm, cones, steps, levels)
    d = np.abs(ao.astype(np.float64) - ref)
    assert np.isfinite(ao).all()
    assert np.sqrt(np.mean(d ** 2)) <= 1e-5, np.sqrt(np.mean(d ** 2))
    assert d.max() <= 2e-3, d.max()
    assert 0.0 <= ao.min() and ao.max() <= 1.0


def test_cone_ao_no_early_exit_is_smooth(ctx):
    """Without the early exit the march has no discontinuity: max error is at float rounding level."""
    f = frame(n=10_000, seed=22)
    nrm = synth.random_normals(f.n, 6)
    ao, vol, _ = run_ao(ctx, f, nrm, ao_mode=p2v.AO_CONE, ao_cones=8, ao_steps=32, ao_levels=3, ao_early_exit=0)
    ref = cone_oracle(f, vol, nrm, 8, 32, 3, early_exit=0)
    assert np.abs(ao - ref).max() <= 2e-5


def test_cone_ao_empty_volume_is_unoccluded(ctx):
    f = frame(n=2000, seed=23)
    nrm = synth.random_normals(f.n, 7)
    ao, vol, _ = run_ao(ctx, f, nrm, ao_mode=p2v.AO_CONE, ao_cones=3, ao_volume_scale=1e-30, normalize=0)
    assert np.allclose(ao, 1.0, atol=1e-6)


def test_zero_normal_means_no_occlusion(ctx):
    f = frame(n=5000, seed=24)
    nrm = synth.random_normals(f.n, 8)
    nrm[::7] = 0.0
    ao, _, _ = run_ao(ctx, f, nrm, ao_mode=p2v.AO_CONE, ao_cones=3)
    assert np.all(ao[::7] == 1.0)


@pytest.mark.parametrize("mode", [p2v.AO_AOSPHERE_AXES, p2v.AO_AOSPHERE_NORMAL])
def test_aosphere_vs_fp64(ctx, mode):
    f = frame(n=20_000, seed=25)
    nrm = synth.random_normals(f.n, 9)
    s = (24, 20, 28)
    ao, _, _ = run_ao(ctx, f, nrm, ao_mode=mode, aos_sizex=s[0], aos_sizey=s[1], aos_sizez=s[2], aos_step_len=0.5,
                      aos_gen_fac=1.0, aos_eval_fac=1.0)
    tex = oracle.aosphere_volume_f64(f.xyzr, f.bbox, s, 1.0)
    ref = oracle.aosphere_ao_f64(tex, f.bbox, f.xyzr, nrm, 0 if mode == p2v.AO_AOSPHERE_AXES else 1, 0.5, 1.0)
    d = np.abs(ao.astype(np.float64) - ref)
    assert d.max() <= 1e-5 * max(1.0, np.abs(ref).max()), d.max()


@pytest.mark.parametrize("mode", [p2v.AO_AOSPHERE_AXES, p2v.AO_AOSPHERE_NORMAL])
@pytest.mark.parametrize("rule, plane", [(p2v.AOS_DEPOSIT_GLSL, None), (p2v.AOS_DEPOSIT_CPU, "oblique"),
                                         (p2v.AOS_DEPOSIT_CPU, "unset")])
def test_aosphere_deposit_rules_vs_fp64(ctx, mode, rule, plane):
    """The two deposit rules of AOSphereRenderer against the FP64 restatement: createVolumeGLSL's (the point's
    pixel: floor clamped to [0, s_inner] in x and y, the host's z slice + 1) and createVolumeCPU's with the
    ao::clipData discard, for an oblique plane through the box centre and for the renderer's plane when no
    clip plane is connected (all zeros: dot - d = 0 >= 0 drops every particle, so the volume stays empty and
    AO is 1, up to the rounding of the normal's squared length)."""
    f = frame(n=20_000, seed=26)
    nrm = synth.random_normals(f.n, 10)
    s = (22, 26, 18)
    cp = None
    if plane == "oblique":
        nv = np.array([0.3, -0.5, 0.81], np.float32)
        nv /= np.linalg.norm(nv)
        ctr = 0.5 * (np.array(f.bbox[:3], np.float32) + np.array(f.bbox[3:], np.float32))
        cp = [float(nv[0]), float(nv[1]), float(nv[2]), float(np.dot(ctr, nv))]
    elif plane == "unset":
        cp = [0.0, 0.0, 0.0, 0.0]
    ao, _, _ = run_ao(ctx, f, nrm, ao_mode=mode, aos_sizex=s[0], aos_sizey=s[1], aos_sizez=s[2], aos_step_len=0.5,
                      aos_gen_fac=1.0, aos_eval_fac=1.0, aos_deposit=rule, aos_clip=int(cp is not None),
                      aos_clip_plane=cp if cp is not None else [0.0] * 4)
    tex = oracle.aosphere_volume_f64(f.xyzr, f.bbox, s, 1.0, glsl_rule=rule, clip_plane=cp)
    ref = oracle.aosphere_ao_f64(tex, f.bbox, f.xyzr, nrm, 0 if mode == p2v.AO_AOSPHERE_AXES else 1, 0.5, 1.0)
    d = np.abs(ao.astype(np.float64) - ref)
    assert d.max() <= 1e-5 * max(1.0, np.abs(ref).max()), d.max()
    if plane == "unset":
        assert np.all(tex == 0) and np.abs(ao - 1.0).max() <= 1e-6  # |n|^2 = 1 up to rounding
    else:
        assert tex.sum() > 0


@pytest.mark.parametrize("mode", [p2v.AO_CONE, p2v.AO_AOSPHERE_AXES])
def test_library_gradient_normals_match_host_normals(ctx, mode):
    """P2V_NORMALS_GRADIENT computes each particle's normal on the device from the frame's density grid (-grad rho,
    central differences, periodic on cyclic axes, trilinear at the particle). The AO it gives equals the AO of
    the same normals computed on the host (synth.gradient_normals, FP64) and passed as list normals: the cone
    march runs without early exit, so the difference is the normals' rounding only."""
    f = synth.lj_liquid(cells=20, res=48, seed=33)
    ctx.set_params(sizex=48, sizey=48, sizez=48, normalize=1, ao_mode=p2v.AO_NONE, ao_normals=p2v.NORMALS_LIST)
    vol = np.empty(48 ** 3, np.float32)
    ctx.run_frame([p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR)], f.bbox, vol)
    nrm = synth.gradient_normals(f.xyzr, vol.reshape(48, 48, 48), f.bbox)
    extra = dict(ao_cones=8, ao_steps=32, ao_levels=3, ao_early_exit=0) if mode == p2v.AO_CONE else \
        dict(aos_sizex=20, aos_sizey=20, aos_sizez=20)
    host, _, _ = run_ao(ctx, f, nrm, ao_mode=mode, ao_normals=p2v.NORMALS_LIST, **extra)
    ctx.set_params(ao_normals=p2v.NORMALS_GRADIENT)
    ao = np.full(f.n, np.nan, np.float32)
    ctx.run_frame([p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR, ao_out=ao)], f.bbox)  # no list normals
    ctx.set_params(ao_normals=p2v.NORMALS_LIST)
    d = np.abs(ao.astype(np.float64) - host)
    assert np.isfinite(ao).all()
    assert np.sqrt(np.mean(d ** 2)) <= 1e-5 and d.max() <= 1e-3, (np.sqrt(np.mean(d ** 2)), d.max())


def test_gradient_normals_ao_pipeline_lj_small(ctx):
    """A small LJ-liquid frame with gradient normals (the headline workload's normal definition)."""
    f = synth.lj_liquid(cells=24, res=64, seed=31)
    ctx.set_params(sizex=64, sizey=64, sizez=64, normalize=1, ao_mode=p2v.AO_NONE)
    vol = np.empty(64 ** 3, np.float32)
    ctx.run_frame([p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR)], f.bbox, vol)
    nrm = synth.gradient_normals(f.xyzr, vol.reshape(64, 64, 64), f.bbox)
    ao, vol2, _ = run_ao(ctx, f, nrm, ao_mode=p2v.AO_CONE, ao_cones=8, ao_steps=32, ao_levels=3)
    assert np.array_equal(vol2.reshape(-1), vol)
    ref = cone_oracle(f, vol2, nrm, 8, 32, 3)
    d = np.abs(ao - ref)
    assert np.sqrt(np.mean(d ** 2)) <= 1e-5 and d.max() <= 2e-3


@pytest.mark.parametrize("early_exit,steps", [(1, 32), (0, 32), (1, 0), (1, 40)])
def test_warp_march_equals_thread_march(ctx, early_exit, steps):
    """P2V_AO_MARCH_WARP (one warp per cone of a particle, its lanes taking the steps 32 at a time, the march's
    recurrence replayed over the shuffled samples) gives the bits of the thread-per-particle march, with and
    without early exit, with the step table of the reference's growth rule (steps 0) and with more than 32
    steps (two rounds of lanes)."""
    f = synth.lj_liquid(cells=20, res=48, seed=36)
    nrm = synth.random_normals(f.n, 37)
    nrm[::97] = 0.0  # particles without a normal: AO 1
    kw = dict(ao_cones=8, ao_steps=steps, ao_levels=3, ao_early_exit=early_exit, ao_mode=p2v.AO_CONE)
    a, _, _ = run_ao(ctx, f, nrm, ao_march=p2v.AO_MARCH_THREAD, **kw)
    b, _, _ = run_ao(ctx, f, nrm, ao_march=p2v.AO_MARCH_WARP, **kw)
    assert np.array_equal(a, b)
    assert (b[::97] == 1.0).all()


@pytest.mark.parametrize("march", [p2v.AO_MARCH_THREAD, p2v.AO_MARCH_WARP])
def test_brick_order_gives_the_same_bits(ctx, march):
    """ao_brick_order: the cone march takes the sorted particles in brick-major order (bricks of 16 x 4 x 4
    cells: a stable reordering of the cell order's row segments); every particle's AO keeps its bits. The
    frame's 66^3 cells leave partial bricks along every axis."""
    f = synth.lj_liquid(cells=24, res=64, seed=38)
    nrm = synth.random_normals(f.n, 39)
    kw = dict(ao_cones=8, ao_steps=32, ao_levels=3, ao_mode=p2v.AO_CONE, ao_march=march)
    a, _, _ = run_ao(ctx, f, nrm, ao_brick_order=0, **kw)
    b, _, _ = run_ao(ctx, f, nrm, ao_brick_order=1, **kw)
    assert np.array_equal(a, b)
    c, _, _ = run_ao(ctx, f, nrm, ao_brick_order=1, ao_normals=p2v.NORMALS_GRADIENT, **kw)
    d, _, _ = run_ao(ctx, f, nrm, ao_brick_order=0, ao_normals=p2v.NORMALS_GRADIENT, **kw)
    assert np.array_equal(c, d)
