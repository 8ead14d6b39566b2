"""GPU tests of the learned AO: the training kernels' gradients against the FP64 CPU MLP, the BF16
tensor-core inference against the FP64 forward, training on cone-march pairs, the cone-march fallback
outside the training range, save/load, and what the network gains over the plain cone march."""
import os
import time

import numpy as np
import pytest

import oracle
from megamol_gb300 import build as nbuild
from megamol_gb300 import p2v, synth

pytestmark = pytest.mark.gpu

AO = dict(ao_volume=p2v.AOVOL_DENSITY, ao_volume_scale=1.0, ao_cones=8, ao_steps=32, ao_levels=3, ao_apex_deg=50.0,
          ao_offset=0.01, ao_strength=1.0, ao_cone_length=0.8, ao_early_exit=1)


@pytest.fixture(scope="module")
def ctx():
    nbuild.build()
    c = p2v.Context(0)
    yield c
    c.close()


def random_params(seed=0, scale=0.2):
    rng = np.random.default_rng(seed)
    return rng.normal(0.0, scale, p2v.MLP_PARAMS).astype(np.float32)


def test_gradients_match_fp64(ctx):
    rng = np.random.default_rng(1)
    w = random_params(1)
    ctx.mlp_set_weights(w)
    x = rng.uniform(0, 1, (96, p2v.MLP_INPUTS)).astype(np.float32)
    x[:, p2v.MLP_INPUTS - 6:p2v.MLP_INPUTS - 3] = synth.random_normals(96, 2)
    t = rng.uniform(0, 1, 96).astype(np.float32)
    g, loss = ctx.mlp_gradients(x, t)
    l64, _, g64 = oracle.mlp_f64(w.astype(np.float64), x, t)
    assert abs(loss - l64) <= 1e-5 * max(1.0, l64)
    rel = np.abs(g - g64).max() / np.abs(g64).max()
    assert rel <= 1e-4, rel


def test_tensor_core_inference_matches_fp64(ctx):
    rng = np.random.default_rng(3)
    w = random_params(3, 0.15)
    ctx.mlp_set_weights(w)
    x = rng.uniform(0, 1, (1000, p2v.MLP_INPUTS)).astype(np.float32)
    x[:, p2v.MLP_INPUTS - 6:p2v.MLP_INPUTS - 3] = synth.random_normals(1000, 4)
    y = ctx.mlp_infer(x)
    _, y64, _ = oracle.mlp_f64(w.astype(np.float64), x, None, grads=False)
    # BF16 weights and features (8 mantissa bits), FP32 accumulation
    assert np.abs(y - y64).max() <= 1.5e-2, np.abs(y - y64).max()
    assert np.sqrt(np.mean((y - y64) ** 2)) <= 3e-3


def set_ao(ctx, f, mode, normalize=1, kernel=p2v.KERNEL_BUMP, **over):
    ctx.set_params(sizex=f.res[0], sizey=f.res[1], sizez=f.res[2], normalize=normalize, sigma=1.0, cyclX=1, cyclY=1,
                   cyclZ=1, accumulate=p2v.ACCUM_EXACT, forSurfaceReconstruction=0, mass_normalize=0,
                   kernel=kernel, ao_mode=mode, **dict(AO, **over))


def with_normals(ctx, f, kernel=p2v.KERNEL_BUMP):
    set_ao(ctx, f, p2v.AO_NONE, kernel=kernel)
    vol = np.empty(f.res[0] * f.res[1] * f.res[2], np.float32)
    ctx.run_frame([p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR)], f.bbox, vol)
    return synth.gradient_normals(f.xyzr, vol.reshape(f.res[2], f.res[1], f.res[0]), f.bbox)


def ao_of(ctx, f, nrm, mode, **over):
    set_ao(ctx, f, mode, **over)
    ao = np.full(f.n, np.nan, np.float32)
    ctx.run_frame([p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR, normals=nrm, ao_out=ao)], f.bbox)
    return ao


@pytest.fixture(scope="module")
def trained(ctx):
    """Train on two small LJ-liquid frames (cone-march pairs); the tests infer on frames of other seeds."""
    ctx.mlp_clear()
    total = 0
    for seed in (41, 42):
        f = synth.lj_liquid(cells=32, res=80, seed=seed)
        nrm = with_normals(ctx, f)
        set_ao(ctx, f, p2v.AO_CONE)
        total = ctx.mlp_collect([p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR, normals=nrm)], f.bbox, 120_000,
                                seed)
    rep = ctx.mlp_train(epochs=16, batch=2048, lr=3e-3, lr_decay=0.8, seed=7)
    return total, rep


def test_training_converges(trained):
    total, rep = trained
    assert total >= 200_000
    assert rep["pairs_val"] > 0 and rep["steps"] > 0
    assert rep["val_rmse"] <= 0.02, rep


def test_learned_ao_matches_cone_march_and_is_faster(ctx, trained):
    """On a frame the network never saw: AO RMSE <= 0.02 against the plain cone march (the accuracy bar),
    well below the constant predictor's, and an AO stage faster than the march it replaces."""
    f = synth.lj_liquid(cells=32, res=80, seed=43)
    nrm = with_normals(ctx, f)
    plain = ao_of(ctx, f, nrm, p2v.AO_CONE)
    learned = ao_of(ctx, f, nrm, p2v.AO_LEARNED)
    st = ctx.stats()
    rmse = float(np.sqrt(np.mean((learned - plain) ** 2)))
    base = float(np.sqrt(np.mean((plain.mean() - plain) ** 2)))  # the constant predictor
    assert np.isfinite(learned).all()
    assert rmse <= 0.02, (rmse, st["ao_fallback"])
    assert rmse < 0.5 * base, (rmse, base)
    # AO stage time: the network against the cone march it replaces
    t_plain = min(_ao_ms(ctx, f, nrm, p2v.AO_CONE) for _ in range(3))
    t_learn = min(_ao_ms(ctx, f, nrm, p2v.AO_LEARNED) for _ in range(3))
    assert t_learn < t_plain, (t_learn, t_plain)


def _ao_ms(ctx, f, nrm, mode):
    set_ao(ctx, f, mode)
    ao = np.empty(f.n, np.float32)
    ctx.run_frame([p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR, normals=nrm, ao_out=ao)], f.bbox)
    return ctx.stats()["ms_ao"]


def test_fallback_outside_training_range_is_the_cone_march(ctx, trained):
    """With a 10x density-to-occlusion scale the liquid's texels saturate, so its cone samples lie above the
    training range (scale 1): those particles take the cone march, and their AO equals the plain cone march
    bit for bit."""
    f = synth.lj_liquid(cells=32, res=80, seed=44)
    nrm = with_normals(ctx, f)
    plain = ao_of(ctx, f, nrm, p2v.AO_CONE, ao_volume_scale=10.0)
    learned = ao_of(ctx, f, nrm, p2v.AO_LEARNED, ao_volume_scale=10.0)
    nfb = ctx.stats()["ao_fallback"]
    assert nfb > 0
    same = np.sum(learned == plain)
    assert same >= nfb


def test_mma_wait_runs_out_and_the_context_survives(ctx, trained):
    """The tensor-core kernel's bounded completion wait: with the test hook its first MMA is never issued, so its
    mbarrier gets no arrival; after mma_wait_polls polls every CTA records the timeout, frees its TMEM and
    returns. p2v_run_frame reports P2V_ETIMEOUT, and the next frame on the same context runs normally and gives
    the bits of a frame before the timeout."""
    f = synth.lj_liquid(cells=16, res=40, seed=45)
    nrm = with_normals(ctx, f)
    before = ao_of(ctx, f, nrm, p2v.AO_LEARNED)
    set_ao(ctx, f, p2v.AO_LEARNED, mma_wait_polls=64, test_hold_mma=1)
    ao = np.empty(f.n, np.float32)
    with pytest.raises(p2v.P2VError) as err:
        ctx.run_frame([p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR, normals=nrm, ao_out=ao)], f.bbox)
    assert err.value.status == p2v.ETIMEOUT
    assert ctx.stats()["device_error"] != 0
    ctx.set_params(mma_wait_polls=0, test_hold_mma=0)
    after = ao_of(ctx, f, nrm, p2v.AO_LEARNED)
    assert ctx.stats()["device_error"] == 0
    assert np.array_equal(before, after)


def test_save_load_roundtrip(ctx, trained, tmp_path):
    w = ctx.mlp_get_weights()
    path = str(tmp_path / "ao_mlp.bin")
    ctx.mlp_save(path)
    c2 = p2v.Context(0)
    c2.mlp_load(path)
    assert np.array_equal(c2.mlp_get_weights(), w)
    x = np.random.default_rng(5).uniform(0, 1, (256, p2v.MLP_INPUTS)).astype(np.float32)
    assert np.array_equal(c2.mlp_infer(x), ctx.mlp_infer(x))
    c2.close()


def test_cone_features_vs_fp64():
    """The learned AO's features of every particle (collected through p2v_mlp_collect, in binning order) against
    the FP64 restatement (oracle.cone_features_f64): the AO pyramid as the GPU built it, rounded to the 8-bit
    UNORM texels the texture units read, sampled along each cone of the MDAO frame at the feature steps,
    linear within and between levels; then the unit normal and the surface point in volume coordinates. The
    texture units weight x, y and z with 8-bit fractions, hence the tolerance. The 44^3 grid puts the steps on
    all three levels, with level blends."""
    c = p2v.Context(0)
    try:
        f = synth.uniform(n=30_000, edge=40.0, res=44, seed=9)
        f.xyzr[:, 3] = np.random.default_rng(9).uniform(0.4, 0.8, f.n).astype(np.float32)
        nrm = synth.random_normals(f.n, 10)
        set_ao(c, f, p2v.AO_CONE)
        c.mlp_clear()
        c.mlp_collect([p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR, normals=nrm)], f.bbox, f.n, 0)
        x, t = c.mlp_pairs()
        _, order, _ = c.binning()
        assert x.shape == (f.n, p2v.MLP_INPUTS) and np.all(t >= 0)
        L = AO["ao_levels"]
        levels = [c.ao_volume(l).astype(np.float64) for l in range(L)]
        levels[0] = np.clip(levels[0] * AO["ao_volume_scale"], 0.0, 1.0)
        tex = [np.round(np.clip(lv, 0.0, 1.0) * 255.0) / 255.0 for lv in levels]  # 8-bit UNORM texels
        h = oracle.spacing_f64(f.bbox, f.res)
        bmin = [np.float64(np.float32(f.bbox[a] - 0.5 * h[a])) for a in range(3)]
        ibs = [np.float64(np.float32(1.0 / (f.res[a] * h[a]))) for a in range(3)]
        dirs = oracle.cone_dirs(AO["ao_cones"], np.deg2rad(np.float32(AO["ao_apex_deg"])))
        ts, lods = oracle.cone_steps(float(dirs[0, 3]), offset=AO["ao_offset"], cone_length=AO["ao_cone_length"],
                                     shortest_edge=float(min(f.res)), max_lod=float(L - 1), steps=AO["ao_steps"])
        fl = lods[oracle.mlp_feature_steps(len(ts))]
        assert fl.min() < 1.0 and fl.max() == L - 1 and np.any(fl != np.floor(fl)), fl  # all levels, blends
        ref = oracle.cone_features_f64(tex, dirs, ts, lods, f.xyzr[order], nrm[order], bmin, ibs)
        ns = p2v.MLP_INPUTS - 6
        e = np.abs(x[:, :ns].astype(np.float64) - ref[:, :ns])
        assert np.abs(x[:, ns:ns + 3] - ref[:, ns:ns + 3]).max() <= 1e-6
        assert np.abs(x[:, ns + 3:] - ref[:, ns + 3:]).max() <= 1e-5
        # 8-bit texels and 8-bit filter weights in x, y and z: each axis' weight moves a sample by up to 1/512 of
        # the neighbouring texels' difference
        assert e.max() <= 6e-3, e.max()
        assert np.sqrt(np.mean(e ** 2)) <= 5e-4, np.sqrt(np.mean(e ** 2))
    finally:
        c.close()


def test_learned_ao_uniform_100k_gauss3():
    """The small plain-method workload (100k particles, 128^3, Gaussian 3-sigma kernel): a network trained on
    eight frames of other seeds reaches AO RMSE <= 0.02 against the plain cone march on the seed-1 frame."""
    c = p2v.Context(0)
    try:
        c.mlp_clear()
        for k in range(8):
            f = synth.uniform(n=100_000, seed=101 + k)
            nrm = with_normals(c, f, kernel=p2v.KERNEL_GAUSS3)
            set_ao(c, f, p2v.AO_CONE, kernel=p2v.KERNEL_GAUSS3)
            c.mlp_collect([p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR, normals=nrm)], f.bbox, 100_000,
                          seed=k)
        rep = c.mlp_train(epochs=16, batch=2048, lr=3e-3, lr_decay=0.85, seed=7)
        f = synth.uniform(n=100_000, seed=1)
        nrm = with_normals(c, f, kernel=p2v.KERNEL_GAUSS3)
        plain = ao_of(c, f, nrm, p2v.AO_CONE, kernel=p2v.KERNEL_GAUSS3)
        learned = ao_of(c, f, nrm, p2v.AO_LEARNED, kernel=p2v.KERNEL_GAUSS3)
        rmse = float(np.sqrt(np.mean((learned.astype(np.float64) - plain) ** 2)))
        assert np.isfinite(learned).all()
        assert rmse <= 0.02, (rmse, rep, c.stats()["ao_fallback"])
    finally:
        c.close()


def test_brick_order_gives_the_same_bits(ctx, trained):
    """ao_brick_order: the learned AO (features, tensor-core inference, fallback march) takes the sorted particles
    in brick-major order; every particle's AO keeps its bits."""
    f = synth.lj_liquid(cells=24, res=64, seed=47)
    nrm = with_normals(ctx, f)
    a = ao_of(ctx, f, nrm, p2v.AO_LEARNED, ao_brick_order=0)
    b = ao_of(ctx, f, nrm, p2v.AO_LEARNED, ao_brick_order=1)
    ctx.set_params(ao_brick_order=0)
    assert np.array_equal(a, b)


def test_learned_ao_with_gradient_normals(ctx, trained):
    """P2V_NORMALS_GRADIENT with the learned AO (normals down the density gradient computed by the library,
    also in brick order). Against the same frame with the host's FP64 gradient normals passed as list normals
    the normals differ in their last bits only: the AO agrees to 2e-3 RMS (features rounded to BF16)."""
    f = synth.lj_liquid(cells=24, res=64, seed=48)
    nrm = with_normals(ctx, f)
    a = ao_of(ctx, f, nrm, p2v.AO_LEARNED)
    b = ao_of(ctx, f, None, p2v.AO_LEARNED, ao_normals=p2v.NORMALS_GRADIENT)
    c = ao_of(ctx, f, None, p2v.AO_LEARNED, ao_normals=p2v.NORMALS_GRADIENT, ao_brick_order=1)
    ctx.set_params(ao_normals=p2v.NORMALS_LIST, ao_brick_order=0)
    assert np.isfinite(b).all()
    assert np.array_equal(b, c)
    d = np.abs(a.astype(np.float64) - b)
    assert np.sqrt(np.mean(d ** 2)) <= 2e-3 and d.max() <= 0.1, (np.sqrt(np.mean(d ** 2)), d.max())


def test_ao_kernel_timing_and_texture_rates(ctx, trained):
    """The frame statistics bracket the AO stage's main kernel alone (the inference, or the plain march) and
    count the inference's texture fetches per particle; the texture-rate probe the benchmark divides by
    reports the units' coherent rate above their incoherent one."""
    f = synth.lj_liquid(cells=32, res=80, seed=43)
    nrm = with_normals(ctx, f)
    ao_of(ctx, f, nrm, p2v.AO_LEARNED)
    st = ctx.stats()
    per_sample = st["ao_fetches"] / p2v.MLP_CONES
    assert st["ao_fetches"] % p2v.MLP_CONES == 0 and p2v.MLP_FSTEPS <= per_sample <= 2 * p2v.MLP_FSTEPS, st
    assert 0.0 < st["ms_ao_kernel"] <= st["ms_ao"], st
    ao_of(ctx, f, nrm, p2v.AO_CONE)
    st = ctx.stats()
    assert st["ao_fetches"] == 0 and 0.0 < st["ms_ao_kernel"] <= st["ms_ao"], st
    coherent, incoherent = p2v.measure_texture_rate(0), p2v.measure_texture_rate(1)
    assert coherent > incoherent > 0.0, (coherent, incoherent)
