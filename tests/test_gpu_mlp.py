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
    x[:, 128:] = synth.random_normals(96, 2)
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
    x[:, 128:] = synth.random_normals(1000, 4)
    y = ctx.mlp_infer(x)
    _, y64, _ = oracle.mlp_f64(w.astype(np.float64), x, None, grads=False)
    # BF16 weights and features (8 mantissa bits), FP32 accumulation
    assert np.abs(y - y64).max() <= 1.5e-2, np.abs(y - y64).max()
    assert np.sqrt(np.mean((y - y64) ** 2)) <= 3e-3


def set_ao(ctx, f, mode, normalize=1, **over):
    ctx.set_params(sizex=f.res[0], sizey=f.res[1], sizez=f.res[2], normalize=normalize, sigma=1.0, cyclX=1, cyclY=1,
                   cyclZ=1, accumulate=p2v.ACCUM_EXACT, forSurfaceReconstruction=0, mass_normalize=0,
                   kernel=p2v.KERNEL_BUMP, ao_mode=mode, **dict(AO, **over))


def with_normals(ctx, f):
    set_ao(ctx, f, p2v.AO_NONE)
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
    """Train on two small LJ-liquid frames (cone-march pairs), like the headline model at smaller size."""
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
    assert rep["val_rmse"] <= 0.03, rep


def test_learned_ao_matches_cone_march_and_is_faster(ctx, trained):
    f = synth.lj_liquid(cells=32, res=80, seed=43)
    nrm = with_normals(ctx, f)
    plain = ao_of(ctx, f, nrm, p2v.AO_CONE)
    learned = ao_of(ctx, f, nrm, p2v.AO_LEARNED)
    st = ctx.stats()
    rmse = float(np.sqrt(np.mean((learned - plain) ** 2)))
    base = float(np.sqrt(np.mean((plain.mean() - plain) ** 2)))  # the constant predictor
    assert np.isfinite(learned).all()
    assert rmse <= 0.03, (rmse, st["ao_fallback"])
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
    """With a 10x density-to-occlusion scale the liquid's texels saturate, so its stencils lie above the
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
