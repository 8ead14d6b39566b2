"""CPU checks of the AO restatements in the oracle: the FP32 cone pipeline (the CPU baseline's timing
stand-in) against the FP64 restatement, and known answers of the learned AO's FP64 feature restatement."""
import numpy as np

import oracle
from megamol_gb300 import synth

AO = dict(offset=0.01, strength=1.0, cone_length=0.8, steps=32, border=0)


def _frame():
    f = synth.uniform(n=20_000, edge=30.0, res=40, seed=21)
    vol = oracle.density_f32(f.xyzr, f.bbox, f.res, (1, 1, 1), 1.0, oracle.BUMP, 2)
    vol, _, _ = oracle.normalize_minmax_f32(vol)
    grid = vol.reshape(f.res[2], f.res[1], f.res[0])
    h = oracle.spacing_f64(f.bbox, f.res)
    bmin = [f.bbox[a] - 0.5 * h[a] for a in range(3)]
    bsize = [f.res[a] * h[a] for a in range(3)]
    return f, grid, bmin, bsize


def test_mip_levels_f32_match_fp64():
    _, grid, _, _ = _frame()
    lv32 = oracle.mip_levels_f32(grid, 4, 1.0, nthreads=2)
    lv64 = oracle.mip_chain_f64(grid, 4, 1.0)
    assert np.array_equal(lv32[0], grid)
    for a, b in zip(lv32[1:], lv64[1:]):
        assert a.shape == b.shape
        assert np.abs(a - b).max() <= 1e-6


def test_cone_ao_f32_matches_fp64():
    """Without early exit the march is continuous and the FP32 pipeline differs from FP64 by rounding only;
    with it, a cone that crosses 0.99 one step apart in the two precisions moves its particle's AO, so only
    the RMS is tight."""
    f, grid, bmin, bsize = _frame()
    nrm = synth.random_normals(f.n, 22)
    dirs = oracle.cone_dirs(8, np.deg2rad(np.float32(50.0)))
    idx = np.arange(0, f.n, 7)
    kw = dict(AO, shortest_edge=float(min(f.res)), max_lod=2.0, sat_scale=1.0)
    lv32 = oracle.mip_levels_f32(grid, 3, 1.0, nthreads=2)
    lv64 = oracle.mip_chain_f64(grid, 3, 1.0)
    for ee, max_bar, rms_bar in ((0, 2e-5, 2e-6), (1, 2e-2, 2e-4)):
        a32 = oracle.cone_ao_f32(lv32, dirs, f.xyzr[idx], nrm[idx], bmin, bsize, nthreads=2, early_exit=ee, **kw)
        a64 = oracle.cone_ao_f64(lv64, dirs, f.xyzr[idx], nrm[idx], bmin, bsize, early_exit=ee, **kw)
        e = np.abs(a32.astype(np.float64) - a64)
        assert e.max() <= max_bar and np.sqrt(np.mean(e ** 2)) <= rms_bar, (ee, e.max(), np.sqrt(np.mean(e ** 2)))


def test_cone_features_known_answers():
    """Every cone sample of a constant volume c reads c wherever the 2x2x2 texel block lies inside the volume
    (at every level: the /8 mip of an interior block of c is c), and 0 in an empty volume; the last six
    features are the unit normal and the surface point in normalised coordinates."""
    c = 0.37
    levels = [np.full((32, 32, 32), c), np.full((16, 16, 16), c), np.full((8, 8, 8), c)]
    dirs = oracle.cone_dirs(8, np.deg2rad(np.float32(50.0)))
    t, lod = oracle.cone_steps(float(dirs[0, 3]), offset=0.01, cone_length=0.1, shortest_edge=32.0, max_lod=2.0,
                               steps=32)
    xyzr = np.array([[16.0, 16.0, 16.0, 0.5], [10.0, 20.0, 12.0, 0.25]], np.float32)
    nrm = np.array([[0.0, 0.0, 2.0], [1.0, 1.0, 0.0]], np.float32)
    x = oracle.cone_features_f64(levels, dirs, t, lod, xyzr, nrm, (0.0, 0.0, 0.0), (1 / 32, 1 / 32, 1 / 32))
    ns = 8 * oracle.MLP_FSTEPS
    assert x.shape == (2, ns + 6)
    assert np.allclose(x[:, :ns], c, atol=1e-12)
    n = nrm / np.linalg.norm(nrm, axis=1, keepdims=True)
    assert np.allclose(x[:, ns:ns + 3], n)
    assert np.allclose(x[:, ns + 3:], (xyzr[:, :3] + xyzr[:, 3:] * n) / 32)
    z = oracle.cone_features_f64([L * 0 for L in levels], dirs, t, lod, xyzr, nrm, (0, 0, 0), (1 / 32,) * 3)
    assert np.all(z[:, :ns] == 0)
    assert oracle.mlp_feature_steps(32) == [0, 6, 12, 19, 25, 31]
    assert oracle.mlp_feature_steps(32, 9) == [0, 4, 8, 12, 16, 19, 23, 27, 31]


def test_gradient_normals_f32_match_host_normals():
    """The FP32 restatement of the library's gradient normals (the CPU baseline's normals stage) against the
    host's FP64 normals of the workloads (synth.gradient_normals): the same unit vectors up to rounding."""
    f = synth.lj_liquid(cells=20, res=48, seed=33)
    vol = oracle.density_f32(f.xyzr, f.bbox, f.res, (1, 1, 1), 1.0, oracle.BUMP, 2)
    vol, _, _ = oracle.normalize_minmax_f32(vol)
    g = vol.reshape(48, 48, 48)
    a = oracle.gradient_normals_f32(g, f.bbox, f.res, f.xyzr, nthreads=2)
    b = synth.gradient_normals(f.xyzr, g, f.bbox)
    assert np.abs(np.linalg.norm(a, axis=1) - 1).max() <= 1e-5
    assert np.abs(a - b).max() <= 1e-3 and np.sqrt(np.mean((a - b) ** 2)) <= 1e-5
