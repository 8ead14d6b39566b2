"""CPU tests of the oracle itself: the FP32 restatement must reproduce the reference module's golden
outputs bit for bit, and the FP64 restatement must agree with them within the reference's own float error."""
import numpy as np
import pytest

import oracle
from tests import golden_io as G

NAMES = G.golden_names()


def test_golden_fixtures_present():
    assert len(NAMES) >= 7


@pytest.mark.parametrize("name", NAMES)
def test_restatement_f32_bitexact_vs_reference_golden(name):
    c = G.load(name)
    xyzr = G.case_xyzr(c)
    bbox, res = G.grid(c)
    v = oracle.density_f32(xyzr, bbox, res, c["cyclic"], float(c["sigma"]), oracle.BUMP, nthreads=1)
    v, mn, mx = oracle.normalize_minmax_f32(v, apply=bool(c["normalize"]))
    assert np.array_equal(v, c["volume"]), f"max diff {np.abs(v - c['volume']).max()}"
    assert float(np.float32(c["min_value"])) == mn or bool(c["normalize"])


@pytest.mark.parametrize("name", NAMES)
def test_fp64_restatement_close_to_reference_golden(name):
    c = G.load(name)
    xyzr = G.case_xyzr(c)
    bbox, res = G.grid(c)
    v64 = oracle.density_f64(xyzr, bbox, res, c["cyclic"], float(c["sigma"]), oracle.BUMP)
    if bool(c["normalize"]):
        v64, _, _ = oracle.normalize_f64(v64, "minmax")
    ref = c["volume"].astype(np.float64)
    err = np.abs(v64 - ref).max() / max(np.abs(v64).max(), 1e-30)
    # the reference rounds node positions and distances in float; that costs it up to ~1e-5 of the max
    assert err < 2e-5, err


def test_surface_box_adjustment_vs_reference_golden():
    """The restated box adjustment publishes the reference module's grid bit for bit: rewritten sizex /
    sizey, origin, extents and slice distances (ParticlesToDensity.cpp:249-288, 749-799)."""
    c = G.load("surface_box")
    bbox, res = G.grid(c)
    f = np.float32
    assert list(res) == [int(v) for v in c["out_res"]] and list(res) != [int(v) for v in c["res"]]
    for a in range(3):
        ext = abs(f(bbox[a + 3]) - f(bbox[a]))
        assert f(bbox[a]) == c["origin"][a] and ext == c["extents"][a]
        assert ext / f(res[a] - 1) == c["slice_dists"][a]
    assert c["volume"].shape == tuple(res[::-1])


@pytest.mark.skipif(not oracle.reference_available(), reason="reference module build not present")
@pytest.mark.parametrize("seed", range(8))
def test_surface_box_adjustment_vs_live_reference(seed):
    """Random boxes (offsets, flat and tall aspect ratios) and slot resolutions: the restated box adjustment
    publishes the module's resolution, origin, extents and slice distances bit for bit."""
    rng = np.random.default_rng(300 + seed)
    lo = rng.uniform(-50, 50, 3)
    hi = lo + rng.uniform(0.5, 40, 3) * rng.choice([0.2, 1.0, 3.0], 3)
    bbox = tuple(float(v) for v in np.concatenate([lo, hi]).astype(np.float32))
    res = tuple(int(v) for v in rng.integers(6, 40, 3))
    xyz = rng.uniform(lo, hi, (200, 3)).astype(np.float32)
    _, meta = oracle.reference_density([dict(type=1, data=xyz, stride=0, radius=0.3, count=200)], bbox, res,
                                       (0, 0, 0), False, 1.0, surface=True)
    bb, rr = oracle.modify_bbox_f32(bbox, res)
    f = np.float32
    assert list(rr) == meta["resolution"]
    for a in range(3):
        ext = abs(f(bb[a + 3]) - f(bb[a]))
        assert f(bb[a]) == f(meta["origin"][a]) and ext == f(meta["extents"][a])
        assert ext / f(rr[a] - 1) == f(meta["slice_dists"][a])


def test_kat_single_particle_on_node():
    """A particle on node (5,5,5) of a unit grid, r = 1: the bump at d=0 is exp(-1); nodes at distance
    1 lie on the support boundary and get exactly 0 (ParticlesToDensity.cpp:472-476)."""
    c = G.load("kat_two_particles")
    v = c["volume"]
    e1 = np.exp(-1.0)  # libm expf is within 1 ulp of this
    assert abs(float(v[5, 5, 5]) - e1) <= 1e-7
    assert v[5, 5, 6] == 0.0 and v[5, 6, 5] == 0.0
    # the particle at the box minimum wraps onto the far faces with unwrapped distances
    assert v[10, 10, 10] == 0.0 and abs(float(v[0, 0, 0]) - e1) <= 1e-7


def test_zero_radius_contributes_nothing():
    c = G.load("zero_radius")
    xyzr = G.case_xyzr(c)
    keep = xyzr[xyzr[:, 3] > 0]
    v = oracle.density_f32(keep, c["bbox"], c["res"], c["cyclic"], 1.0, oracle.BUMP, 1)
    assert np.array_equal(v, c["volume"])


def test_threaded_restatement_matches_serial_within_rounding():
    c = G.load("uniform_cyclic")
    xyzr = G.case_xyzr(c)
    a = oracle.density_f32(xyzr, c["bbox"], c["res"], c["cyclic"], 1.0, oracle.BUMP, 1)
    b = oracle.density_f32(xyzr, c["bbox"], c["res"], c["cyclic"], 1.0, oracle.BUMP, 4)
    assert np.abs(a - b).max() <= 1e-6 * np.abs(a).max()


@pytest.mark.skipif(not oracle.reference_available(), reason="reference module build not present")
def test_restatement_matches_live_reference_threads():
    rng = np.random.default_rng(5)
    xyz = rng.uniform(0, 20, size=(5000, 3)).astype(np.float32)
    L = [dict(type=1, data=xyz, stride=0, radius=0.55, count=5000)]
    vr, _ = oracle.reference_density(L, (0, 0, 0, 20, 20, 20), (24, 24, 24), (1, 1, 1), False, 1.0)
    xyzr = np.concatenate([xyz, np.full((5000, 1), 0.55, np.float32)], 1)
    import os
    T = int(os.environ.get("OMP_NUM_THREADS", "0")) or os.cpu_count()
    v = oracle.density_f32(xyzr, (0, 0, 0, 20, 20, 20), (24, 24, 24), (1, 1, 1), 1.0, oracle.BUMP, T)
    assert np.array_equal(v, vr)


def test_mip_constant_volume():
    """Mip of a constant c is c inside; dimensions that collapse to 1 are attenuated by the fixed /8
    (mdao_mipmap_compute_main.comp.glsl:16-23)."""
    src = np.full((8, 6, 4), 0.5)
    m1 = oracle.mip_step_f64(src)
    assert m1.shape == (4, 3, 2) and np.allclose(m1, 0.5)
    m2 = oracle.mip_step_f64(m1)  # (2, 1, 1): every output still has 8 children
    assert m2.shape == (2, 1, 1) and np.allclose(m2, 0.5)
    m3 = oracle.mip_step_f64(np.full((4, 1, 2), 0.5))  # y is already 1: only 4 children, still /8
    assert m3.shape == (2, 1, 1) and np.allclose(m3, 0.5 * 4 / 8)


def test_support_misses_nodes_known_answers():
    """The FP64 test of a support holding no grid node (nodes at 0, 1, ..., 10 on every axis, h = 1): a
    particle midway between two node planes in z with radius 0.3 misses every node, one within its radius
    of a plane does not, and the Gaussian kernel's support (3 sigma r) reaches the planes."""
    bbox, res = (0.0, 0.0, 0.0, 10.0, 10.0, 10.0), (11, 11, 11)
    x = np.array([[2.0, 3.0, 4.5, 0.3],     # z midway: |4.5 - 4| = |5 - 4.5| = 0.5 > 0.3
                  [2.0, 3.0, 4.25, 0.3],    # 0.25 from the plane z = 4
                  [2.0, 3.0, 4.5, 0.6],     # radius beyond half the spacing
                  [2.5, 3.5, 4.5, 0.45]],   # midway on every axis
                 np.float32)
    assert oracle.support_misses_nodes_f64(x, bbox, res).tolist() == [True, False, False, True]
    assert oracle.support_misses_nodes_f64(x, bbox, res, sigma=1.0, kernel=1).tolist() == [False] * 4
