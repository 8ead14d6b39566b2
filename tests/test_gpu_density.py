"""GPU parity tests of the density path, called through the C ABI (megamol_gb300.p2v -> libp2v.so).

Bars: against the FP64 oracle, max-rel error (max|a-b| / max|b|) <= 1e-6 (the target is 1e-5); against
the reference module's own FP32 output (golden fixtures) the difference is bounded by the reference's
float rounding, <= 2e-5 of the maximum. Integer metadata (resolution, slice distances) must be identical.
"""
import os

import numpy as np
import pytest

import oracle
from megamol_gb300 import build as nbuild
from megamol_gb300 import p2v, synth
from tests import golden_io as G

pytestmark = pytest.mark.gpu
NT = os.cpu_count() or 1


@pytest.fixture(scope="module")
def ctx():
    nbuild.build()
    c = p2v.Context(0)
    yield c
    c.close()


def run(ctx, lists, bbox, res, cyclic=(1, 1, 1), normalize=False, sigma=1.0, kernel=p2v.KERNEL_BUMP, mass=False,
        out=None, accumulate=p2v.ACCUM_EXACT, surface=False, out_res=None):
    """One frame; `out_res` sizes the host output when the module rewrites the resolution (surface)."""
    ctx.set_params(sizex=int(res[0]), sizey=int(res[1]), sizez=int(res[2]), cyclX=int(cyclic[0]),
                   cyclY=int(cyclic[1]), cyclZ=int(cyclic[2]), normalize=int(bool(normalize)), sigma=float(sigma),
                   kernel=kernel, mass_normalize=int(mass), forSurfaceReconstruction=int(bool(surface)),
                   accumulate=accumulate)
    r = out_res if out_res is not None else res
    if out is None:
        out = np.full(int(r[0]) * int(r[1]) * int(r[2]), np.nan, np.float32)
    meta = ctx.run_frame(lists, bbox, out)
    if isinstance(out, np.ndarray):
        r = meta["resolution"]
        out = out.reshape(int(r[2]), int(r[1]), int(r[0]))
    return out, meta


def maxrel(a, b):
    b = np.asarray(b, np.float64)
    return float(np.abs(np.asarray(a, np.float64) - b).max() / max(np.abs(b).max(), 1e-300))


def golden_lists(c):
    return [p2v.ParticleList(np.ascontiguousarray(L["data"]), L["type"], count=L["count"], stride=L["stride"],
                             global_radius=L["radius"]) for L in c["lists"]]


ACCUM = [p2v.ACCUM_EXACT, p2v.ACCUM_KAHAN]


@pytest.mark.parametrize("accumulate", ACCUM)
@pytest.mark.parametrize("name", G.golden_names())
def test_golden_vs_reference_and_fp64(ctx, name, accumulate):
    c = G.load(name)
    bbox, res = G.grid(c)  # the surface case's adjusted box, restated bit-exactly against the reference
    vol, meta = run(ctx, golden_lists(c), c["bbox"], c["res"], c["cyclic"], bool(c["normalize"]), float(c["sigma"]),
                    accumulate=accumulate, surface=bool(c["surface"]), out_res=res)
    ref = c["volume"]
    assert meta["resolution"] == [int(x) for x in res] and vol.shape == ref.shape
    xyzr = G.case_xyzr(c)
    v64 = oracle.density_f64(xyzr, bbox, res, c["cyclic"], float(c["sigma"]), oracle.BUMP, NT)
    if bool(c["normalize"]):
        v64, _, _ = oracle.normalize_f64(v64, "minmax")
    assert maxrel(vol, v64) <= 1e-6, f"{name}: vs FP64 {maxrel(vol, v64):.3e}"
    assert maxrel(vol, ref) <= 2e-5, f"{name}: vs reference {maxrel(vol, ref):.3e}"
    assert meta["slice_dists"] == [float(x) for x in c["slice_dists"]]
    if int(c["surface"]):
        assert meta["origin"] == [float(x) for x in c["origin"]]
        assert meta["extents"] == [float(x) for x in c["extents"]]
    if bool(c["normalize"]):
        assert meta["min_value"] == 0.0 and meta["max_value"] == 1.0
    else:
        assert abs(meta["max_value"] - float(c["max_value"])) <= 2e-5 * abs(float(c["max_value"]))


@pytest.mark.parametrize("accumulate", ACCUM)
def test_deterministic_bitwise(ctx, accumulate):
    f = synth.uniform(n=200_000, edge=60.0, res=96, seed=3)
    L = [p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR)]
    a, _ = run(ctx, L, f.bbox, f.res, accumulate=accumulate)
    b, _ = run(ctx, L, f.bbox, f.res, accumulate=accumulate)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    # the exact mode is independent of the particle order: shuffle the input and compare bitwise
    if accumulate == p2v.ACCUM_EXACT:
        perm = np.random.default_rng(0).permutation(f.n)
        c, _ = run(ctx, [p2v.ParticleList(np.ascontiguousarray(f.xyzr[perm]), p2v.VERTDATA_FLOAT_XYZR)], f.bbox,
                   f.res, accumulate=accumulate)
        assert np.array_equal(a.view(np.uint32), c.view(np.uint32))


def test_device_buffers_match_host_buffers(ctx):
    torch = pytest.importorskip("torch")
    f = synth.uniform(n=50_000, edge=30.0, res=40, seed=4)
    host, _ = run(ctx, [p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR)], f.bbox, f.res)
    dx = torch.from_numpy(f.xyzr).cuda()
    dout = torch.empty(40 * 40 * 40, dtype=torch.float32, device="cuda")
    run(ctx, [p2v.ParticleList(dx, p2v.VERTDATA_FLOAT_XYZR, count=f.n)], f.bbox, f.res, out=dout)
    torch.cuda.synchronize()
    assert np.array_equal(dout.cpu().numpy().reshape(40, 40, 40), host)


def test_gauss3_and_mass_normalisation(ctx):
    f = synth.uniform(n=30_000, edge=30.0, res=40, seed=5)
    f.xyzr[:, 3] = np.random.default_rng(1).uniform(0.3, 0.7, f.n).astype(np.float32)
    L = [p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR)]
    raw, _ = run(ctx, L, f.bbox, f.res, kernel=p2v.KERNEL_GAUSS3)
    v64 = oracle.density_f64(f.xyzr, f.bbox, f.res, (1, 1, 1), 1.0, oracle.GAUSS3, NT)
    assert maxrel(raw, v64) <= 1e-6
    vm, meta = run(ctx, L, f.bbox, f.res, kernel=p2v.KERNEL_GAUSS3, mass=True)
    h = oracle.spacing_f64(f.bbox, f.res)
    mass = vm.astype(np.float64).sum() * h[0] * h[1] * h[2]
    assert abs(mass - f.n) <= 1e-5 * f.n
    m64, _, _ = oracle.normalize_f64(v64, "mass", f.n, h)
    assert maxrel(vm, m64) <= 1e-6


def test_invalid_particles_are_dropped(ctx):
    f = synth.uniform(n=20_000, edge=20.0, res=24, seed=6)
    x = f.xyzr.copy()
    x[::97, 0] = np.nan
    x[5::101, 3] = 0.0
    x[7::103, 3] = -1.0
    x[9::107, 1] = np.inf
    vol, _ = run(ctx, [p2v.ParticleList(x, p2v.VERTDATA_FLOAT_XYZR)], f.bbox, f.res)
    ok = np.isfinite(x).all(1) & (x[:, 3] > 0)
    v64 = oracle.density_f64(x[ok], f.bbox, f.res, (1, 1, 1), 1.0, oracle.BUMP, NT)
    assert maxrel(vol, v64) <= 1e-6
    st = ctx.stats()
    assert st["particles_dropped"] == int((~ok).sum())
    assert st["particles_binned"] == int(ok.sum())


def test_empty_frame(ctx):
    vol, meta = run(ctx, [], (0, 0, 0, 1, 1, 1), (8, 8, 8), normalize=False)
    assert np.all(vol == 0)
    # the reference divides by (max - min) = 0 when normalising an empty grid; so does this library
    vol, meta = run(ctx, [], (0, 0, 0, 1, 1, 1), (8, 8, 8), normalize=True)
    assert np.all(np.isnan(vol))


@pytest.mark.parametrize("accumulate", ACCUM)
def test_out_of_box_particles_open_and_cyclic(ctx, accumulate):
    rng = np.random.default_rng(8)
    x = np.zeros((8000, 4), np.float32)
    x[:, :3] = rng.uniform(-6, 26, size=(8000, 3))
    x[:, 3] = rng.uniform(0.4, 1.6, 8000)
    for cyc in [(0, 0, 0), (1, 1, 1), (0, 1, 0)]:
        for sigma in (1.0, 1.7):
            vol, _ = run(ctx, [p2v.ParticleList(x, p2v.VERTDATA_FLOAT_XYZR)], (0, 0, 0, 20, 20, 20), (21, 18, 23),
                         cyc, sigma=sigma, accumulate=accumulate)
            v64 = oracle.density_f64(x, (0, 0, 0, 20, 20, 20), (21, 18, 23), cyc, sigma, oracle.BUMP, NT)
            assert maxrel(vol, v64) <= 1e-6, (cyc, sigma)


def test_surface_reconstruction_box(ctx):
    f = synth.uniform(n=5000, edge=10.0, res=16, seed=9)
    m = p2v.ParticlesToDensity(0, sizex=16, sizey=16, sizez=20, forSurfaceReconstruction=1, normalize=0)
    vol, meta = m.get_data([p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR)], f.bbox)
    # modifyBBox makes voxels cubic and rewrites sizex / sizey (ParticlesToDensity.cpp:749-799)
    assert meta["resolution"][2] == 20
    sd = meta["slice_dists"]
    assert vol.shape == tuple(meta["resolution"][::-1])
    bb = meta["bbox"]
    assert (tuple(bb), tuple(meta["resolution"])) == oracle.modify_bbox_f32(f.bbox, (16, 16, 20))
    v64 = oracle.density_f64(f.xyzr, bb, meta["resolution"], (1, 1, 1), 1.0, oracle.BUMP, NT)
    assert maxrel(vol, v64) <= 1e-6
    assert m.param("sizex") == meta["resolution"][0]
    assert abs(sd[0] - sd[2]) < 0.2 * sd[2]


def test_surface_reconstruction_rejects_flat_box(ctx):
    """A box without depth would divide by a zero voxel spacing in the box adjustment (the reference's
    float-to-int conversions are then undefined): the frame is rejected and the context stays usable."""
    x = np.zeros((10, 4), np.float32)
    x[:, :2] = np.random.default_rng(1).uniform(0, 1, (10, 2))
    x[:, 3] = 0.5
    ctx.set_params(sizex=8, sizey=8, sizez=8, forSurfaceReconstruction=1, normalize=0, cyclX=0, cyclY=0, cyclZ=0)
    with pytest.raises(p2v.P2VError):
        ctx.run_frame([p2v.ParticleList(x, p2v.VERTDATA_FLOAT_XYZR)], (0, 0, 0, 1, 1, 0), None)
    vol, meta = run(ctx, [p2v.ParticleList(x, p2v.VERTDATA_FLOAT_XYZR)], (0, 0, 0, 1, 1, 1), (8, 8, 8))
    assert meta["resolution"] == [8, 8, 8] and np.isfinite(vol).all()


@pytest.mark.parametrize("seed,accumulate", [(0, p2v.ACCUM_EXACT), (1, p2v.ACCUM_KAHAN)])
def test_lj_liquid_full_size(ctx, seed, accumulate):
    """The headline workload at full size (4M particles, 256^3), against the FP64 oracle."""
    f = synth.lj_liquid(seed=2 + seed)
    vol, meta = run(ctx, [p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR)], f.bbox, f.res, accumulate=accumulate)
    v64 = oracle.density_f64(f.xyzr, f.bbox, f.res, (1, 1, 1), 1.0, oracle.BUMP, NT)
    err = maxrel(vol, v64)
    assert err <= 1e-6, err
    st = ctx.stats()
    assert st["particles_binned"] == f.n and st["device_error"] == 0


@pytest.mark.parametrize("cyclic", [(1, 1, 1), (0, 0, 0)])
def test_particles_whose_support_misses_every_node(ctx, cyclic):
    """A frame of flat voxels (3.1 units in z against radii of 0.3-0.9, as in the mixed-phase frame) on the
    radix path (86 cells per particle): the binning sorts the particles whose support holds no node after all
    others and the gather never visits them. The grid is bit-identical to the one of plain cell keys (the AO
    brick order keeps them) and matches the FP64 oracle."""
    rng = np.random.default_rng(77)
    n = 40_000
    x = np.empty((n, 4), np.float32)
    x[:, :2] = rng.uniform(0, 40, (n, 2))
    x[:, 2] = rng.uniform(0, 400, n)
    x[:, 3] = rng.uniform(0.3, 0.9, n)
    bbox, res = (0.0, 0.0, 0.0, 40.0, 40.0, 400.0), (160, 160, 129)
    L = [p2v.ParticleList(x, p2v.VERTDATA_FLOAT_XYZR)]
    ctx.set_params(ao_brick_order=0)
    flagged, _ = run(ctx, L, bbox, res, cyclic=cyclic)
    flagged = flagged.copy()
    keys, order, start = ctx.binning()
    nbins = start.size - 1
    assert ctx.stats()["cell_max_count"] == 0  # the radix path
    miss = oracle.support_misses_nodes_f64(x, bbox, res)
    pf = np.zeros(n, bool)
    pf[order[keys > nbins]] = True
    assert pf.sum() > 0.3 * n and np.all(miss[pf]), (pf.sum(), miss.sum())
    ctx.set_params(ao_brick_order=1)
    try:
        plain, _ = run(ctx, L, bbox, res, cyclic=cyclic)
        assert ctx.binning()[0].max() <= nbins
    finally:
        ctx.set_params(ao_brick_order=0)
    assert np.array_equal(flagged.view(np.uint32), plain.view(np.uint32))
    v64 = oracle.density_f64(x, bbox, res, cyclic, 1.0, oracle.BUMP, NT)
    assert maxrel(flagged, v64) <= 1e-6
