"""GPU tests of the intensity (aggregator 1) and vector (aggregator 2) aggregators of ParticlesToDensity.

Against the reference's own output (golden fixtures made by the compiled module, tests/golden/agg_*.npz) and
against the FP64 restatement. Bars: intensity max|a-b| <= 2e-5 of max|b| against the reference (its float
node positions) and <= 1e-6 against FP64. Vector volume, over the voxels whose weight sum is a normal float:
<= 1e-5 of max|b| against FP64 and <= 2e-3 against the reference, whose float distances move kernel tails
(exp(-1/(1-q^2)) near q = 1) by up to about 0.5 % where two particles' tails meet. Voxels reached only by
tails whose float sum is subnormal hold the quotient of two sums of a few bits, which depends on how each
exponential rounds subnormal results (the C library's and the GPU's differ there): within 5 % of max|b| of
the reference's value. Colour types: the first channel as float, the global colour as r / 255."""
import glob
import os

import numpy as np
import pytest

import oracle
from megamol_gb300 import build as nbuild
from megamol_gb300 import p2v
from tests import golden_io as G

pytestmark = pytest.mark.gpu
AGG = sorted(os.path.basename(p)[4:-4] for p in glob.glob(os.path.join(G.GOLDEN, "agg_*.npz")))


@pytest.fixture(scope="module")
def ctx():
    nbuild.build()
    c = p2v.Context(0)
    yield c
    c.close()


def load_agg(name):
    z = np.load(os.path.join(G.GOLDEN, f"agg_{name}.npz"))
    c = {k: z[k] for k in z.files}
    lists = []
    for i in range(int(c["nlists"])):
        L = dict(type=int(c[f"l{i}_type"]), data=c[f"l{i}_data"], stride=int(c[f"l{i}_stride"]),
                 radius=float(c[f"l{i}_radius"]), count=int(c[f"l{i}_count"]))
        for k in ("icol", "dir"):
            if f"l{i}_{k}" in c:
                L[k] = c[f"l{i}_{k}"]
        lists.append(L)
    c["lists"] = lists
    return c


def run(ctx, c, lists, agg):
    res = [int(v) for v in c["res"]]
    cyc = [int(v) for v in c["cyclic"]]
    ctx.set_params(aggregator=agg, sizex=res[0], sizey=res[1], sizez=res[2], cyclX=cyc[0], cyclY=cyc[1],
                   cyclZ=cyc[2], normalize=int(c["normalize"]), sigma=float(c["sigma"]), kernel=p2v.KERNEL_BUMP,
                   accumulate=p2v.ACCUM_EXACT, mass_normalize=0, ao_mode=p2v.AO_NONE, forSurfaceReconstruction=0)
    comps = 3 if agg == 2 else 1
    out = np.empty(res[0] * res[1] * res[2] * comps, np.float32)
    meta = ctx.run_frame(lists, [float(v) for v in c["bbox"]], out)
    assert meta["components"] == comps
    return out.reshape(res[2], res[1], res[0], comps) if comps == 3 else out.reshape(res[2], res[1], res[0]), meta


def p2v_lists(c):
    out = []
    for L in c["lists"]:
        kw = {}
        if "icol" in L:
            kw = dict(colour=np.ascontiguousarray(L["icol"], np.float32), colour_type=p2v.COLDATA_FLOAT_I)
        if "dir" in L:
            kw = dict(normals=np.ascontiguousarray(L["dir"], np.float32))
        out.append(p2v.ParticleList(L["data"], L["type"], count=L["count"], stride=L["stride"],
                                    global_radius=L["radius"], **kw))
    return out


def fp64_reference(c, agg):
    xyzr = np.concatenate([G.list_to_xyzr(L) for L in c["lists"]])
    res = [int(v) for v in c["res"]]
    cyc = [int(v) for v in c["cyclic"]]
    bbox = [float(v) for v in c["bbox"]]
    if agg == 1:
        w = np.concatenate([L["icol"] for L in c["lists"]])
        v = oracle.density_weighted(xyzr, w, bbox, res, cyc, float(c["sigma"]), fp64=True)
        if int(c["normalize"]):
            v = (v - v.min()) / (v.max() - v.min())
        return v, None
    d = np.concatenate([L["dir"] for L in c["lists"]])
    sig = float(c["sigma"])
    v3 = oracle.density_weighted(xyzr, d, bbox, res, cyc, sig, fp64=True)
    w = oracle.density_f64(xyzr, bbox, res, cyc, sig)
    v3 = v3 / np.where(w == 0.0, 1.0, w)[..., None]
    dens = np.sqrt((v3 ** 2).sum(-1))
    if int(c["normalize"]):
        lo, hi = min(dens.min(), np.finfo(np.float32).max), max(dens.max(), 0.0)
        v3 = (v3 - lo) / (hi - lo)
    return v3, w


@pytest.mark.parametrize("name", AGG)
def test_aggregator_vs_reference_and_fp64(ctx, name):
    c = load_agg(name)
    agg = int(c["aggregator"])
    got, meta = run(ctx, c, p2v_lists(c), agg)
    ref = c["volume"].reshape(got.shape).astype(np.float64)
    scale = np.abs(ref).max()
    err_ref = np.abs(got - ref).max() / scale
    exact, w64 = fp64_reference(c, agg)
    if agg == 1:
        err_64 = np.abs(got - exact).max() / np.abs(exact).max()
        assert err_ref <= 2e-5, err_ref
        assert err_64 <= 1e-6, err_64
    else:
        # voxels whose weight sum is a normal float: the FP64 bar; where it is subnormal (kernel tails below
        # FLT_MIN) the reference and the GPU both divide sums of a few bits, rounded by their own exponentials
        normal = w64 >= np.finfo(np.float32).tiny
        err_64 = np.abs(got - exact)[normal].max() / np.abs(exact).max()
        err_ref = np.abs(got - ref)[normal].max() / scale
        assert err_ref <= 2e-3, err_ref
        assert err_64 <= 1e-5, err_64
        assert np.abs(got - ref)[~normal].max(initial=0.0) <= 0.05 * scale
        assert np.all(got[w64 == 0.0] == (ref[w64 == 0.0]))
    if int(c["normalize"]):
        assert (meta["min_value"], meta["max_value"]) == (0.0, 1.0)
    else:
        assert abs(meta["min_value"] - float(c["min_value"])) <= 2e-5 * scale
        assert abs(meta["max_value"] - float(c["max_value"])) <= 2e-3 * scale


@pytest.mark.parametrize("kind", ["uint8_rgba", "float_rgb", "double_i", "ushort_rgba", "global"])
def test_intensity_from_colour_types(ctx, kind):
    rng = np.random.default_rng(3)
    n = 6000
    xyzr = np.column_stack([rng.uniform(0, 16, (n, 3)), rng.uniform(0.5, 1.0, n)]).astype(np.float32)
    if kind == "uint8_rgba":
        col = rng.integers(0, 256, (n, 4)).astype(np.uint8)
        w, ct = col[:, 0].astype(np.float32), p2v.COLDATA_UINT8_RGBA
    elif kind == "float_rgb":
        col = rng.uniform(-2, 2, (n, 3)).astype(np.float32)
        w, ct = col[:, 0], p2v.COLDATA_FLOAT_RGB
    elif kind == "double_i":
        col = rng.uniform(0, 9, (n, 1))
        w, ct = col[:, 0].astype(np.float32), p2v.COLDATA_DOUBLE_I
    elif kind == "ushort_rgba":
        col = rng.integers(0, 65536, (n, 4)).astype(np.uint16)
        w, ct = col[:, 0].astype(np.float32), p2v.COLDATA_USHORT_RGBA
    else:
        col, ct = None, p2v.COLDATA_NONE
        w = np.full(n, np.float32(77) / np.float32(255), np.float32)
    L = p2v.ParticleList(xyzr, p2v.VERTDATA_FLOAT_XYZR, colour=col, colour_type=ct, global_colour=(77, 1, 2, 255))
    res, bbox = (18, 17, 19), (0, 0, 0, 16, 16, 16)
    ctx.set_params(aggregator=1, sizex=res[0], sizey=res[1], sizez=res[2], cyclX=1, cyclY=1, cyclZ=1, normalize=0,
                   sigma=1.0, kernel=p2v.KERNEL_BUMP, accumulate=p2v.ACCUM_EXACT, mass_normalize=0,
                   ao_mode=p2v.AO_NONE)
    out = np.empty(res[0] * res[1] * res[2], np.float32)
    ctx.run_frame([L], bbox, out)
    exact = oracle.density_weighted(xyzr, w, bbox, res, fp64=True)
    assert np.abs(out.reshape(exact.shape) - exact).max() <= 1e-6 * np.abs(exact).max()


def test_aggregators_are_deterministic_and_reject_bad_settings(ctx):
    c = load_agg("ivec_cyclic")
    a, _ = run(ctx, c, p2v_lists(c), 2)
    b, _ = run(ctx, c, p2v_lists(c), 2)
    assert np.array_equal(a, b)
    ctx.set_params(aggregator=3)
    with pytest.raises(p2v.P2VError):
        ctx.run_frame(p2v_lists(c), [float(v) for v in c["bbox"]], None)
    ctx.set_params(aggregator=1, accumulate=p2v.ACCUM_KAHAN)
    with pytest.raises(p2v.P2VError):
        ctx.run_frame(p2v_lists(c), [float(v) for v in c["bbox"]], None)
    ctx.set_params(aggregator=0, accumulate=p2v.ACCUM_EXACT)


@pytest.mark.parametrize("name", ["ivec_cyclic", "ivec_mixed_norm"])
def test_vector_grid_outputs(ctx, name):
    """The vector aggregator's outParticles / outInfo grid (p2v_get_vector_grid). Bit for bit against the
    float32 restatement applied to the GPU's own direction volume (the finish, the stable descending sort
    by density and the compaction); against the reference's grid: the same node set up to nodes reached only
    by tails whose float sums are subnormal, and directions within 2e-3 on nodes of normal weight."""
    c = load_agg(name)
    norm = int(c["normalize"])
    res = [int(v) for v in c["res"]]
    bbox = [float(v) for v in c["bbox"]]
    raw = dict(c)
    raw["normalize"] = np.int32(0)
    ctx.set_params(vector_grid=1)
    v3, _ = run(ctx, raw, p2v_lists(c), 2)           # the finished, not normalised volume
    ctx.set_params(vector_grid=1)
    run(ctx, c, p2v_lists(c), 2)
    g = ctx.vector_grid()
    mine = oracle.vector_grid_f32(v3, bbox, res, norm)
    assert g["count"] == mine["count"]
    for k in ("positions", "directions", "colours", "info"):
        assert np.array_equal(g[k], mine[k]), k
    assert g["global_radius"] == float(c["vg_radius"])
    assert np.array_equal(g["col_min"][:6], c["vg_col_min"][:6]) and np.array_equal(g["col_max"][:6],
                                                                                  c["vg_col_max"][:6])
    # against the reference module's grid
    _, w64 = fp64_reference(c, 2)
    ref_pos = c["vg_positions"]
    key = lambda p: {tuple(r): i for i, r in enumerate(p.tolist())}
    gi, ri = key(g["positions"]), key(ref_pos)
    sub = w64 < np.finfo(np.float32).tiny
    flat_sub = set(np.flatnonzero(sub.ravel()).tolist())
    h = [np.float32(abs(np.float32(bbox[a + 3]) - np.float32(bbox[a]))) / np.float32(res[a] - 1) for a in range(3)]

    def node(p):
        ix = [int(round((p[a] - bbox[a]) / float(h[a]))) for a in range(3)]
        return ix[0] + (ix[1] + ix[2] * res[1]) * res[0]

    for p in set(gi) ^ set(ri):          # nodes in one grid only: subnormal tails
        assert node(p) in flat_sub
    both = [p for p in set(gi) & set(ri) if node(p) not in flat_sub]
    assert len(both) > 0.5 * len(ri)
    a = np.array([g["directions"][gi[p]] for p in both])
    b = np.array([c["vg_directions"][ri[p]] for p in both])
    assert np.abs(a - b).max() <= 2e-3
