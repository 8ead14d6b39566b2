"""The intensity and vector aggregators of the CPU restatement against MegaMol's own ParticlesToDensity
(compiled from the reference tree where it exists): bit-exact with one thread."""
import os

import numpy as np
import pytest

import oracle

# the reference's OpenMP team size; the restatement reproduces its static partition and thread-grid sum
T = int(os.environ.get("OMP_NUM_THREADS", "0")) or os.cpu_count()


def frame(rng, n=3000):
    xyz = rng.uniform(0, 20, (n, 3)).astype(np.float32)
    xyzr = np.column_stack([xyz, np.full(n, 0.9, np.float32)])
    inten = rng.uniform(-1.0, 3.0, n).astype(np.float32)
    dirs = rng.normal(size=(n, 3)).astype(np.float32)
    return xyz, xyzr, inten, dirs


needs_ref = pytest.mark.skipif(not oracle.reference_available(), reason="reference tree not compiled here")


@needs_ref
@pytest.mark.parametrize("normalize", [False, True])
def test_intensity_aggregator_bit_exact(normalize):
    rng = np.random.default_rng(7)
    xyz, xyzr, inten, _ = frame(rng)
    res, bbox = (22, 20, 24), (0, 0, 0, 20, 20, 20)
    ref, meta = oracle.reference_density([dict(type=1, data=xyz, stride=0, radius=0.9, count=len(xyz), icol=inten)],
                                         bbox, res, (1, 1, 1), normalize, 1.0, aggregator=1)
    mine = oracle.density_weighted(xyzr, inten, bbox, res, nthreads=T)
    mine, mn, mx = oracle.normalize_minmax_f32(mine, normalize)
    assert np.array_equal(ref.reshape(-1), mine.reshape(-1))
    assert meta["min_value"] == (0.0 if normalize else mn) and meta["max_value"] == (1.0 if normalize else mx)


@needs_ref
@pytest.mark.parametrize("normalize", [False, True])
def test_vector_aggregator_bit_exact(normalize):
    rng = np.random.default_rng(8)
    xyz, xyzr, _, dirs = frame(rng)
    res, bbox = (18, 21, 19), (0, 0, 0, 20, 20, 20)
    ref, meta = oracle.reference_density([dict(type=1, data=xyz, stride=0, radius=0.9, count=len(xyz), dir=dirs)],
                                         bbox, res, (1, 0, 1), normalize, 1.0, aggregator=2)
    v3 = oracle.density_weighted(xyzr, dirs, bbox, res, cyclic=(1, 0, 1), nthreads=T)
    w = oracle.density_f32(xyzr, bbox, res, cyclic=(1, 0, 1), nthreads=T)
    mine, mn, mx = oracle.vector_finish_f32(v3, w, normalize)
    assert np.array_equal(ref.reshape(-1), mine.reshape(-1))
    if normalize:
        assert (meta["min_value"], meta["max_value"]) == (0.0, 1.0)
    else:
        assert (meta["min_value"], meta["max_value"]) == (mn, mx)


def _colour_list(kind, rng, n=900):
    """One particle list with colour data of `kind`, the colour interleaved after the vertex record (the MMPLD
    layout), and the weights the intensity aggregator reads from it."""
    def interleaved(vt, v, ct, c):
        rec = np.concatenate([np.ascontiguousarray(v).view(np.uint8).reshape(len(v), -1),
                              np.ascontiguousarray(c).view(np.uint8).reshape(len(c), -1)], 1)
        return dict(type=vt, data=rec.copy(), stride=rec.shape[1], count=len(v), col_type=ct,
                    col_offset=v.itemsize * v.shape[1], col_stride=rec.shape[1], radius=0.8)

    xyz = rng.uniform(0, 20, (n, 3)).astype(np.float32)
    if kind == "uint8_rgba":
        c = rng.integers(0, 256, (n, 4)).astype(np.uint8)
        return interleaved(1, xyz, 2, c), c[:, 0].astype(np.float32)
    if kind == "uint8_rgb":
        c = rng.integers(0, 256, (n, 3)).astype(np.uint8)
        return interleaved(1, xyz, 1, c), c[:, 0].astype(np.float32)
    if kind == "float_rgb":
        xyzr = np.column_stack([xyz, rng.uniform(0.4, 1.2, n)]).astype(np.float32)
        c = rng.uniform(-2, 3, (n, 3)).astype(np.float32)
        return dict(interleaved(2, xyzr, 3, c), radius=0.0), c[:, 0]
    if kind == "float_rgba":
        c = rng.uniform(-1, 1, (n, 4)).astype(np.float32)
        return interleaved(1, xyz, 4, c), c[:, 0]
    if kind == "ushort_rgba":
        c = rng.integers(0, 65536, (n, 4)).astype(np.uint16)
        return interleaved(4, xyz.astype(np.float64), 6, c), c[:, 0].astype(np.float32)
    if kind == "double_i":
        c = rng.uniform(-5, 5, (n, 1))
        return interleaved(3, rng.integers(0, 20, (n, 3)).astype(np.uint16), 7, c), c[:, 0].astype(np.float32)
    # COLDATA_NONE: the global colour's red channel
    return (dict(type=1, data=xyz, stride=0, count=n, radius=0.85, col_type=0, global_colour=(77, 5, 6, 255)),
            np.full(n, np.float32(77) / np.float32(255), np.float32))


@needs_ref
@pytest.mark.parametrize("kind", ["uint8_rgba", "uint8_rgb", "float_rgb", "float_rgba", "ushort_rgba", "double_i",
                                  "global"])
def test_intensity_from_every_colour_type_bit_exact(kind):
    """The intensity aggregator reads the first colour channel through SimpleSphericalParticles' accessor
    (ParticlesToDensity.cpp:483,508-516; SimpleSphericalParticles.h:123-177, Accessor.h:88-90,136-147): the raw
    value as float for UINT8 / USHORT / FLOAT / DOUBLE data (with every vertex type), and the global colour's
    red channel / 255 for COLDATA_NONE. The weights restated that way give the module's volume bit for bit
    (one list per frame: the module's OpenMP partition is per list)."""
    from tests import golden_io as G

    L, w = _colour_list(kind, np.random.default_rng(12))
    res, bbox = (21, 19, 23), (0, 0, 0, 20, 20, 20)
    ref, _ = oracle.reference_density([L], bbox, res, (1, 0, 1), False, 1.0, aggregator=1)
    mine = oracle.density_weighted(G.list_to_xyzr(L), w, bbox, res, cyclic=(1, 0, 1), nthreads=T)
    assert np.array_equal(ref.reshape(-1), mine.reshape(-1))


def test_weighted_fp64_is_linear():
    rng = np.random.default_rng(9)
    _, xyzr, inten, dirs = frame(rng, 800)
    res, bbox = (12, 12, 12), (0, 0, 0, 20, 20, 20)
    a = oracle.density_weighted(xyzr, inten, bbox, res, fp64=True)
    b = oracle.density_weighted(xyzr, 4.0 * inten, bbox, res, fp64=True)  # exact scaling in float32
    assert np.allclose(b, 4.0 * a, rtol=1e-12, atol=1e-12)
    ones = oracle.density_weighted(xyzr, np.ones(len(xyzr), np.float32), bbox, res, fp64=True)
    assert np.allclose(ones, oracle.density_f64(xyzr, bbox, res), rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("name", ["ivec_cyclic", "ivec_mixed_norm"])
def test_vector_grid_restatement_matches_reference_fixture(name):
    """The outParticles / outInfo grid of the vector aggregator (ParticlesToDensity.cpp:306-380, 628-727)
    restated in numpy float32 from the restatement's volume equals, bit for bit, what MegaMol's module
    produced for the fixture (one OpenMP thread)."""
    from tests import golden_io as G
    from tests.test_gpu_aggregators import load_agg

    c = load_agg(name)
    xyzr = np.concatenate([G.list_to_xyzr(L) for L in c["lists"]])
    d = np.concatenate([L["dir"] for L in c["lists"]])
    res = [int(v) for v in c["res"]]
    bbox = [float(v) for v in c["bbox"]]
    cyc = [int(v) for v in c["cyclic"]]
    v3 = oracle.density_weighted(xyzr, d, bbox, res, cyc, float(c["sigma"]))
    w = oracle.density_f32(xyzr, bbox, res, cyc, float(c["sigma"]))
    fin, mn, mx = oracle.vector_finish_f32(v3, w, False)
    g = oracle.vector_grid_f32(fin, bbox, res, int(c["normalize"]))
    assert g["count"] == int(c["vg_count"])
    for k in ("positions", "directions", "colours", "info"):
        assert np.array_equal(g[k], c[f"vg_{k}"]), k
    assert g["global_radius"] == c["vg_radius"]
    # the table's column ranges: the box, [-1, 1] for the directions, the published density range
    assert np.array_equal(c["vg_col_min"][:3], np.float32(bbox[:3])) and np.all(c["vg_col_min"][3:6] == -1)
    assert np.array_equal(c["vg_col_max"][:3], np.float32(bbox[3:])) and np.all(c["vg_col_max"][3:6] == 1)
    if int(c["normalize"]):
        assert (c["vg_col_min"][6], c["vg_col_max"][6]) == (0.0, 1.0)
    else:
        assert (c["vg_col_min"][6], c["vg_col_max"][6]) == (np.float32(mn), np.float32(mx))
