"""Generate golden vectors from MegaMol's own modules: ParticlesToDensity (density, aggregators, surface box),
DatRawWriter (dat/raw files) and MMPLDDataSource (MMPLD frames as the module publishes them).

Runs the reference's unmodified modules (compiled by ``oracle/Makefile`` target ``ref`` into
``oracle/_ref``) on small seeded inputs and stores inputs, parameters and the reference output as
``tests/golden/{p2d,agg,datraw,mmpld}_<case>.npz``. The reference tree exists only on the development
machine, so the fixtures are committed and the tests read them from here.

Usage:  python tests/golden/make_golden.py [prefix]   (only the fixtures whose name starts with prefix;
        OMP_NUM_THREADS is forced to 1: the reference's
        float sums then run in particle order, the order the CPU restatement reproduces bit-exactly)
"""
from __future__ import annotations

import os
import sys

os.environ["OMP_NUM_THREADS"] = "1"
HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import numpy as np  # noqa: E402

import oracle  # noqa: E402

VERT_FLOAT_XYZ, VERT_FLOAT_XYZR, VERT_SHORT_XYZ, VERT_DOUBLE_XYZ = 1, 2, 3, 4


def _case_uniform(rng, n, edge, r):
    xyz = rng.uniform(0, edge, size=(n, 3)).astype(np.float32)
    return [dict(type=VERT_FLOAT_XYZ, data=xyz, stride=0, radius=r, count=n)]


def cases():
    rng = np.random.default_rng(20240601)
    out = {}
    # 1. uniform, global radius, cyclic, sigma 1 (the reference defaults except the resolution)
    out["uniform_cyclic"] = dict(lists=_case_uniform(rng, 6000, 30.0, 0.5), bbox=(0, 0, 0, 30, 30, 30),
                                 res=(32, 32, 32), cyclic=(1, 1, 1), normalize=False, sigma=1.0)
    # 2. the same kind of data, non-cyclic, min-max normalised (ParticlesToDensity.cpp:676-682)
    out["uniform_open_norm"] = dict(lists=_case_uniform(rng, 6000, 30.0, 0.6), bbox=(0, 0, 0, 30, 30, 30),
                                    res=(32, 24, 28), cyclic=(0, 0, 0), normalize=True, sigma=1.0)
    # 3. per-particle radii, FLOAT_XYZR with a padded stride, sigma > 1 (footprint truncation)
    n = 4000
    rec = np.zeros((n, 5), np.float32)
    rec[:, :3] = rng.uniform(-5, 25, size=(n, 3))
    rec[:, 3] = rng.uniform(0.3, 1.4, size=n)
    rec[:, 4] = 123.0
    out["xyzr_stride_sigma2"] = dict(lists=[dict(type=VERT_FLOAT_XYZR, data=rec, stride=20, radius=0.0, count=n)],
                                     bbox=(-5, -5, -5, 25, 25, 25), res=(30, 30, 30), cyclic=(1, 0, 1),
                                     normalize=False, sigma=2.0)
    # 4. several lists of different vertex types, particles partly outside the box, sigma < 1
    xyz_d = rng.uniform(-2, 22, size=(2500, 3)).astype(np.float64)
    xyz_s = rng.integers(0, 20, size=(1500, 3)).astype(np.uint16)
    xyz_f = rng.uniform(0, 20, size=(2000, 3)).astype(np.float32)
    out["multilist_types"] = dict(lists=[
        dict(type=VERT_DOUBLE_XYZ, data=xyz_d, stride=0, radius=0.7, count=2500),
        dict(type=VERT_SHORT_XYZ, data=xyz_s, stride=0, radius=0.9, count=1500),
        dict(type=VERT_FLOAT_XYZ, data=xyz_f, stride=0, radius=0.45, count=2000),
    ], bbox=(0, 0, 0, 20, 20, 20), res=(25, 21, 23), cyclic=(1, 1, 0), normalize=False, sigma=0.8)
    # 5. footprint wider than the grid: cyclic wrap visits nodes several times (ParticlesToDensity.cpp:583-603)
    out["wide_footprint_wrap"] = dict(lists=_case_uniform(rng, 300, 10.0, 3.1), bbox=(0, 0, 0, 10, 10, 10),
                                      res=(6, 5, 7), cyclic=(1, 1, 1), normalize=False, sigma=1.0)
    # 6. one particle exactly on a node and one at the box minimum (known-answer test)
    one = np.array([[5.0, 5.0, 5.0], [0.0, 0.0, 0.0]], np.float32)
    out["kat_two_particles"] = dict(lists=[dict(type=VERT_FLOAT_XYZ, data=one, stride=0, radius=1.0, count=2)],
                                    bbox=(0, 0, 0, 10, 10, 10), res=(11, 11, 11), cyclic=(1, 1, 1),
                                    normalize=False, sigma=1.0)
    # 7. zero radius particles contribute nothing (ParticlesToDensity.cpp:523-524)
    rec0 = np.zeros((500, 4), np.float32)
    rec0[:, :3] = rng.uniform(0, 10, size=(500, 3))
    rec0[:250, 3] = 0.0
    rec0[250:, 3] = 0.8
    out["zero_radius"] = dict(lists=[dict(type=VERT_FLOAT_XYZR, data=rec0, stride=0, radius=0.0, count=500)],
                              bbox=(0, 0, 0, 10, 10, 10), res=(16, 16, 16), cyclic=(0, 0, 0), normalize=False,
                              sigma=1.0)
    # 8. forSurfaceReconstruction: the module grows the box and rewrites sizex / sizey for cubic voxels
    #    (ParticlesToDensity.cpp:234-235, 749-799); a flat, off-origin box with per-particle radii
    rec1 = np.zeros((3000, 4), np.float32)
    rec1[:, 0] = rng.uniform(-3.0, 17.0, 3000)
    rec1[:, 1] = rng.uniform(0.5, 12.5, 3000)
    rec1[:, 2] = rng.uniform(1.0, 25.0, 3000)
    rec1[:, 3] = rng.uniform(0.4, 1.1, 3000)
    out["surface_box"] = dict(lists=[dict(type=VERT_FLOAT_XYZR, data=rec1, stride=0, radius=0.0, count=3000)],
                              bbox=(-3.0, 0.5, 1.0, 17.0, 12.5, 25.0), res=(16, 16, 20), cyclic=(0, 0, 0),
                              normalize=False, sigma=1.0, surface=True)
    return out


def agg_cases():
    """The intensity (aggregator 1) and vector (aggregator 2) aggregators; colour data are COLDATA_FLOAT_I and
    directions DIRDATA_FLOAT_XYZ, the types the reference harness passes through."""
    rng = np.random.default_rng(20240917)
    out = {}
    xyz = rng.uniform(0, 24, size=(5000, 3)).astype(np.float32)
    out["icol_cyclic"] = dict(aggregator=1, lists=[dict(type=VERT_FLOAT_XYZ, data=xyz, stride=0, radius=0.8,
                                                        count=5000, icol=rng.uniform(-1, 3, 5000).astype(np.float32))],
                              bbox=(0, 0, 0, 24, 24, 24), res=(26, 24, 25), cyclic=(1, 1, 1), normalize=False,
                              sigma=1.0)
    rec = np.zeros((4000, 4), np.float32)
    rec[:, :3] = rng.uniform(-2, 22, size=(4000, 3))
    rec[:, 3] = rng.uniform(0.4, 1.2, size=4000)
    out["icol_open_norm"] = dict(aggregator=1, lists=[dict(type=VERT_FLOAT_XYZR, data=rec, stride=0, radius=0.0,
                                                           count=4000, icol=rng.uniform(0, 5, 4000).astype(np.float32))],
                                 bbox=(0, 0, 0, 20, 20, 20), res=(21, 23, 20), cyclic=(0, 0, 0), normalize=True,
                                 sigma=1.0)
    xyz2 = rng.uniform(0, 20, size=(4500, 3)).astype(np.float32)
    out["ivec_cyclic"] = dict(aggregator=2, lists=[dict(type=VERT_FLOAT_XYZ, data=xyz2, stride=0, radius=0.9,
                                                        count=4500, dir=rng.normal(size=(4500, 3)).astype(np.float32))],
                              bbox=(0, 0, 0, 20, 20, 20), res=(22, 20, 21), cyclic=(1, 1, 1), normalize=False,
                              sigma=1.0)
    rec2 = np.zeros((3500, 4), np.float32)
    rec2[:, :3] = rng.uniform(0, 20, size=(3500, 3))
    rec2[:, 3] = rng.uniform(0.5, 1.3, size=3500)
    out["ivec_mixed_norm"] = dict(aggregator=2, lists=[dict(type=VERT_FLOAT_XYZR, data=rec2, stride=0, radius=0.0,
                                                            count=3500,
                                                            dir=rng.uniform(-2, 2, (3500, 3)).astype(np.float32))],
                                  bbox=(0, 0, 0, 20, 20, 20), res=(20, 22, 24), cyclic=(1, 0, 1), normalize=True,
                                  sigma=1.0)
    return out


def datraw_cases():
    """Volumes for MegaMol's DatRawWriter: a scalar grid and a 3-component grid with a five-digit frame."""
    rng = np.random.default_rng(20241203)
    return {
        "scalar": dict(volume=rng.uniform(-1, 5, 5 * 4 * 3).astype(np.float32), resolution=(5, 4, 3), components=1,
                       slice_dists=(0.787402, 1.2345678, 2.5), origin=(-1.25, 0.0, 3e-7), frame=7, frame_count=10),
        "vector": dict(volume=rng.normal(size=3 * 2 * 2 * 3).astype(np.float32), resolution=(3, 2, 2), components=3,
                       slice_dists=(1.0 / 3.0, 1e10, 0.125), origin=(-0.0, 123456.789, -2.5e-12), frame=12345,
                       frame_count=20000),
    }


def mmpld_cases():
    from tests import mmpld_io
    rng = np.random.default_rng(20241204)
    out = {}
    for version in (100, 101, 102, 103):
        lists = mmpld_io.mixed_lists(rng)
        out[f"v{version}"] = dict(version=version, frames=[(0.25, lists), (1.5, lists[3:7]), (2.75, [])],
                                  bbox=(-5, -5, -5, 15, 15, 15), clipbox=(-6, -6, -6, 16, 16, 16.5))
    return out


def main(only=None):
    oracle.build(with_reference=True)
    import tempfile
    for name, c in mmpld_cases().items():
        if only and not f"mmpld_{name}".startswith(only):
            continue
        from tests import mmpld_io
        with tempfile.TemporaryDirectory() as d:
            fpath = os.path.join(d, f"{name}.mmpld")
            mmpld_io.write(fpath, c["frames"], version=c["version"], bbox=c["bbox"], clipbox=c["clipbox"])
            raw = open(fpath, "rb").read()
            r = oracle.reference_mmpld(fpath)
        d = dict(mmpld=np.frombuffer(raw, np.uint8), frames=np.int64(r["frames"]),
                 bbox=np.array(r["bbox"], np.float32), clipbox=np.array(r["clipbox"], np.float32))
        for fi, lists in enumerate(r["frame_lists"]):
            d[f"f{fi}_nlists"] = np.int64(len(lists))
            for li, L in enumerate(lists):
                vb = oracle.VERTEX_RECORD_BYTES.get(L["vert_type"], 0)
                cb = oracle.COLOUR_RECORD_BYTES.get(L["col_type"], 0)
                # strides as the records lie in the frame (the getters report 0 for packed records)
                vs = L["vert_stride"] or vb
                cs = L["col_stride"] or cb
                d[f"f{fi}_l{li}_meta"] = np.array(
                    [L["vert_type"], L["col_type"], L["count"], L["global_radius"], *L["global_colour"], L["col_min"],
                     L["col_max"], vs, cs, *L["bbox"], L["clusters"], L["cluster_bytes"]], np.float64)
                d[f"f{fi}_l{li}_vertex"] = L["vertex"]
                d[f"f{fi}_l{li}_colour"] = L["colour"]
        path = os.path.join(HERE, f"mmpld_{name}.npz")
        np.savez_compressed(path, **d)
        print(f"{path}: {len(raw)} B file, {r['frames']} frames")
    for name, c in datraw_cases().items():
        if only and not f"datraw_{name}".startswith(only):
            continue
        with tempfile.TemporaryDirectory() as d:
            assert oracle.reference_write_datraw(os.path.join(d, "vol_"), c["frame"], c["volume"], c["resolution"],
                                                 c["components"], c["slice_dists"], c["origin"], c["frame_count"])
            stem = os.path.join(d, f"vol_{c['frame']:04d}")
            dat = open(stem + ".dat", "rb").read()
            raw = open(stem + ".raw", "rb").read()
        path = os.path.join(HERE, f"datraw_{name}.npz")
        np.savez_compressed(path, dat=np.frombuffer(dat, np.uint8), raw=np.frombuffer(raw, np.uint8),
                            volume=c["volume"], resolution=np.array(c["resolution"], np.uint64),
                            components=np.int64(c["components"]), slice_dists=np.array(c["slice_dists"], np.float32),
                            origin=np.array(c["origin"], np.float32), frame=np.int64(c["frame"]),
                            frame_count=np.int64(c["frame_count"]))
        print(f"{path}: {len(dat)} B header, {len(raw)} B raw")
    for name, c in agg_cases().items():
        if only and not f"agg_{name}".startswith(only):
            continue
        vol, meta = oracle.reference_density(c["lists"], c["bbox"], c["res"], c["cyclic"], c["normalize"], c["sigma"],
                                             aggregator=c["aggregator"])
        d = dict(aggregator=np.int32(c["aggregator"]), bbox=np.array(c["bbox"], np.float32),
                 res=np.array(c["res"], np.int32), cyclic=np.array(c["cyclic"], np.int32),
                 normalize=np.int32(c["normalize"]), sigma=np.float32(c["sigma"]), nlists=np.int32(len(c["lists"])),
                 volume=vol, components=np.int32(meta["components"]), min_value=np.float64(meta["min_value"]),
                 max_value=np.float64(meta["max_value"]))
        if c["aggregator"] == 2:
            # the outParticles / outInfo outputs of the vector aggregator (ParticlesToDensity.cpp:306-380)
            vg = oracle.reference_vector_grid(c["lists"], c["bbox"], c["res"], c["cyclic"], c["normalize"],
                                              c["sigma"])
            assert np.array_equal(vg["volume"], vol)
            for k in ("positions", "directions", "colours", "info", "col_min", "col_max"):
                d[f"vg_{k}"] = vg[k]
            d["vg_count"] = np.int64(vg["count"])
            d["vg_radius"] = np.float32(vg["global_radius"])
        for i, L in enumerate(c["lists"]):
            d[f"l{i}_type"] = np.int32(L["type"])
            d[f"l{i}_data"] = np.ascontiguousarray(L["data"])
            d[f"l{i}_stride"] = np.int32(L["stride"])
            d[f"l{i}_radius"] = np.float32(L["radius"])
            d[f"l{i}_count"] = np.int64(L["count"])
            if "icol" in L:
                d[f"l{i}_icol"] = L["icol"]
            if "dir" in L:
                d[f"l{i}_dir"] = L["dir"]
        path = os.path.join(HERE, f"agg_{name}.npz")
        np.savez_compressed(path, **d)
        print(f"{path}: volume {vol.shape} range [{vol.min():.6g}, {vol.max():.6g}]")
    for name, c in cases().items():
        if only and not f"p2d_{name}".startswith(only):
            continue
        surface = bool(c.get("surface", False))
        vol, meta = oracle.reference_density(c["lists"], c["bbox"], c["res"], c["cyclic"], c["normalize"], c["sigma"],
                                             surface=surface)
        d = dict(bbox=np.array(c["bbox"], np.float32), res=np.array(c["res"], np.int32),
                 cyclic=np.array(c["cyclic"], np.int32), normalize=np.int32(c["normalize"]),
                 sigma=np.float32(c["sigma"]), nlists=np.int32(len(c["lists"])), volume=vol,
                 min_value=np.float64(meta["min_value"]), max_value=np.float64(meta["max_value"]),
                 slice_dists=np.array(meta["slice_dists"], np.float32))
        if surface:
            # the module's published grid after the box adjustment
            d.update(surface=np.int32(1), out_res=np.array(meta["resolution"], np.int32),
                     origin=np.array(meta["origin"], np.float32), extents=np.array(meta["extents"], np.float32))
        for i, L in enumerate(c["lists"]):
            d[f"l{i}_type"] = np.int32(L["type"])
            d[f"l{i}_data"] = np.ascontiguousarray(L["data"])
            d[f"l{i}_stride"] = np.int32(L["stride"])
            d[f"l{i}_radius"] = np.float32(L["radius"])
            d[f"l{i}_count"] = np.int64(L["count"])
        path = os.path.join(HERE, f"p2d_{name}.npz")
        np.savez_compressed(path, **d)
        print(f"{path}: volume {vol.shape} range [{vol.min():.6g}, {vol.max():.6g}]")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
