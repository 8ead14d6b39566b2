"""MMPLD reader (p2v_mmpld_*) on files written in the layout of MegaMol's reader, CPU only."""
import os

import numpy as np
import pytest

from tests import mmpld_io
from megamol_gb300 import p2v


def as_array(L, dtype, comps, which="vertex"):
    """The list's per-particle records as a (count, comps) array read through the pointer and stride."""
    import ctypes as C

    ptr = L.data if which == "vertex" else L.colour
    stride = L.stride if which == "vertex" else L.colour_stride
    buf = (C.c_uint8 * (stride * L.count)).from_address(ptr)
    raw = np.frombuffer(buf, np.uint8).reshape(L.count, stride)
    item = np.dtype(dtype).itemsize
    return raw[:, :item * comps].copy().view(dtype).reshape(L.count, comps)


def make_lists(rng):
    n1, n2, n3, n4 = 37, 50, 11, 23
    xyzr = rng.uniform(0, 10, (n1, 4)).astype(np.float32)
    rgba8 = rng.integers(0, 255, (n1, 4)).astype(np.uint8)
    xyz = rng.uniform(0, 10, (n2, 3)).astype(np.float32)
    inten = rng.uniform(-1, 3, (n2, 1)).astype(np.float32)
    sxyz = rng.integers(0, 60000, (n3, 3)).astype(np.uint16)
    dxyz = rng.uniform(0, 10, (n4, 3)).astype(np.float64)
    drgb = rng.uniform(0, 1, (n4, 3)).astype(np.float32)
    lists = [dict(vt=2, ct=2, count=n1, records=mmpld_io.records(xyzr, rgba8), bbox=(0, 1, 2, 3, 4, 5)),
             dict(vt=1, ct=3, count=n2, records=mmpld_io.records(xyz, inten), radius=0.7, irange=(-1.0, 3.0)),
             dict(vt=3, ct=0, count=n3, records=mmpld_io.records(sxyz), radius=1.5, colour=(9, 8, 7, 6)),
             dict(vt=4, ct=4, count=n4, records=mmpld_io.records(dxyz, drgb), radius=0.25),
             dict(vt=0, ct=0, count=5, records=b"", colour=(1, 2, 3, 4))]
    return lists, (xyzr, rgba8, xyz, inten, sxyz, dxyz, drgb)


@pytest.mark.parametrize("version", [100, 101, 102, 103])
def test_read_all_list_types(tmp_path, version):
    rng = np.random.default_rng(version)
    lists, (xyzr, rgba8, xyz, inten, sxyz, dxyz, drgb) = make_lists(rng)
    frames = [(0.5, lists), (1.5, lists[:2]), (2.5, [])]
    path = tmp_path / f"t{version}.mmpld"
    mmpld_io.write(path, frames, version=version)
    f = p2v.Mmpld(path)
    assert (f.version, f.frames) == (version, 3)
    assert f.bbox == [0, 0, 0, 10, 10, 10] and f.clipbox == [-1, -1, -1, 11, 11, 11]
    L, info, ts, buf = f.read(0)
    assert ts == (0.5 if version >= 102 else 0.0)
    assert [l.vertex_type for l in L] == [2, 1, 3, 4, 0]
    assert [l.colour_type for l in L] == [p2v.COLDATA_UINT8_RGBA, p2v.COLDATA_FLOAT_I, p2v.COLDATA_NONE,
                                          p2v.COLDATA_FLOAT_RGB, p2v.COLDATA_NONE]
    assert [l.count for l in L] == [37, 50, 11, 23, 5]
    assert np.array_equal(as_array(L[0], np.float32, 4), xyzr)
    assert np.array_equal(as_array(L[0], np.uint8, 4, "colour"), rgba8)
    assert np.array_equal(as_array(L[1], np.float32, 3), xyz)
    assert np.array_equal(as_array(L[1], np.float32, 1, "colour"), inten)
    assert np.array_equal(as_array(L[2], np.uint16, 3), sxyz)
    assert np.array_equal(as_array(L[3], np.float64, 3), dxyz)
    assert np.array_equal(as_array(L[3], np.float32, 3, "colour"), drgb)
    # global radius: the file's for types 1, 3, 4 and 0.05 otherwise (MMPLDDataSource.cpp:158-163)
    assert [round(l.global_radius, 6) for l in L] == [0.05, 0.7, 1.5, 0.25, 0.05]
    assert L[2].global_colour[:3] == (9, 8, 7) and L[0].global_colour[:3] == (192, 192, 192)
    assert info[1]["intensity_range"] == [-1.0, 3.0] and info[0]["intensity_range"] == [0.0, 1.0]
    if version >= 103:
        assert info[0]["bbox"] == [0, 1, 2, 3, 4, 5]
    else:
        assert info[0]["bbox"] == f.bbox
    if version == 101:
        assert info[0]["clusters"] == 2
    L1, _, ts1, _ = f.read(1)
    assert len(L1) == 2 and ts1 == (1.5 if version >= 102 else 1.0)
    L2, _, _, _ = f.read(2)
    assert L2 == []
    f.close()


def test_rejects_bad_files(tmp_path):
    p = tmp_path / "bad.mmpld"
    p.write_bytes(b"MMPLX\0" + bytes(100))
    with pytest.raises(p2v.P2VError):
        p2v.Mmpld(p)
    rng = np.random.default_rng(1)
    lists, _ = make_lists(rng)
    good = tmp_path / "good.mmpld"
    mmpld_io.write(good, [(0.0, lists)], version=103)
    data = good.read_bytes()
    trunc = tmp_path / "trunc.mmpld"
    trunc.write_bytes(data[:-40])  # frame table points past the end
    with pytest.raises(p2v.P2VError):
        p2v.Mmpld(trunc)
    with pytest.raises(p2v.P2VError):
        p2v.Mmpld(tmp_path / "missing.mmpld")


def test_corrupt_list_count_is_an_error(tmp_path):
    rng = np.random.default_rng(2)
    lists, _ = make_lists(rng)
    lists[0]["count"] = 10 ** 9  # records run past the frame
    p = tmp_path / "corrupt.mmpld"
    mmpld_io.write(p, [(0.0, lists)], version=103)
    f = p2v.Mmpld(p)
    with pytest.raises(p2v.P2VError):
        f.read(0)


# ---- parity with MegaMol's own reader -------------------------------------------------------------------
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MMPLD_GOLDEN = sorted(n[6:-4] for n in os.listdir(GOLDEN) if n.startswith("mmpld_") and n.endswith(".npz"))
RECORD_BYTES = ({0: 0, 1: 12, 2: 16, 3: 6, 4: 24}, {0: 0, 1: 3, 2: 4, 3: 12, 4: 16, 5: 4, 6: 8, 7: 8})


def packed_records(ptr, stride, count, nbytes):
    """The `nbytes` leading bytes of each of `count` records `stride` apart, packed."""
    import ctypes as C

    if count == 0 or nbytes == 0:
        return np.zeros(0, np.uint8)
    buf = (C.c_uint8 * (stride * (count - 1) + nbytes)).from_address(ptr)
    raw = np.frombuffer(buf, np.uint8)
    idx = (np.arange(count)[:, None] * stride + np.arange(nbytes)[None, :]).ravel()
    return raw[idx].copy()


def compare_with_reference(f, ref_frames, ref_bbox, ref_clipbox, frame_lists):
    """Our reader `f` against what MMPLDDataSource published: the extent (GetExtent, :469-481) and per frame
    every list's types, count, global radius and colour, colour map range, record strides, the version 1.3
    list box, the version 1.1 cluster count, and the vertex and colour bytes."""
    assert f.frames == ref_frames
    assert f.bbox == list(ref_bbox) and f.clipbox == list(ref_clipbox)
    for fi, ref_lists in enumerate(frame_lists):
        lists, info, _, buf = f.read(fi, max_lists=256)
        assert len(lists) == len(ref_lists), fi
        for L, li, R in zip(lists, info, ref_lists):
            meta = R["meta"]
            vt, ct, count = int(meta[0]), int(meta[1]), int(meta[2])
            assert (L.vertex_type, L.colour_type, L.count) == (vt, ct, count)
            assert np.float32(L.global_radius) == np.float32(meta[3])
            assert tuple(L.global_colour) == tuple(int(x) for x in meta[4:8])
            assert [np.float32(x) for x in li["intensity_range"]] == [np.float32(meta[8]), np.float32(meta[9])]
            vb, cb = RECORD_BYTES[0][vt], RECORD_BYTES[1][ct]
            if vb:
                assert L.stride == int(meta[10])
                assert np.array_equal(packed_records(L.data, L.stride, count, vb), R["vertex"])
            if cb:
                assert L.colour_stride == int(meta[11])
                assert np.array_equal(packed_records(L.colour, L.colour_stride, count, cb), R["colour"])
            if f.version >= 103:
                assert [np.float32(x) for x in li["bbox"]] == [np.float32(x) for x in meta[12:18]]
            assert li["clusters"] == int(meta[18])
        del buf


@pytest.mark.parametrize("name", MMPLD_GOLDEN)
def test_reader_matches_reference_reader_golden(tmp_path, name):
    """Golden frames published by MegaMol's own MMPLDDataSource (tests/golden/make_golden.py): every vertex
    and colour type, lists without vertex data, unknown colour types, empty lists and frames."""
    z = np.load(os.path.join(GOLDEN, f"mmpld_{name}.npz"))
    path = tmp_path / f"{name}.mmpld"
    path.write_bytes(z["mmpld"].tobytes())
    frame_lists = []
    for fi in range(int(z["frames"])):
        frame_lists.append([dict(meta=z[f"f{fi}_l{li}_meta"], vertex=z[f"f{fi}_l{li}_vertex"],
                                 colour=z[f"f{fi}_l{li}_colour"]) for li in range(int(z[f"f{fi}_nlists"]))])
    f = p2v.Mmpld(path)
    compare_with_reference(f, int(z["frames"]), z["bbox"], z["clipbox"], frame_lists)
    f.close()


def _reference_reader_built():
    import oracle
    return os.path.exists(oracle.REF_MMPLD_SO)


@pytest.mark.skipif(not _reference_reader_built(), reason="reference MMPLDDataSource build not present")
@pytest.mark.parametrize("seed", range(6))
def test_reader_matches_live_reference_reader(tmp_path, seed):
    """Random files (versions, list mixes, several frames) read by both readers."""
    import oracle
    rng = np.random.default_rng(1000 + seed)
    version = [100, 101, 102, 103][seed % 4]
    frames = []
    for _ in range(int(rng.integers(1, 4))):
        lists = mmpld_io.mixed_lists(rng)
        keep = rng.permutation(len(lists))[:int(rng.integers(0, len(lists) + 1))]
        frames.append((float(rng.uniform(0, 10)), [lists[k] for k in keep]))
    path = tmp_path / f"r{seed}.mmpld"
    mmpld_io.write(path, frames, version=version, bbox=tuple(rng.uniform(-9, 0, 3)) + tuple(rng.uniform(1, 9, 3)))
    r = oracle.reference_mmpld(path)
    frame_lists = []
    for lists in r["frame_lists"]:
        out = []
        for L in lists:
            vb = oracle.VERTEX_RECORD_BYTES.get(L["vert_type"], 0)
            cb = oracle.COLOUR_RECORD_BYTES.get(L["col_type"], 0)
            meta = np.array([L["vert_type"], L["col_type"], L["count"], L["global_radius"], *L["global_colour"],
                             L["col_min"], L["col_max"], L["vert_stride"] or vb, L["col_stride"] or cb, *L["bbox"],
                             L["clusters"], L["cluster_bytes"]], np.float64)
            out.append(dict(meta=meta, vertex=L["vertex"], colour=L["colour"]))
        frame_lists.append(out)
    f = p2v.Mmpld(path)
    compare_with_reference(f, r["frames"], r["bbox"], r["clipbox"], frame_lists)
    f.close()
