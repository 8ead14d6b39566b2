"""The dat/raw writer (p2v_write_datraw) against MegaMol's own volume::DatRawWriter
(plugins/volume/src/DatRawWriter.cpp:58-186): byte-identical .dat headers and .raw payloads for host
volumes, against fixtures the reference module wrote (tests/golden/datraw_*.npz) and, where the reference
tree is compiled here, against the module run live; the same refusals (empty prefix, bare directory,
frame past the frame count). The device path (streamed through pinned buffers) is in test_gpu_datraw.py."""
import glob
import os

import numpy as np
import pytest

import oracle
from megamol_gb300 import build as nbuild
from megamol_gb300 import p2v
from tests import golden_io as G

CASES = sorted(os.path.basename(p)[7:-4] for p in glob.glob(os.path.join(G.GOLDEN, "datraw_*.npz")))


@pytest.fixture(scope="module", autouse=True)
def lib():
    nbuild.build()
    return p2v.library()


def load(name):
    z = np.load(os.path.join(G.GOLDEN, f"datraw_{name}.npz"))
    return {k: z[k] for k in z.files}


def meta_of(c):
    return dict(resolution=[int(v) for v in c["resolution"]], components=int(c["components"]),
                slice_dists=[float(v) for v in c["slice_dists"]], origin=[float(v) for v in c["origin"]])


def read_pair(stem):
    with open(stem + ".dat", "rb") as f:
        dat = f.read()
    with open(stem + ".raw", "rb") as f:
        raw = f.read()
    return dat, raw


@pytest.mark.parametrize("name", CASES)
def test_host_volume_matches_reference_fixture(tmp_path, name):
    c = load(name)
    frame = int(c["frame"])
    p2v.write_datraw(str(tmp_path / "vol_"), frame, c["volume"], meta_of(c), int(c["frame_count"]))
    dat, raw = read_pair(str(tmp_path / f"vol_{frame:04d}"))
    assert dat == bytes(c["dat"])
    assert raw == bytes(c["raw"])


@pytest.mark.skipif(not os.path.exists(oracle.REF_DATRAW_SO), reason="reference writer not compiled here")
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_host_volume_matches_reference_live(tmp_path, seed):
    rng = np.random.default_rng(seed)
    res = [int(v) for v in rng.integers(2, 9, 3)]
    comps = int(rng.choice([1, 3]))
    vol = rng.normal(size=int(np.prod(res)) * comps).astype(np.float32) * np.float32(10.0 ** rng.integers(-8, 9))
    sd = rng.uniform(1e-3, 50.0, 3).astype(np.float32)
    org = rng.uniform(-1e4, 1e4, 3).astype(np.float32)
    frame = int(rng.integers(0, 3000))
    (tmp_path / "ref").mkdir()
    (tmp_path / "gpu").mkdir()
    assert oracle.reference_write_datraw(str(tmp_path / "ref" / "v"), frame, vol, res, comps, sd, org, frame + 1)
    meta = dict(resolution=res, components=comps, slice_dists=sd.tolist(), origin=org.tolist())
    p2v.write_datraw(str(tmp_path / "gpu" / "v"), frame, vol, meta, frame + 1)
    assert read_pair(str(tmp_path / "ref" / f"v{frame:04d}")) == read_pair(str(tmp_path / "gpu" / f"v{frame:04d}"))


def test_refusals_match_the_reference(tmp_path):
    c = load(CASES[0])
    meta = meta_of(c)
    for prefix, frame, count in [("", 0, 1), (str(tmp_path) + "/", 0, 1), (str(tmp_path / "x"), 5, 5)]:
        with pytest.raises(p2v.P2VError):
            p2v.write_datraw(prefix, frame, c["volume"], meta, count)
        if os.path.exists(oracle.REF_DATRAW_SO):
            assert not oracle.reference_write_datraw(prefix, frame, c["volume"], meta["resolution"],
                                                     meta["components"], meta["slice_dists"], meta["origin"], count)
    assert not os.path.exists(str(tmp_path / "x0005.dat"))
    small = np.zeros(3, np.float32)   # capacity below the resolution
    with pytest.raises(p2v.P2VError):
        p2v.write_datraw(str(tmp_path / "y"), 0, small, meta)
