"""MMPLD frames through the GPU pipeline: a frame read by p2v_mmpld_read_frame (lists pointing into the
frame buffer, interleaved colour records in the stride) gives the same grid as the same particles passed as
packed arrays."""
import numpy as np
import pytest

from megamol_gb300 import build as nbuild
from megamol_gb300 import p2v
from tests import mmpld_io

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    nbuild.build()
    c = p2v.Context(0)
    yield c
    c.close()


def test_mmpld_frame_equals_packed_lists(ctx, tmp_path):
    rng = np.random.default_rng(5)
    a = np.concatenate([rng.uniform(0, 20, (30_000, 3)), rng.uniform(0.3, 0.8, (30_000, 1))], 1).astype(np.float32)
    ca = rng.integers(0, 255, (30_000, 4)).astype(np.uint8)
    b = rng.uniform(0, 20, (20_000, 3)).astype(np.float32)
    cb = rng.uniform(0, 1, (20_000, 1)).astype(np.float32)
    lists = [dict(vt=2, ct=2, count=a.shape[0], records=mmpld_io.records(a, ca)),
             dict(vt=1, ct=3, count=b.shape[0], records=mmpld_io.records(b, cb), radius=0.6, irange=(0.0, 1.0))]
    path = tmp_path / "f.mmpld"
    mmpld_io.write(path, [(0.0, lists), (1.0, lists[1:])], version=103, bbox=(0, 0, 0, 20, 20, 20))
    f = p2v.Mmpld(path)
    L, _, _, buf = f.read(0)
    ctx.set_params(sizex=40, sizey=40, sizez=40, ao_mode=p2v.AO_NONE, normalize=1, kernel=p2v.KERNEL_BUMP)
    got = np.empty(40 ** 3, np.float32)
    ctx.run_frame(L, f.bbox, got)
    ref = np.empty(40 ** 3, np.float32)
    ctx.run_frame([p2v.ParticleList(a, p2v.VERTDATA_FLOAT_XYZR),
                   p2v.ParticleList(b, p2v.VERTDATA_FLOAT_XYZ, global_radius=0.6)], f.bbox, ref)
    assert np.array_equal(got, ref)
    f.close()
