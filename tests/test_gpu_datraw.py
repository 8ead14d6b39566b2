"""The dat/raw writer's device path: a grid still in device memory (the context's last grid, or a CUDA
tensor) streams to the raw file through two pinned buffers; the files equal those of the host path
byte for byte, on a grid larger than one 32 MiB staging chunk."""
import numpy as np
import pytest

from megamol_gb300 import build as nbuild
from megamol_gb300 import p2v, synth

pytestmark = pytest.mark.gpu


def test_device_grid_streams_like_the_host_copy(tmp_path):
    nbuild.build()
    ctx = p2v.Context(0)
    try:
        f = synth.uniform(n=200_000, edge=100.0, res=208, seed=5)   # 208^3 floats = 34.4 MiB
        ctx.set_params(sizex=f.res[0], sizey=f.res[1], sizez=f.res[2], normalize=1, ao_mode=p2v.AO_NONE)
        host = np.empty(f.res[0] * f.res[1] * f.res[2], np.float32)
        meta = ctx.run_frame([p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR)], f.bbox, host)
        p2v.write_datraw(str(tmp_path / "host_"), 3, host, meta, 4)
        p2v.write_datraw(str(tmp_path / "dev_"), 3, None, meta, 4, ctx=ctx)
        a = [(tmp_path / f"host_0003.{e}").read_bytes() for e in ("dat", "raw")]
        b = [(tmp_path / f"dev_0003.{e}").read_bytes() for e in ("dat", "raw")]
        assert a[0].replace(b"host_", b"dev_") == b[0]
        assert len(a[1]) == host.nbytes and a[1] == b[1]
        torch = pytest.importorskip("torch")
        t = torch.from_numpy(host).cuda()
        p2v.write_datraw(str(tmp_path / "tensor_"), 3, t, meta, 4)
        assert (tmp_path / "tensor_0003.raw").read_bytes() == a[1]
    finally:
        ctx.close()
