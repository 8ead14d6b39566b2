"""The allocation-free AOSphere AO entry point, called through the C ABI.

It exists for callers that cannot allocate device memory while they compute AO (a renderer recording a
CUDA graph, a host with a fixed memory budget). Its output must equal what the allocating entry point
(p2v_run_frame with an AOSphere AO mode) produces for the same particles, on two calls in a row (the
static scratch keeps the previous call's contents, so the second call checks that it is cleared).
This file is collected last so a failure here cannot hide another test's result."""
import ctypes as C

import numpy as np
import pytest

from megamol_gb300 import build as nbuild
from megamol_gb300 import p2v, synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [p2v.AO_AOSPHERE_AXES, p2v.AO_AOSPHERE_NORMAL])
def test_noalloc_aosphere_matches_allocating_entry_point(mode):
    torch = pytest.importorskip("torch")
    nbuild.build()
    lib = p2v.library()
    f = synth.uniform(n=30_000, edge=25.0, res=32, seed=91)
    f.xyzr[:, 3] = np.random.default_rng(92).uniform(0.3, 0.9, f.n).astype(np.float32)
    nrm3 = synth.random_normals(f.n, 93)
    size = (40, 36, 44)

    ctx = p2v.Context(0)
    ctx.set_params(sizex=16, sizey=16, sizez=16, ao_mode=mode, aos_sizex=size[0], aos_sizey=size[1],
                   aos_sizez=size[2], aos_step_len=0.5, aos_gen_fac=1.0, aos_eval_fac=1.0)
    ref = np.full(f.n, np.nan, np.float32)
    ctx.run_frame([p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR, normals=nrm3, ao_out=ref)], f.bbox)
    ctx.close()

    d_xyzr = torch.from_numpy(f.xyzr).cuda()
    nrm4 = np.zeros((f.n, 4), np.float32)
    nrm4[:, :3] = nrm3
    d_nrm = torch.from_numpy(nrm4).cuda()
    clip = (C.c_float * 6)(*f.bbox)
    vs = (C.c_int32 * 3)(*size)
    for call in range(2):
        d_ao = torch.full((f.n,), float("nan"), dtype=torch.float32, device="cuda")
        st = lib.p2v_aosphere_ao_noalloc(d_xyzr.data_ptr(), d_nrm.data_ptr(), f.n, clip, vs, 0.5, 1.0, 1.0, mode,
                                         d_ao.data_ptr(), None)
        assert st == p2v.OK, f"call {call}: status {st}"
        torch.cuda.synchronize()
        got = d_ao.cpu().numpy()
        assert np.abs(got - ref).max() <= 1e-5, f"call {call}: max diff {np.abs(got - ref).max()}"


def test_noalloc_rejects_volumes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    lib = p2v.library()
    d = torch.zeros((4, 4), dtype=torch.float32, device="cuda")
    ao = torch.zeros(4, dtype=torch.float32, device="cuda")
    clip = (C.c_float * 6)(0, 0, 0, 1, 1, 1)
    edge = round(p2v.NOALLOC_MAX_VOXELS ** (1 / 3))
    assert edge ** 3 == p2v.NOALLOC_MAX_VOXELS
    too_big = (C.c_int32 * 3)(edge + 1, edge, edge)
    st = lib.p2v_aosphere_ao_noalloc(d.data_ptr(), d.data_ptr(), 4, clip, too_big, 0.5, 1.0, 1.0,
                                     p2v.AO_AOSPHERE_AXES, ao.data_ptr(), None)
    assert st == p2v.EINVAL


def test_noalloc_rejects_sizes_whose_product_wraps():
    """(2^21, 2^21, 2^22) voxels multiply to 2^64, which wraps to 0 in 64 bits; the size check must still
    reject it. With count 0 no kernel would run even if the check let it through."""
    torch = pytest.importorskip("torch")
    lib = p2v.library()
    ao = torch.zeros(4, dtype=torch.float32, device="cuda")
    clip = (C.c_float * 6)(0, 0, 0, 1, 1, 1)
    for size in [(1 << 21, 1 << 21, 1 << 22), (1 << 30, 1 << 30, 1 << 4), (3, 3, p2v.NOALLOC_MAX_VOXELS + 1)]:
        vs = (C.c_int32 * 3)(*size)
        st = lib.p2v_aosphere_ao_noalloc(ao.data_ptr(), ao.data_ptr(), 0, clip, vs, 0.5, 1.0, 1.0,
                                         p2v.AO_AOSPHERE_AXES, ao.data_ptr(), None)
        assert st == p2v.EINVAL, size
