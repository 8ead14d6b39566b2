"""Full-size GPU checks of the two large workloads, through size-independent properties:

* the large mixed-phase frame (64,000,000 particles: FCC slab + gas, radii 0.5/0.8/1.2, 512^3 grid) and the
  learned-AO inference set (16,000,000 uniform particles of the small case's structure, 695^3 grid);
* each grid is deterministic bit for bit, and a z-slab of it equals the FP64 oracle computed from the
  particles that reach the slab (sharding.slab_particle_mask) within the density bar (1e-6 of the slab
  maximum); the cell binning stays sorted with consistent cell starts;
* on the 16M set (Gaussian 3-sigma kernel) the learned AO, trained only on cone-march pairs of the two
  smaller configurations (uniform 100k Gaussian frames and LJ frames), stays within RMSE 0.02 of the plain
  cone march and marches only a small fraction of the particles through the fallback."""
import numpy as np
import pytest

import oracle
from megamol_gb300 import build as nbuild
from megamol_gb300 import p2v, sharding, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    nbuild.build()
    c = p2v.Context(0)
    yield c
    c.close()


def density(ctx, f, kernel=p2v.KERNEL_BUMP):
    ctx.set_params(sizex=f.res[0], sizey=f.res[1], sizez=f.res[2], cyclX=1, cyclY=1, cyclZ=1, normalize=0,
                   sigma=1.0, kernel=kernel, accumulate=p2v.ACCUM_EXACT, ao_mode=p2v.AO_NONE, mass_normalize=0)
    vol = np.empty(f.res[0] * f.res[1] * f.res[2], np.float32)
    ctx.run_frame([p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR)], f.bbox, vol)
    return vol.reshape(f.res[2], f.res[1], f.res[0])


def check_slab(f, grid, z0, z1, kernel):
    keep = sharding.slab_particle_mask(f.xyzr, f.bbox, f.res, True, z0, z1,
                                       1.0 if kernel == p2v.KERNEL_BUMP else 3.0)
    ref = oracle.density_f64(f.xyzr[keep], f.bbox, f.res, (1, 1, 1), 1.0, kernel, 1)[z0:z1]
    got = grid[z0:z1].astype(np.float64)
    assert ref.max() > 0
    assert np.abs(got - ref).max() <= 1e-6 * np.abs(ref).max()


def check_binning(ctx, n):
    keys, order, start = ctx.binning()
    assert keys.size == n and np.all(np.diff(keys.astype(np.int64)) >= 0)
    assert np.array_equal(np.sort(order), np.arange(n, dtype=np.uint32))
    for b in np.unique(keys)[:: max(1, np.unique(keys).size // 64)]:
        if b < start.size - 1:
            assert start[b] <= start[b + 1] and np.all(keys[start[b]:start[b + 1]] == b)


def test_mixed_phase_64M(ctx):
    f = synth.mixed_phase()
    assert f.n == 64_000_000 and f.res == (512, 512, 512)
    g1 = density(ctx, f)
    check_binning(ctx, f.n)
    g2 = density(ctx, f)
    assert np.array_equal(g1, g2)
    for z0 in (0, 200, 504):
        check_slab(f, g1, z0, z0 + 8, p2v.KERNEL_BUMP)


def _gradient_normals(ctx, f, kernel):
    ctx.set_params(sizex=f.res[0], sizey=f.res[1], sizez=f.res[2], cyclX=1, cyclY=1, cyclZ=1, normalize=1,
                   sigma=1.0, kernel=kernel, ao_mode=p2v.AO_NONE, mass_normalize=0)
    vol = np.empty(f.res[0] * f.res[1] * f.res[2], np.float32)
    ctx.run_frame([p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR)], f.bbox, vol)
    return synth.gradient_normals(f.xyzr, vol.reshape(f.res[2], f.res[1], f.res[0]), f.bbox)


def test_uniform_16M_density_and_learned_ao(ctx):
    """The learned-AO inference set (16M particles of the small case's structure, Gaussian 3-sigma kernel):
    density against FP64 on a slab, and the learned AO trained on pairs of the two smaller configurations only
    (uniform 100k Gaussian frames and LJ frames, other seeds) within RMSE 0.02 of the plain cone march."""
    n = 16_000_000
    scale = (n / 100_000) ** (1.0 / 3.0)
    f = synth.uniform(n=n, edge=100.0 * scale, res=int(round(128 * scale)), seed=1)
    g = density(ctx, f, p2v.KERNEL_GAUSS3)
    check_slab(f, g, 300, 306, p2v.KERNEL_GAUSS3)
    ao_params = dict(ao_volume=p2v.AOVOL_DENSITY, ao_volume_scale=1.0, ao_cones=8, ao_steps=32, ao_levels=3,
                     ao_apex_deg=50.0, ao_offset=0.01, ao_strength=1.0, ao_cone_length=0.8, ao_early_exit=1)
    ctx.mlp_clear()
    train = [(synth.uniform(n=100_000, seed=10 + k), 100_000, p2v.KERNEL_GAUSS3) for k in range(10)]
    train += [(synth.lj_liquid(seed=s), 500_000, p2v.KERNEL_BUMP) for s in (3, 4)]
    for k, (t, npairs, kern) in enumerate(train):
        nt = _gradient_normals(ctx, t, kern)
        ctx.set_params(**ao_params)
        ctx.mlp_collect([p2v.ParticleList(t.xyzr, p2v.VERTDATA_FLOAT_XYZR, normals=nt)], t.bbox, npairs, seed=k)
    ctx.mlp_train(seed=3)
    nrm = _gradient_normals(ctx, f, p2v.KERNEL_GAUSS3)
    ctx.set_params(**ao_params)
    plain = np.empty(f.n, np.float32)
    ctx.set_params(ao_mode=p2v.AO_CONE)
    ctx.run_frame([p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR, normals=nrm, ao_out=plain)], f.bbox, None)
    learned = np.empty(f.n, np.float32)
    ctx.set_params(ao_mode=p2v.AO_LEARNED)
    ctx.run_frame([p2v.ParticleList(f.xyzr, p2v.VERTDATA_FLOAT_XYZR, normals=nrm, ao_out=learned)], f.bbox, None)
    st = ctx.stats()
    rmse = float(np.sqrt(np.mean((learned.astype(np.float64) - plain) ** 2)))
    assert np.isfinite(learned).all() and 0.0 <= learned.min() and learned.max() <= 1.0
    assert rmse <= 0.02, rmse
    assert st["ao_fallback"] <= 0.05 * f.n, st["ao_fallback"]
