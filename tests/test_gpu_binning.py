"""GPU test of the cell binning: the sort of the bin keys must equal a CPU stable sort bit for bit (sorted
keys, permutation and cell starts), for ordinary, ragged, out-of-box, invalid and crowded inputs and at the
full LJ-liquid size (4,000,000 particles, 256^3 grid, 25-bit keys). Both sorting paths are covered: the
counting sort by cell (cells of at most 32 particles, ordered by index within the cell) and the radix sort,
alone (cell table much larger than the particle count) or as the fallback for a fuller cell."""
import numpy as np
import pytest

import oracle
from megamol_gb300 import build as nbuild
from megamol_gb300 import p2v, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    nbuild.build()
    c = p2v.Context(0)
    yield c
    c.close()


def check(ctx, xyzr, bbox, res, lists=None):
    ctx.set_params(sizex=res[0], sizey=res[1], sizez=res[2], ao_mode=p2v.AO_NONE, normalize=0,
                   forSurfaceReconstruction=0)
    ctx.run_frame(lists or [p2v.ParticleList(xyzr, p2v.VERTDATA_FLOAT_XYZR)], bbox, None)
    keys, order, start = ctx.binning()
    rk, ro, rs = oracle.binning(xyzr, bbox, res)
    nbins = rs.size - 1
    if keys.size and keys.max() > nbins:
        # the radix path sorts the particles whose support holds no node after all others, by a key bit above
        # the cells: each of them must miss every node (FP64), and the order must be the stable sort by
        # (that bit, cell)
        flag = 1 << int(nbins).bit_length()
        n = keys.size
        pf = np.zeros(n, bool)
        pf[order[keys > nbins]] = True
        assert np.all(oracle.support_misses_nodes_f64(xyzr, bbox, res)[pf])
        ck = np.empty(n, np.uint32)
        ck[ro] = rk
        ro = np.lexsort((np.arange(n), ck, pf)).astype(np.uint32)
        rk = (ck[ro] | np.where(pf[ro], flag, 0)).astype(np.uint32)
        rs = np.searchsorted(rk, np.arange(nbins + 1, dtype=np.int64), side="left").astype(np.uint32)
    assert np.array_equal(keys, rk)
    assert np.array_equal(order, ro)
    assert np.array_equal(start, rs)
    return ctx.stats()["cell_max_count"]


COUNTING = range(1, 33)   # cell_max_count of a frame the counting sort took


def test_uniform_frame(ctx):
    f = synth.uniform(n=200_000, edge=50.0, res=64, seed=3)
    assert check(ctx, f.xyzr, f.bbox, f.res) in COUNTING


@pytest.mark.parametrize("fill,invalid", [(32, 0), (33, 0), (1, 32), (1, 33)])
def test_cell_occupancy_limit(ctx, fill, invalid):
    """One cell holding exactly `fill` particles, `invalid` particles with a NaN coordinate (they share
    the invalid key): 32 stays with the counting sort, 33 sends the frame through the radix sort."""
    rng = np.random.default_rng(fill + 100 * invalid)
    n = 40_000
    x = np.empty((n, 4), np.float32)
    x[:, :3] = rng.uniform(0, 30, (n, 3))
    x[:, 3] = 0.6
    # move every particle of cell (10, 10, 10) out, then put `fill` particles into it at scattered indices
    h = 30.0 / 29.0
    cell = np.floor(x[:, :3] / np.float32(h)).astype(int)
    hit = np.all(cell == 10, axis=1)
    x[hit, :3] = np.float32(0.1)
    idx = rng.choice(np.flatnonzero(~hit), fill + invalid, replace=False)
    x[idx[:fill], :3] = rng.uniform(10.05 * h, 10.95 * h, (fill, 3)).astype(np.float32)
    x[idx[fill:], 1] = np.nan
    m = check(ctx, x, (0.0, 0.0, 0.0, 30.0, 30.0, 30.0), (30, 30, 30))
    assert (m in COUNTING) == (max(fill, invalid) <= 32), m


def test_out_of_box_invalid_and_crowded(ctx):
    rng = np.random.default_rng(4)
    n = 150_000
    x = np.empty((n, 4), np.float32)
    x[:, :3] = rng.uniform(-20, 60, (n, 3))       # a third outside the box: underflow / overflow bins
    x[:, 3] = rng.uniform(0.2, 1.0, n)
    x[::11, :3] = np.float32(17.25)                # one crowded cell (~14k particles)
    x[5::97, 3] = 0.0                              # invalid radius
    x[7::101, 1] = np.nan                          # invalid coordinate
    assert check(ctx, x, (0.0, 0.0, 0.0, 40.0, 40.0, 40.0), (48, 40, 56)) > 32   # the radix fallback


def test_ragged_sizes(ctx):
    rng = np.random.default_rng(5)
    for n in (1, 31, 4095, 4096, 4097, 70_001):
        x = np.concatenate([rng.uniform(0, 10, (n, 3)), np.full((n, 1), 0.5)], 1).astype(np.float32)
        m = check(ctx, x, (0, 0, 0, 10, 10, 10), (20, 20, 20))
        assert (m == 0) == (22 ** 3 > 64 * n), (n, m)   # a sparse frame: the radix sort alone


def test_mixed_list_types(ctx):
    rng = np.random.default_rng(6)
    a = rng.uniform(0, 30, (5000, 3)).astype(np.float64)
    b = rng.integers(0, 30, (3000, 3)).astype(np.uint16)
    c = np.concatenate([rng.uniform(0, 30, (4000, 3)), np.full((4000, 1), 0.7)], 1).astype(np.float32)
    lists = [p2v.ParticleList(a, p2v.VERTDATA_DOUBLE_XYZ, global_radius=0.5),
             p2v.ParticleList(b, p2v.VERTDATA_SHORT_XYZ, global_radius=0.6),
             p2v.ParticleList(c, p2v.VERTDATA_FLOAT_XYZR)]
    packed = np.concatenate([np.column_stack([a.astype(np.float32), np.full(len(a), 0.5, np.float32)]),
                             np.column_stack([b.astype(np.float32), np.full(len(b), 0.6, np.float32)]), c])
    check(ctx, packed, (0, 0, 0, 30, 30, 30), (33, 30, 31), lists=lists)


def test_lj_liquid_full_size(ctx):
    f = synth.lj_liquid(seed=2)
    assert check(ctx, f.xyzr, f.bbox, f.res) in COUNTING


@pytest.mark.parametrize("n", [1, 2, 37])
def test_long_empty_runs(ctx, n):
    """A sparse frame on a 160^3 grid (4.3M cells): the cell starts of runs of up to millions of empty cells,
    which the fill takes in chunks of 8192 cells."""
    rng = np.random.default_rng(90 + n)
    x = np.empty((n, 4), np.float32)
    x[:, :3] = rng.uniform(0, 100, (n, 3))
    x[:, 3] = 0.5
    h = np.float32(100.0 / 159.0)
    if n >= 2:  # the second particle 50 rows of cells after the first: a run of about 8100 cells between them
        x[1, :3] = x[0, :3]
        x[1, 1] += np.float32(50.0) * h
        x[1, 0] = np.float32(0.25) * h
    assert check(ctx, x, (0.0, 0.0, 0.0, 100.0, 100.0, 100.0), (160, 160, 160)) == 0   # the radix sort


@pytest.mark.parametrize("with_ao", [False, True])
def test_lookback_wait_runs_out_and_the_context_survives(ctx, with_ao):
    """The radix sort's bounded decoupled look-back: with the test hook the second tile of the first pass never
    publishes its digit counts, so the tiles after it poll sort_wait_polls times, record the timeout, and the
    sort's unfinished output is replaced by a valid one (every particle in the invalid cell, identity order)
    before a later stage reads it. p2v_run_frame reports P2V_ETIMEOUT; the next frame on the same context gives
    the bits of a frame before the timeout. with_ao: the AO stages (mip levels, gradient normals, cone march)
    run on that output as well."""
    rng = np.random.default_rng(95)
    n = 30_000  # 8 sort tiles of 4096 keys; 162^3 cells > 64 n: the radix sort alone
    x = np.empty((n, 4), np.float32)
    x[:, :3] = rng.uniform(0, 50, (n, 3))
    x[:, 3] = rng.uniform(0.4, 0.6, n)
    bbox = (0.0, 0.0, 0.0, 50.0, 50.0, 50.0)
    ao_params = dict(ao_mode=p2v.AO_CONE, ao_volume=p2v.AOVOL_DENSITY, ao_volume_scale=1.0, ao_cones=8,
                     ao_steps=32, ao_levels=3, ao_normals=p2v.NORMALS_GRADIENT) if with_ao else dict(ao_mode=p2v.AO_NONE)

    def frame():
        ctx.set_params(sizex=160, sizey=160, sizez=160, normalize=1, forSurfaceReconstruction=0, **ao_params)
        vol = np.full(160 ** 3, np.nan, np.float32)
        ao = np.full(n, np.nan, np.float32)
        ctx.run_frame([p2v.ParticleList(x, p2v.VERTDATA_FLOAT_XYZR, ao_out=ao if with_ao else None)], bbox, vol)
        return vol, ao

    before = frame()
    assert ctx.stats()["cell_max_count"] == 0  # the radix path
    ctx.set_params(sort_wait_polls=1000, test_hold_sort=1)
    with pytest.raises(p2v.P2VError) as err:
        frame()
    assert err.value.status == p2v.ETIMEOUT
    ctx.set_params(sort_wait_polls=0, test_hold_sort=0)
    after = frame()
    assert np.array_equal(before[0], after[0])
    assert np.array_equal(before[1], after[1], equal_nan=True)
    ctx.set_params(ao_mode=p2v.AO_NONE, ao_normals=p2v.NORMALS_LIST)
