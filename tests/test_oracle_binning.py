"""Known answers of the binning restatement (oracle.bin_keys / oracle.binning), CPU only."""
import numpy as np

import oracle


def test_bin_keys_known_answers():
    bbox = (0.0, 0.0, 0.0, 9.0, 9.0, 9.0)  # h = 1 for res 10
    res = (10, 10, 10)
    x = np.array([[0.0, 0.0, 0.0, 0.5],    # cell 0 -> bin 1
                  [9.0, 9.0, 9.0, 0.5],    # cell 9 -> bin 10
                  [-0.5, 4.2, 10.7, 0.5],  # cells -1, 4, 10 -> bins 0, 5, 11
                  [-7.0, 25.0, 3.0, 0.5],  # clamped to -1 and 10
                  [1.0, 2.0, 3.0, 0.0],    # radius 0: invalid
                  [np.nan, 1.0, 1.0, 0.5]], np.float32)
    keys, nbins = oracle.bin_keys(x, bbox, res)
    nb = 12
    assert nbins == nb ** 3
    k = lambda bx, by, bz: (bz * nb + by) * nb + bx
    assert list(keys) == [k(1, 1, 1), k(10, 10, 10), k(0, 5, 11), k(0, 11, 4), nbins, nbins]


def test_binning_is_a_stable_sort_with_cell_starts():
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.uniform(-1, 11, (500, 3)), rng.uniform(0.1, 1, (500, 1))], 1).astype(np.float32)
    x[::7, :3] = x[0, :3]  # many particles in one cell: order inside a cell = input order
    sk, order, start = oracle.binning(x, (0, 0, 0, 10, 10, 10), (8, 8, 8))
    assert np.all(np.diff(sk.astype(np.int64)) >= 0)
    same = order[sk == sk[np.searchsorted(sk, oracle.bin_keys(x[:1], (0, 0, 0, 10, 10, 10), (8, 8, 8))[0][0])]]
    assert np.all(np.diff(same.astype(np.int64)) > 0)
    for b in (0, 5, 100, len(start) - 2):
        assert np.all(sk[start[b]:start[b + 1]] == b)
