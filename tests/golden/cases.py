"""Small deterministic box sets shared by the fixture generator and the tests.

Each case is (name, boxes[n, 2*dims+1] uint32 RectInfo rows, range). They
cover the edge cases of the reference's semantics: closed intervals
(touching faces, edges and corners overlap), zero-extent boxes, identical
boxes with distinct rids, coordinates at range-1, a box spanning the whole
domain, cells far above 256 boxes, empty and single-box scenes, ragged sizes.
"""
from __future__ import annotations

import numpy as np

R24 = 1 << 24


def _rect(rows, dims):
    a = np.asarray(rows, dtype=np.uint32).reshape(-1, 2 * dims)
    rid = np.arange(a.shape[0], dtype=np.uint32)[:, None]
    return np.ascontiguousarray(np.concatenate([a, rid], axis=1))


def _random(n, dims, rng_seed, range_, side_max, side_min=0):
    rng = np.random.default_rng(rng_seed)
    lo = rng.integers(0, range_, size=(n, dims), dtype=np.int64)
    side = rng.integers(side_min, side_max + 1, size=(n, dims), dtype=np.int64)
    hi = np.minimum(lo + side, range_ - 1)
    rows = np.empty((n, 2 * dims), dtype=np.int64)
    rows[:, 0::2] = lo
    rows[:, 1::2] = hi
    return _rect(rows, dims)


def cases():
    out = []
    # touching faces / edges / corners and a gap of one unit (3-D)
    out.append(("touching3d", _rect([
        [0, 10, 0, 10, 0, 10],
        [10, 20, 0, 10, 0, 10],      # shares the face x=10 with box 0
        [21, 30, 0, 10, 0, 10],      # one unit away from box 1
        [20, 20, 10, 10, 10, 10],    # point on the corner of box 1
        [0, 30, 11, 11, 0, 30],      # thin slab one unit above boxes 0,1
        [5, 5, 5, 5, 5, 5],          # point inside box 0
        [5, 5, 5, 5, 5, 5],          # identical point (distinct rid)
    ], 3), 64))
    out.append(("touching2d", _rect([
        [0, 4, 0, 4], [4, 8, 4, 8], [9, 9, 0, 8], [8, 8, 8, 8], [0, 15, 0, 0], [15, 15, 15, 15],
    ], 2), 16))
    out.append(("empty3d", np.zeros((0, 7), dtype=np.uint32), 100))
    out.append(("single3d", _rect([[1, 2, 1, 2, 1, 2]], 3), 100))
    out.append(("pair_max_coord", _rect([[R24 - 1, R24 - 1] * 3, [R24 - 2, R24 - 1] * 3], 3), R24))
    # many identical boxes: one cell far above 256 and 512 boxes
    out.append(("identical700", _rect([[100, 200, 100, 200, 100, 200]] * 700, 3), 1000))
    # one box spanning the domain plus small ones
    big = _random(3000, 3, 7, 1 << 16, 300)
    big[0, :6] = [0, (1 << 16) - 1] * 3
    out.append(("domain_box", big, 1 << 16))
    # random ragged sizes, 2-D and 3-D, dense and sparse
    out.append(("rand3d_1001", _random(1001, 3, 1, 10000, 400), 10000))
    out.append(("rand2d_4097", _random(4097, 2, 2, 1 << 20, 20000), 1 << 20))
    out.append(("rand3d_dense_20000", _random(20000, 3, 3, 4096, 120), 4096))
    out.append(("rand3d_points_30000", _random(30000, 3, 4, 64, 0), 64))  # many coincident points
    out.append(("rand3d_mixed_50000", _random(50000, 3, 5, 1 << 24, 400000, 1), 1 << 24))
    return out
