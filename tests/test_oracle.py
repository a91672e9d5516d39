"""The oracle (CPU restatement of the reference path) pinned against the
reference's own published results and cross-checked with brute force."""
import ctypes
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))


def test_glibc_rand_restatement_matches_libc():
    libc = ctypes.CDLL("libc.so.6")
    for seed in (1, 100, 12345):
        libc.srand(seed)
        ref = [libc.rand() for _ in range(2000)]
        assert O.rand_sequence(seed, 2000) == ref


def test_golden_test1_uu_10m_pairs():
    """benchmarks/test1/filter_file:7 and test2/filter_file:7: 49 514 252
    pairs for check.PBIG -n 10000000 -S 100 -g 10000 -t UU (srand(100))."""
    boxes = O.harness_boxes(10_000_000, S=100, range_=10000, sim="UU")
    _, st = O.grid_pairs(boxes, 10000, count_only=True)
    assert st["pairs"] == 49_514_252
    assert st["cs"] == 128


@pytest.mark.slow
def test_golden_test3_un_10m_pairs_and_phase_stats():
    """benchmarks/test3/filter_file: 1 121 815 231 intersections, 16 683 783 392
    compared pairs, E = 26 668 901, 493 039 cells, 200 096 jobs, 219 batches,
    largest cell 3 543 (cs = 128), all reproduced by the restatement."""
    boxes = O.harness_boxes(10_000_000, S=100, range_=10000, sim="UN")
    _, st = O.grid_pairs(boxes, 10000, count_only=True)
    assert st["pairs"] == 1_121_815_231
    assert st["comp_pairs"] == 16_683_783_392
    assert st["entries"] == 26_668_901
    assert st["ncells"] == 493_039
    assert st["jobs"] == 200_096
    assert st["batches"] == 219
    assert st["max_cell"] == 3543
    assert st["cs"] == 128


def _rand_boxes(n, dims, seed, range_, side):
    rng = np.random.default_rng(seed)
    lo = rng.integers(0, range_, size=(n, dims))
    hi = np.minimum(lo + rng.integers(0, side + 1, size=(n, dims)), range_ - 1)
    rows = np.empty((n, 2 * dims), dtype=np.uint32)
    rows[:, 0::2] = lo
    rows[:, 1::2] = hi
    return np.ascontiguousarray(np.concatenate([rows, np.arange(n, dtype=np.uint32)[:, None]], axis=1))


@pytest.mark.parametrize("dims,cs", [(2, 0), (2, 1), (2, 16), (2, 1024), (2, 1 << 14),
                                     (3, 0), (3, 32), (3, 64), (3, 1024), (3, 1 << 14)])
def test_grid_restatement_equals_brute_force(dims, cs):
    b = _rand_boxes(3000, dims, 10 + dims, 10000, 300 if dims == 3 else 60)
    g, st = O.grid_pairs(b, 10000, cs=cs)
    assert np.array_equal(g, O.brute_pairs(b))
    assert st["pairs"] == len(g)


@pytest.mark.parametrize("dims", [2, 3])
def test_merged_mode_reports_the_same_pairs(dims):
    """MERGED=1 (h_merge_grids + d_postcounting) changes the work, not the
    pair set."""
    b = _rand_boxes(5000, dims, 3, 10000, 200 if dims == 3 else 40)
    a, st0 = O.grid_pairs(b, 10000, cs=256)
    m, st1 = O.grid_pairs(b, 10000, cs=256, merged=True)
    assert np.array_equal(a, m)
    assert st1["comp_pairs"] != st0["comp_pairs"] or st1["entries"] != st0["entries"]


def test_fixtures_reproduce():
    files = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))
    assert len(files) >= 16
    for f in files:
        z = np.load(f)
        boxes, rng, pairs = z["boxes"], int(z["range"]), z["pairs"]
        if len(boxes) == 0:
            assert len(pairs) == 0
            continue
        g, _ = O.grid_pairs(boxes, rng)
        assert np.array_equal(g, pairs), f
