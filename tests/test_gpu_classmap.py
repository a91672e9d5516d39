"""Parity at non-default work-list class maps (PBIG2_OPT_CLASS_MAP) and
merged-mode block limits (PBIG2_OPT_MERGE_LIMIT): the pair set must not
depend on which pair kernel takes a cell, nor on how cells are merged."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from pbig_gb300 import Engine, gen

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))

MAPS = [0x6666665544421000,   # 17..32 to one warp per cell
        0x6666665544444000,   # 5..32 to one warp per cell (the one-launch choice)
        0x6666665554321000,   # 65..128 to one block per cell
        0x6666665555321000,   # 33..128 to one block per cell
        0x6666665544331000,   # 9..16 in lane groups of 32
        0x6666665544322100,   # 3..8 in lane groups of 8 and 16
        0x6666666666666660]   # everything as 32x32 tile tasks


def canon(p):
    return O.sort_pairs(np.asarray(p, dtype=np.uint32).reshape(-1, 2))


@pytest.fixture(scope="module")
def eng():
    e = Engine(0)
    yield e
    e.close()


@pytest.mark.parametrize("one_launch", [True, False])
@pytest.mark.parametrize("name", ["rand3d_1001", "identical700", "rand2d_4097", "cfg2_clustered3d_16384",
                                  "touching3d"])
def test_fixture_at_every_map(eng, name, one_launch):
    z = np.load(os.path.join(HERE, "golden", name + ".npz"))
    boxes, rng, want = z["boxes"], int(z["range"]), z["pairs"]
    eng.set_one_launch(one_launch)
    try:
        for m in MAPS:
            eng.set_class_map(m)
            for _ in range(2):  # (a first result too large for a launch's buffers is redone)
                n = eng.self_intersect(boxes, rng)
                assert n == len(want), hex(m)
                assert np.array_equal(canon(eng.pairs()), want), hex(m)
            assert eng.stats()["class_map"] == m
    finally:
        eng.set_class_map(0)
        eng.set_one_launch(True)


def test_clustered_scene_and_red_blue_at_every_map(eng):
    """300 000 clustered boxes (cells of every class at the tuned size) and a
    red/blue query against the oracle."""
    boxes = gen.clustered3d(300000, seed=8)
    want, _ = O.grid_pairs(boxes, gen.RANGE, cs=1 << 16)
    red, blue = gen.mixed3d(60000, seed=2), gen.mixed3d(60000, seed=3)
    u = np.concatenate([red, blue])
    u[len(red):, -1] += len(red)
    allp = O.brute_pairs(u)
    cross = allp[(allp[:, 0] < len(red)) & (allp[:, 1] >= len(red))].copy()
    cross[:, 1] -= len(red)
    try:
        for m in MAPS:
            eng.set_class_map(m)
            assert eng.self_intersect(boxes, gen.RANGE, cell_shift=16) == len(want), hex(m)
            assert np.array_equal(canon(eng.pairs()), want), hex(m)
            assert eng.bipartite_intersect(red, blue, gen.RANGE) == len(cross), hex(m)
            got = eng.pairs()
            assert np.array_equal(got[np.lexsort((got[:, 1], got[:, 0]))], cross), hex(m)
        eng.set_class_map(0)
        eng.self_intersect(boxes, gen.RANGE, cell_shift=16)
        assert eng.stats()["class_map"] == 0x6666665544321000
    finally:
        eng.set_class_map(0)


@pytest.mark.parametrize("limit", [16, 64, 1024, 8192])
def test_merged_mode_at_other_block_limits(eng, limit):
    """The merge limit changes the blocks, not the pairs; the limit of the
    reference's build (256) is checked against the oracle's statistics in
    the merged-mode tests."""
    z = np.load(os.path.join(HERE, "golden", "rand3d_1001.npz"))
    boxes, rng, want = z["boxes"], int(z["range"]), z["pairs"]
    big = gen.clustered3d(100000, seed=6)
    want_big, _ = O.grid_pairs(big, gen.RANGE, cs=1 << 17)
    eng.set_merged(True)
    eng.set_merge_limit(limit)
    try:
        assert eng.self_intersect(boxes, rng) == len(want)
        assert np.array_equal(canon(eng.pairs()), want)
        assert eng.self_intersect(big, gen.RANGE, cell_shift=17) == len(want_big)
        st = eng.stats()
        assert st["merge_limit"] == limit and st["merged_blocks"] > 0
        assert np.array_equal(canon(eng.pairs()), want_big)
    finally:
        eng.set_merged(False)
        eng.set_merge_limit(0)
