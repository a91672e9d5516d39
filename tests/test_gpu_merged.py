"""MERGED=1 mode (pbig2_set_option(PBIG2_OPT_MERGED)) against the oracle's
restatement of the reference's merged build (h_merge_grids,
src/pbig/pbig.cu:1066-1251, and the first-visit rule of d_postcounting,
:223-318): the same pair set as ever, and the merged build's own work
statistics -- cell entries, numCompPairs, 256-row jobs, largest block, pair
tests. The plain mode's statistics are checked against the unmerged build."""
import numpy as np
import pytest

from oracle import oracle as O
from pbig_gb300 import gen

pytestmark = pytest.mark.gpu


def canon(p):
    return O.sort_pairs(np.asarray(p, dtype=np.uint32).reshape(-1, 2))


CASES = {
    # the reference harness's generator (main.cc:223-335), uniform centres,
    # range 10 000, cell size 128 -> 79^3 cells
    "harness_uu_3d": lambda: (O.harness_boxes(100000, S=100, range_=10000, sim="UU", seed=100), 10000, 128),
    "harness_uu_3d_s300": lambda: (O.harness_boxes(60000, S=300, range_=10000, sim="UU", seed=7), 10000, 128),
    "harness_uu_2d": lambda: (O.harness_boxes(50000, S=100, range_=10000, sim="UU", seed=3, dims=2), 10000, 64),
    # the build's own workloads on a fine grid (many sparse cells to merge)
    "clustered_3d": lambda: (gen.clustered3d(200000, seed=3), gen.RANGE, 1 << 17),
    "plain_2d": lambda: (gen.uniform2d(65536, seed=0), gen.RANGE, 1 << 14),
}


@pytest.mark.parametrize("merged", [False, True], ids=["plain", "merged"])
@pytest.mark.parametrize("name", sorted(CASES))
def test_work_statistics_of_the_reference_build(engine, name, merged):
    boxes, rng, cs = CASES[name]()
    want, st = O.grid_pairs(boxes, rng, cs=cs, merged=merged)
    engine.set_merged(merged)
    try:
        n = engine.self_intersect(boxes, rng, cell_shift=int(cs).bit_length() - 1)
        s = engine.stats()
        got = canon(engine.pairs())
    finally:
        engine.set_merged(False)
    assert n == len(want) and np.array_equal(got, want)
    assert s["entries"] == st["entries"]
    assert s["comp_pairs"] == st["comp_pairs"]
    assert s["jobs"] == st["jobs"]
    assert s["max_cell"] == st["max_cell"]
    assert s["pair_tests"] == st["tests"]
    assert (s["merged_blocks"] > 0) == merged


def test_merged_red_blue_pairs(engine):
    """The merged grid serves red/blue queries too (same cross pairs)."""
    red, blue = gen.mixed3d(60000, seed=0), gen.mixed3d(60000, seed=1)
    n0 = engine.bipartite_intersect(red, blue, gen.RANGE, cell_shift=17)
    want = engine.pairs()
    engine.set_merged(True)
    try:
        n1 = engine.bipartite_intersect(red, blue, gen.RANGE, cell_shift=17)
        got = engine.pairs()
        blocks = engine.stats()["merged_blocks"]
    finally:
        engine.set_merged(False)
    order = lambda p: p[np.lexsort((p[:, 1], p[:, 0]))]
    assert n1 == n0 and blocks > 0 and np.array_equal(order(got), order(want))
