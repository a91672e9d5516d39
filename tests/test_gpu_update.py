"""Resident scenes and incremental updates (pbig2_scene_*): after every move
the scene's full pair list equals a fresh query of the moved boxes, and the
removed / added lists are exactly the pairs that involve a moved box before
and after the move."""
import numpy as np
import pytest

from oracle import oracle as O
from pbig_gb300 import PbigError, Scene, gen
from pbig_gb300.serve import move_indices

pytestmark = pytest.mark.gpu


def canon(p):
    return O.sort_pairs(np.asarray(p, dtype=np.uint32).reshape(-1, 2))


def touching(pairs, moved):
    m = np.zeros(int(max(pairs.max() if len(pairs) else 0, moved.max())) + 1, dtype=bool)
    m[moved] = True
    return canon(pairs[m[pairs[:, 0]] | m[pairs[:, 1]]]) if len(pairs) else canon(pairs)


@pytest.mark.parametrize("dims", [2, 3])
def test_moves_keep_the_pair_set_exact(engine, dims):
    boxes = gen.clustered3d(200000, seed=11) if dims == 3 else gen.uniform2d(100000, seed=5, side=(0.002, 0.01))
    if dims == 2:
        boxes = np.ascontiguousarray(boxes)
    sc = Scene(engine, boxes, gen.RANGE)
    try:
        cur = boxes.copy()
        before = canon(sc.pairs())
        assert sc.npairs == len(before)
        assert np.array_equal(before, O.grid_pairs(cur, gen.RANGE)[0])
        for step in range(6):
            idx = move_indices(len(cur), 0.01 if step % 2 == 0 else 0.05, 100 + step)
            nb = cur[idx].copy()
            if dims == 3:
                tmp = cur.copy()
                gen.move3d(tmp, idx, 7 + step, sigma=0.002)
                nb = tmp[idx]
            else:  # 2-D: shift by a seeded amount, clipped to the range
                rng = np.random.default_rng(step)
                d = rng.integers(-20000, 20000, size=(len(idx), 2))
                for a in range(2):
                    lo = np.clip(nb[:, 2 * a].astype(np.int64) + d[:, a], 0, gen.RANGE - 1)
                    w = nb[:, 2 * a + 1].astype(np.int64) - nb[:, 2 * a]
                    nb[:, 2 * a] = lo
                    nb[:, 2 * a + 1] = np.minimum(lo + w, gen.RANGE - 1)
            nr, na = sc.move(idx, nb)
            after_boxes = cur.copy()
            after_boxes[idx] = nb
            want = O.grid_pairs(after_boxes, gen.RANGE)[0]
            got = canon(sc.pairs())
            assert np.array_equal(got, want), step
            rem, add = sc.delta()
            assert nr == len(rem) and na == len(add)
            assert np.array_equal(canon(rem), touching(before, idx))
            assert np.array_equal(canon(add), touching(want, idx))
            cur, before = after_boxes, want
    finally:
        sc.close()


def test_slack_overflow_rebuilds_the_grid(engine):
    """Moving many boxes into one place overflows the slack of its cells; the
    grid is rebuilt and the results stay exact."""
    boxes = gen.scene3d(50000, seed=3)
    sc = Scene(engine, boxes, gen.RANGE, cell_shift=16)
    try:
        idx = np.arange(0, 50000, 10, dtype=np.uint32)
        nb = boxes[idx].copy()
        nb[:, [0, 2, 4]] = 5000000
        nb[:, [1, 3, 5]] = 5000000 + 1000
        nr, na = sc.move(idx, nb)
        cur = boxes.copy()
        cur[idx] = nb
        assert np.array_equal(canon(sc.pairs()), O.grid_pairs(cur, gen.RANGE)[0])
        assert na >= len(idx) * (len(idx) - 1) // 2  # all moved boxes are identical now
    finally:
        sc.close()


def test_bad_moves_are_refused(engine):
    boxes = gen.scene3d(20000, seed=4)
    sc = Scene(engine, boxes, gen.RANGE)
    try:
        idx = np.array([5, 9, 5], dtype=np.uint32)
        with pytest.raises(PbigError):
            sc.move(idx, boxes[idx])
        bad = boxes[[1, 2]].copy()
        bad[0, 0], bad[0, 1] = 100, 50  # min > max
        with pytest.raises(PbigError):
            sc.move(np.array([1, 2], dtype=np.uint32), bad)
        wrong = boxes[[1, 2]].copy()
        wrong[:, 6] = [2, 1]  # rid must be the index
        with pytest.raises(PbigError):
            sc.move(np.array([1, 2], dtype=np.uint32), wrong)
        # the scene is unchanged and still usable
        assert np.array_equal(canon(sc.pairs()), O.grid_pairs(boxes, gen.RANGE)[0])
        sc.move(np.array([3], dtype=np.uint32), boxes[[3]])
        assert np.array_equal(canon(sc.pairs()), O.grid_pairs(boxes, gen.RANGE)[0])
    finally:
        sc.close()


def test_delta_only_scene(engine):
    """PBIG2_SCENE_DELTA_ONLY: the moves report the same delta, no full list."""
    boxes = gen.clustered3d(100000, seed=12)
    sc = Scene(engine, boxes, gen.RANGE, keep_pairs=False)
    try:
        before = O.grid_pairs(boxes, gen.RANGE)[0]
        idx = move_indices(len(boxes), 0.02, 9)
        cur = boxes.copy()
        gen.move3d(cur, idx, 9, sigma=0.002)
        sc.move(idx, cur[idx])
        rem, add = sc.delta()
        after = O.grid_pairs(cur, gen.RANGE)[0]
        assert np.array_equal(canon(rem), touching(before, idx))
        assert np.array_equal(canon(add), touching(after, idx))
        with pytest.raises(PbigError):
            sc.pairs()
    finally:
        sc.close()
