"""Randomised parity: many small scenes of every shape the engine handles --
2-D and 3-D, ranges from 2^4 to 2^32, zero-extent, identical and touching
boxes, boxes spanning the whole range, random and forced cell sizes -- self,
red/blue and batched queries, each compared exactly with the all-pairs brute
force of the oracle (the reference's closed-interval test,
src/pbig/pbig.cu:562-577)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def canon(p):
    return O.sort_pairs(np.asarray(p, dtype=np.uint32).reshape(-1, 2))


def random_scene(rs, n, dims, rng):
    """n boxes in [0, rng) with a mix of extents: points, small, large, the
    whole range, duplicates, and faces that touch on a lattice."""
    lo = rs.integers(0, rng, size=(n, dims), dtype=np.int64)
    kind = rs.integers(0, 6, size=n)
    ext = np.zeros((n, dims), dtype=np.int64)
    small = max(1, rng // 64)
    ext[kind == 1] = rs.integers(0, small + 1, size=((kind == 1).sum(), dims))
    ext[kind == 2] = rs.integers(0, max(2, rng // 4), size=((kind == 2).sum(), dims))
    ext[kind == 3] = rng  # clipped below: spans to the end
    # kind 4: lattice boxes whose faces touch their neighbours
    lat = max(1, rng // 16)
    lo[kind == 4] = (lo[kind == 4] // lat) * lat
    ext[kind == 4] = lat
    hi = np.minimum(lo + ext, rng - 1)
    # kind 5: duplicates of earlier boxes
    dup = np.nonzero(kind == 5)[0]
    if len(dup):
        src = rs.integers(0, n, size=len(dup))
        lo[dup], hi[dup] = lo[src], hi[src]
    boxes = np.empty((n, 2 * dims + 1), dtype=np.uint32)
    for d in range(dims):
        boxes[:, 2 * d] = lo[:, d]
        boxes[:, 2 * d + 1] = hi[:, d]
    boxes[:, 2 * dims] = np.arange(n, dtype=np.uint32)
    return boxes


def scene_params(seed):
    rs = np.random.default_rng(1000 + seed)
    dims = int(rs.choice([2, 3]))
    rng = int(2 ** rs.integers(4, 33)) if seed % 7 else int(rs.integers(2, 100000))
    rng = min(rng, (1 << 32) - 1)
    n = int(rs.integers(0, 2500))
    return rs, dims, rng, n


@pytest.mark.parametrize("seed", range(40))
def test_random_self(engine, seed):
    """Each scene through the one-launch path (these scenes are small) and
    through the regular multi-launch pipeline."""
    rs, dims, rng, n = scene_params(seed)
    boxes = random_scene(rs, n, dims, rng)
    want = O.brute_pairs(boxes)
    top = max(1, int(rng - 1).bit_length())
    shifts = [None] + sorted(set(int(s) for s in rs.integers(max(0, top - 9), top + 1, size=2)))
    try:
        for one_launch in (True, False):
            engine.set_one_launch(one_launch)
            for s in shifts:
                if s is not None and (((rng + (1 << s) - 1) >> s) ** dims) > 1 << 25:
                    continue  # a box may cover fewer than 2^26 cells
                got = engine.self_intersect(boxes, rng, cell_shift=s)
                assert got == len(want), (seed, s, one_launch)
                assert np.array_equal(canon(engine.pairs()), want), (seed, s, one_launch)
    finally:
        engine.set_one_launch(True)


@pytest.mark.parametrize("seed", range(12))
def test_random_red_blue(engine, seed):
    rs, dims, rng, n = scene_params(100 + seed)
    red = random_scene(rs, max(1, n), dims, rng)
    blue = random_scene(rs, int(rs.integers(1, 2500)), dims, rng)
    union = np.concatenate([red, blue])
    union[len(red):, -1] += len(red)
    allp = O.brute_pairs(np.ascontiguousarray(union))
    cross = allp[(allp[:, 0] < len(red)) & (allp[:, 1] >= len(red))]
    want = O.sort_pairs(np.stack([cross[:, 0], cross[:, 1] - len(red)], axis=1).astype(np.uint32))
    got = engine.bipartite_intersect(red, blue, rng)
    assert got == len(want), seed
    assert np.array_equal(O.sort_pairs(engine.pairs()), want), seed


@pytest.mark.parametrize("seed", range(6))
def test_random_batches(engine, seed):
    """Scenes of one dimensionality and range, uneven sizes (empty ones
    included), resolved in one batched query; each scene's pairs (scene-local
    indices) equal its brute force."""
    rs = np.random.default_rng(5000 + seed)
    dims = int(rs.choice([2, 3]))
    rng = int(2 ** rs.integers(8, 31))
    parts = [random_scene(rs, int(rs.integers(0, 1500)), dims, rng) for _ in range(int(rs.integers(2, 30)))]
    offs = np.zeros(len(parts) + 1, dtype=np.uint64)
    for i, b in enumerate(parts):
        offs[i + 1] = offs[i] + len(b)
    allb = np.ascontiguousarray(np.concatenate(parts)) if int(offs[-1]) else np.zeros((0, 2 * dims + 1), np.uint32)
    if int(offs[-1]) == 0:
        return
    total = engine.batch_intersect(allb, offs, rng)
    so = engine.scene_offsets()
    res = engine.pairs()
    assert int(so[-1]) == total
    for i, b in enumerate(parts):
        want = O.brute_pairs(b) if len(b) else np.zeros((0, 2), np.uint32)
        assert np.array_equal(canon(res[int(so[i]):int(so[i + 1])]), want), (seed, i)


@pytest.mark.parametrize("seed", range(16))
def test_random_merged_and_records(engine, seed):
    """The same kind of scenes through the reference's merged build (sparse
    cells merged into blocks, pbig.cu:1066-1251 and 223-318) and through its
    Rice record stream (pbig.cu:788-920), decoded by the oracle's restatement
    of decode.cc:38-131: both give the brute-force pair set."""
    rs, dims, rng, n = scene_params(200 + seed)
    boxes = random_scene(rs, max(n, 1), dims, rng)
    want = O.brute_pairs(boxes)
    engine.set_merged(True)
    try:
        got = engine.self_intersect(boxes, rng)
        merged = canon(engine.pairs())
    finally:
        engine.set_merged(False)
    assert got == len(want), seed
    assert np.array_equal(merged, want), seed
    engine.set_records(True)
    try:
        got = engine.self_intersect(boxes, rng)
        words, start_i, recs = engine.records()
    finally:
        engine.set_records(False)
    assert got == len(want), seed
    dec = O.decode_rice(words, start_i, recs) if len(words) else np.zeros((0, 2), np.uint32)
    assert np.array_equal(canon(dec), want), seed
