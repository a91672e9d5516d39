"""Coarser-grid retry of the automatic cell size.

A box outside the tuner's sample can cover 2^26 cells or more at the cell
size chosen from the sample (cells are enumerated with 32-bit indices). The
reference has no answer for it: it aborts on oversized cells
(src/pbig/pbig.cu:1613-1614) and silently skips cell ids past the grid
(:212). This engine reruns such a query on grids twice as coarse per axis
until every box fits, and later queries of the same scene start at the size
that fitted. These tests show that the rerun gives exactly the brute-force
pair set on every path that takes it: self queries with pageable, page-locked
and device input, red/blue queries, batched scenes, and the legacy pbig.h
API with cs = 0.

The scene: 20,000 3-D boxes of side < 64 in a 2^18 range plus, at index
12345 (outside every sample the tuner takes), one box spanning the range.
The tuner picks a cell size of at most 2^9 (the spanning box would then
cover at least 2^27 cells); the reruns end at 2^10 or coarser.
"""
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle as O
from pbig_gb300 import Engine, build, tune_shift

HERE = os.path.dirname(os.path.abspath(__file__))
RANGE = 1 << 18
BIG = 12345


def _scene(n=20001, seed=21, big_at=BIG):
    r = np.random.default_rng(seed)
    lo = r.integers(0, RANGE - 64, size=(n, 3), dtype=np.int64)
    hi = lo + r.integers(0, 64, size=(n, 3))
    b = np.empty((n, 7), dtype=np.uint32)
    b[:, 0:6:2] = lo
    b[:, 1:6:2] = hi
    b[:, 6] = np.arange(n, dtype=np.uint32)
    if big_at is not None:
        b[big_at, :6] = [0, RANGE - 1] * 3
    return b


def _canon(p):
    return O.sort_pairs(np.asarray(p, dtype=np.uint32).reshape(-1, 2))


def _fits(shift):
    return ((RANGE >> shift) ** 3) < (1 << 26)


@pytest.fixture(autouse=True)
def _regular_pipeline(request):
    """The rerun belongs to the regular pipeline: a one-launch query's grid
    has at most 2^20 cells, so no box can cover 2^26 of them."""
    if "engine" not in request.fixturenames:
        yield
        return
    eng = request.getfixturevalue("engine")
    eng.set_one_launch(False)
    try:
        yield
    finally:
        eng.set_one_launch(True)


def test_tuner_picks_a_size_the_spanning_box_overflows():
    """(CPU) The scene really exercises the rerun: the tuner's sample misses
    the spanning box and its choice is too fine for it."""
    b = _scene()
    s = tune_shift(b, RANGE, 4096)
    assert not _fits(s), s
    # the spanning box alone would be seen and fitted
    assert _fits(tune_shift(b[BIG:BIG + 1].copy(), RANGE, 4096))


@pytest.mark.gpu
@pytest.mark.parametrize("loc", ["pageable", "pinned", "device"])
def test_self_query_reruns_on_a_coarser_grid(loc):
    """A fresh context each time: the tuner's memory of earlier queries of the
    scene would otherwise skip the rerun."""
    import torch
    b = _scene()
    want = O.brute_pairs(b)
    assert (want == BIG).any()
    if loc == "pageable":
        src = b
    elif loc == "pinned":
        src = torch.from_numpy(b.view(np.int32)).pin_memory()
    else:
        src = torch.from_numpy(b.view(np.int32)).cuda()
    with Engine(0) as engine:
        engine.set_one_launch(False)
        n = engine.self_intersect(src, RANGE)
        st = engine.stats()
        assert n == len(want)
        assert np.array_equal(_canon(engine.pairs()), want)
        assert st["grid_retries"] >= 1 and _fits(st["cell_shift"]), st
        assert st["bad_boxes"] == 0
        first = st["cell_shift"]
        # the same scene again: the remembered size fits at once
        assert engine.self_intersect(src, RANGE) == len(want)
        st2 = engine.stats()
        assert st2["grid_retries"] == 0 and st2["cell_shift"] == first, st2
        assert np.array_equal(_canon(engine.pairs()), want)


@pytest.mark.gpu
def test_bipartite_query_reruns_on_a_coarser_grid():
    b = _scene(big_at=None)
    red = b[:10000].copy()
    blue = b[10000:].copy()
    blue[:, 6] = np.arange(len(blue), dtype=np.uint32)
    blue[BIG - 10000, :6] = [0, RANGE - 1] * 3  # union index 12345
    u = np.concatenate([red, blue])
    u[10000:, 6] += 10000
    allp = O.brute_pairs(u)
    cross = allp[(allp[:, 0] < 10000) & (allp[:, 1] >= 10000)].copy()
    cross[:, 1] -= 10000
    assert len(cross) >= 10000 and (cross[:, 1] == BIG - 10000).sum() == 10000
    with Engine(0) as engine:
        n = engine.bipartite_intersect(red, blue, RANGE)
        st = engine.stats()
        got = engine.pairs()
    assert n == len(cross) and st["grid_retries"] >= 1 and _fits(st["cell_shift"]), st
    order = np.lexsort((got[:, 1], got[:, 0]))
    assert np.array_equal(got[order], cross)


def _batch():
    """48 scenes: scene 17 holds 5000 small boxes (side < 64, so its tuner
    picks 2^8 from its 64-box sample) and the spanning box at a local index
    that neither the per-scene host sample (rows floor(k * 5000 / 64)) nor the
    strided device sample of the whole batch reaches; the other scenes hold
    boxes of side 1024..2047 and get coarse grids of their own."""
    r = np.random.default_rng(3)
    sizes = r.integers(200, 5000, size=48)
    sizes[17] = 5000
    parts = []
    for i, k in enumerate(sizes):
        b = _scene(int(k), seed=100 + i, big_at=None)
        if i != 17:
            lo = r.integers(0, RANGE - 2048, size=(int(k), 3))
            b[:, 0:6:2] = lo
            b[:, 1:6:2] = lo + r.integers(1024, 2048, size=(int(k), 3))
        parts.append(b)
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    n = int(offs[-1])
    stride = n // min(n, 64 * 48)
    host_rows = {k * 5000 // 64 for k in range(64)}
    local = next(j for j in range(100, 5000) if j not in host_rows and (int(offs[17]) + j) % stride)
    parts[17][local, :6] = [0, RANGE - 1] * 3
    return parts, offs


@pytest.mark.gpu
@pytest.mark.parametrize("loc", ["host", "device"])
def test_batch_with_one_spanning_box_reruns_every_scene(engine, loc):
    """Every scene is coarsened and every scene's pair list equals its brute
    force."""
    import torch
    parts, offs = _batch()
    allb = np.ascontiguousarray(np.concatenate(parts))
    src = allb if loc == "host" else torch.from_numpy(allb.view(np.int32)).cuda()
    total = engine.batch_intersect(src, offs, RANGE)
    st = engine.stats()
    assert st["grid_retries"] >= 1 and st["bad_boxes"] == 0, st
    so = engine.scene_offsets()
    assert int(so[-1]) == total
    res = engine.pairs()
    for i, b in enumerate(parts):
        want = O.brute_pairs(b)
        got = _canon(res[int(so[i]):int(so[i + 1])])
        assert np.array_equal(got, want), i


@pytest.mark.gpu
def test_legacy_api_with_cs_zero_reruns(tmp_path):
    """pbig_init(num, range, cs = 0, ...) + pbig_check through a recording
    report: three steps, each the oracle's pair set. The scene has 300 001
    boxes, more than a one-launch query takes, so the regular pipeline and
    its rerun serve it."""
    d = os.path.join(HERE, "clients", "recording")
    exe = build.compile_client([os.path.join(HERE, "clients", "legacy_client.cc"), os.path.join(d, "report.cc")],
                               str(tmp_path / "client"), include_first=[d])
    b = _scene(n=300001)
    want, _ = O.grid_pairs(b, RANGE, cs=1 << 12)
    f = tmp_path / "boxes.bin"
    b.tofile(f)
    env = dict(os.environ, PBIG_PAIRS_OUT=str(tmp_path / "pairs.bin"))
    r = subprocess.run([exe, str(f), str(len(b)), str(RANGE), "3", "0"], capture_output=True, text=True, env=env,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "WARNING" not in r.stdout
    assert r.stdout.count(f"Number of pairs = {len(want)}") == 3
    got = np.fromfile(tmp_path / "pairs.bin", dtype=np.uint32)
    assert np.array_equal(_canon(got), want)
