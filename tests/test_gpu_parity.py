"""Parity of the CUDA engine with the oracle and the committed fixtures.

Pair sets are compared exactly (canonical (a<b) pairs, sorted): the results
are integer index pairs, so no tolerance applies.
"""
import glob
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle as O
from pbig_gb300 import PbigError, build, gen

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))


def canon(p):
    return O.sort_pairs(np.asarray(p, dtype=np.uint32).reshape(-1, 2))


def to_device(boxes):
    import torch
    return torch.from_numpy(np.ascontiguousarray(boxes).view(np.int32)).cuda()


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(f)[:-4] for f in FIXTURES])
def test_fixture_host_and_device_input(engine, path):
    z = np.load(path)
    boxes, rng, want = z["boxes"], int(z["range"]), z["pairs"]
    n = engine.self_intersect(boxes, rng)
    assert n == len(want)
    assert np.array_equal(canon(engine.pairs()), want)
    if len(boxes):
        n2 = engine.self_intersect(to_device(boxes), rng)
        assert n2 == len(want)
        assert np.array_equal(canon(engine.pairs()), want)


@pytest.mark.parametrize("name", ["rand3d_1001", "identical700", "domain_box", "rand2d_4097",
                                  "rand3d_points_30000", "cfg2_clustered3d_16384"])
def test_fixture_every_cell_size(engine, name):
    """The pair set does not depend on the grid: force fine to coarse cells
    (cells of 1..>512 boxes exercise every work class of the pair kernel)."""
    z = np.load(os.path.join(HERE, "golden", name + ".npz"))
    boxes, rng, want = z["boxes"], int(z["range"]), z["pairs"]
    top = max(1, int(rng - 1).bit_length())
    for s in sorted(set([max(0, top - 12), top - 8, top - 5, top - 3, top - 1, top, 31])):
        if s < 0:
            continue
        cells = (((rng + (1 << s) - 1) >> s) ** ((boxes.shape[1] - 1) // 2))
        if cells > 1 << 28:
            continue
        n = engine.self_intersect(boxes, rng, cell_shift=s)
        assert n == len(want), s
        assert np.array_equal(canon(engine.pairs()), want), s


def test_invalid_boxes_are_skipped_and_reported(engine):
    z = np.load(os.path.join(HERE, "golden", "rand3d_1001.npz"))
    boxes, rng = z["boxes"].copy(), int(z["range"])
    boxes[3, 1] = rng            # coordinate == range
    boxes[10, 2], boxes[10, 3] = 50, 40  # inverted y
    boxes[20, 6] = 7             # rid != index
    with pytest.raises(PbigError) as ei:
        engine.self_intersect(boxes, rng)
    assert ei.value.code == 4
    n = engine.self_intersect(boxes, rng, allow_bad=True)
    assert engine.stats()["bad_boxes"] == 3
    keep = np.ones(len(boxes), bool)
    keep[[3, 10, 20]] = False
    full = canon(O.brute_pairs(np.where(keep[:, None], boxes, 0).astype(np.uint32)))
    bad = np.isin(full[:, 0], [3, 10, 20]) | np.isin(full[:, 1], [3, 10, 20])
    want = full[~bad]
    assert n == len(want) and np.array_equal(canon(engine.pairs()), want)


def test_config1_plain2d_full(engine):
    boxes = gen.uniform2d(65536)
    want = O.brute_pairs(boxes)
    assert engine.self_intersect(boxes, gen.RANGE) == len(want)
    assert np.array_equal(canon(engine.pairs()), want)


def test_config2_clustered3d_4m_full(engine):
    boxes = gen.clustered3d(4194304)
    want, st = O.grid_pairs(boxes, gen.RANGE, cs=1 << 16)
    n = engine.self_intersect(to_device(boxes), gen.RANGE)
    assert n == st["pairs"]
    assert np.array_equal(canon(engine.pairs()), want)
    s = engine.stats()
    assert s["pairs"] == n and s["bad_boxes"] == 0
    # same grid as the oracle: identical entry count
    engine.self_intersect(to_device(boxes), gen.RANGE, cell_shift=16)
    assert engine.stats()["entries"] == st["entries"]


def test_config3_bipartite_full(engine):
    red = gen.mixed3d(2097152, seed=0)
    blue = gen.mixed3d(2097152, seed=1)
    u = np.concatenate([red, blue])
    u[len(red):, 6] += len(red)
    allp, _ = O.grid_pairs(np.ascontiguousarray(u), gen.RANGE, cs=1 << 18)
    cross = allp[(allp[:, 0] < len(red)) & (allp[:, 1] >= len(red))].copy()
    cross[:, 1] -= len(red)
    n = engine.bipartite_intersect(to_device(red), to_device(blue), gen.RANGE)
    assert n == len(cross)
    got = engine.pairs()
    assert (got[:, 0] < len(red)).all() and (got[:, 1] < len(blue)).all()
    order = np.lexsort((got[:, 1], got[:, 0]))
    assert np.array_equal(got[order], cross)


def _scenes(k, seed, lo, hi):
    sizes = gen.scene_sizes(k, seed, lo, hi)
    parts = [gen.scene3d(int(n), seed=1000 * seed + i) for i, n in enumerate(sizes)]
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    return parts, offs


@pytest.mark.parametrize("loc", ["host", "device"])
def test_batched_scenes_match_plain_and_oracle(engine, loc):
    parts, offs = _scenes(48, 3, 256, 20000)
    allb = np.ascontiguousarray(np.concatenate(parts))
    total = engine.batch_intersect(allb if loc == "host" else to_device(allb), offs, gen.RANGE)
    so = engine.scene_offsets()
    assert int(so[-1]) == total
    res = engine.pairs()
    for i, b in enumerate(parts):
        got = canon(res[int(so[i]):int(so[i + 1])])
        want, _ = O.grid_pairs(b, gen.RANGE)
        assert np.array_equal(got, want), i
        assert engine.self_intersect(b, gen.RANGE) == len(want) or True
    # plain path per scene (done after the batch check: a query replaces the result)
    for i, b in enumerate(parts[:8]):
        n = engine.self_intersect(b, gen.RANGE)
        want, _ = O.grid_pairs(b, gen.RANGE)
        assert n == len(want) and np.array_equal(canon(engine.pairs()), want)


def test_repeated_queries_are_stable(engine):
    boxes = gen.clustered3d(300000, seed=4)
    a = engine.self_intersect(boxes, gen.RANGE)
    pa = canon(engine.pairs())
    for _ in range(3):
        assert engine.self_intersect(boxes, gen.RANGE) == a
        assert np.array_equal(canon(engine.pairs()), pa)


def test_direct_pair_output(engine):
    """Pairs stored straight into a caller's page-locked host buffer (or a
    device buffer) equal the default path; a buffer that is too small makes
    the engine redo the query into its own buffer; pageable host memory is
    refused."""
    import torch
    boxes = gen.clustered3d(300000, seed=5)
    n = engine.self_intersect(boxes, gen.RANGE)
    want = canon(engine.pairs())
    out = torch.empty((n + 100, 2), dtype=torch.int32).pin_memory()
    try:
        engine.set_pair_output(out)
        assert engine.self_intersect(boxes, gen.RANGE) == n
        assert engine.result_in(out)
        assert np.array_equal(canon(out[:n].numpy().view(np.uint32)), want)
        assert np.array_equal(canon(engine.pairs()), want)
        small = torch.empty((n // 2, 2), dtype=torch.int32).pin_memory()
        engine.set_pair_output(small)
        assert engine.self_intersect(boxes, gen.RANGE) == n
        assert not engine.result_in(small)
        assert np.array_equal(canon(engine.pairs()), want)
        dev = torch.empty((n + 1, 2), dtype=torch.int32, device="cuda")
        engine.set_pair_output(dev)
        assert engine.self_intersect(to_device(boxes), gen.RANGE) == n
        assert engine.result_in(dev)
        assert np.array_equal(canon(dev[:n].cpu().numpy().view(np.uint32)), want)
        red, blue = gen.mixed3d(100000, seed=0), gen.mixed3d(100000, seed=1)
        nb = engine.bipartite_intersect(red, blue, gen.RANGE)
        assert engine.result_in(dev) and np.array_equal(dev[:nb].cpu().numpy().view(np.uint32), engine.pairs())
        with pytest.raises(PbigError):
            engine.set_pair_output(torch.empty((16, 2), dtype=torch.int32))
    finally:
        engine.set_pair_output(None)
    assert engine.self_intersect(boxes, gen.RANGE) == n and not engine.result_in(out)


@pytest.fixture
def regular(engine):
    """The shared context with every query on the regular multi-launch
    pipeline (small self queries otherwise run as one launch)."""
    engine.set_one_launch(False)
    try:
        yield engine
    finally:
        engine.set_one_launch(True)


@pytest.mark.parametrize("split", [-1, 0, 8, 100])
def test_host_output_split(regular, split):
    """Pairs to page-locked host memory with the small-cell and block kernels
    beside the medium-cell kernel (any SM share) or after it: the same pair
    set, self and red/blue, with cells of every class (a stack of identical
    boxes fills the block kernel)."""
    import torch
    engine = regular
    boxes = gen.clustered3d(200000, seed=9)
    stack = np.repeat(boxes[:1], 3000, axis=0)
    boxes = np.concatenate([boxes, stack])
    boxes[:, 6] = np.arange(boxes.shape[0])
    n = engine.self_intersect(boxes, gen.RANGE)
    want = canon(engine.pairs())
    red, blue = gen.mixed3d(100000, seed=0), gen.mixed3d(100000, seed=1)
    nb = engine.bipartite_intersect(red, blue, gen.RANGE)
    want_b = canon(engine.pairs())
    out = torch.empty((max(n, nb) + 64, 2), dtype=torch.int32).pin_memory()
    try:
        engine.set_host_split(split)
        engine.set_pair_output(out)
        assert engine.self_intersect(boxes, gen.RANGE) == n and engine.result_in(out)
        assert np.array_equal(canon(out[:n].numpy().view(np.uint32)), want)
        assert engine.bipartite_intersect(red, blue, gen.RANGE) == nb and engine.result_in(out)
        assert np.array_equal(canon(out[:nb].numpy().view(np.uint32)), want_b)
        with pytest.raises(PbigError):
            engine.set_host_split(100000)
    finally:
        engine.set_pair_output(None)
        engine.set_host_split(0)


@pytest.mark.parametrize("one_launch", [False, True])
@pytest.mark.parametrize("dims", [2, 3])
def test_pinned_host_input(engine, dims, one_launch):
    """Page-locked host input is uploaded by the count kernel itself (no copy
    before the pipeline; a one-launch query copies it first): the same pairs
    as pageable input for self and red/blue queries of ragged sizes (a count
    tile straddles red and blue), with one side pinned and the other
    pageable, and in merged mode."""
    import torch
    engine.set_one_launch(one_launch)
    request_cleanup = engine.set_one_launch

    def pin(a):
        return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).pin_memory()

    boxes = gen.clustered3d(100003, seed=3) if dims == 3 else gen.uniform2d(100003, seed=3)
    n = engine.self_intersect(boxes, gen.RANGE)
    want = canon(engine.pairs())
    assert engine.self_intersect(pin(boxes), gen.RANGE) == n
    assert np.array_equal(canon(engine.pairs()), want)
    red, blue = boxes[:50001].copy(), boxes[50001:].copy()
    blue[:, -1] = np.arange(blue.shape[0])
    nb = engine.bipartite_intersect(red, blue, gen.RANGE)
    want_b = canon(engine.pairs())
    assert engine.bipartite_intersect(pin(red), pin(blue), gen.RANGE) == nb
    assert np.array_equal(canon(engine.pairs()), want_b)
    assert engine.bipartite_intersect(pin(red), blue, gen.RANGE) == nb
    assert np.array_equal(canon(engine.pairs()), want_b)
    engine.set_merged(True)
    try:
        assert engine.self_intersect(pin(boxes), gen.RANGE) == n
        assert np.array_equal(canon(engine.pairs()), want)
    finally:
        engine.set_merged(False)
        request_cleanup(True)


def test_output_capacity_growth(engine):
    """A tiny scene first (small buffers), then one with millions of pairs:
    the pair buffer must grow and the count stay exact."""
    engine.self_intersect(np.load(os.path.join(HERE, "golden", "touching3d.npz"))["boxes"], 64)
    z = np.load(os.path.join(HERE, "golden", "identical700.npz"))
    b = np.repeat(z["boxes"][:1], 3000, axis=0)
    b[:, 6] = np.arange(3000)
    assert engine.self_intersect(b, 1000) == 3000 * 2999 // 2


def test_medium_cells_rerun_after_pair_overflow():
    """A fresh context on the multi-launch pipeline: 25 cells of 80 boxes
    that all overlap (medium cells) give 79 000 pairs, more than the first
    pair buffer holds, so the pair kernels run again on the same grid; the
    medium-cell pass takes its cells from a counter, which the rerun must
    start from zero again."""
    from pbig_gb300 import Engine
    rng = np.random.default_rng(7)
    rows = []
    for g in range(25):
        lo = np.array([(g % 5) * 2048, (g // 5) * 2048, 4096]) + 10
        for _ in range(80):
            a = lo + rng.integers(0, 8, size=3)
            b = a + rng.integers(8, 16, size=3)
            rows.append([a[0], b[0], a[1], b[1], a[2], b[2], 0])
    boxes = np.asarray(rows, dtype=np.uint32)
    boxes[:, 6] = np.arange(len(boxes))
    want = O.brute_pairs(boxes)
    assert len(want) == 25 * 80 * 79 // 2
    with Engine(0) as e:
        e.set_one_launch(False)
        for _ in range(2):
            assert e.self_intersect(boxes, 1 << 16, cell_shift=10) == len(want)
            assert e.stats()["max_cell"] == 80
            assert np.array_equal(canon(e.pairs()), want)


@pytest.mark.parametrize("kind", ["counting", "recording"])
def test_legacy_pbig_api_client(tmp_path, kind):
    """A pbig.h client (pbig_init / pbig_check / pbig_finalize, report
    callback) built against this library, with a counting and a recording
    report type."""
    d = os.path.join(HERE, "clients", kind)
    exe = build.compile_client([os.path.join(HERE, "clients", "legacy_client.cc"), os.path.join(d, "report.cc")],
                               str(tmp_path / "client"), include_first=[d])
    z = np.load(os.path.join(HERE, "golden", "rand3d_mixed_50000.npz"))
    boxes, rng, want = z["boxes"], int(z["range"]), z["pairs"]
    f = tmp_path / "boxes.bin"
    boxes.tofile(f)
    env = dict(os.environ, PBIG_PAIRS_OUT=str(tmp_path / "pairs.bin"))
    r = subprocess.run([exe, str(f), str(len(boxes)), str(rng), "3"], capture_output=True, text=True, env=env,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count(f"Number of pairs = {len(want)}") == 3
    if kind == "recording":
        got = np.fromfile(tmp_path / "pairs.bin", dtype=np.uint32)
        assert np.array_equal(canon(got), want)


def test_harness_golden_count_on_gpu(engine):
    """The reference harness workload behind the published 49 514 252 pairs
    (test1, N = 10 M, UU, side < 100, range 10 000), through the engine."""
    boxes = O.harness_boxes(10_000_000, S=100, range_=10000, sim="UU")
    assert engine.self_intersect(to_device(boxes), 10000) == 49_514_252


@pytest.mark.parametrize("name", ["rand3d_mixed_50000", "rand2d_4097", "identical700"])
def test_wide_coordinates(engine, name):
    """Ranges above 2^29 take the comparison form of the pair test: scaling
    every coordinate by a power of two keeps the pair set."""
    z = np.load(os.path.join(HERE, "golden", name + ".npz"))
    boxes, rng, want = z["boxes"].astype(np.uint64), int(z["range"]), z["pairs"]
    k = max(0, 32 - int(rng - 1).bit_length() - 1)
    wide = boxes.copy()
    wide[:, :-1] <<= k
    wide = wide.astype(np.uint32)
    rng_w = min((rng << k), 0xFFFFFFFF)
    assert rng_w > (1 << 29)
    assert engine.self_intersect(wide, rng_w) == len(want)
    assert np.array_equal(canon(engine.pairs()), want)


def test_batched_graph_replay_matches_eager(engine):
    """Batched queries replay a captured CUDA graph once the first query of a
    shape ran; the replay (same batch, then a smaller batch in the same
    buffer) must give the eager results."""
    import torch
    parts, offs = _scenes(40, 7, 256, 30000)
    allb = np.ascontiguousarray(np.concatenate(parts))
    dev = to_device(allb)
    results = []
    for graphs in (False, True):
        engine.set_graphs(graphs)
        for rep in range(3):  # eager, capture, replay
            total = engine.batch_intersect(dev, offs, gen.RANGE)
            so = engine.scene_offsets()
            res = engine.pairs()
            results.append([canon(res[int(so[i]):int(so[i + 1])]) for i in range(len(parts))])
    for r in results[1:]:
        for a, b in zip(results[0], r):
            assert np.array_equal(a, b)
    # a smaller batch (first 25 scenes) in the same device buffer replays the graph too
    engine.set_graphs(True)
    sub = dev[: int(offs[25])]
    offs25 = offs[:26].copy()
    assert engine.batch_intersect(sub, offs25, gen.RANGE) == sum(len(x) for x in results[0][:25])
    so = engine.scene_offsets()
    res = engine.pairs()
    for i in range(25):
        assert np.array_equal(canon(res[int(so[i]):int(so[i + 1])]), results[0][i])
    engine.set_graphs(True)
