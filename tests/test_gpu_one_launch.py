"""One-launch queries of small scenes (PBIG2_OPT_ONE_LAUNCH).

A self query of at most 262 144 boxes runs as one cooperative kernel: the
cell size chosen on the device, count, scan, scatter and every pair pass,
separated by grid barriers. These tests compare it with the regular
multi-launch pipeline and with the oracle on every fixture, at forced cell
sizes from fine to a single cell (cells of 1 to more than 512 boxes, so every
work class and the tile tasks of huge cells run inside the one launch), with
a result larger than the pair buffer it was given, and they let a barrier's
bounded wait run out.
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O
from pbig_gb300 import Engine, PbigError, gen
from pbig_gb300.engine import ETIMEOUT

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))


def canon(p):
    return O.sort_pairs(np.asarray(p, dtype=np.uint32).reshape(-1, 2))


def to_device(boxes):
    import torch
    return torch.from_numpy(np.ascontiguousarray(boxes).view(np.int32)).cuda()


@pytest.fixture(scope="module")
def two():
    """A context on each path."""
    one, reg = Engine(0), Engine(0)
    reg.set_one_launch(False)
    yield one, reg
    one.close()
    reg.close()


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(f)[:-4] for f in FIXTURES])
def test_fixture_one_launch_and_regular(two, path):
    one, reg = two
    z = np.load(path)
    boxes, rng, want = z["boxes"], int(z["range"]), z["pairs"]
    if len(boxes) == 0 or len(boxes) > 1 << 18:
        pytest.skip("not a one-launch size")
    for src in (boxes, to_device(boxes)):
        # (a first result larger than the context's pair buffer is redone by
        # the regular pipeline; the repeat fits in one launch)
        for _ in range(2):
            n1 = one.self_intersect(src, rng)
            assert n1 == len(want)
            assert np.array_equal(canon(one.pairs()), want)
        assert one.stats()["kernels"] == 1, one.stats()
        n2 = reg.self_intersect(src, rng)
        assert reg.stats()["kernels"] > 1
        assert n2 == n1 and np.array_equal(canon(reg.pairs()), want)


@pytest.mark.parametrize("name", ["rand3d_1001", "identical700", "rand2d_4097", "rand3d_points_30000",
                                  "cfg2_clustered3d_16384", "domain_box"])
def test_every_cell_size_in_one_launch(two, name):
    one, _ = two
    z = np.load(os.path.join(HERE, "golden", name + ".npz"))
    boxes, rng, want = z["boxes"], int(z["range"]), z["pairs"]
    dims = (boxes.shape[1] - 1) // 2
    top = max(1, int(rng - 1).bit_length())
    ran = 0
    for s in range(max(0, top - 12), 32):
        cells = ((rng + (1 << s) - 1) >> s) ** dims
        if cells > 1 << 20:
            continue
        # (a first query whose entries, tile tasks or pairs exceed the
        # capacities the launch was given is redone by the regular pipeline
        # and raises them; the repeat runs in one launch)
        for _ in range(2):
            n = one.self_intersect(boxes, rng, cell_shift=s)
            assert n == len(want), s
            assert np.array_equal(canon(one.pairs()), want), s
        assert one.stats()["kernels"] == 1 and one.stats()["cell_shift"] == s
        ran += 1
    assert ran >= 3


def test_config1_in_one_launch(two):
    one, reg = two
    boxes = gen.uniform2d(65536)
    want = O.brute_pairs(boxes)
    dev = to_device(boxes)
    for _ in range(3):  # repeated launches advance the barriers' count
        assert one.self_intersect(dev, gen.RANGE) == len(want)
        assert one.stats()["kernels"] == 1
        assert np.array_equal(canon(one.pairs()), want)
    assert reg.self_intersect(dev, gen.RANGE) == len(want)


def test_result_larger_than_the_buffer_is_redone():
    """700 identical boxes give 244 650 pairs, more than a fresh context's
    pair buffer for 700 boxes: the launch reports the overflow, the regular
    pipeline redoes the query, and the next one-launch query fits."""
    z = np.load(os.path.join(HERE, "golden", "identical700.npz"))
    boxes, rng, want = z["boxes"], int(z["range"]), z["pairs"]
    assert len(want) > 1 << 16
    with Engine(0) as e:
        assert e.self_intersect(boxes, rng) == len(want)
        assert e.stats()["kernels"] > 1
        assert np.array_equal(canon(e.pairs()), want)
        assert e.self_intersect(boxes, rng) == len(want)
        assert e.stats()["kernels"] == 1
        assert np.array_equal(canon(e.pairs()), want)


def test_bounded_barrier_wait_runs_out():
    """The barriers' count of the next launch is set far ahead of every
    arrival: each block gives up after its bounded wait, the query returns
    ETIMEOUT, and the context then answers correctly."""
    z = np.load(os.path.join(HERE, "golden", "rand3d_1001.npz"))
    boxes, rng, want = z["boxes"], int(z["range"]), z["pairs"]
    with Engine(0) as e:
        assert e.self_intersect(boxes, rng) == len(want)
        e._L.pbig2_set_option(e._ctx, 5, 2)
        with pytest.raises(PbigError) as ei:
            e.self_intersect(boxes, rng)
        assert ei.value.code == ETIMEOUT
        for _ in range(2):
            assert e.self_intersect(boxes, rng) == len(want)
            assert e.stats()["kernels"] == 1
            assert np.array_equal(canon(e.pairs()), want)


def test_back_to_back_beside_other_work(two):
    """Launches on the context's own stream while torch's default stream
    runs other device work (a 256 MB memset before each query, no host
    synchronisation in between): the launch's blocks start at different
    times as the other kernel leaves the SMs, and every result must still be
    exact. Config 1 (a 64 x 64 grid: each block sums the chunks itself) and a
    clustered 3-D scene on 64 x 64 x 64 cells (the chunk totals shared
    through a barrier)."""
    import torch
    one, _ = two
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    st = None  # the context's own stream, not ordered with torch's default stream
    b1 = gen.uniform2d(65536, seed=0)
    b3 = gen.clustered3d(100000, seed=4)
    for boxes, shift in ((b1, None), (b3, 18)):
        want = O.brute_pairs(boxes)
        dev = to_device(boxes)
        for i in range(60):
            flush.zero_()
            n = one.self_intersect(dev, gen.RANGE, cell_shift=shift, stream=st)
            assert n == len(want), (i, n, len(want))
            assert one.stats()["kernels"] == 1
            if i % 20 == 19:
                assert np.array_equal(canon(one.pairs()), want)
