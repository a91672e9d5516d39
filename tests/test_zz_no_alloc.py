"""The allocation-free entry point, pbig2_self_intersect_noalloc, called
through the C ABI.

It serves callers that cannot allocate device memory during a query: a
process whose device memory is all owned by another allocator (a caching
allocator that reserved the GPU), or a latency-critical loop that cannot
afford the device-wide synchronization of cudaMalloc/cudaFree. All its
intermediate buffers live in a fixed scratch array inside the library, so
every call reuses what the previous call left behind.

Its pairs must equal the oracle's (the CPU restatement of the reference
pipeline) and those of the allocating entry point, pbig2_self_intersect, on
two calls in a row. Collected last so that a failure here does not hide the
others; it passes alone in a fresh process as well as after them.
"""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import oracle as O
from pbig_gb300 import Engine, gen
from pbig_gb300.engine import AUTO, ECAPACITY, EINVAL, lib

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def _noalloc(d_boxes, n, dims, rng, d_out, cap, shift=AUTO, out_offset_bytes=0):
    npairs = C.c_uint64(12345)
    out_ptr = d_out.data_ptr() + out_offset_bytes if d_out is not None else 0
    rc = lib().pbig2_self_intersect_noalloc(C.c_void_p(d_boxes.data_ptr()), n, dims, rng, shift,
                                            C.c_void_p(out_ptr), cap, C.byref(npairs), None)
    return rc, npairs.value


def _err():
    return lib().pbig2_noalloc_last_error().decode()


def _device(boxes):
    import torch
    return torch.from_numpy(np.ascontiguousarray(boxes).view(np.int32)).cuda()


def _run_twice(boxes, rng, want, shift=AUTO):
    """Two calls in a row (the second reuses the scratch the first left) must
    both return exactly `want`, the oracle's sorted (a<b) pair list."""
    import torch
    dims = (boxes.shape[1] - 1) // 2
    d_boxes = _device(boxes)
    cap = len(want) + 1024
    d_out = torch.zeros((cap, 2), dtype=torch.int32, device="cuda")
    for _ in range(2):
        d_out.fill_(-1)
        torch.cuda.synchronize()
        rc, n = _noalloc(d_boxes, boxes.shape[0], dims, rng, d_out, cap, shift)
        assert rc == 0, _err()
        assert n == len(want)
        got = O.sort_pairs(d_out[:n].cpu().numpy().view(np.uint32))
        assert np.array_equal(got, want)


@pytest.mark.parametrize("which", ["clustered3d", "uniform2d"])
def test_noalloc_matches_oracle_and_allocating_entry_point_twice(which):
    if which == "clustered3d":
        boxes = gen.clustered3d(200000, seed=9)
    else:
        boxes = gen.uniform2d(65536, seed=0)
    rng = gen.RANGE
    want, _ = O.grid_pairs(boxes, rng)
    with Engine(0) as e:
        n_ref = e.self_intersect(boxes, rng)
        assert n_ref == len(want)
        assert np.array_equal(O.sort_pairs(e.pairs()), want)
    _run_twice(boxes, rng, want)


def _small_boxes(n, dims, seed, range_, side_max):
    r = np.random.default_rng(seed)
    lo = r.integers(0, range_, size=(n, dims), dtype=np.int64)
    hi = np.minimum(lo + r.integers(0, side_max + 1, size=(n, dims)), range_ - 1)
    rows = np.empty((n, 2 * dims + 1), dtype=np.uint32)
    rows[:, 0:2 * dims:2] = lo
    rows[:, 1:2 * dims:2] = hi
    rows[:, -1] = np.arange(n, dtype=np.uint32)
    return rows


@pytest.mark.parametrize("shift", [AUTO, 0, 1, 2, 12])
def test_noalloc_point_like_boxes_in_a_wide_range(shift):
    """Boxes under 2 units wide in a 2^24 range: the automatic cell size (and
    the explicit shifts 0..2) would give a grid of 2^66..2^72 cells in 3-D;
    the cell count saturates and the grid is coarsened to fit the scratch."""
    rng = 1 << 24
    boxes = _small_boxes(30000, 3, 11, rng, 1)
    # clusters of coincident points so that pairs exist
    boxes[1::2, :6] = boxes[0:-1:2, :6]
    want = O.brute_pairs(boxes)
    assert len(want) >= 15000
    _run_twice(boxes, rng, want, shift)


@pytest.mark.parametrize("name,shift", [("rand3d_points_30000", AUTO), ("rand3d_points_30000", 2),
                                        ("rand3d_dense_20000", 10), ("rand3d_mixed_50000", AUTO),
                                        ("rand2d_4097", 14), ("touching3d", 0), ("identical700", AUTO)])
def test_noalloc_fixtures(name, shift):
    z = np.load(os.path.join(HERE, "golden", name + ".npz"))
    _run_twice(z["boxes"], int(z["range"]), z["pairs"], shift)


def test_noalloc_rejects_misaligned_pair_buffer():
    import torch
    boxes = gen.uniform2d(1024, seed=3)
    d = _device(boxes)
    out = torch.zeros((64, 2), dtype=torch.int32, device="cuda")
    rc, n = _noalloc(d, 1024, 2, gen.RANGE, out, 16, out_offset_bytes=4)
    assert rc == EINVAL and n == 0
    assert "8-byte aligned" in _err()


def test_noalloc_rejects_oversized_queries():
    import torch
    d = torch.zeros((300000, 7), dtype=torch.int32, device="cuda")
    out = torch.zeros((16, 2), dtype=torch.int32, device="cuda")
    rc, _ = _noalloc(d, 300000, 3, gen.RANGE, out, 16)
    assert rc == ECAPACITY
    assert "262144" in _err()


def test_noalloc_entry_overflow_reports_zero_pairs_then_recovers():
    """200,000 tiny boxes, each on a corner shared by 8 cells of the coarsened
    grid (64 cells per axis), need 1.6 M cell entries: more than the scratch
    holds. The call says so and leaves *npairs at 0; the next call is exact."""
    import torch
    rng = 1 << 24
    r = np.random.default_rng(5)
    corner = r.choice(63 ** 3, size=200000, replace=False)
    c = np.stack([corner % 63, (corner // 63) % 63, corner // (63 * 63)], axis=1).astype(np.int64) + 1
    boxes = np.empty((200000, 7), dtype=np.uint32)
    boxes[:, 0:6:2] = c * (1 << 18) - 1
    boxes[:, 1:6:2] = c * (1 << 18)
    boxes[:, 6] = np.arange(200000, dtype=np.uint32)
    d = _device(boxes)
    out = torch.zeros((1024, 2), dtype=torch.int32, device="cuda")
    rc, n = _noalloc(d, 200000, 3, rng, out, 1024, shift=18)
    assert rc == ECAPACITY and n == 0
    assert "524288" in _err()
    z = np.load(os.path.join(HERE, "golden", "rand3d_1001.npz"))
    _run_twice(z["boxes"], int(z["range"]), z["pairs"])
