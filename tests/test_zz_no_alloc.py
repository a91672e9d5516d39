"""The allocation-free entry point, pbig2_self_intersect_noalloc, called
through the C ABI.

It serves callers that cannot allocate device memory during a query (their
device memory is owned by another allocator, or they cannot afford the
device-wide synchronization of cudaMalloc/cudaFree): all its intermediate
buffers live in a fixed scratch array inside the library. Its pairs must be
the same set as those of the allocating entry point, pbig2_self_intersect,
on two calls in a row (the second call reuses the scratch the first one
left behind). Collected last so a failure here does not hide the others.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from pbig_gb300 import Engine, gen
from pbig_gb300.engine import lib

pytestmark = pytest.mark.gpu


def _noalloc(d_boxes, n, dims, rng, d_out, cap):
    L = lib()
    npairs = C.c_uint64()
    rc = L.pbig2_self_intersect_noalloc(C.c_void_p(d_boxes.data_ptr()), n, dims, rng, 0xFFFFFFFF,
                                        C.c_void_p(d_out.data_ptr()), cap, C.byref(npairs), None)
    return rc, npairs.value


@pytest.mark.parametrize("which", ["clustered3d", "uniform2d"])
def test_noalloc_matches_allocating_entry_point_twice(which):
    import torch
    if which == "clustered3d":
        boxes, dims = gen.clustered3d(200000, seed=9), 3
    else:
        boxes, dims = gen.uniform2d(65536, seed=0), 2
    rng = gen.RANGE
    with Engine(0) as e:
        n_ref = e.self_intersect(boxes, rng)
        ref = O.sort_pairs(e.pairs())
    d_boxes = torch.from_numpy(boxes.view(np.int32)).cuda()
    cap = n_ref + 1024
    d_out = torch.zeros((cap, 2), dtype=torch.int32, device="cuda")
    for _ in range(2):
        d_out.fill_(-1)
        torch.cuda.synchronize()
        rc, n = _noalloc(d_boxes, boxes.shape[0], dims, rng, d_out, cap)
        assert rc == 0, lib().pbig2_noalloc_last_error().decode()
        assert n == n_ref
        got = O.sort_pairs(d_out[:n].cpu().numpy().view(np.uint32))
        assert np.array_equal(got, ref)


def test_noalloc_rejects_oversized_queries():
    import torch
    d = torch.zeros((300000, 7), dtype=torch.int32, device="cuda")
    out = torch.zeros((16, 2), dtype=torch.int32, device="cuda")
    rc, _ = _noalloc(d, 300000, 3, gen.RANGE, out, 16)
    assert rc == 6  # PBIG2_ECAPACITY
    assert b"262144" in lib().pbig2_noalloc_last_error()
