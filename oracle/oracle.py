"""ORACLE (test infrastructure only): ctypes bindings to ``oracle.c``, the
CPU restatement of the reference's pair-detection path.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg use this module, and only as the checker / timed CPU baseline; the
product (``pbig_gb300``) never imports it.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


class OrcStats(C.Structure):
    _fields_ = [("cs", C.c_uint32), ("shift", C.c_uint32), ("nrc", C.c_uint32), ("ncells", C.c_uint32),
                ("entries", C.c_uint64), ("jobs", C.c_uint64), ("batches", C.c_uint64),
                ("comp_pairs", C.c_uint64), ("pairs", C.c_uint64), ("max_cell", C.c_uint32),
                ("would_abort", C.c_uint32), ("tests", C.c_uint64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "_build", "liborc.so")
        if not os.path.exists(path):
            import sys
            sys.path.insert(0, os.path.dirname(_HERE))
            from pbig_gb300 import build as _b
            _b.build()
        L = C.CDLL(path)
        u32p = C.POINTER(C.c_uint32)
        L.orc_grid_pairs.argtypes = [u32p, C.c_uint32, C.c_int, C.c_uint32, C.c_uint32, C.c_int, C.c_uint64,
                                     C.c_int, u32p, C.c_uint64, C.POINTER(OrcStats)]
        L.orc_grid_pairs.restype = C.c_int
        L.orc_brute_pairs.argtypes = [u32p, C.c_uint32, C.c_int, C.c_int, u32p, C.c_uint64,
                                      C.POINTER(C.c_uint64)]
        L.orc_brute_pairs.restype = C.c_int
        L.orc_decide_cell_size.argtypes = [u32p, C.c_uint32, C.c_int, C.c_uint32, C.c_uint64]
        L.orc_decide_cell_size.restype = C.c_uint32
        L.orc_gen_harness.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_char_p, C.c_uint32, C.c_int, u32p]
        L.orc_gen_harness.restype = C.c_int
        L.orc_sort_pairs.argtypes = [u32p, C.c_uint64]
        L.orc_decode_rice.argtypes = [C.c_void_p, C.c_uint64, u32p, C.c_uint64, u32p, C.c_uint64, u32p, C.c_uint64]
        L.orc_decode_rice.restype = C.c_int64
        L.orc_sort_pairs.restype = None
        L.orc_srand.argtypes = [C.c_void_p, C.c_uint32]
        L.orc_rand.argtypes = [C.c_void_p]
        L.orc_rand.restype = C.c_int32
        _LIB = L
    return _LIB


def _ptr(a: np.ndarray):
    assert a.dtype == np.uint32 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


def threads_default() -> int:
    return os.cpu_count() or 1


def dims_of(boxes: np.ndarray) -> int:
    w = boxes.shape[1]
    assert w in (5, 7), "boxes must be RectInfo rows of 5 (2-D) or 7 (3-D) words"
    return (w - 1) // 2


def grid_pairs(boxes: np.ndarray, range_: int, cs: int = 0, merged: bool = False, threads: int | None = None,
               count_only: bool = False, free_bytes: int = 280 << 30):
    """Reference pipeline on the CPU. Returns (pairs[P,2] sorted or None, stats)."""
    L = lib()
    boxes = np.ascontiguousarray(boxes, dtype=np.uint32)
    n, dims = boxes.shape[0], dims_of(boxes)
    st = OrcStats()
    th = threads or threads_default()
    if count_only:
        rc = L.orc_grid_pairs(_ptr(boxes), n, dims, range_, cs, int(merged), free_bytes, th, None, 0, C.byref(st))
        if rc < 0:
            raise RuntimeError("oracle grid failed")
        return None, st.as_dict()
    cap = max(1024, 4 * n)
    while True:
        out = np.empty((cap, 2), dtype=np.uint32)
        rc = L.orc_grid_pairs(_ptr(boxes), n, dims, range_, cs, int(merged), free_bytes, th, _ptr(out), cap,
                              C.byref(st))
        if rc < 0:
            raise RuntimeError("oracle grid failed")
        if rc == 0:
            break
        cap = int(st.pairs) + 16
    p = out[: st.pairs].copy()
    L.orc_sort_pairs(_ptr(p), p.shape[0])
    return p, st.as_dict()


def brute_pairs(boxes: np.ndarray, threads: int | None = None) -> np.ndarray:
    """All-pairs O(N^2) closed-interval test; sorted canonical pairs."""
    L = lib()
    boxes = np.ascontiguousarray(boxes, dtype=np.uint32)
    n, dims = boxes.shape[0], dims_of(boxes)
    cap = max(1024, 4 * n)
    while True:
        out = np.empty((cap, 2), dtype=np.uint32)
        npairs = C.c_uint64()
        rc = L.orc_brute_pairs(_ptr(boxes), n, dims, threads or threads_default(), _ptr(out), cap,
                               C.byref(npairs))
        if rc == 0:
            break
        cap = int(npairs.value) + 16
    p = out[: npairs.value].copy()
    L.orc_sort_pairs(_ptr(p), p.shape[0])
    return p


def sort_pairs(p: np.ndarray) -> np.ndarray:
    p = np.ascontiguousarray(p, dtype=np.uint32).reshape(-1, 2)
    lo = np.minimum(p[:, 0], p[:, 1])
    hi = np.maximum(p[:, 0], p[:, 1])
    q = np.ascontiguousarray(np.stack([lo, hi], axis=1))
    lib().orc_sort_pairs(_ptr(q), q.shape[0])
    return q


def decode_rice(words: np.ndarray, start_i: np.ndarray, recs: np.ndarray) -> np.ndarray:
    """The reference's decode of a Rice record stream (decode.cc:26-138, with
    the column offset fixed): [P,2] (min, max) pairs in stream order."""
    L = lib()
    w = np.ascontiguousarray(words, dtype=np.uint64)
    si = np.ascontiguousarray(start_i, dtype=np.uint32)
    rc = np.ascontiguousarray(recs, dtype=np.uint32)
    args = [w.ctypes.data_as(C.c_void_p), w.shape[0], _ptr(si), si.shape[0], _ptr(rc), rc.shape[0]]
    n = L.orc_decode_rice(*args, None, 0)
    if n < 0:
        raise ValueError("malformed record stream")
    out = np.empty((n, 2), dtype=np.uint32)
    L.orc_decode_rice(*args, _ptr(out), n)
    return out


def harness_boxes(n: int, S: int = 100, range_: int = 10000, sim: str = "UU", seed: int = 100,
                  dims: int = 3) -> np.ndarray:
    """The reference harness's box generator (src/pbig/main.cc:223-335)."""
    out = np.empty((n, 2 * dims + 1), dtype=np.uint32)
    lib().orc_gen_harness(n, S, range_, sim.encode(), seed, dims, _ptr(out))
    return out


def decide_cell_size(boxes: np.ndarray, range_: int, free_bytes: int = 280 << 30) -> int:
    boxes = np.ascontiguousarray(boxes, dtype=np.uint32)
    return int(lib().orc_decide_cell_size(_ptr(boxes), boxes.shape[0], dims_of(boxes), range_, free_bytes))


def rand_sequence(seed: int, k: int) -> list[int]:
    st = C.create_string_buffer(256)
    L = lib()
    L.orc_srand(st, seed)
    return [L.orc_rand(st) for _ in range(k)]
