"""Seeded synthetic workloads (ctypes over ``csrc/gen.c``).

All boxes are fp32 in [0,1) quantised to PBIG's unsigned-int coordinates with
maxRange ``RANGE = 2**24`` (q(f) = min(floor(f * 2^24), 2^24 - 1)), returned as
``RectInfo`` rows: ``[xmin, xmax, ymin, ymax, (zmin, zmax,) rid]`` (uint32).
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os

import numpy as np

from . import _native

RANGE = 1 << 24

_L = None


def _lib():
    global _L
    if _L is None:
        L = C.CDLL(_native.lib_path("gen"))
        u32p = C.POINTER(C.c_uint32)
        L.pbig_gen_uniform2d.argtypes = [C.c_uint64, C.c_uint64, C.c_double, C.c_double, u32p, C.c_int]
        L.pbig_gen_clustered3d.argtypes = [C.c_uint64, C.c_uint64, C.c_double, C.c_double, u32p, C.c_int]
        L.pbig_gen_mixed3d.argtypes = [C.c_uint64, C.c_uint64, C.c_double, u32p, C.c_int]
        L.pbig_gen_scene3d.argtypes = [C.c_uint64, C.c_uint64, u32p, C.c_int]
        L.pbig_gen_loguniform.argtypes = [C.c_uint64, C.c_uint64, C.c_double, C.c_double]
        L.pbig_gen_loguniform.restype = C.c_uint64
        L.pbig_gen_uniform.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64]
        L.pbig_gen_uniform.restype = C.c_double
        L.pbig_gen_normal.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64]
        L.pbig_gen_normal.restype = C.c_double
        L.pbig_gen_move3d.argtypes = [u32p, u32p, C.c_uint64, C.c_uint64, C.c_double]
        L.pbig_gen_pick.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64, u32p]
        for f in ("log", "exp", "cos2pi", "log_nodiv", "cos2pi_nodiv"):
            fn = getattr(L, "pbig_gen_" + f)
            fn.argtypes = [C.c_double]
            fn.restype = C.c_double
        _L = L
    return _L


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


def _threads():
    return min(32, os.cpu_count() or 1)


def uniform2d(n: int = 65536, seed: int = 0, side=(0.001, 0.005)) -> np.ndarray:
    """Plain 2-D scene: lower corners U[0,1)^2, sides U[side] per axis."""
    out = np.empty((n, 5), dtype=np.uint32)
    _lib().pbig_gen_uniform2d(n, seed, side[0], side[1], _p(out), _threads())
    return out


def clustered3d(n: int = 4194304, seed: int = 0, sigma: float = 0.02, log_sigma: float = 0.5) -> np.ndarray:
    """3-D mixture of 64 isotropic Gaussians (means U[0.1,0.9]^3), sides
    lognormal(ln 0.002, log_sigma) per axis."""
    out = np.empty((n, 7), dtype=np.uint32)
    _lib().pbig_gen_clustered3d(n, seed, sigma, log_sigma, _p(out), _threads())
    return out


def mixed3d(n: int = 2097152, seed: int = 0, large_frac: float = 0.01) -> np.ndarray:
    """3-D uniform centres, sides U[0.001,0.004], a fraction with U[0.02,0.1]."""
    out = np.empty((n, 7), dtype=np.uint32)
    _lib().pbig_gen_mixed3d(n, seed, large_frac, _p(out), _threads())
    return out


def scene3d(n: int, seed: int, out: np.ndarray | None = None) -> np.ndarray:
    """One batched/serving scene: uniform centres, sides U[0.5,2]*n^(-1/3)*0.5
    (written into `out`, a C-contiguous [n,7] uint32 view, when given)."""
    if out is None:
        out = np.empty((n, 7), dtype=np.uint32)
    assert out.shape == (n, 7) and out.dtype == np.uint32 and out.flags.c_contiguous
    _lib().pbig_gen_scene3d(n, seed, _p(out), _threads())
    return out


def scene_batch(count: int = 4096, seed: int = 0, lo: int = 256, hi: int = 262144):
    """Batched-scenes workload: `count` scenes with log-uniform sizes in
    [lo, hi], scene i generated with seed 1000003*seed + i; returns (boxes
    concatenated, scene offsets[count+1])."""
    sizes = scene_sizes(count, seed, lo, hi)
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    boxes = np.empty((int(offs[-1]), 7), dtype=np.uint32)
    for i, n in enumerate(sizes):
        scene3d(int(n), 1000003 * seed + i, out=boxes[int(offs[i]):int(offs[i + 1])])
    return boxes, offs


def scene_sizes(count: int, seed: int, lo: float, hi: float) -> np.ndarray:
    L = _lib()
    return np.array([L.pbig_gen_loguniform(seed, i, lo, hi) for i in range(count)], dtype=np.int64)


def uniform(seed: int, stream: int, idx: int) -> float:
    return _lib().pbig_gen_uniform(seed, stream, idx)


def normal(seed: int, stream: int, idx: int) -> float:
    return _lib().pbig_gen_normal(seed, stream, idx)


def move3d(boxes: np.ndarray, idx: np.ndarray, seed: int, sigma: float = 0.001) -> None:
    """In place: shift the listed boxes by N(0, sigma) per axis and re-quantise."""
    assert boxes.dtype == np.uint32 and boxes.shape[1] == 7 and boxes.flags.c_contiguous
    idx = np.ascontiguousarray(idx, dtype=np.uint32)
    _lib().pbig_gen_move3d(_p(boxes), _p(idx), idx.shape[0], seed, sigma)


def pick(n: int, k: int, seed: int) -> np.ndarray:
    """k distinct sorted indices in [0, n): one drawn uniformly from each of
    k equal strata (seeded)."""
    out = np.empty(k, dtype=np.uint32)
    if _lib().pbig_gen_pick(n, k, seed, _p(out)) != 0:
        raise ValueError("need 0 < k <= n")
    return out


def digest(boxes: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(boxes).tobytes()).hexdigest()
