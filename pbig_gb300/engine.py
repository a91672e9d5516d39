"""Python face of the C ABI (``include/pbig2.h``), via ctypes.

``Engine`` mirrors the reference's ``pbig_init`` / ``pbig_check`` /
``pbig_finalize`` life cycle (src/pbig/pbig.cu:2139, 1962, 141 of awatch/pbig)
with explicit results instead of a callback: a query returns the number of
overlapping pairs and the pairs stay on the device until the next query.

Inputs are PBIG ``RectInfo`` rows (uint32, 5 words in 2-D, 7 in 3-D, rid =
row index): a numpy array (host memory) or a CUDA tensor (device memory;
int32 or uint32, same bit pattern). There is no CPU fallback: without the
CUDA library or a GPU the calls raise.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native

OK, EINVAL, ENOMEM, ECUDA, EINPUT, ETIMEOUT, ECAPACITY, EBUSY = range(8)
HOST, DEVICE = 0, 1
AUTO = 0xFFFFFFFF

EXPORTS = [
    "pbig2_create", "pbig2_destroy", "pbig2_last_error", "pbig2_version", "pbig2_self_intersect",
    "pbig2_bipartite_intersect", "pbig2_batch_intersect", "pbig2_result_pairs", "pbig2_copy_pairs",
    "pbig2_set_pair_output",
    "pbig2_result_scene_offsets", "pbig2_copy_pairs_async", "pbig2_sync", "pbig2_host_alloc",
    "pbig2_host_free", "pbig2_get_stats", "pbig2_tune_shift", "pbig2_self_intersect_noalloc",
    "pbig2_noalloc_last_error", "pbig2_set_option", "pbig2_scene_create", "pbig2_scene_destroy",
    "pbig2_scene_move", "pbig2_scene_delta", "pbig2_scene_pairs", "pbig2_scene_boxes", "pbig2_scene_copy",
    "pbig2_result_records", "pbig2_copy_records", "pbig2_decode_records", "pbig2_serve_batch",
    "pbig2_grid_cells", "pbig2_result_scene_shifts", "pbig2_class_map_auto", "pbig2_class_map_check",
]


class BatchItem(C.Structure):
    """pbig2_batch_item: one scene of a serving batch (pbig2_serve_batch)."""
    _fields_ = [("dev", C.c_void_p), ("host", C.c_void_p), ("n", C.c_uint64), ("rows", C.c_void_p),
                ("idx", C.c_void_p), ("k", C.c_uint64), ("upload", C.c_uint32), ("shift", C.c_uint32)]


class PbigError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"pbig2 error {code}: {msg}")
        self.code = code


class Stats(C.Structure):
    _fields_ = [("boxes", C.c_uint64), ("bad_boxes", C.c_uint64), ("cells", C.c_uint64),
                ("entries", C.c_uint64), ("pair_tests", C.c_uint64), ("pairs", C.c_uint64),
                ("cell_shift", C.c_uint32), ("scenes", C.c_uint32), ("kernels", C.c_uint32),
                ("grid_retries", C.c_uint32), ("device_ms", C.c_double), ("phase_ms", C.c_double * 9),
                ("comp_pairs", C.c_uint64), ("jobs", C.c_uint64), ("max_cell", C.c_uint32),
                ("merged_blocks", C.c_uint32), ("class_map", C.c_uint64), ("merge_limit", C.c_uint32),
                ("pad", C.c_uint32)]

    PHASES = ("count", "scan", "expand", "scatter", "pairs", "group", "pairs_small", "pairs_med", "pairs_block")

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "phase_ms"}
        d["phase_ms"] = dict(zip(self.PHASES, list(self.phase_ms)))
        return d


_LIB = None


def lib():
    """The loaded engine library (built in-tree on first use)."""
    global _LIB
    if _LIB is None:
        L = C.CDLL(_native.lib_path("engine"))
        vp, u64, u32 = C.c_void_p, C.c_uint64, C.c_uint32
        L.pbig2_create.argtypes = [C.c_int, C.POINTER(vp)]
        L.pbig2_destroy.argtypes = [vp]
        L.pbig2_last_error.restype = C.c_char_p
        L.pbig2_self_intersect.argtypes = [vp, vp, u64, u32, u32, u32, C.c_int, vp, C.POINTER(u64)]
        L.pbig2_bipartite_intersect.argtypes = [vp, vp, u64, vp, u64, u32, u32, u32, C.c_int, vp,
                                                C.POINTER(u64)]
        L.pbig2_batch_intersect.argtypes = [vp, vp, C.POINTER(u64), u32, u32, u32, vp, C.c_int, vp,
                                            C.POINTER(u64)]
        L.pbig2_result_pairs.argtypes = [vp, C.POINTER(vp), C.POINTER(u64)]
        L.pbig2_copy_pairs.argtypes = [vp, vp, u64, u64, C.c_int, vp]
        L.pbig2_copy_pairs_async.argtypes = [vp, vp, u64, u64, C.c_int, vp]
        L.pbig2_sync.argtypes = [vp, vp]
        L.pbig2_set_pair_output.argtypes = [vp, vp, u64]
        L.pbig2_scene_create.argtypes = [vp, vp, u64, u32, u32, u32, C.c_int, u32, C.POINTER(vp), C.POINTER(u64)]
        L.pbig2_scene_destroy.argtypes = [vp]
        L.pbig2_scene_move.argtypes = [vp, vp, u64, vp, C.c_int, C.POINTER(u64), C.POINTER(u64)]
        L.pbig2_scene_copy.argtypes = [vp, C.c_int, vp, u64]
        L.pbig2_scene_pairs.argtypes = [vp, C.POINTER(vp), C.POINTER(u64)]
        L.pbig2_result_records.argtypes = [vp, C.POINTER(vp), C.POINTER(u64), C.POINTER(vp), C.POINTER(u64),
                                           C.POINTER(vp), C.POINTER(u64)]
        L.pbig2_copy_records.argtypes = [vp, vp, vp, vp]
        L.pbig2_decode_records.argtypes = [vp, u64, vp, u64, vp, u64, vp, u64, C.POINTER(u64)]
        L.pbig2_result_scene_offsets.argtypes = [vp, C.POINTER(u64), u32]
        L.pbig2_result_scene_shifts.argtypes = [vp, C.POINTER(u32), u32]
        L.pbig2_get_stats.argtypes = [vp, C.POINTER(Stats)]
        L.pbig2_host_alloc.argtypes = [C.c_size_t, C.POINTER(vp)]
        L.pbig2_host_free.argtypes = [vp]
        L.pbig2_tune_shift.argtypes = [vp, u64, u32, u32, u64, C.POINTER(u32)]
        L.pbig2_grid_cells.argtypes = [u32, u32, u32]
        L.pbig2_grid_cells.restype = u64
        L.pbig2_class_map_auto.argtypes = [u32]
        L.pbig2_class_map_auto.restype = u64
        L.pbig2_class_map_check.argtypes = [u64]
        L.pbig2_class_map_check.restype = u32
        L.pbig2_self_intersect_noalloc.argtypes = [vp, u64, u32, u32, u32, vp, u64, C.POINTER(u64), vp]
        L.pbig2_noalloc_last_error.restype = C.c_char_p
        L.pbig2_set_option.argtypes = [vp, C.c_int, C.c_int64]
        L.pbig2_serve_batch.argtypes = [vp, C.POINTER(BatchItem), u32, u32, vp, u64, vp, vp, u64, vp, vp, u64,
                                        C.POINTER(u64), C.POINTER(u64), C.POINTER(C.c_double)]
        _LIB = L
    return _LIB


_LEGACY_STREAM = 0x1  # cudaStreamLegacy


def _check(rc: int, allow=(OK,)) -> int:
    if rc not in allow:
        raise PbigError(rc, lib().pbig2_last_error().decode())
    return rc


def _boxes_arg(boxes):
    """(pointer, n rows, dims, location, keepalive) for a numpy array or a
    CUDA tensor of RectInfo rows."""
    if isinstance(boxes, np.ndarray):
        a = np.ascontiguousarray(boxes, dtype=np.uint32)
        if a.ndim != 2 or a.shape[1] not in (5, 7):
            raise ValueError("boxes must be [n,5] (2-D) or [n,7] (3-D) RectInfo rows")
        return a.ctypes.data, a.shape[0], (a.shape[1] - 1) // 2, HOST, a
    import torch
    t = boxes
    if not isinstance(t, torch.Tensor):
        raise TypeError("boxes must be a numpy array or a torch tensor")
    if t.dim() != 2 or t.shape[1] not in (5, 7) or t.element_size() != 4 or not t.is_contiguous():
        raise ValueError("boxes tensor must be contiguous [n,5] or [n,7] with 4-byte elements")
    loc = DEVICE if t.is_cuda else HOST
    return t.data_ptr(), t.shape[0], (t.shape[1] - 1) // 2, loc, t


@dataclass
class Result:
    npairs: int
    rc: int


class Engine:
    """One CUDA device, its buffers and stream (not thread-safe)."""

    def __init__(self, device: int = 0):
        self._L = lib()
        ctx = C.c_void_p()
        _check(self._L.pbig2_create(device, C.byref(ctx)))
        self._ctx = ctx
        self.device = device
        self.last_rc = OK
        self._keep = None
        self._out = None
        self._nscenes = 1

    def close(self):
        if getattr(self, "_ctx", None):
            self._L.pbig2_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @staticmethod
    def _stream(stream):
        """None: the context's own stream. A torch stream or a raw handle
        otherwise; torch's default stream (handle 0) becomes CUDA's legacy
        default stream, so the query is ordered with torch's work on it (a
        null handle would select the context's own non-blocking stream)."""
        if stream is None:
            return None
        h = getattr(stream, "cuda_stream", stream)
        return C.c_void_p(h if h else _LEGACY_STREAM)

    def self_intersect(self, boxes, range_: int, cell_shift: int | None = None, stream=None,
                       allow_bad: bool = False) -> int:
        """All overlapping pairs of one scene; returns the pair count."""
        ptr, n, dims, loc, keep = _boxes_arg(boxes)
        self._keep = keep
        out = C.c_uint64()
        rc = self._L.pbig2_self_intersect(self._ctx, C.c_void_p(ptr), n, dims, range_,
                                          AUTO if cell_shift is None else cell_shift, loc,
                                          self._stream(stream), C.byref(out))
        self.last_rc = _check(rc, (OK, EINPUT) if allow_bad else (OK,))
        self._nscenes = 1
        return out.value

    def bipartite_intersect(self, red, blue, range_: int, cell_shift: int | None = None, stream=None) -> int:
        """Pairs (red index, blue index) of overlapping red/blue boxes."""
        pr, nr, dr, lr, kr = _boxes_arg(red)
        pb, nb, db, lb, kb = _boxes_arg(blue)
        if dr != db or lr != lb:
            raise ValueError("red and blue must have the same dims and memory location")
        self._keep = (kr, kb)
        out = C.c_uint64()
        rc = self._L.pbig2_bipartite_intersect(self._ctx, C.c_void_p(pr), nr, C.c_void_p(pb), nb, dr, range_,
                                               AUTO if cell_shift is None else cell_shift, lr,
                                               self._stream(stream), C.byref(out))
        self.last_rc = _check(rc)
        self._nscenes = 1
        return out.value

    def batch_intersect(self, boxes, scene_offsets, range_: int, cell_shifts=None, stream=None) -> int:
        """Independent scenes (concatenated boxes, scene_offsets[n_scenes+1])."""
        ptr, n, dims, loc, keep = _boxes_arg(boxes)
        offs = np.ascontiguousarray(scene_offsets, dtype=np.uint64)
        ns = offs.shape[0] - 1
        if ns < 1 or int(offs[-1]) != n:
            raise ValueError("scene_offsets must end at the number of boxes")
        sh = None
        if cell_shifts is not None:
            sh = np.ascontiguousarray(cell_shifts, dtype=np.uint32)
        self._keep = (keep, offs, sh)
        out = C.c_uint64()
        rc = self._L.pbig2_batch_intersect(self._ctx, C.c_void_p(ptr),
                                           offs.ctypes.data_as(C.POINTER(C.c_uint64)), ns, dims, range_,
                                           None if sh is None else C.c_void_p(sh.ctypes.data), loc,
                                           self._stream(stream), C.byref(out))
        self.last_rc = _check(rc)
        self._nscenes = ns
        return out.value

    def serve_batch(self, items, range_: int, cat_dev: int, cat_rows: int, stage_host: int, stage_dev: int,
                    stage_rows: int, stream, pairs_host: int, pairs_cap: int):
        """One serving batch in native code (pbig2_serve_batch): items is a
        ctypes array of BatchItem (cell sizes written back). Returns (rc,
        pairs, per-item pair offsets, host phase ms); rc is OK or ECAPACITY
        (a buffer too small: the pairs stay on the device)."""
        ns = len(items)
        npairs = C.c_uint64()
        offs = np.zeros(ns + 1, dtype=np.uint64)
        ph = (C.c_double * 4)()
        rc = self._L.pbig2_serve_batch(self._ctx, items, ns, range_, C.c_void_p(cat_dev), cat_rows,
                                       C.c_void_p(stage_host), C.c_void_p(stage_dev), stage_rows,
                                       self._stream(stream), C.c_void_p(pairs_host), pairs_cap, C.byref(npairs),
                                       offs.ctypes.data_as(C.POINTER(C.c_uint64)), ph)
        self.last_rc = _check(rc, (OK, ECAPACITY))
        self._nscenes = ns
        return rc, npairs.value, offs, list(ph)

    def scene_offsets(self) -> np.ndarray:
        ns = self._nscenes
        out = np.empty(ns + 1, dtype=np.uint64)
        _check(self._L.pbig2_result_scene_offsets(self._ctx, out.ctypes.data_as(C.POINTER(C.c_uint64)), ns))
        return out

    def scene_shifts(self, n_scenes: int | None = None) -> np.ndarray:
        """Cell size (log2) of every scene of the last query (1 for a self or
        red/blue query)."""
        ns = self._nscenes if n_scenes is None else n_scenes
        out = np.empty(ns, dtype=np.uint32)
        _check(self._L.pbig2_result_scene_shifts(self._ctx, out.ctypes.data_as(C.POINTER(C.c_uint32)), ns))
        return out

    def pairs(self, first: int = 0, count: int | None = None) -> np.ndarray:
        """Pairs of the last query as a host [P,2] uint32 array."""
        n = self.result_count()
        count = n - first if count is None else count
        out = np.empty((count, 2), dtype=np.uint32)
        _check(self._L.pbig2_copy_pairs(self._ctx, C.c_void_p(out.ctypes.data), first, count, HOST, None))
        return out

    def pairs_into(self, dst, first: int = 0, stream=None) -> None:
        """Copy the result into a preallocated host (pinned or not) or device
        buffer: a tensor/array of shape [P,2] with 4-byte elements."""
        if isinstance(dst, np.ndarray):
            ptr, loc, count = dst.ctypes.data, HOST, dst.shape[0]
        else:
            ptr, loc, count = dst.data_ptr(), (DEVICE if dst.is_cuda else HOST), dst.shape[0]
        _check(self._L.pbig2_copy_pairs_async(self._ctx, C.c_void_p(ptr), first, count, loc, self._stream(stream)))

    def set_pair_output(self, dst) -> None:
        """Later self/bipartite queries store their pairs straight into dst
        (a page-locked host or a device tensor [cap,2] of 4-byte elements);
        None restores the context's own buffer. A result larger than dst is
        redone into the context's buffer (``result_in(dst)`` tells)."""
        if dst is None:
            _check(self._L.pbig2_set_pair_output(self._ctx, None, 0))
            self._out = None
            return
        if dst.dim() != 2 or dst.shape[1] != 2 or dst.element_size() != 4 or not dst.is_contiguous():
            raise ValueError("pair output must be a contiguous [cap,2] tensor of 4-byte elements")
        _check(self._L.pbig2_set_pair_output(self._ctx, C.c_void_p(dst.data_ptr()), dst.shape[0]))
        self._out = dst

    def result_in(self, dst) -> bool:
        """True when the last result's pairs are in dst (set_pair_output)."""
        return dst is not None and self.device_pairs()[0] == dst.data_ptr()

    def sync(self, stream=None):
        _check(self._L.pbig2_sync(self._ctx, self._stream(stream)))

    def device_pairs(self):
        """(device pointer, count) of the resident result."""
        p = C.c_void_p()
        n = C.c_uint64()
        _check(self._L.pbig2_result_pairs(self._ctx, C.byref(p), C.byref(n)))
        return p.value, n.value

    def result_count(self) -> int:
        return self.device_pairs()[1]

    def set_merged(self, on: bool) -> None:
        """The reference's MERGED=1 build: sparse cells merged into blocks of
        at most 256 entries, pairs tested per block (same pair set, the merged
        build's work statistics)."""
        _check(self._L.pbig2_set_option(self._ctx, 2, int(bool(on))))

    def set_records(self, on: bool) -> None:
        """Self queries return the reference's Rice record stream (PBIG2_OPT_RICE)."""
        _check(self._L.pbig2_set_option(self._ctx, 3, int(bool(on))))

    def records(self):
        """(words uint64, StartI uint32, Recs uint32) of the last record-mode
        query, copied to the host."""
        vp = C.c_void_p
        w, si, rc = vp(), vp(), vp()
        nw, nc, ne = C.c_uint64(), C.c_uint64(), C.c_uint64()
        _check(self._L.pbig2_result_records(self._ctx, C.byref(w), C.byref(nw), C.byref(si), C.byref(nc),
                                            C.byref(rc), C.byref(ne)))
        words = np.empty(nw.value, dtype=np.uint64)
        start_i = np.empty(nc.value, dtype=np.uint32)
        recs = np.empty(ne.value, dtype=np.uint32)
        _check(self._L.pbig2_copy_records(self._ctx, vp(words.ctypes.data), vp(start_i.ctypes.data),
                                          vp(recs.ctypes.data)))
        return words, start_i, recs

    def set_host_split(self, sms: int) -> None:
        """SMs of the small-cell and block kernels beside the medium-cell
        kernel when pairs go to page-locked host memory (0: automatic, a
        quarter; negative: one after another)."""
        _check(self._L.pbig2_set_option(self._ctx, 4, int(sms)))

    def set_one_launch(self, on: bool) -> None:
        """Run small self queries (at most 262 144 boxes) as one cooperative
        kernel launch (on by default); off: the regular pipeline."""
        _check(self._L.pbig2_set_option(self._ctx, 5, int(bool(on))))

    def set_class_map(self, cmap: int) -> None:
        """Which pair kernel takes a cell of n boxes (PBIG2_OPT_CLASS_MAP):
        nibble ceil(log2 n) names the list; 0 restores the automatic choice."""
        _check(self._L.pbig2_set_option(self._ctx, 6, int(cmap) - (1 << 64) if cmap >= 1 << 63 else int(cmap)))

    def set_merge_limit(self, limit: int) -> None:
        """Merged mode's block limit in boxes (PBIG2_OPT_MERGE_LIMIT; 0: 256)."""
        _check(self._L.pbig2_set_option(self._ctx, 7, int(limit)))

    def set_graphs(self, on: bool) -> None:
        """Capture/replay batched queries as CUDA graphs (on by default)."""
        _check(self._L.pbig2_set_option(self._ctx, 1, int(bool(on))))

    def stats(self) -> dict:
        s = Stats()
        _check(self._L.pbig2_get_stats(self._ctx, C.byref(s)))
        return s.as_dict()


def decode_records(words: np.ndarray, start_i: np.ndarray, recs: np.ndarray) -> np.ndarray:
    """pbig2_decode_records: a Rice record stream (host arrays) -> [P,2] pairs."""
    L = lib()
    w = np.ascontiguousarray(words, dtype=np.uint64)
    si = np.ascontiguousarray(start_i, dtype=np.uint32)
    rc = np.ascontiguousarray(recs, dtype=np.uint32)
    n = C.c_uint64()
    vp = C.c_void_p
    args = (vp(w.ctypes.data), w.shape[0], vp(si.ctypes.data), si.shape[0], vp(rc.ctypes.data), rc.shape[0])
    _check(L.pbig2_decode_records(*args, None, 0, C.byref(n)), (OK, ECAPACITY))
    out = np.empty((n.value, 2), dtype=np.uint32)
    _check(L.pbig2_decode_records(*args, vp(out.ctypes.data), n.value, C.byref(n)))
    return out


class Scene:
    """A resident scene (pbig2_scene_*): boxes, a grid with slack and the
    full pair list stay on the device; move() re-bins only the moved boxes
    and reports the pairs they had before and have after the move."""

    def __init__(self, engine: Engine, boxes: np.ndarray, range_: int, cell_shift: int | None = None,
                 keep_pairs: bool = True):
        self._L = engine._L
        self._eng = engine  # the scene uses the engine's stream and buffers
        ptr, n, dims, loc, keep = _boxes_arg(boxes)
        self.dims = dims
        sc = C.c_void_p()
        out = C.c_uint64()
        _check(self._L.pbig2_scene_create(engine._ctx, C.c_void_p(ptr), n, dims, range_,
                                           AUTO if cell_shift is None else cell_shift, loc,
                                           0 if keep_pairs else 1, C.byref(sc), C.byref(out)))
        self._sc = sc
        self.npairs = out.value
        self.nremoved = self.nadded = 0

    def move(self, idx, new_boxes) -> tuple[int, int]:
        """Boxes idx get the coordinates of new_boxes (RectInfo rows whose rid
        is the index); returns (pairs the moved boxes had, pairs they have)."""
        idx = np.ascontiguousarray(idx, dtype=np.uint32)
        nb = np.ascontiguousarray(new_boxes, dtype=np.uint32)
        if nb.shape != (idx.shape[0], 2 * self.dims + 1):
            raise ValueError("new_boxes must hold one RectInfo row per index")
        r, a = C.c_uint64(), C.c_uint64()
        _check(self._L.pbig2_scene_move(self._sc, C.c_void_p(idx.ctypes.data), idx.shape[0],
                                        C.c_void_p(nb.ctypes.data), HOST, C.byref(r), C.byref(a)))
        self.nremoved, self.nadded = r.value, a.value
        return r.value, a.value

    def _copy(self, which: int, count: int, out=None) -> np.ndarray:
        if out is None:
            out = np.empty((count, 2), dtype=np.uint32)
        elif out.shape[0] < count or out.shape[1:] != (2,) or out.dtype.itemsize != 4 or not out.flags.c_contiguous:
            raise ValueError("output array too small or not a contiguous [n,2] array of 4-byte elements")
        _check(self._L.pbig2_scene_copy(self._sc, which, C.c_void_p(out.ctypes.data), count))
        return out[:count]

    def pairs(self) -> np.ndarray:
        p = C.c_void_p()
        n = C.c_uint64()
        _check(self._L.pbig2_scene_pairs(self._sc, C.byref(p), C.byref(n)))
        return self._copy(0, n.value)

    def delta(self, out_removed=None, out_added=None) -> tuple[np.ndarray, np.ndarray]:
        """(pairs the moved boxes had, pairs they have) of the last move, as
        host arrays (written into the given arrays -- page-locked ones make
        the copies fast -- when passed)."""
        return self._copy(1, self.nremoved, out_removed), self._copy(2, self.nadded, out_added)

    def close(self):
        if getattr(self, "_sc", None):
            self._L.pbig2_scene_destroy(self._sc)
            self._sc = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tune_shift(boxes: np.ndarray, range_: int, sample: int = 4096) -> int:
    a = np.ascontiguousarray(boxes, dtype=np.uint32)
    out = C.c_uint32()
    _check(lib().pbig2_tune_shift(C.c_void_p(a.ctypes.data), a.shape[0], (a.shape[1] - 1) // 2, range_, sample,
                                  C.byref(out)))
    return out.value
