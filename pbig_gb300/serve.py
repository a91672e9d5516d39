"""Continuous-batching request loop for scene queries.

Requests arrive over time. Each is either a *query* of a new scene (its boxes
come from the host) or an *update* of a resident scene (a fraction of its
boxes moved in place); either way the answer is the scene's full set of
overlapping pairs, copied to the host.

The server keeps every scene's boxes resident on the device (with its cell
size, chosen once by the autotuner) under a device-memory budget; when a new
batch does not fit, the device copies of the least recently used idle scenes
are dropped (their host copies stay, and a later request uploads them again). Whenever one of its slots
(an engine context with its own stream and buffers) is free it takes every
pending request it can admit -- requests that arrived while other batches
were on the GPU -- and resolves them as one batched query; two slots keep
two batches in flight, so the copies and the host work of one overlap the
kernels of the other. A scene is in at most one batch at a time.

A batch's work after the admission decision -- cell sizes of new scenes,
update rows, uploads, concatenation, the batched query and the download of
the pairs -- is one native call (pbig2_serve_batch) that holds no
interpreter lock, so the slot threads and the dispatcher run concurrently.
"""
from __future__ import annotations

import collections
import gc
import sys
import threading
import time
from dataclasses import dataclass

import numpy as np

from . import gen
from .engine import AUTO, ECAPACITY, BatchItem, Engine, tune_shift

BOX_BYTES = 28
WORK_BYTES_PER_BOX = 160  # device working memory of a query per box (grid, entries, lists, pairs)


@dataclass
class Request:
    rid: int
    arrival: float             # seconds, relative to the start of the run
    scene: int
    kind: str                  # "query" or "update"
    boxes: np.ndarray | None = None     # query: host RectInfo rows
    move_frac: float = 0.01    # update: fraction of boxes moved
    move_seed: int = 0
    move_sigma: float = 0.001
    idx: np.ndarray | None = None       # update: indices of the moved boxes (sorted, distinct)
    rows: np.ndarray | None = None      # update: their new RectInfo rows
    # filled by the server
    start: float = 0.0
    done: float = 0.0
    npairs: int = 0
    pairs: np.ndarray | None = None
    batch: int = -1
    snapshot: np.ndarray | None = None  # scene boxes as queried (kept when the server records them)
    nboxes: int = 0


class _Arena:
    """First-fit allocator over one device allocation of int32 words: the
    resident scenes live in it, so uploading a scene never calls cudaMalloc
    (which blocks the whole device) while requests wait. Blocks are rounded
    to 64 words (256 bytes)."""

    def __init__(self, torch, words: int, device: int):
        self.buf = torch.empty(max(64, words), dtype=torch.int32, device=f"cuda:{device}")
        self.free = [(0, self.buf.shape[0])]  # (offset, length), sorted by offset

    @staticmethod
    def _round(words: int) -> int:
        return (words + 63) & ~63

    def alloc(self, words: int):
        w = self._round(words)
        for i, (off, ln) in enumerate(self.free):
            if ln >= w:
                if ln == w:
                    del self.free[i]
                else:
                    self.free[i] = (off + w, ln - w)
                return off
        return None

    def release(self, off: int, words: int) -> None:
        w = self._round(words)
        i = 0
        while i < len(self.free) and self.free[i][0] < off:
            i += 1
        self.free.insert(i, (off, w))
        # coalesce with the neighbours
        if i + 1 < len(self.free) and self.free[i][0] + self.free[i][1] == self.free[i + 1][0]:
            self.free[i] = (off, self.free[i][1] + self.free[i + 1][1])
            del self.free[i + 1]
        if i > 0 and self.free[i - 1][0] + self.free[i - 1][1] == self.free[i][0]:
            self.free[i - 1] = (self.free[i - 1][0], self.free[i - 1][1] + self.free[i][1])
            del self.free[i]


@dataclass
class Scene:
    sid: int
    host: np.ndarray           # master copy (host)
    dev: object                # torch tensor [n,7] int32 on the device
    shift: int
    last_used: float = 0.0
    busy: bool = False
    arena_off: int | None = None  # where dev lives in the server's arena

    @property
    def bytes(self) -> int:
        return self.host.shape[0] * BOX_BYTES


class Server:
    def __init__(self, device: int = 0, budget_bytes: int = 40 << 30, slots: int = 2,
                 max_batch_boxes: int = 64 << 20, keep_pairs: bool = True, keep_snapshots: bool = False,
                 copy_pairs: bool = True, reserve_boxes: int = 0):
        import torch
        self.torch = torch
        self.device = device
        self.budget = budget_bytes
        self.max_batch_boxes = max_batch_boxes
        self.keep_pairs = keep_pairs
        self.keep_snapshots = keep_snapshots
        self.copy_pairs = copy_pairs
        self.scenes: "collections.OrderedDict[int, Scene]" = collections.OrderedDict()
        self.resident_bytes = 0
        self.inflight_bytes = 0
        self.pending: collections.deque[Request] = collections.deque()
        self.done: list[Request] = []
        self.lock = threading.Condition()
        self.engines = [Engine(device) for _ in range(slots)]
        for e in self.engines:
            e.set_graphs(False)  # every batch has a new layout
        # each slot orders its uploads and its batch on its own stream, and
        # downloads pairs into its own page-locked buffer
        self.streams = [torch.cuda.Stream(device=device) for _ in range(slots)]
        # capacity reserved up front: a synthetic batch of reserve_boxes boxes
        # (four scenes) through every slot grows its engine buffers, and the
        # page-locked pair buffers start at twice as many pairs, so batches up
        # to that size allocate nothing (no cudaMalloc / cudaHostAlloc while
        # requests wait)
        pairs0 = max(1 << 20, 2 * reserve_boxes)
        self.pinned = [torch.empty((pairs0, 2), dtype=torch.int32).pin_memory() for _ in range(slots)]
        # per-slot device buffer the batch's scenes are concatenated into
        self.catbuf = [torch.empty((max(reserve_boxes, 1 << 16), 7), dtype=torch.int32, device=f"cuda:{device}")
                       for _ in range(slots)]
        self.arena = _Arena(torch, budget_bytes // 4, device)
        if reserve_boxes:
            q = reserve_boxes // 4
            parts = [gen.scene3d(q, 424242 + k) for k in range(4)]
            offs = np.array([0, q, 2 * q, 3 * q, 4 * q], dtype=np.uint64)
            boxes = torch.from_numpy(np.concatenate(parts).view(np.int32)).to(f"cuda:{device}")
            shifts = np.array([tune_shift(b, gen.RANGE, 256) for b in parts], dtype=np.uint32)
            for e, st in zip(self.engines, self.streams):
                e.batch_intersect(boxes, offs, gen.RANGE, cell_shifts=shifts, stream=st)
                e.sync(st)
            del boxes
        # staged update rows (7 words and the box index), host and device
        self.staging = [torch.empty((1 << 16, 8), dtype=torch.int32).pin_memory() for _ in range(slots)]
        self.stage_dev = [torch.empty((1 << 16, 8), dtype=torch.int32, device=f"cuda:{device}")
                          for _ in range(slots)]
        self.free_slots = list(range(slots))
        self.batches = 0
        gc.collect()  # before the clock starts: serve() runs with the collector paused
        self.t0 = time.perf_counter()
        self.busy_time = 0.0
        self.evictions = 0
        self.refused = 0
        self.phase_s = collections.defaultdict(float)  # host seconds per batch phase (summed)
        self.batch_log: list[tuple] = []  # (start s, boxes, requests, prepare, concat, query, download ms)

    # ---- request intake -------------------------------------------------
    def now(self) -> float:
        return time.perf_counter() - self.t0

    def submit(self, req: Request) -> None:
        with self.lock:
            self.pending.append(req)
            self.lock.notify_all()

    # ---- memory ---------------------------------------------------------
    def _evict_for(self, need: int, protect: set[int]) -> bool:
        """Drop the device copies of idle scenes (least recently used first)
        until `need` more bytes fit the budget; False if impossible."""
        while self.resident_bytes + self.inflight_bytes + need > self.budget:
            victim = None
            for sid, sc in self.scenes.items():
                if sc.dev is not None and not sc.busy and sid not in protect:
                    victim = sc
                    break
            if victim is None:
                return False
            self._drop(victim)
        return True

    def _drop(self, sc: Scene) -> None:
        """Forget a scene's device copy (its host copy stays)."""
        if sc.arena_off is not None:
            self.arena.release(sc.arena_off, sc.host.size)
            sc.arena_off = None
        sc.dev = None
        self.resident_bytes -= sc.bytes
        self.evictions += 1

    def _place(self, sc: Scene, dev: str) -> None:
        """Give a scene a device home (its rows are copied by the batch's
        native step): in the arena (evicting idle scenes, least recently used
        first, when it is too fragmented), else through the caching
        allocator."""
        torch = self.torch
        with self.lock:
            off = self.arena.alloc(sc.host.size)
            while off is None:
                victim = next((v for v in self.scenes.values()
                               if v.dev is not None and not v.busy and v.arena_off is not None), None)
                if victim is None:
                    break
                self._drop(victim)
                off = self.arena.alloc(sc.host.size)
        if off is None:
            sc.dev = torch.empty((sc.host.shape[0], 7), dtype=torch.int32, device=dev)
            return
        sc.arena_off = off
        sc.dev = self.arena.buf[off:off + sc.host.size].view(sc.host.shape[0], 7)

    def _take_batch(self) -> list[Request]:
        """Pending requests that can run now (caller holds the lock)."""
        batch, boxes, keep = [], 0, collections.deque()
        in_batch: set[int] = set()
        while self.pending:
            r = self.pending.popleft()
            sc = self.scenes.get(r.scene)
            if r.scene in in_batch or (sc is not None and sc.busy):
                keep.append(r)          # its scene is already in a batch
                continue
            if r.kind == "update" and sc is None:
                keep.append(r)          # the scene is not resident yet (its query is still pending)
                continue
            n = sc.host.shape[0] if sc is not None else r.boxes.shape[0]
            if batch and boxes + n > self.max_batch_boxes:
                keep.append(r)
                continue
            upload = sc is None or sc.dev is None
            need = (n * BOX_BYTES if upload else 0) + n * WORK_BYTES_PER_BOX
            if not self._evict_for(need, in_batch):
                if not batch and not self.scenes_busy():
                    self.refused += 1   # cannot fit even alone: refused
                else:
                    keep.append(r)
                continue
            self.inflight_bytes += n * WORK_BYTES_PER_BOX
            if upload:
                self.resident_bytes += n * BOX_BYTES
            if sc is None:
                sc = Scene(r.scene, r.boxes, None, -1)
                self.scenes[r.scene] = sc
            sc.busy = True
            self.scenes.move_to_end(r.scene)
            in_batch.add(r.scene)
            batch.append(r)
            boxes += n
        keep.extend(self.pending)
        self.pending = keep
        return batch

    def scenes_busy(self) -> bool:
        return any(sc.busy for sc in self.scenes.values())

    # ---- batch execution (slot thread) ------------------------------------
    def _run_batch(self, slot: int, batch: list[Request]) -> None:
        """A batch on one slot: device homes for scenes that need an upload
        (Python, under the server lock), then one native call
        (pbig2_serve_batch, no interpreter lock held) does the rest -- cell
        sizes of new scenes, update rows into the host and device copies,
        uploads, concatenation, the batched query and the download of the
        pairs into the slot's page-locked buffer."""
        torch = self.torch
        eng = self.engines[slot]
        t_start = self.now()
        for r in batch:
            r.start = t_start
        scenes = [self.scenes[r.scene] for r in batch]
        dev = f"cuda:{self.device}"
        stream = self.streams[slot]
        tp = [time.perf_counter()]
        items = (BatchItem * len(batch))()
        keep = []  # arrays the native step reads
        staged = total = 0
        for i, (r, sc) in enumerate(zip(batch, scenes)):
            r.nboxes = sc.host.shape[0]
            upload = sc.dev is None
            if upload:
                self._place(sc, dev)
            it = items[i]
            it.dev = sc.dev.data_ptr()
            it.host = sc.host.ctypes.data
            it.n = sc.host.shape[0]
            if r.kind == "update":
                rows = np.ascontiguousarray(r.rows, dtype=np.uint32)
                idx = np.ascontiguousarray(r.idx, dtype=np.uint32)
                keep += [rows, idx]
                it.rows, it.idx, it.k = rows.ctypes.data, idx.ctypes.data, idx.shape[0]
                if not upload:
                    staged += idx.shape[0]
            it.upload = 1 if upload else 0
            it.shift = sc.shift if sc.shift >= 0 else AUTO
            total += sc.host.shape[0]
        if self.staging[slot].shape[0] < staged:
            self.staging[slot] = torch.empty((int(staged * 1.25) + 1024, 8), dtype=torch.int32).pin_memory()
            self.stage_dev[slot] = torch.empty((int(staged * 1.25) + 1024, 8), dtype=torch.int32, device=dev)
        if len(batch) > 1 and self.catbuf[slot].shape[0] < total:
            self.catbuf[slot] = torch.empty((total, 7), dtype=torch.int32, device=dev)
        tp.append(time.perf_counter())
        buf = self.pinned[slot]
        rc, npairs, so, ph = eng.serve_batch(items, gen.RANGE, self.catbuf[slot].data_ptr(),
                                             self.catbuf[slot].shape[0], self.staging[slot].data_ptr(),
                                             self.stage_dev[slot].data_ptr(), self.staging[slot].shape[0],
                                             stream, buf.data_ptr(), buf.shape[0])
        if rc == ECAPACITY:  # more pairs than the slot's page-locked buffer holds: grow it, copy again
            self.pinned[slot] = torch.empty((int(npairs * 1.25) + 1024, 2), dtype=torch.int32).pin_memory()
            buf = self.pinned[slot]
            eng.pairs_into(buf[:npairs], stream=stream)
            eng.sync(stream)
        tp.append(time.perf_counter())
        allp = None
        if self.keep_pairs:
            allp = buf[:npairs].numpy().view(np.uint32)
            if self.copy_pairs:  # the pinned buffer is reused by the slot's next batch
                allp = allp.copy()
        t_done = self.now()
        for i, (r, sc) in enumerate(zip(batch, scenes)):
            sc.shift = int(items[i].shift)
            r.npairs = int(so[i + 1] - so[i])
            if self.keep_pairs:
                r.pairs = allp[int(so[i]):int(so[i + 1])]
            if self.keep_snapshots:
                r.snapshot = sc.host.copy()
            r.done = t_done
            r.batch = self.batches
        py_ms = (tp[1] - tp[0]) * 1e3
        with self.lock:
            for name, v in zip(("prepare", "concat", "query", "download"), (py_ms + ph[0], ph[1], ph[2], ph[3])):
                self.phase_s[name] += v * 1e-3
            # (start s, boxes, requests, prepare, concat, query, download ms, Python part of the preparation ms)
            self.batch_log.append((t_start, sum(r.nboxes for r in batch), len(batch),
                                   py_ms + ph[0], ph[1], ph[2], ph[3], py_ms))
            self.batches += 1
            self.busy_time += t_done - t_start
            for sc in scenes:
                sc.busy = False
                sc.last_used = t_done
                self.inflight_bytes -= sc.host.shape[0] * WORK_BYTES_PER_BOX
            self.done.extend(batch)
            self.free_slots.append(slot)
            self.lock.notify_all()

    # ---- dispatcher ----------------------------------------------------------
    def serve(self, n_expected: int, timeout: float = 600.0) -> None:
        """Dispatch until n_expected requests have completed (or were refused).

        While it runs, the interpreter switches threads every 0.2 ms (not the
        default 5 ms: a slot thread waiting for the GIL would add that to a
        request's latency) and the cyclic garbage collector is paused (the
        constructor collected once), so no collection pause lands in the
        middle of a batch; both are restored on return."""
        switch = sys.getswitchinterval()
        gc_on = gc.isenabled()
        gc.disable()
        sys.setswitchinterval(min(switch, 0.0002))
        try:
            self._serve(n_expected, timeout)
        finally:
            sys.setswitchinterval(switch)
            if gc_on:
                gc.enable()

    def _serve(self, n_expected: int, timeout: float) -> None:
        threads = []
        deadline = time.perf_counter() + timeout
        while True:
            with self.lock:
                while True:
                    if len(self.done) + self.refused >= n_expected:
                        for t in threads:
                            t.join()
                        return
                    if time.perf_counter() > deadline:
                        raise TimeoutError("serving loop timed out")
                    if self.free_slots and self.pending:
                        batch = self._take_batch()
                        if batch:
                            slot = self.free_slots.pop()
                            break
                    self.lock.wait(timeout=0.05)
            t = threading.Thread(target=self._run_batch, args=(slot, batch), daemon=True)
            t.start()
            threads = [x for x in threads if x.is_alive()] + [t]

    def close(self):
        for e in self.engines:
            e.close()


def move_indices(n: int, frac: float, seed: int) -> np.ndarray:
    """round(frac * n) (at least 1) distinct box indices, seeded, sorted."""
    k = min(n, max(1, int(round(frac * n))))
    return gen.pick(n, k, seed)


def pinned_boxes(n: int) -> np.ndarray:
    """A page-locked [n,7] uint32 host array (fast host<->device copies)."""
    import torch
    return torch.empty((n, 7), dtype=torch.int32).pin_memory().numpy().view(np.uint32)


def make_requests(duration: float, rate: float = 2000.0, seed: int = 0, lo: int = 1024, hi: int = 1 << 20,
                  update_frac: float = 0.3, move_frac: float = 0.01, pinned: bool = True) -> list[Request]:
    """Seeded request stream: Poisson arrivals, `update_frac` of them updates
    of an earlier scene (uniform over the scenes queried before), the rest
    queries of new scenes with log-uniform sizes in [lo, hi] (the batched
    scenes' generator). An update carries the indices and new rows of the
    moved boxes, as a client that owns its scene would send them: the
    clients' copies of the scenes are moved here, in arrival order."""
    reqs, t, i, scene_ids = [], 0.0, 0, []
    client: dict[int, np.ndarray] = {}  # scene -> the client's current boxes
    first_req: dict[int, int] = {}      # scene -> its query request
    while True:
        u = gen.uniform(seed, 20, i)
        t += -np.log(1.0 - u) / rate
        if t >= duration:
            break
        if scene_ids and gen.uniform(seed, 21, i) < update_frac:
            sid = scene_ids[int(gen.uniform(seed, 22, i) * len(scene_ids))]
            r = Request(i, t, sid, "update", move_frac=move_frac, move_seed=seed * 1000003 + i)
            if sid not in client:
                client[sid] = reqs[first_req[sid]].boxes.copy()
            cur = client[sid]
            r.idx = move_indices(cur.shape[0], r.move_frac, r.move_seed)
            gen.move3d(cur, r.idx, r.move_seed, r.move_sigma)
            r.rows = cur[r.idx]
            reqs.append(r)
        else:
            n = int(gen.scene_sizes(1, seed * 7919 + i, lo, hi)[0])
            sid = len(scene_ids)
            scene_ids.append(sid)
            first_req[sid] = len(reqs)
            out = pinned_boxes(n) if pinned else None
            reqs.append(Request(i, t, sid, "query", boxes=gen.scene3d(n, seed=seed * 1000003 + i, out=out)))
        i += 1
    return reqs


def feed(server: Server, reqs: list[Request]) -> threading.Thread:
    """Submit each request at its arrival time (relative to server.t0)."""
    def run():
        for r in reqs:
            dt = r.arrival - server.now()
            if dt > 0:
                time.sleep(dt)
            server.submit(r)
    th = threading.Thread(target=run, daemon=True)
    th.start()
    return th


def latency_summary(reqs: list[Request]) -> dict:
    lat = np.array([r.done - r.arrival for r in reqs if r.done > 0])
    pairs = sum(r.npairs for r in reqs)
    boxes = sum(r.nboxes for r in reqs)
    span = max(r.done for r in reqs) - min(r.arrival for r in reqs)
    return {"requests": len(reqs), "p50_ms": float(np.percentile(lat, 50) * 1e3),
            "p99_ms": float(np.percentile(lat, 99) * 1e3), "mean_ms": float(lat.mean() * 1e3),
            "max_ms": float(lat.max() * 1e3), "pairs": pairs, "boxes": boxes, "span_s": span,
            "pairs_per_s": pairs / span, "boxes_per_s": boxes / span}
