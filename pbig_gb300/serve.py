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

The engine calls release the GIL (ctypes), so the slot threads run
concurrently.
"""
from __future__ import annotations

import collections
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import gen
from .engine import Engine, tune_shift

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
    # filled by the server
    start: float = 0.0
    done: float = 0.0
    npairs: int = 0
    pairs: np.ndarray | None = None
    batch: int = -1
    snapshot: np.ndarray | None = None  # scene boxes as queried (kept when the server records them)
    nboxes: int = 0


@dataclass
class Scene:
    sid: int
    host: np.ndarray           # master copy (host)
    dev: object                # torch tensor [n,7] int32 on the device
    shift: int
    last_used: float = 0.0
    busy: bool = False

    @property
    def bytes(self) -> int:
        return self.host.shape[0] * BOX_BYTES


class Server:
    def __init__(self, device: int = 0, budget_bytes: int = 40 << 30, slots: int = 2,
                 max_batch_boxes: int = 64 << 20, keep_pairs: bool = True, keep_snapshots: bool = False,
                 copy_pairs: bool = True):
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
        self.pinned = [torch.empty((1 << 20, 2), dtype=torch.int32).pin_memory() for _ in range(slots)]
        self.staging = [torch.empty((1 << 16, 8), dtype=torch.int32).pin_memory() for _ in range(slots)]
        self.free_slots = list(range(slots))
        self.batches = 0
        self.t0 = time.perf_counter()
        self.busy_time = 0.0
        self.evictions = 0
        self.refused = 0
        self.phase_s = collections.defaultdict(float)  # host seconds per batch phase (summed)

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
            victim.dev = None
            self.resident_bytes -= victim.bytes
            self.evictions += 1
        return True

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
        torch = self.torch
        eng = self.engines[slot]
        t_start = self.now()
        for r in batch:
            r.start = t_start
        scenes = [self.scenes[r.scene] for r in batch]
        dev = f"cuda:{self.device}"
        stream = self.streams[slot]
        tp = [time.perf_counter()]
        with torch.cuda.stream(stream):
            self._prepare(batch, scenes, dev, slot)
            tp.append(time.perf_counter())
            offs = np.zeros(len(batch) + 1, dtype=np.uint64)
            for i, sc in enumerate(scenes):
                offs[i + 1] = offs[i] + sc.host.shape[0]
            cat = torch.cat([sc.dev for sc in scenes]) if len(scenes) > 1 else scenes[0].dev
            shifts = np.array([sc.shift for sc in scenes], dtype=np.uint32)
            tp.append(time.perf_counter())
            total = eng.batch_intersect(cat, offs, gen.RANGE, cell_shifts=shifts, stream=stream)
            so = eng.scene_offsets()
            tp.append(time.perf_counter())
            if self.keep_pairs:
                if self.pinned[slot].shape[0] < total:
                    self.pinned[slot] = torch.empty((int(total * 1.25) + 1024, 2), dtype=torch.int32).pin_memory()
                buf = self.pinned[slot][:total]
                eng.pairs_into(buf, stream=stream)
                eng.sync(stream)
                allp = buf.numpy().view(np.uint32)
                if self.copy_pairs:  # the pinned buffer is reused by the slot's next batch
                    allp = allp.copy()
        tp.append(time.perf_counter())
        t_done = self.now()
        for i, r in enumerate(batch):
            r.npairs = int(so[i + 1] - so[i])
            if self.keep_pairs:
                r.pairs = allp[int(so[i]):int(so[i + 1])]
            r.done = t_done
            r.batch = self.batches
        with self.lock:
            for k, name in enumerate(("prepare", "concat", "query", "download")):
                if k + 1 < len(tp):
                    self.phase_s[name] += tp[k + 1] - tp[k]
            self.batches += 1
            self.busy_time += t_done - t_start
            for sc in scenes:
                sc.busy = False
                sc.last_used = t_done
                self.inflight_bytes -= sc.host.shape[0] * WORK_BYTES_PER_BOX
            self.done.extend(batch)
            self.free_slots.append(slot)
            self.lock.notify_all()

    def _prepare(self, batch, scenes, dev, slot) -> None:
        """Apply updates and make the batch's scenes device-resident (on the
        current stream). The moved rows of every update in the batch go up
        in one copy through the slot's page-locked staging buffer (free
        again: the slot's previous batch ended with a stream synchronize)."""
        torch = self.torch
        moved = []  # (scene, indices) of updates whose scene stays resident
        for r, sc in zip(batch, scenes):
            r.nboxes = sc.host.shape[0]
            if sc.shift < 0:  # first query of the scene: tune its cell size once
                sc.shift = tune_shift(sc.host, gen.RANGE, 256)
            if r.kind == "update":  # move a fraction of the boxes (host master copy)
                idx = move_indices(sc.host.shape[0], r.move_frac, r.move_seed)
                gen.move3d(sc.host, idx, r.move_seed, r.move_sigma)
                if sc.dev is not None:
                    moved.append((sc, idx))
            if sc.dev is None:  # not on the device (new or dropped): upload it whole
                sc.dev = torch.from_numpy(sc.host.view(np.int32)).to(dev, non_blocking=True)
            if self.keep_snapshots:
                r.snapshot = sc.host.copy()
        if moved:
            k = sum(idx.shape[0] for _, idx in moved)
            if self.staging[slot].shape[0] < k:
                self.staging[slot] = torch.empty((int(k * 1.25) + 1024, 8), dtype=torch.int32).pin_memory()
            st = self.staging[slot][:k].numpy()
            a = 0
            for sc, idx in moved:  # row = [7 coordinate/rid words, box index]
                b = a + idx.shape[0]
                np.take(sc.host.view(np.int32), idx, axis=0, out=st[a:b, :7])
                st[a:b, 7] = idx.view(np.int32)
                a = b
            up = self.staging[slot][:k].to(dev, non_blocking=True)
            a = 0
            for sc, idx in moved:
                b = a + idx.shape[0]
                sc.dev.index_copy_(0, up[a:b, 7].long(), up[a:b, :7])
                a = b

    # ---- dispatcher ----------------------------------------------------------
    def serve(self, n_expected: int, timeout: float = 600.0) -> None:
        """Dispatch until n_expected requests have completed (or were refused)."""
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
    scenes' generator)."""
    reqs, t, i, scene_ids = [], 0.0, 0, []
    while True:
        u = gen.uniform(seed, 20, i)
        t += -np.log(1.0 - u) / rate
        if t >= duration:
            break
        if scene_ids and gen.uniform(seed, 21, i) < update_frac:
            sid = scene_ids[int(gen.uniform(seed, 22, i) * len(scene_ids))]
            reqs.append(Request(i, t, sid, "update", move_frac=move_frac, move_seed=seed * 1000003 + i))
        else:
            n = int(gen.scene_sizes(1, seed * 7919 + i, lo, hi)[0])
            sid = len(scene_ids)
            scene_ids.append(sid)
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
