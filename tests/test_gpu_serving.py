"""The serving loop: continuous batching of scene queries and updates.

Each request's pair set, whatever batch it was mixed into, must equal the
oracle's pairs of the scene as it was when the request ran, and the pairs of
that scene queried alone on the engine.
"""
import numpy as np
import pytest

from oracle import oracle as O
from pbig_gb300 import gen, serve

pytestmark = pytest.mark.gpu


def _check_alone(engine, reqs):
    for r in reqs:
        assert r.done > 0, r.rid
        want, _ = O.grid_pairs(r.snapshot, gen.RANGE)
        got = O.sort_pairs(r.pairs)
        assert r.npairs == len(want), r.rid
        assert np.array_equal(got, want), r.rid
        n = engine.self_intersect(r.snapshot, gen.RANGE)
        assert n == r.npairs
        assert np.array_equal(O.sort_pairs(engine.pairs()), want), r.rid


def test_serving_results_equal_alone_and_in_the_mix(engine):
    reqs = serve.make_requests(0.08, rate=2000, seed=5, lo=256, hi=20000)
    srv = serve.Server(keep_snapshots=True)
    th = serve.feed(srv, reqs)
    srv.serve(len(reqs), timeout=120)
    th.join()
    srv.close()
    assert srv.refused == 0
    assert any(r.kind == "update" for r in reqs)
    sizes = np.bincount([r.batch for r in reqs])
    assert sizes.max() > 1, "no request was batched with another"
    _check_alone(engine, reqs)
    s = serve.latency_summary(reqs)
    assert s["p99_ms"] >= s["p50_ms"] > 0


def test_serving_under_a_small_memory_budget(engine):
    """A budget far below the scenes' total: device copies are dropped and
    re-uploaded, answers unchanged."""
    reqs = serve.make_requests(0.05, rate=2000, seed=6, lo=20000, hi=60000)
    total = sum(r.boxes.shape[0] for r in reqs if r.boxes is not None) * serve.BOX_BYTES
    srv = serve.Server(budget_bytes=max(total // 4, 40 << 20), keep_snapshots=True)
    th = serve.feed(srv, reqs)
    srv.serve(len(reqs), timeout=120)
    th.join()
    srv.close()
    assert srv.evictions > 0
    assert srv.refused == 0
    _check_alone(engine, reqs)
