"""The cell-size autotuner (host code, no GPU needed): its choices on the
benchmark workloads, and the grids it must never pick -- a single cell for a
scene of many small boxes, a grid on which a sampled box covers 2^26 cells or
more (the count kernel would skip it), or a grid far larger than the scene."""
import numpy as np
import pytest

from pbig_gb300 import gen
from pbig_gb300.engine import tune_shift


def cells_per_axis(rng, s):
    return (rng + (1 << s) - 1) >> s


def grid_cells(rng, s, dims):
    return cells_per_axis(rng, s) ** dims


def box_cells(boxes, s):
    dims = (boxes.shape[1] - 1) // 2
    lo = boxes[:, 0:2 * dims:2].astype(np.int64) >> s
    hi = boxes[:, 1:2 * dims:2].astype(np.int64) >> s
    return (hi - lo + 1).prod(axis=1)


def small_boxes(n, dims, rng, side, seed):
    rs = np.random.default_rng(seed)
    lo = rs.integers(0, rng - side, size=(n, dims), dtype=np.int64)
    hi = lo + rs.integers(0, side, size=(n, dims))
    b = np.empty((n, 2 * dims + 1), dtype=np.uint32)
    for d in range(dims):
        b[:, 2 * d], b[:, 2 * d + 1] = lo[:, d], hi[:, d]
    b[:, -1] = np.arange(n)
    return b


def test_benchmark_workload_choices():
    """The cell sizes the benchmark lines report (clustered 4M: 2^16; plain
    2-D and the red/blue union: 2^18)."""
    assert tune_shift(gen.clustered3d(4194304, seed=0), gen.RANGE) == 16
    assert tune_shift(gen.uniform2d(65536, seed=0), gen.RANGE) == 18
    red, blue = gen.mixed3d(2097152, seed=0), gen.mixed3d(2097152, seed=1)
    union = np.concatenate([red, blue])
    union[len(red):, -1] += len(red)
    assert tune_shift(union, gen.RANGE) == 18


@pytest.mark.parametrize("dims", [2, 3])
@pytest.mark.parametrize("where", [0, 12345])
def test_one_box_spanning_the_range(dims, where):
    """20 000 boxes of side < 64 and one spanning the whole 2^24 range (in the
    tuner's sample at index 0, outside it at 12345): a grid on which the big
    box fits, not a single cell, not far larger than the scene."""
    rng, n = 1 << 24, 20000
    b = small_boxes(n, dims, rng, 64, seed=77)
    b[where, 0:2 * dims:2], b[where, 1:2 * dims:2] = 0, rng - 1
    s = tune_shift(b, rng)
    assert 0 <= s <= 31
    assert box_cells(b, s).max() < 1 << 26
    assert 1 < grid_cells(rng, s, dims) <= max(4096, 64 * n)


def test_two_boxes_at_the_largest_coordinate():
    """Two boxes in a 2^24 range: a grid of a few cells, not 2^30."""
    rng = 1 << 24
    b = np.array([[rng - 1] * 6 + [0], [rng - 2, rng - 1] * 3 + [1]], dtype=np.uint32)
    assert grid_cells(rng, tune_shift(b, rng), 3) <= 4096


@pytest.mark.parametrize("seed", range(40))
def test_sampled_boxes_always_fit(seed):
    """Scenes of at most 4096 boxes are sampled whole: at the chosen cell size
    no box covers 2^26 cells or more, and the grid holds fewer than 2^32 cells."""
    rs = np.random.default_rng(4000 + seed)
    dims = int(rs.choice([2, 3]))
    rng = int(min(2 ** int(rs.integers(6, 33)), (1 << 32) - 1))
    n = int(rs.integers(1, 4096))
    side = max(1, rng >> int(rs.integers(1, 20)))
    b = small_boxes(n, dims, rng, min(side, rng - 1) or 1, seed=seed)
    k = int(rs.integers(0, 4))  # a few boxes spanning most of the range
    for i in rs.integers(0, n, size=k):
        b[i, 0:2 * dims:2], b[i, 1:2 * dims:2] = 0, rng - 1
    s = tune_shift(b, rng)
    assert 0 <= s <= 31
    assert box_cells(b, s).max() < 1 << 26
    assert grid_cells(rng, s, dims) < 1 << 32


def analytic_shift(b, rng):
    """Restatement of the per-scene tuner of batched queries (the engine's
    cost model with T = E^2 / 2C on the rows floor(k * n / m), k < m =
    min(n, 64)), in the same double arithmetic."""
    n = b.shape[0]
    dims = (b.shape[1] - 1) // 2

    def nrc(s):
        return (rng + (1 << s) - 1) >> s

    def coarsest():
        s = 31
        while s > 0 and nrc(s - 1) <= 1:
            s -= 1
        return s

    if n == 0:
        return coarsest()
    m = min(n, 64)
    smp = b[[k * n // m for k in range(m)]].astype(np.int64)
    lo, hi = smp[:, 0:2 * dims:2], smp[:, 1:2 * dims:2]
    ok = ((lo <= hi) & (hi < rng)).all(axis=1)
    ext, good = int((hi - lo + 1)[ok].sum()), int(ok.sum())
    mean = ext / ((good if good else 1) * dims)
    s0 = int(mean).bit_length() - 1 if mean >= 2.0 else 0
    scale = n / m
    s_win = min(31, s0 + 3)
    best, best_s = 1e300, None
    for s in range(max(0, s0 - 2), 32):
        if s == s_win + 1 and best < 1e300:
            break
        C = float(nrc(s))
        for _ in range(1, dims):
            C = C * float(nrc(s))
        if C > 4.0e9:
            continue
        if s > s_win and C > max(4096.0, 64.0 * n):
            continue
        E, cmax = 0.0, 0.0
        for i in np.nonzero(ok)[0]:
            c = 1.0
            for d in range(dims):
                c = c * float((int(hi[i, d]) >> s) - (int(lo[i, d]) >> s) + 1)
            E += c
            cmax = max(cmax, c)
        if E / m > 64.0 or cmax >= float(1 << 26):
            continue
        E = E * scale
        T = E * E / (2.0 * C)
        occ = 2.0 * T / max(E, 1.0) + 1.0
        f = occ / 96.0 if occ / 96.0 > 1.0 else 1.0
        cost = (2.4e-12 * C + 80.0e-12 * E) + (0.9e-12 * f) * T
        if cost < best:
            best, best_s = cost, s
    return coarsest() if best_s is None else best_s
