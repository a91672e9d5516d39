"""The batched workload at full size: 4,096 independent 3-D scenes of
log-uniform sizes in [256, 262,144] boxes (1.54e8 boxes in all), every
scene's cell size chosen inside the call by the device tuner (its choices
must equal a restatement of the cost model). Each scene's pair list must equal
the plain single-scene path's list (all 4,096 scenes, compared on the device
after sorting) and the oracle's (a stratified sample: the 20 largest scenes
and every 128th scene in size order).

The reference has no batched mode; it runs one pbig_check per scene
(src/pbig/pbig.cu:1962-1981), which is what the plain path and the oracle
stand for here.
"""
import numpy as np
import pytest

from oracle import oracle as O
from pbig_gb300 import Engine, gen
from test_tuner import analytic_shift

pytestmark = pytest.mark.gpu


def _keys(t):
    import torch
    k = (t[:, 0].to(torch.int64) << 32) | t[:, 1].to(torch.int64)
    return torch.sort(k).values


def test_full_batched_workload_scene_by_scene():
    import torch
    boxes, offs = gen.scene_batch(4096, seed=0)
    sizes = np.diff(offs).astype(np.int64)
    dev = torch.from_numpy(boxes.view(np.int32)).cuda()
    with Engine(0) as e:
        total = e.batch_intersect(dev, offs, gen.RANGE)  # cell sizes tuned in the call
        so = e.scene_offsets()
        assert int(so[-1]) == total
        res = torch.empty((total, 2), dtype=torch.int32, device="cuda")
        e.pairs_into(res)
        e.sync()
        assert e.stats()["bad_boxes"] == 0
        # the device tuner's choice for every scene equals the cost model's
        shifts = e.scene_shifts()
        want_shifts = [analytic_shift(boxes[int(offs[i]):int(offs[i + 1])], gen.RANGE) for i in range(4096)]
        assert np.array_equal(shifts, np.array(want_shifts, dtype=np.uint32))
        # every scene against the plain path
        bad = []
        for i in range(4096):
            a, b = int(offs[i]), int(offs[i + 1])
            k = e.self_intersect(dev[a:b], gen.RANGE)
            mine = res[int(so[i]):int(so[i + 1])]
            if k != mine.shape[0]:
                bad.append(i)
                continue
            if k:
                plain = torch.empty((k, 2), dtype=torch.int32, device="cuda")
                e.pairs_into(plain)
                e.sync()
                if not torch.equal(_keys(mine), _keys(plain)):
                    bad.append(i)
        assert not bad, bad[:20]
        host = res.cpu().numpy().view(np.uint32)
    # a stratified sample against the oracle, the largest scenes included
    order = np.argsort(sizes)
    sample = sorted(set(order[-20:].tolist()) | set(order[::128].tolist()))
    assert sizes[order[-1]] > 250000
    for i in sample:
        want, _ = O.grid_pairs(boxes[int(offs[i]):int(offs[i + 1])], gen.RANGE)
        got = O.sort_pairs(host[int(so[i]):int(so[i + 1])])
        assert np.array_equal(got, want), (i, int(sizes[i]))
