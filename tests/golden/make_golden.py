"""Regenerates tests/golden/*.npz from the oracle.

Every fixture holds the boxes of a case, its range and the sorted canonical
pair list (a < b). The pair lists come from the oracle's restatement of the
reference pipeline (auto cell size, reference heuristic) and are checked
against the all-pairs brute force before they are written; the workload
fixtures also record the SHA-256 of the generated boxes so the generator's
cross-machine determinism is tested too.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

from cases import cases  # noqa: E402

from oracle import oracle as O  # noqa: E402
from pbig_gb300 import gen  # noqa: E402


def workload_cases():
    return [
        ("cfg1_plain2d_8192", gen.uniform2d(65536)[:8192].copy(), gen.RANGE),
        ("cfg2_clustered3d_16384", gen.clustered3d(16384), gen.RANGE),
        ("cfg3_red_4096", gen.mixed3d(4096, seed=0), gen.RANGE),
        ("scene_3000", gen.scene3d(3000, seed=11), gen.RANGE),
    ]


def main():
    digests = {}
    for name, boxes, rng in cases() + workload_cases():
        p, st = O.grid_pairs(boxes, rng) if len(boxes) else (np.zeros((0, 2), np.uint32), {})
        b = O.brute_pairs(boxes) if len(boxes) else np.zeros((0, 2), np.uint32)
        assert p.shape == b.shape and (p == b).all(), name
        np.savez_compressed(os.path.join(HERE, name + ".npz"), boxes=boxes, range=np.uint64(rng), pairs=p)
        digests[name] = gen.digest(boxes)
        print(f"{name}: {len(boxes)} boxes, {len(p)} pairs")
    # digests of full-size generated workloads (first rows) for determinism checks
    full = {
        "cfg1_full": gen.digest(gen.uniform2d(65536)),
        "cfg2_first_262144": gen.digest(gen.clustered3d(262144)),
        "cfg3_blue_first_65536": gen.digest(gen.mixed3d(65536, seed=1)),
        "scene_100000_seed5": gen.digest(gen.scene3d(100000, seed=5)),
    }
    digests.update(full)
    with open(os.path.join(HERE, "digests.json"), "w") as f:
        json.dump(digests, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
