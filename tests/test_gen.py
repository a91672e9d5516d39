"""Seeded workload generators: determinism (committed digests, identical on
x86-64 and aarch64) and the shapes the workloads are specified with."""
import json
import math
import os

import numpy as np

from pbig_gb300 import gen

HERE = os.path.dirname(os.path.abspath(__file__))


def test_digests_match_committed():
    with open(os.path.join(HERE, "golden", "digests.json")) as f:
        want = json.load(f)
    got = {
        "cfg1_full": gen.digest(gen.uniform2d(65536)),
        "cfg2_first_262144": gen.digest(gen.clustered3d(262144)),
        "cfg3_blue_first_65536": gen.digest(gen.mixed3d(65536, seed=1)),
        "scene_100000_seed5": gen.digest(gen.scene3d(100000, seed=5)),
        "cfg1_plain2d_8192": gen.digest(gen.uniform2d(65536)[:8192].copy()),
        "cfg2_clustered3d_16384": gen.digest(gen.clustered3d(16384)),
    }
    for k, v in got.items():
        assert want[k] == v, k


def test_own_math_accuracy():
    L = gen._lib()
    for x in [1e-300, 1e-10, 0.1, 0.5, 0.75, 0.999999, 1.0]:
        assert abs(L.pbig_gen_log(x) - math.log(x)) <= 1e-15 * max(1.0, abs(math.log(x)))
    for x in np.linspace(-30, 5, 301):
        assert abs(L.pbig_gen_exp(x) - math.exp(x)) <= 1e-14 * math.exp(x)
    for u in np.linspace(0, 1, 1001, endpoint=False):
        assert abs(L.pbig_gen_cos2pi(u) - math.cos(2 * math.pi * u)) <= 1e-14
        assert abs(L.pbig_gen_cos2pi_nodiv(u) - math.cos(2 * math.pi * u)) <= 1e-14
    for x in [1e-300, 1e-10, 0.1, 0.5, 0.75, 0.999999, 1.0]:
        assert abs(L.pbig_gen_log_nodiv(x) - math.log(x)) <= 1e-15 * max(1.0, abs(math.log(x)))


def test_update_moves():
    from pbig_gb300 import serve
    idx = serve.move_indices(150000, 0.01, 3)
    assert len(idx) == 1500 and len(np.unique(idx)) == 1500 and np.all(np.diff(idx.astype(np.int64)) > 0)
    assert idx.max() < 150000
    assert len(serve.move_indices(7, 1.0, 1)) == 7 and len(serve.move_indices(256, 0.01, 1)) == 3
    b0 = gen.scene3d(150000, 3)
    b = b0.copy()
    gen.move3d(b, idx, 5)
    untouched = np.setdiff1d(np.arange(150000), idx)
    assert np.array_equal(b[untouched], b0[untouched]) and np.array_equal(b[:, 6], b0[:, 6])
    d = (b[idx, 0].astype(np.int64) - b0[idx, 0]) / gen.RANGE
    assert abs(np.median(np.abs(d)) / 0.6745 - 0.001) < 1e-4  # N(0, 0.001) displacement


def test_workload_shapes():
    b = gen.uniform2d(65536)
    ext = (b[:, 1] - b[:, 0]) / gen.RANGE
    assert b.shape == (65536, 5) and (b[:, 4] == np.arange(65536)).all()
    inner = (b[:, 1] < gen.RANGE - 1) & (b[:, 3] < gen.RANGE - 1)  # boxes not clipped at 1.0
    assert 0.0009 < ext[inner].min() and ext.max() < 0.00501
    c = gen.clustered3d(200000)
    e = (c[:, 1:6:2].astype(np.int64) - c[:, 0:6:2]) / gen.RANGE
    assert abs(np.median(e) - 0.002) < 0.0002
    assert (c[:, 0:6:2] <= c[:, 1:6:2]).all() and (c[:, :6] < gen.RANGE).all()
    m = gen.mixed3d(200000)
    me = (m[:, 1] - m[:, 0]) / gen.RANGE
    large = (me > 0.015).mean()
    assert 0.007 < large < 0.013
    sizes = gen.scene_sizes(4096, 0, 256, 262144)
    assert sizes.min() >= 256 and sizes.max() <= 262144
    assert 30000 < sizes.mean() < 46000
