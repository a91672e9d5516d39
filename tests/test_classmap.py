"""The work-list class map (PBIG2_OPT_CLASS_MAP) and its automatic choice,
on the CPU through the C ABI: which list each cell-size bucket goes to, and
the maps the engine refuses."""
from pbig_gb300 import engine

DEFAULT = 0x6666665544321000
ONE_LAUNCH = 0x6666665544444000


def _nib(m, L):
    return (m >> (4 * L)) & 15


def test_automatic_maps():
    f = engine.lib().pbig2_class_map_auto
    assert f(0) == DEFAULT and f(1) == ONE_LAUNCH
    # default: each bucket to the smallest list that holds it
    assert [_nib(DEFAULT, L) for L in range(1, 16)] == [0, 0, 1, 2, 3, 4, 4, 5, 5, 6, 6, 6, 6, 6, 6]
    # one launch: cells of 5..32 boxes (buckets 3..5) to the one-warp-per-cell list
    assert [_nib(ONE_LAUNCH, L) for L in range(1, 16)] == [0, 0, 4, 4, 4, 4, 4, 5, 5, 6, 6, 6, 6, 6, 6]


def test_map_check():
    f = engine.lib().pbig2_class_map_check
    assert f(DEFAULT) == 0 and f(ONE_LAUNCH) == 0
    assert f(0x6666665554321000) == 0   # 65..128 to the block list
    assert f(0x6666666666666660) == 0   # everything as tile tasks
    assert f(0x6666665543321000) == 6   # 33..64 to lane groups of 32: too small
    assert f(0x6666666644321000) == 0
    assert f(0x6666655544321000) == 10  # 513..1024 to the block list: too small
    assert f(0x5666665544321000) == 15  # the last bucket must be tile tasks
    assert f(0x6666665544321700) == 2   # no list 7
    assert f(0x6666665544321100) == 0   # 3..4 boxes in lane groups of 8
