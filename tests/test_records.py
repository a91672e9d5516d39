"""The Rice record stream (src/pbig/pbig.cu:788-920, decode.cc:38-131):
hand-made streams decoded by the oracle's restatement of the reference's
decode (column offset fixed) and by pbig2_decode_records (host code, no GPU
needed); and, on the GPU, the engine's record mode against its flat pairs."""
import numpy as np
import pytest

from oracle import oracle as O

UNUSED = 0x0FFFFF11


def record(row_tile, col_tile, row, cols):
    b = bytes([row_tile, col_tile]) + int(row).to_bytes(2, "little") + len(cols).to_bytes(2, "little") + bytes(cols)
    b += b"\0" * (-len(b) % 8)
    return list(np.frombuffer(b, dtype=np.uint64))


def stream(blocks):
    w = []
    for gid, recs in blocks:
        w += [UNUSED, gid]
        for r in recs:
            w += record(*r)
    return np.array(w, dtype=np.uint64)


def test_handmade_stream_decodes_with_the_fixed_offset():
    # two cells: cell 3 holds entries 10..14 (boxes 100..104), cell 7 entries
    # 20..(20+300) (boxes 500+k); records in both tiles of cell 7
    start_i = np.zeros(8, dtype=np.uint32)
    start_i[3], start_i[7] = 10, 20
    recs = np.zeros(400, dtype=np.uint32)
    recs[10:15] = np.arange(100, 105)
    recs[20:320] = 500 + np.arange(300)
    w = stream([(3, [(0, 0, 0, [1, 2]), (0, 0, 3, [4])]),
                (7, [(0, 1, 5, [0, 43]), (1, 1, 2, list(range(9)))])])
    got = O.decode_rice(w, start_i, recs)
    want = [(100, 101), (100, 102), (103, 104),
            (505, 756), (505, 799)] + [(758, 756 + k) if 756 + k > 758 else (756 + k, 758) for k in range(9)]
    assert [tuple(p) for p in got] == [tuple(p) for p in want]
    from pbig_gb300.engine import decode_records
    assert np.array_equal(decode_records(w, start_i, recs), got)


def test_malformed_streams_are_refused():
    from pbig_gb300 import PbigError
    from pbig_gb300.engine import decode_records
    start_i = np.zeros(4, dtype=np.uint32)
    recs = np.arange(8, dtype=np.uint32)
    bad = [stream([(9, [(0, 0, 0, [1])])]),             # cell out of range
           stream([(1, [(0, 0, 0, [200])])]),           # column past the entries
           np.array([5, 1], dtype=np.uint64)]           # no block header
    for w in bad:
        with pytest.raises((ValueError, PbigError)):
            O.decode_rice(w, start_i, recs)
            decode_records(w, start_i, recs)
        with pytest.raises(PbigError):
            decode_records(w, start_i, recs)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["clustered", "big_cells", "huge_cell", "plain2d", "merged"])
def test_record_mode_against_flat_pairs(engine, case):
    from pbig_gb300 import PbigError, gen
    from pbig_gb300.engine import decode_records
    if case == "clustered":
        boxes, rng, shift = gen.clustered3d(300000, seed=8), gen.RANGE, None
    elif case == "big_cells":  # cells of 129..512 boxes: row and column tiles past the first
        boxes, rng, shift = gen.clustered3d(300000, seed=8), gen.RANGE, 18
    elif case == "huge_cell":  # one cell of 3000 identical boxes (tile tasks)
        z = np.load(__file__.replace("test_records.py", "golden/identical700.npz"))
        boxes = np.repeat(z["boxes"][:1], 3000, axis=0)
        boxes[:, 6] = np.arange(3000)
        rng, shift = 1000, None
    elif case == "plain2d":
        boxes, rng, shift = gen.uniform2d(65536, seed=0), gen.RANGE, None
    else:
        boxes, rng, shift = gen.clustered3d(200000, seed=3), gen.RANGE, 17
    n_flat = engine.self_intersect(boxes, rng, cell_shift=shift)
    flat = O.sort_pairs(engine.pairs())
    engine.set_records(True)
    engine.set_merged(case == "merged")
    try:
        n_rec = engine.self_intersect(boxes, rng, cell_shift=shift)
        words, start_i, recs = engine.records()
        with pytest.raises(PbigError):
            engine.pairs()  # the result is a stream, not pairs
        red = gen.mixed3d(1000, seed=0)
        with pytest.raises(PbigError):
            engine.bipartite_intersect(red, red, gen.RANGE)
    finally:
        engine.set_records(False)
        engine.set_merged(False)
    assert n_rec == n_flat
    assert words.shape[0] > 0 and words[0] == UNUSED
    ref = O.decode_rice(words, start_i, recs)
    assert np.array_equal(O.sort_pairs(ref), flat)
    assert np.array_equal(decode_records(words, start_i, recs), ref)
