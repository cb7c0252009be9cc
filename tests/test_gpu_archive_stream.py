"""Arrays exchanged with TiledArray programs through the byte stream of
DistArray::serialize on one rank (tagpu_array_serialize /
tagpu_array_deserialize).  Streams built by hand from the field order
(tests/ta_stream.py) are read back tile for tile, and the engine writes the
same bytes for the same array."""
import os

import numpy as np
import pytest

import ta_stream
from helpers import gpu_operand

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ta():
    import tiledarray_gb300 as ta
    return ta


def _hand_built(sparse):
    rng = np.random.default_rng(4)
    hm = [[0, 2, 5, 10, 17], [3, 4, 9, 11, 20]]    # the second mode starts at 3
    nt = [len(h) - 1 for h in hm]
    tiles, norms = {}, np.zeros(nt, np.float32)
    for i in range(nt[0]):
        for j in range(nt[1]):
            if sparse and (i + j) % 3 == 1:
                continue
            shp = (hm[0][i + 1] - hm[0][i], hm[1][j + 1] - hm[1][j])
            t = rng.integers(-9, 10, shp).astype(np.float64)
            vol = max(t.size, 1)
            norms[i, j] = np.float32(np.linalg.norm(t)) / np.float32(vol)
            if sparse and norms[i, j] == 0:
                continue
            tiles[(i, j)] = t
    return hm, tiles, (norms if sparse else None)


@pytest.mark.parametrize("sparse", [True, False])
def test_hand_built_stream_round_trip(ta, world, tmp_path, sparse):
    hm, tiles, norms = _hand_built(sparse)
    raw = ta_stream.write(hm, tiles, norms, type_hash=0x1234abcd5678ef90, pmap_hash=77)
    p = tmp_path / "in.bin"
    p.write_bytes(raw)
    A, th, ph = ta.DistArray.deserialize(world, str(p), sparse=sparse)
    assert (th, ph) == (0x1234abcd5678ef90, 77)
    assert A.info().dense == (not sparse)
    off = A.tile_offsets()
    data = A.download()
    nt1 = len(hm[1]) - 1
    for (i, j), t in tiles.items():
        o = off[i * nt1 + j]
        assert o >= 0
        assert np.array_equal(data[o:o + t.size], t.ravel())
    if sparse:
        assert np.array_equal(A.norms(), norms.ravel())
        assert sum(1 for o in off if o >= 0) == len(tiles)
    # the engine writes the same bytes back
    q = tmp_path / "out.bin"
    A.serialize(str(q), 0x1234abcd5678ef90, 77)
    assert q.read_bytes() == raw


def test_generated_array_stream(ta, world, tmp_path):
    h = [0, 48, 130, 300, 301, 420]
    A, _ = gpu_operand(ta, world, [h, h, [0, 7, 16]], 9, 0, kind=0,
                       tile_scale=np.arange(5 * 5 * 2) % 4)
    p = tmp_path / "g.bin"
    A.serialize(str(p), 5, 6)
    B, th, ph = ta.DistArray.deserialize(world, str(p))
    assert (th, ph) == (5, 6)
    assert np.array_equal(A.norms(), B.norms())
    assert np.array_equal(A.tile_offsets(), B.tile_offsets())
    assert np.array_equal(A.download(), B.download())
    # the stream equals the hand-written restatement of the same array
    nt = [len(h) - 1, len(h) - 1, 2]
    off, data = A.tile_offsets(), A.download()
    hm = [h, h, [0, 7, 16]]
    tiles = {}
    for o in range(len(off)):
        if off[o] < 0:
            continue
        idx = np.unravel_index(o, nt)
        shp = tuple(hm[d][idx[d] + 1] - hm[d][idx[d]] for d in range(3))
        tiles[tuple(int(x) for x in idx)] = data[off[o]:off[o] + int(np.prod(shp))].reshape(shp)
    assert p.read_bytes() == ta_stream.write(hm, tiles, A.norms().reshape(nt), 5, 6)


def test_rejects_multi_rank_and_damaged_streams(ta, world, tmp_path):
    hm, tiles, norms = _hand_built(True)
    p = tmp_path / "w2.bin"
    p.write_bytes(ta_stream.write(hm, tiles, norms, world=(2, 0)))
    with pytest.raises(ta.TAGPUError, match="multi-rank"):
        ta.DistArray.deserialize(world, str(p))
    raw = ta_stream.write(hm, tiles, norms)
    p.write_bytes(raw[:len(raw) - 8])
    with pytest.raises(ta.TAGPUError, match="truncated"):
        ta.DistArray.deserialize(world, str(p))
