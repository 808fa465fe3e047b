"""Index scheme of the FP32 own-cell pair pass (k_pair_own32 in
rbc3d_gb300/csrc/pair.cu), restated on the CPU: one CTA per (target tile T,
source tile S >= T) of a cell's points in tiles of 128, thread t taking
target T*128 + t and at step s the source pair 2*((t + s) mod 64); off the
diagonal each evaluation is added to both points.  Every ordered pair of a
cell's points must be taken exactly once, and at every step the 32 lanes of
a warp must touch distinct sources (their per-warp sums are written without
atomics)."""
import numpy as np
import pytest

TILE = 128


def tile_pair(r, ntile):
    t = 0
    while r >= ntile - t:
        r -= ntile - t
        t += 1
    return t, t + r


@pytest.mark.parametrize("nv", [1, 8, 127, 128, 129, 300, 1250])
def test_every_ordered_pair_once(nv):
    ntile = (nv + TILE - 1) // TILE
    seen = np.zeros((nv, nv), dtype=np.int64)
    blocks = set()
    for r in range(ntile * (ntile + 1) // 2):
        T, S = tile_pair(r, ntile)
        assert 0 <= T <= S < ntile
        blocks.add((T, S))
        tid = np.arange(TILE)
        k = T * TILE + tid
        for step in range(TILE // 2):
            j = 2 * ((tid + step) & (TILE // 2 - 1))
            # lanes of one warp touch distinct sources
            for w in range(TILE // 32):
                lanes = j[32 * w:32 * (w + 1)]
                assert len(set(lanes.tolist())) == 32
            for off in (0, 1):
                js = S * TILE + j + off
                ok = (k < nv) & (js < nv)
                np.add.at(seen, (k[ok], js[ok]), 1)
                if S != T:
                    np.add.at(seen, (js[ok], k[ok]), 1)
    assert len(blocks) == ntile * (ntile + 1) // 2
    assert (seen == 1).all()


def test_mask_rows_staged_cover_the_tile():
    """The target tile's latitude rings (ring-major order, nlon points a
    ring) fit in the staged rows: at most (TILE - 1) // nlon + 2 of them."""
    for nlat, nlon in [(25, 50), (12, 24), (64, 128), (6, 8), (3, 200)]:
        nv = nlat * nlon
        cap = min(nlat, (TILE - 1) // nlon + 2)
        for T in range((nv + TILE - 1) // TILE):
            lat0 = T * TILE // nlon
            last = min(nlat - 1, (T * TILE + TILE - 1) // nlon)
            nrow = last - lat0 + 1
            assert 1 <= nrow <= cap
            k = np.arange(T * TILE, min(nv, T * TILE + TILE))
            assert ((k // nlon - lat0 >= 0) & (k // nlon - lat0 < nrow)).all()
