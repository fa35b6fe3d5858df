"""The neighbour table of the uniform-tile skipping (host code, no GPU):
every tile the engine may skip must have its whole 3-cell halo ring inside
the interiors of the eight tiles it lists, each in the right direction, so
that eight uniform records with one value prove the halo box uniform.
Random patch sets of one level (patches aligned as the base level's are,
and arbitrary clustered boxes; touching, never overlapping), and the tiles
the rules should take."""
import ctypes as C

import numpy as np
import pytest

from enlightning_gb300 import _lib

DIRS = [(-1, -1), (0, -1), (1, -1), (-1, 0), (1, 0), (-1, 1), (0, 1), (1, 1)]  # (dx, dy) with dy < 0 above


def _table(boxes):
    b = np.ascontiguousarray(np.asarray(boxes, np.int32).reshape(-1, 4))
    cap = 64
    while True:
        tiles = np.zeros((cap, 4), np.int32)
        nbr = np.zeros((cap, 8), np.int32)
        n = C.c_int()
        st = _lib.lib().enl_tile_neighbours(b.ctypes.data_as(C.c_void_p) if len(b) else None, len(b),
                                            tiles.ctypes.data_as(C.c_void_p), nbr.ctypes.data_as(C.c_void_p),
                                            cap, C.byref(n))
        if st == 0:
            return tiles[: n.value], nbr[: n.value]
        assert n.value > cap
        _lib.lib().enl_get_last_error()  # the ENL_ERR_ARG of a short buffer, consumed
        cap = n.value


def _check(tiles, nbr):
    """Every listed neighbour set covers the halo ring, direction by direction."""
    skippable = 0
    for t, (i0, j0, w, h) in enumerate(tiles):
        if nbr[t, 0] < 0:
            continue
        skippable += 1
        assert w == 32 and h == 8, (t, w, h)
        cover = np.zeros((h + 6, w + 6), bool)
        for m, (dx, dy) in enumerate(DIRS):
            q = nbr[t, m]
            assert 0 <= q < len(tiles) and q != t
            qi, qj, qw, qh = tiles[q]
            # the neighbour lies in its direction
            assert (qi >= i0 + w) if dx > 0 else ((qi + qw <= i0) if dx < 0 else (qi == i0))
            assert (qj >= j0 + h) if dy > 0 else ((qj + qh <= j0) if dy < 0 else (qj == j0))
            # its interior, in the tile's box coordinates
            a0, a1 = max(qi - (i0 - 3), 0), min(qi + qw - (i0 - 3), w + 6)
            b0, b1 = max(qj - (j0 - 3), 0), min(qj + qh - (j0 - 3), h + 6)
            if a0 < a1 and b0 < b1:
                cover[b0:b1, a0:a1] = True
        cover[3:3 + h, 3:3 + w] = True  # the tile itself
        assert cover.all(), (t, i0, j0)
    return skippable


def _random_boxes(rng, aligned):
    boxes, occ = [], np.zeros((64, 64), bool)  # occupancy in units of 16 cells
    for _ in range(40):
        if aligned:
            gi, gj = int(rng.integers(0, 8)) * 8, int(rng.integers(0, 8)) * 8  # multiples of 128 cells
            wi, wj = 8, 8
        else:
            gi, gj = int(rng.integers(0, 60)), int(rng.integers(0, 60))
            wi, wj = int(rng.integers(1, 5)), int(rng.integers(1, 5))
        if gi + wi > 64 or gj + wj > 64 or occ[gj:gj + wj, gi:gi + wi].any():
            continue
        occ[gj:gj + wj, gi:gi + wi] = True
        ilo, jlo = 16 * gi + (0 if aligned else int(rng.integers(0, 3)) * 2), 16 * gj
        ihi, jhi = 16 * (gi + wi) - 1, 16 * (gj + wj) - 1
        boxes.append((ilo, ihi, jlo, jhi))
    return boxes


@pytest.mark.parametrize("seed", range(6))
def test_listed_neighbours_hold_the_halo_ring(seed):
    rng = np.random.default_rng(seed)
    for aligned in (True, False):
        boxes = _random_boxes(rng, aligned)
        tiles, nbr = _table(boxes)
        assert len(tiles) == sum(((b[1] - b[0] + 32) // 32) * ((b[3] - b[2] + 8) // 8) for b in boxes)
        _check(tiles, nbr)


def test_interior_and_cross_patch_tiles_are_taken():
    # one 256 x 256 patch: the 6 x 30 tiles off its border ring
    tiles, nbr = _table([(0, 255, 0, 255)])
    assert (nbr[:, 0] >= 0).sum() == 6 * 30 == _check(tiles, nbr)
    # four aligned 256 x 256 patches in a square: across the patches every
    # tile off the outer ring of the 512 x 512 square
    tiles, nbr = _table([(0, 255, 0, 255), (256, 511, 0, 255), (0, 255, 256, 511), (256, 511, 256, 511)])
    assert (nbr[:, 0] >= 0).sum() == 14 * 62 == _check(tiles, nbr)
    # a patch whose last column of tiles is 2 cells wide: the tiles beside it
    # cannot take their right halo from it
    tiles, nbr = _table([(0, 97, 0, 63)])
    for t, (i0, j0, w, h) in enumerate(tiles):
        if i0 == 64:
            assert nbr[t, 0] < 0
    _check(tiles, nbr)
