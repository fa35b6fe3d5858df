"""The coarse-fine halo the engine interpolates (host code, no GPU): the
band sweep of enl_halo_segments against a direct construction — cells
within 3 (Chebyshev) of the patch union, inside the level, in no patch —
on random patch sets, touching boxes and the level's edges included."""
import ctypes as C

import numpy as np
import pytest
from scipy.ndimage import binary_dilation

from enlightning_gb300 import _lib


def _segments(boxes, nx, ny):
    b = np.ascontiguousarray(np.asarray(boxes, np.int32).reshape(-1, 4))
    cap = 64
    while True:
        out = np.zeros((cap, 3), np.int32)
        n = C.c_int()
        st = _lib.lib().enl_halo_segments(b.ctypes.data_as(C.c_void_p) if len(b) else None, len(b), nx, ny,
                                          out.ctypes.data_as(C.c_void_p), cap, C.byref(n))
        if st == 0:
            return [tuple(int(v) for v in s) for s in out[: n.value]]
        assert n.value > cap
        _lib.lib().enl_get_last_error()  # the ENL_ERR_ARG of a short buffer, consumed
        cap = n.value


def _direct(boxes, nx, ny):
    cover = np.zeros((ny, nx), bool)
    for ilo, ihi, jlo, jhi in boxes:
        cover[jlo:jhi + 1, ilo:ihi + 1] = True
    halo = binary_dilation(cover, structure=np.ones((7, 7), bool)) & ~cover
    segs = []
    for j in range(ny):
        row = halo[j]
        i = 0
        while i < nx:
            if row[i]:
                k = i
                while k + 1 < nx and row[k + 1]:
                    k += 1
                segs.append((j, i, k))
                i = k + 1
            else:
                i += 1
    return segs


@pytest.mark.parametrize("seed", range(30))
def test_halo_segments_match_direct_construction(seed):
    rng = np.random.default_rng(seed)
    nx, ny = int(rng.integers(8, 150)), int(rng.integers(8, 150))
    boxes = []
    for _ in range(int(rng.integers(1, 14))):
        ilo, jlo = int(rng.integers(0, nx)), int(rng.integers(0, ny))
        boxes.append((ilo, min(nx - 1, ilo + int(rng.integers(0, 40))), jlo, min(ny - 1, jlo + int(rng.integers(0, 40)))))
    assert _segments(boxes, nx, ny) == _direct(boxes, nx, ny)


def test_halo_segments_edge_cases():
    assert _segments([], 10, 10) == []
    assert _segments([(0, 9, 0, 9)], 10, 10) == []  # the whole level: no halo
    one = _segments([(4, 4, 4, 4)], 9, 9)
    assert one == _direct([(4, 4, 4, 4)], 9, 9) and len(one) == 8  # 7 rows, the middle one split
    touching = [(0, 4, 0, 4), (5, 9, 0, 4)]  # neighbours: no halo between them
    assert _segments(touching, 20, 12) == _direct(touching, 20, 12)
