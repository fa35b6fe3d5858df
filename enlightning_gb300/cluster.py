"""Clustering of tagged cells into patch boxes (host side of regridding).

The reference delegates this to SAMRAI's BergerRigoutsos box generator
(main.C:261-265, input.txt:123-127: efficiency_tolerance 0.70,
combine_efficiency 0.80).  This is a from-scratch implementation of the
published Berger-Rigoutsos signature algorithm (Berger & Rigoutsos, IEEE
Trans. SMC 21(5), 1991): shrink a box to the bounding box of its tags; accept
it when the fraction of tagged cells reaches the efficiency; otherwise cut it
at a zero of the tag signature (a hole), else at the strongest inflection of
the signature (largest jump of its second difference), else in the middle of
its longest side.  Boxes are finally chopped so that no side exceeds
max_size.  Boxes are (ilo, ihi, jlo, jhi), inclusive.
"""
from __future__ import annotations

import numpy as np


def _bbox(t):
    rows = np.flatnonzero(t.any(axis=1))
    cols = np.flatnonzero(t.any(axis=0))
    if rows.size == 0:
        return None
    return cols[0], cols[-1], rows[0], rows[-1]


def _cut(sig, min_size):
    """Cut position c (box splits into [0, c) and [c, n)) or None."""
    n = sig.size
    lo, hi = min_size, n - min_size
    if hi < lo:
        return None
    zeros = np.flatnonzero(sig[lo:hi + 1] == 0) + lo
    if zeros.size:
        mid = (n - 1) / 2.0
        z = zeros[np.argmin(np.abs(zeros - mid))]
        return int(max(lo, min(hi, z if z >= lo else lo)))
    if n >= 4:
        lap = sig[:-2] - 2 * sig[1:-1] + sig[2:]
        jump = np.abs(np.diff(lap))
        # candidate cut between i+1 and i+2 for jump index i
        cand = np.arange(jump.size) + 2
        ok = (cand >= lo) & (cand <= hi) & (np.sign(lap[:-1]) != np.sign(lap[1:]))
        if ok.any():
            jj = np.where(ok, jump, -1)
            if jj.max() > 0:
                return int(cand[np.argmax(jj)])
    return int(n // 2) if n // 2 >= lo and n // 2 <= hi else None


def cluster_tags(tags: np.ndarray, efficiency=0.7, min_size=8, max_size=128, allowed=None):
    """Boxes covering every tag.  With ``allowed`` (same shape, bool) every
    box is also kept inside the allowed cells (proper nesting): a box that
    reaches outside is cut where its columns or rows start or stop leaving
    the allowed region, down to single cells if need be."""
    tags = np.asarray(tags, dtype=bool)
    if allowed is not None:
        allowed = np.asarray(allowed, dtype=bool)
        tags = tags & allowed
    out = []
    bb = _bbox(tags)
    if bb is None:
        return out
    stack = [bb]
    while stack:
        ilo, ihi, jlo, jhi = stack.pop()
        sub = tags[jlo:jhi + 1, ilo:ihi + 1]
        b = _bbox(sub)
        if b is None:
            continue
        ilo, ihi, jlo, jhi = ilo + b[0], ilo + b[1], jlo + b[2], jlo + b[3]
        sub = tags[jlo:jhi + 1, ilo:ihi + 1]
        nxb, nyb = ihi - ilo + 1, jhi - jlo + 1
        if allowed is not None:
            bad = ~allowed[jlo:jhi + 1, ilo:ihi + 1]
            if bad.any():
                cut = _nesting_cut(bad)
                if cut is None:
                    continue
                ax, c = cut
                if ax == "x":
                    stack.append((ilo, ilo + c - 1, jlo, jhi))
                    stack.append((ilo + c, ihi, jlo, jhi))
                else:
                    stack.append((ilo, ihi, jlo, jlo + c - 1))
                    stack.append((ilo, ihi, jlo + c, jhi))
                continue
        eff = sub.sum() / float(nxb * nyb)
        if eff >= efficiency:
            out.append((ilo, ihi, jlo, jhi))
            continue
        sx = sub.sum(axis=0)  # signature along x
        sy = sub.sum(axis=1)
        order = [(nxb, "x"), (nyb, "y")]
        order.sort(reverse=True)
        done = False
        for _, ax in order:
            sig = sx if ax == "x" else sy
            c = _cut(sig, min_size)
            if c is None or c <= 0 or c >= sig.size:
                continue
            if ax == "x":
                stack.append((ilo, ilo + c - 1, jlo, jhi))
                stack.append((ilo + c, ihi, jlo, jhi))
            else:
                stack.append((ilo, ihi, jlo, jlo + c - 1))
                stack.append((ilo, ihi, jlo + c, jhi))
            done = True
            break
        if not done:
            out.append((ilo, ihi, jlo, jhi))
    return chop(out, max_size)


def _nesting_cut(bad):
    """Cut separating columns (rows) that contain disallowed cells from those
    that do not, on the longer side first; None for a 1x1 box."""
    ny, nx = bad.shape
    colbad = bad.any(axis=0)
    rowbad = bad.any(axis=1)
    for ax, sig, n in sorted((("x", colbad, nx), ("y", rowbad, ny)), key=lambda t: -t[2]):
        if n < 2:
            continue
        ch = np.flatnonzero(sig[1:] != sig[:-1]) + 1
        if ch.size:
            return ax, int(ch[np.argmin(np.abs(ch - n / 2.0))])
    if nx >= ny and nx >= 2:
        return "x", nx // 2
    if ny >= 2:
        return "y", ny // 2
    return None


def erode_allowed(allowed, passes):
    """Proper-nesting mask: `passes` erosions by the 3x3 square, the outside
    of the map counting as allowed."""
    if passes <= 0:
        return np.asarray(allowed, bool)
    from scipy.ndimage import binary_erosion
    return binary_erosion(allowed, structure=np.ones((3, 3), bool), iterations=passes, border_value=1)


def cluster_tags_native(tags, efficiency=0.7, min_size=8, max_size=128, allowed=None, nest_erode=0):
    """cluster_tags(tags, ..., allowed=erode_allowed(allowed, nest_erode)) in
    the library's C++ (enl_cluster_tags): the same boxes in the same order,
    with summed-area tables instead of array scans."""
    import ctypes as C

    from . import _lib
    def as_bytes(m):  # bool maps are passed as their bytes, without a copy
        m = np.ascontiguousarray(m)
        return m.view(np.uint8) if m.dtype == np.bool_ else np.ascontiguousarray(m, dtype=np.uint8)

    t = as_bytes(tags)
    ny, nx = t.shape
    a = None if allowed is None else as_bytes(allowed)
    cap = 1024
    while True:
        out = np.zeros((cap, 4), np.int32)
        n = C.c_int()
        st = _lib.lib().enl_cluster_tags(t.ctypes.data_as(C.c_void_p),
                                         None if a is None else a.ctypes.data_as(C.c_void_p), nx, ny,
                                         int(nest_erode), float(efficiency), int(min_size), int(max_size),
                                         out.ctypes.data_as(C.c_void_p), cap, C.byref(n))
        if st == 0:
            return [tuple(int(v) for v in b) for b in out[: n.value]]
        if n.value <= cap:
            _lib.check(st, "enl_cluster_tags")
        cap = n.value


def chop(boxes, max_size):
    out = []
    for ilo, ihi, jlo, jhi in boxes:
        nx, ny = ihi - ilo + 1, jhi - jlo + 1
        kx = -(-nx // max_size)
        ky = -(-ny // max_size)
        xs = np.linspace(ilo, ihi + 1, kx + 1).round().astype(int)
        ys = np.linspace(jlo, jhi + 1, ky + 1).round().astype(int)
        for a in range(kx):
            for b in range(ky):
                out.append((int(xs[a]), int(xs[a + 1] - 1), int(ys[b]), int(ys[b + 1] - 1)))
    return out
