"""Host-side regridding logic (CPU): clustering covers every tag, respects
proper nesting and the size limits; box arithmetic."""
import numpy as np
import pytest

from enlightning_gb300.cluster import chop, cluster_tags
from enlightning_gb300.engine import box_difference


def _cover(boxes, shape):
    m = np.zeros(shape, bool)
    for b in boxes:
        m[b[2]:b[3] + 1, b[0]:b[1] + 1] = True
    return m


@pytest.mark.parametrize("seed", range(6))
def test_cluster_covers_tags_and_respects_nesting(seed):
    rng = np.random.default_rng(seed)
    ny, nx = 64, 96
    tags = np.zeros((ny, nx), bool)
    for _ in range(5):
        x, y = rng.integers(5, nx - 5), rng.integers(5, ny - 5)
        r = rng.integers(2, 8)
        Y, X = np.mgrid[0:ny, 0:nx]
        tags |= (X - x) ** 2 + (Y - y) ** 2 < r * r
    allowed = np.zeros((ny, nx), bool)
    allowed[4:60, 6:90] = True
    allowed[30:50, 40:55] = False  # a hole in the coarse level
    boxes = cluster_tags(tags, efficiency=0.7, min_size=2, max_size=16, allowed=allowed)
    cov = _cover(boxes, tags.shape)
    assert (cov >= (tags & allowed)).all()               # every allowed tag covered
    assert not (cov & ~allowed).any()                     # proper nesting
    assert all(b[1] - b[0] < 16 and b[3] - b[2] < 16 for b in boxes)
    # boxes do not overlap
    total = sum((b[1] - b[0] + 1) * (b[3] - b[2] + 1) for b in boxes)
    assert total == cov.sum()


def test_cluster_efficiency_on_two_blobs():
    tags = np.zeros((40, 40), bool)
    tags[2:8, 2:8] = True
    tags[30:36, 30:38] = True
    boxes = cluster_tags(tags, efficiency=0.7, min_size=1, max_size=64)
    assert sorted(boxes) == [(2, 7, 2, 7), (30, 37, 30, 35)]


def test_chop_and_box_difference():
    assert chop([(0, 99, 0, 9)], 32) == [(0, 24, 0, 9), (25, 49, 0, 9), (50, 74, 0, 9), (75, 99, 0, 9)]
    d = box_difference([(0, 9, 0, 9)], [(3, 5, 2, 20)])
    m = _cover(d, (12, 12))
    ref = _cover([(0, 9, 0, 9)], (12, 12)) & ~_cover([(3, 5, 2, 20)], (12, 12))
    assert (m == ref).all()


def _random_tag_map(rng, ny, nx, kind):
    tags = np.zeros((ny, nx), bool)
    if kind == "blobs":
        Y, X = np.mgrid[0:ny, 0:nx]
        for _ in range(rng.integers(1, 8)):
            x, y, r = rng.integers(0, nx), rng.integers(0, ny), rng.integers(1, 12)
            tags |= (X - x) ** 2 + (Y - y) ** 2 < r * r
    elif kind == "walk":  # a thin random-walk channel like the line source's
        x, y = nx / 2, ny - 2.0
        for _ in range(6 * (nx + ny)):
            a = -np.pi / 2 + rng.normal(0, 0.7)
            x, y = x + np.cos(a) * 0.7, y + np.sin(a) * 0.7
            if 0 <= int(y) < ny and 0 <= int(x) < nx:
                tags[int(y), max(0, int(x) - 1):int(x) + 2] = True
    else:  # sparse noise
        tags = rng.random((ny, nx)) < 0.03
    return tags


@pytest.mark.parametrize("seed", range(24))
def test_native_clustering_equals_specification(seed):
    """enl_cluster_tags (C++, summed-area tables) returns exactly the boxes,
    in the same order, of the array-based cluster_tags."""
    from enlightning_gb300.cluster import cluster_tags_native
    rng = np.random.default_rng(1000 + seed)
    ny, nx = int(rng.integers(8, 120)), int(rng.integers(8, 160))
    tags = _random_tag_map(rng, ny, nx, ["blobs", "walk", "noise"][seed % 3])
    allowed = None
    if seed % 2:
        allowed = np.ones((ny, nx), bool)
        for _ in range(3):
            x0, y0 = rng.integers(0, nx), rng.integers(0, ny)
            allowed[y0:y0 + rng.integers(1, 20), x0:x0 + rng.integers(1, 30)] = False
    kw = dict(efficiency=float(rng.choice([0.5, 0.7, 0.9])), min_size=int(rng.integers(1, 5)),
              max_size=int(rng.integers(4, 40)), allowed=allowed)
    ref = cluster_tags(tags, **kw)
    got = cluster_tags_native(tags, **kw)
    assert got == ref
    if allowed is not None:  # the nesting erosion done inside the native call
        from enlightning_gb300.cluster import erode_allowed
        for passes in (1, 2):
            kw2 = dict(kw, allowed=erode_allowed(allowed, passes))
            assert cluster_tags_native(tags, **dict(kw, nest_erode=passes)) == cluster_tags(tags, **kw2)


def test_native_clustering_edge_cases():
    from enlightning_gb300.cluster import cluster_tags_native
    assert cluster_tags_native(np.zeros((5, 7), bool)) == []
    one = np.zeros((5, 7), bool)
    one[2, 3] = True
    assert cluster_tags_native(one, min_size=1) == cluster_tags(one, min_size=1) == [(3, 3, 2, 2)]
    full = np.ones((40, 300), bool)
    assert cluster_tags_native(full, max_size=64) == cluster_tags(full, max_size=64)
    nothing_allowed = np.zeros((5, 7), bool)
    assert cluster_tags_native(one, allowed=nothing_allowed) == []


@pytest.mark.parametrize("seed", range(12))
def test_native_clustering_of_the_tag_window(seed):
    """The native regrid clusters only the window of the tagged blocks'
    bounding box grown by the erosion passes (clamped to the map) and shifts
    the boxes back: the same boxes as clustering the whole map."""
    from enlightning_gb300.cluster import cluster_tags_native
    rng = np.random.default_rng(2000 + seed)
    ny, nx = int(rng.integers(30, 120)), int(rng.integers(30, 160))
    tags = np.zeros((ny, nx), bool)
    sub = _random_tag_map(rng, ny // 2, nx // 2, ["blobs", "walk", "noise"][seed % 3])
    y0, x0 = int(rng.integers(0, ny - ny // 2 + 1)), int(rng.integers(0, nx - nx // 2 + 1))
    tags[y0:y0 + ny // 2, x0:x0 + nx // 2] = sub
    allowed = np.ones((ny, nx), bool)
    for _ in range(4):
        ax, ay = rng.integers(0, nx), rng.integers(0, ny)
        allowed[ay:ay + rng.integers(1, 20), ax:ax + rng.integers(1, 30)] = False
    kw = dict(efficiency=float(rng.choice([0.5, 0.7, 0.9])), min_size=int(rng.integers(1, 5)),
              max_size=int(rng.integers(4, 40)))
    if not tags.any():
        return
    jj, ii = np.nonzero(tags)
    for passes in (0, 1, 2, 3):
        full = cluster_tags_native(tags, allowed=allowed, nest_erode=passes, **kw)
        wx0, wx1 = max(0, ii.min() - passes), min(nx - 1, ii.max() + passes)
        wy0, wy1 = max(0, jj.min() - passes), min(ny - 1, jj.max() + passes)
        win = cluster_tags_native(tags[wy0:wy1 + 1, wx0:wx1 + 1], allowed=allowed[wy0:wy1 + 1, wx0:wx1 + 1],
                                  nest_erode=passes, **kw)
        assert [(a + wx0, b + wx0, c + wy0, d + wy0) for a, b, c, d in win] == full
