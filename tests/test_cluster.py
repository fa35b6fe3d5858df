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
