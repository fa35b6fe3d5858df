"""Why the line-source workloads use a CFL reduction for dt.

The reference's time step is cfl*min(dx)/c (enlightning.C:433-456).  For a
10 p0 line source the flow reaches several hundred m/s and that step is
unstable; dt = cfl*dx/max(|u|,|v|)+c keeps the same run finite.  Both runs
use the oracle (the restated Fortran) on a small patch.
"""
import math

import numpy as np

from enlightning_gb300 import workloads
from enlightning_gb300.constants import default_params


def _run(adaptive, steps=14):
    import oracle as ora
    prm = default_params()
    n, dx = 96, (0.5, 0.5)
    rng = np.random.default_rng(1)
    segs = workloads.random_walk_channel(rng, nseg=8, start=(24.0, 36.0), heading_deg=-90.0)
    H = np.zeros((n + 6, n + 6))
    ora.paint_source(n + 6, n + 6, (-1.5, -1.5), dx, H, 30, amp=10 * prm["p0"],
                     spread=workloads.gaussian_spread(1.0), segs=segs)
    w = workloads.state_from_dp(H, prm)
    box = (0, n - 1, 0, n - 1)
    P = ora.Patch(box, (0.0, 0.0), dx)
    P.w_scr[...] = w
    P.w_cur[...] = P.interior(w)
    ora.update_state(dx, (-1.5, -1.5), (-3, n + 2, -3, n + 2), (0, 0), P.w_scr, P.pres, P.temp, prm)
    for _ in range(steps):
        if adaptive:
            wc = P.w_cur
            smax = max(np.abs(wc[1] / wc[0]).max(), np.abs(wc[2] / wc[0]).max()) + prm["c"]
            dt = 0.5 * min(dx) / smax
        else:
            dt = 0.5 * min(dx) / prm["c"]
        with np.errstate(all="ignore"):
            ora.advance(P, prm, "hybrid_high_llf", dt, 1, domain=((0, 0), (n * dx[0], n * dx[1])))
        if not np.isfinite(P.w_cur).all():
            return False
    return True


def test_reference_dt_is_unstable_for_line_source(ora):
    ora.set_threads(4)
    assert _run(adaptive=False) is False


def test_cfl_reduction_keeps_line_source_finite(ora):
    ora.set_threads(4)
    assert _run(adaptive=True) is True
