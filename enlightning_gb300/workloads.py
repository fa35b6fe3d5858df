"""Seeded synthetic initial conditions of the benchmark workloads.

None of the workloads uses a public dataset; every input is generated here.
A Gaussian overpressure dp(x, y) is mapped onto the reference's 5-field state
(rho, rho*u, rho*v, rho*s, rho*T_n) by inverting the equation of state of
update_state.m4:90-94 at s = 0 and c_lr = 0:

    dp / c^2 = drho + (gamma - 1) / (2 rho0) * drho^2      (positive root)

with u = v = s = 0 and T_n = T(rho, s = 0) = T0 * exp(-R log(rho0/rho) / c_v)
(update_state.m4:103-105), so the nitrogen mode starts in equilibrium.
"""
from __future__ import annotations

import math

import numpy as np


def drho_from_dp(dp, p):
    k = (p["gamma1"] - 1.0) / (2.0 * p["rho0"])
    x = np.asarray(dp, dtype=np.float64) / (p["c"] ** 2)
    return (-1.0 + np.sqrt(1.0 + 4.0 * k * x)) / (2.0 * k)


def state_from_dp(dp, p):
    """(5, ...) state for an overpressure field dp (any shape)."""
    rho = p["rho0"] + drho_from_dp(dp, p)
    T = p["T0"] * np.exp((0.0 - p["R"] * np.log(p["rho0"] / rho)) / p["c_v"])
    z = np.zeros_like(rho)
    return np.stack([rho, z, z, z, rho * T])


def gaussian_dp(nx, ny, amp, sigma_cells, cx=None, cy=None):
    """Overpressure amp * exp(-r^2 / (2 sigma^2)), r in cells, centred by default."""
    cx = (nx - 1) / 2.0 if cx is None else cx
    cy = (ny - 1) / 2.0 if cy is None else cy
    X, Y = np.meshgrid(np.arange(nx, dtype=np.float64), np.arange(ny, dtype=np.float64))
    return amp * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2.0 * sigma_cells ** 2))


def pulse_patch_state(nx, ny, p, amp_frac=0.1, sigma_cells=8.0, g=3):
    """Single-pulse patch: ghosted (5, ny+2g, nx+2g) array, interior set."""
    w = np.zeros((5, ny + 2 * g, nx + 2 * g))
    dp = gaussian_dp(nx, ny, amp_frac * p["p0"], sigma_cells)
    w[:, g:g + ny, g:g + nx] = state_from_dp(dp, p)
    # ghosts: ambient until the first boundary fill
    amb = state_from_dp(np.zeros((1,)), p)[:, 0]
    for k in range(5):
        m = np.ones((ny + 2 * g, nx + 2 * g), bool)
        m[g:g + ny, g:g + nx] = False
        w[k][m] = amb[k]
    return w


def pulse_dt(p, dx):
    """enlightning.C:433-456: cfl * min(dx) / c."""
    return p["cfl"] * (min(dx) / p["c"])


def rankine_hugoniot(mach, gamma=1.4):
    """Post-shock ratios (rho2/rho1, p2/p1) and the flow speed factor u2/c1."""
    m2 = mach * mach
    r = (gamma + 1.0) * m2 / ((gamma - 1.0) * m2 + 2.0)
    pr = 1.0 + 2.0 * gamma / (gamma + 1.0) * (m2 - 1.0)
    u2 = mach * (1.0 - 1.0 / r)
    return r, pr, u2


def random_walk_channel(rng, nseg=200, start=(0.0, 0.0), heading_deg=-90.0, seg_len=(1.0, 3.0),
                        turn_deg=16.0):
    """Seeded 2-D random walk: nseg segments, lengths U(seg_len), turns U(+-turn_deg).

    Returns an array (nseg, 4) of (x0, y0, x1, y1) in metres, in the manner of
    the reference's channel generator (matlab/LightningChannel.m:48-89).
    """
    segs = np.zeros((nseg, 4))
    x, y = start
    h = math.radians(heading_deg)
    for n in range(nseg):
        h += math.radians(rng.uniform(-turn_deg, turn_deg))
        L = rng.uniform(*seg_len)
        x1, y1 = x + L * math.cos(h), y + L * math.sin(h)
        segs[n] = (x, y, x1, y1)
        x, y = x1, y1
    return segs


# ---------------------------------------------------------------------------
# multi-level workloads
# ---------------------------------------------------------------------------

SRC_POINT, SRC_SINE, SRC_LIGHTNING = 10, 20, 30


def gaussian_spread(sigma):
    """Reference spread for exp(-ln2 r^2/spread^2) equal to exp(-r^2/(2 sigma^2))."""
    return sigma * math.sqrt(2.0 * math.log(2.0))


def line_source(prm, nx0=4096, ny0=2048, dx0=0.5, nlevels=3, seed=100, nseg=200, precision=1,
                variant="hybrid_high_llf", learned=False, base_patch=256, cfl=0.5, amp_frac=10.0,
                sigma_cells=2.0, min_size=16, max_size=256, native_regrid=True, dense=False, tile_order=0):
    """Thunder-like line source on a multi-level hierarchy (synthetic).

    A seeded random-walk channel of `nseg` segments (lengths U(1, 3) m, turns
    U(-16, 16) deg) starting high in the domain and heading down deposits a
    Gaussian overpressure amp_frac*p0 of sigma = sigma_cells base cells per
    segment with the reference's capsule-union painting (enlightning.C:
    2214-2281), evaluated on the device at every level's own resolution and
    converted to the state.  Boundaries as the reference's input.txt:14-18
    (ABSORB left/right/top, REFLECT ground).  The time step is the device CFL
    reduction (cfl * dx_min / max(|u|+c)): the reference's c-only dt
    (enlightning.C:433-456) is unstable for a 10 p0 source.
    """
    from .constants import ABSORB, REFLECT
    from .engine import Engine, Hierarchy

    rng = np.random.default_rng(seed)
    L = nx0 * dx0
    Hh = ny0 * dx0
    segs = random_walk_channel(rng, nseg=nseg, start=(0.5 * L, 0.85 * Hh), heading_deg=-90.0)
    E = Engine(prm, nx0, ny0, (dx0, dx0), nlevels=nlevels, ratio=2, bc=(ABSORB, ABSORB, REFLECT, ABSORB),
               variant=variant, precision=precision, learned=learned, dense=dense, tile_order=tile_order)
    E.set_adaptive_dt(True, cfl)
    Hy = Hierarchy(E, min_size=min_size, max_size=max_size, tag_buffer=2, native=native_regrid)
    Hy.base_patches(base_patch)
    amp = amp_frac * prm["p0"]
    spread = gaussian_spread(sigma_cells * dx0)

    def paint(level):
        E.paint_source(level, SRC_LIGHTNING, amp=amp, spread=spread, segs=segs)
        E.state_from_overpressure(level)

    paint(0)
    for l in range(nlevels - 1):
        Hy.regrid_level(l)
        paint(l + 1)
    return E, Hy, segs


def eos_state(rho, u, v, p, prm):
    """State (5, ...) and T for given rho, velocity and pressure at c_lr = 0,
    inverting update_state.m4:90-94 for rho*s and using T_n = T."""
    k = (prm["gamma1"] - 1.0) / (2.0 * prm["rho0"])
    drho = rho - prm["rho0"]
    rs = prm["c_p"] * ((p - prm["p0"]) / prm["c"] ** 2 - drho - k * drho ** 2)
    T = prm["T0"] * np.exp((rs / rho - prm["R"] * np.log(prm["rho0"] / rho)) / prm["c_v"])
    return np.stack([rho, rho * u, rho * v, rs, rho * T]), T


def mach_shock(prm, seed=0, nx0=1024, ny0=512, dx0=0.1, nlevels=2, mach=1.5, precision=1, learned=False,
               variant="hybrid_high_llf", base_patch=128, cfl=0.5, min_size=32, max_size=128, dense=False, tile_order=0):
    """Planar shock moving +x into ambient air with 1 % i.i.d. density noise.

    Post-shock state from the ideal-gas Rankine-Hugoniot relations at
    gamma = 1.4, mapped onto the reference's state through its equation of
    state (eos_state).  Shock at x = 0.1 L; ABSORB left/right (zero-width
    envelope: zero-gradient ghosts), REFLECT top/bottom; device CFL time step.
    """
    from .constants import ABSORB, REFLECT
    from .engine import Engine, Hierarchy

    rng = np.random.default_rng(seed)
    r, pr, u2f = rankine_hugoniot(mach, 1.4)
    p = dict(prm)
    p["bc_absorb_width"] = 1e-9
    E = Engine(p, nx0, ny0, (dx0, dx0), nlevels=nlevels, ratio=2, bc=(ABSORB, ABSORB, REFLECT, REFLECT),
               variant=variant, precision=precision, learned=learned, dense=dense, tile_order=tile_order)
    E.set_adaptive_dt(True, cfl)
    Hy = Hierarchy(E, min_size=min_size, max_size=max_size, tag_buffer=2)
    Hy.base_patches(base_patch)
    X = np.arange(nx0)[None, :].repeat(ny0, 0)
    post = X < int(0.1 * nx0)
    rho = np.where(post, prm["rho0"] * r, prm["rho0"] * (1.0 + rng.uniform(-0.01, 0.01, (ny0, nx0))))
    pres = np.where(post, prm["p0"] * pr, prm["p0"] + prm["c"] ** 2 * (rho - prm["rho0"]) +
                    prm["c"] ** 2 * (prm["gamma1"] - 1) / (2 * prm["rho0"]) * (rho - prm["rho0"]) ** 2)
    u = np.where(post, u2f * prm["c"], 0.0)
    w, T = eos_state(rho, u, np.zeros_like(u), pres, prm)
    E.set_level_state(0, w, pres, T)
    for l in range(nlevels - 1):
        Hy.regrid_level(l)
    return E, Hy


def shelf_pack(sides, width, gap=8):
    """Origins (x, y) placing squares of the given sides on shelves of a
    canvas `width` wide, `gap` cells apart (gap >= 6 keeps the 3-cell ghost
    bands of neighbours disjoint; multiples of 8 keep TMA-friendly origins)."""
    order = sorted(range(len(sides)), key=lambda k: -sides[k])
    pos = [None] * len(sides)
    x = y = gap
    shelf_h = 0
    for k in order:
        s = sides[k]
        if x + s + gap > width:
            x = gap
            y += shelf_h + gap
            shelf_h = 0
        pos[k] = (x, y)
        x += s + gap
        shelf_h = max(shelf_h, s)
    height = y + shelf_h + gap
    return pos, height


def pulse_batch(prm, seed=7, n=64, side_range=(128, 1024), precision=1, learned=False, variant="hybrid_high_llf",
                width=8192, dx=0.1, dense=False, tile_order=0):
    """Batched independent pulse problems: n square patches with sides drawn
    uniformly from multiples of 32 in side_range, Gaussian overpressure
    U(0.01, 0.5) p0 with sigma U(4, 16) cells at each centre, reflective
    walls, dx = 0.1 m and the reference's dt = cfl*dx/c; all advanced by one
    engine (independent mode: every patch is its own domain)."""
    from .constants import REFLECT
    from .engine import Engine

    rng = np.random.default_rng(seed)
    sides = [int(32 * rng.integers(side_range[0] // 32, side_range[1] // 32 + 1)) for _ in range(n)]
    amps = rng.uniform(0.01, 0.5, n)
    sigmas = rng.uniform(4.0, 16.0, n)
    pos, height = shelf_pack(sides, width)
    height = int(-(-height // 8) * 8)
    E = Engine(prm, width, height, (dx, dx), nlevels=1, bc=(REFLECT,) * 4, variant=variant, precision=precision,
               learned=learned, independent=True, dense=dense, tile_order=tile_order)
    boxes = [(x, x + s - 1, y, y + s - 1) for (x, y), s in zip(pos, sides)]
    E.set_patches(0, boxes)
    k = (prm["gamma1"] - 1.0) / (2.0 * prm["rho0"])
    for (x, y), s, a, sg in zip(pos, sides, amps, sigmas):
        dp = gaussian_dp(s, s, a * prm["p0"], sg)
        w = state_from_dp(dp, prm)
        drho = w[0] - prm["rho0"]
        p = prm["c"] ** 2 * (drho + k * drho ** 2) + prm["p0"]
        T = w[4] / w[0]
        E.set_box_state(0, x, y, w, p, T)
    dt = pulse_dt(prm, (dx, dx))
    return E, boxes, dict(sides=sides, amps=amps, sigmas=sigmas, dt=dt)
