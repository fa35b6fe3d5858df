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
    """Config-1 style patch: ghosted (5, ny+2g, nx+2g) array, interior set."""
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
