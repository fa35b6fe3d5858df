"""Generate tests/golden/enl_golden.npz from the reference's own Fortran source.

Runs fortran/rhs_*.m4 (all nine variants), runge_kutta.m4, update_state.m4 and
tag_cells.m4 of the reference tree through tests/golden/f77interp.py on small
seeded patches and stores inputs and outputs.  The hybrid WENO/DRP switch is
read from the Fortran's own ``tag`` variable at the point where it is tested.

Run it where the reference tree is checked out, giving its root:

    python tests/golden/make_golden.py <reference root>

The fixtures are committed; the tests never read the reference tree.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import f77interp  # noqa: E402

from enlightning_gb300.constants import VARIANTS, default_params  # noqa: E402

G = 3


def make_case(kind: str, seed: int, nx: int, ny: int, if0: int, if1: int, prm: dict):
    """Seeded patch state (w with ghosts) with regions of both switch outcomes."""
    rng = np.random.default_rng(seed)
    NX, NY = nx + 2 * G, ny + 2 * G
    X, Y = np.meshgrid(np.arange(NX, dtype=np.float64), np.arange(NY, dtype=np.float64))
    rho0, T0 = prm["rho0"], prm["T0"]
    if kind == "ambient":
        rho = np.full((NY, NX), rho0)
        u = np.zeros_like(rho)
        v = np.zeros_like(rho)
        s = np.zeros_like(rho)
        Tn = np.full_like(rho, T0)
    elif kind == "smooth":
        # constant + linear regions (DRP) and a Gaussian bump (WENO)
        rho = rho0 + 1e-3 * X + 0.02 * np.exp(-((X - NX * 0.7) ** 2 + (Y - NY * 0.6) ** 2) / 4.0)
        u = 3.0 + 0.5 * np.sin(0.3 * X + 0.2 * Y)
        v = -2.0 + 0.4 * np.cos(0.25 * X - 0.1 * Y)
        s = 5.0 * np.sin(0.2 * X) * np.cos(0.3 * Y)
        Tn = T0 + 2.0 * np.cos(0.15 * X + 0.35 * Y)
    elif kind == "shock":
        step = (X > NX * 0.45).astype(np.float64)
        rho = rho0 * (1.0 + 0.862 * step) + 1e-3 * rng.standard_normal((NY, NX)) * step
        u = 238.0 * step
        v = 1.0 * np.sin(0.4 * Y)
        s = 40.0 * step
        Tn = T0 + 60.0 * step
    else:  # "random"
        rho = rho0 * (1.0 + 0.01 * rng.uniform(-1, 1, (NY, NX)))
        u = 10.0 * rng.standard_normal((NY, NX))
        v = 10.0 * rng.standard_normal((NY, NX))
        s = 20.0 * rng.standard_normal((NY, NX))
        Tn = T0 + 3.0 * rng.standard_normal((NY, NX))
    w = np.ascontiguousarray(np.stack([rho, rho * u, rho * v, rho * s, rho * Tn]))
    H0g = np.ascontiguousarray(
        np.where(rng.uniform(size=(NY, NX)) < 0.5, 0.0, 1e4 * np.exp(-((X - NX / 2) ** 2) / 9.0)))
    return w, H0g


def main(ref: str) -> None:
    fdir = os.path.join(ref, "fortran")
    prm = default_params()
    out: dict[str, np.ndarray] = {}
    cases = [("ambient", 0, 10, 8, 0, 0), ("smooth", 1, 14, 11, 5, -3),
             ("shock", 2, 13, 10, -4, 7), ("random", 3, 9, 12, 0, 2)]
    us = f77interp.load(os.path.join(fdir, "update_state.m4"))
    rk = f77interp.load(os.path.join(fdir, "runge_kutta.m4"))
    tg = f77interp.load(os.path.join(fdir, "tag_cells.m4"))
    rhs_ns = {v: f77interp.load(os.path.join(fdir, f"rhs_{v}.m4"), watch="tag") for v in VARIANTS}
    tol = np.array(prm["tol"], dtype=np.float64)
    for cname, seed, nx, ny, if0, if1 in cases:
        box = (if0, if0 + nx - 1, if1, if1 + ny - 1)
        xlo = np.array([0.35 + 0.1 * seed, -0.2 + 0.05 * seed])
        dx = np.array([0.1, 0.125]) if seed % 2 else np.array([0.5, 0.5])
        w, H0g = make_case(cname, seed, nx, ny, if0, if1, prm)
        NX, NY = nx + 2 * G, ny + 2 * G
        pres = np.zeros((NY, NX))
        temp = np.zeros((NY, NX))
        c_lr = -3.9e-3 if cname == "smooth" else 0.0
        # update_state over the whole ghosted box (box grown by G, zero ghosts)
        us["update_state"](dx, xlo - G * dx, box[0] - G, box[1] + G, box[2] - G, box[3] + G, 0, 0,
                           w.T, pres.T, temp.T, prm["rho0"], prm["c"], prm["gamma1"], prm["c_p"],
                           prm["p0"], prm["T0"], c_lr, prm["c_v"], prm["R_tilde"], prm["M"],
                           prm["R"], 5)
        H0 = np.ascontiguousarray(H0g[G:-G, G:-G])
        pre = f"{cname}/"
        out[pre + "box"] = np.array(box, np.int32)
        out[pre + "xlo"] = xlo
        out[pre + "dx"] = dx
        out[pre + "c_lr"] = np.array(c_lr)
        out[pre + "w"] = w
        out[pre + "pres"] = pres.copy()
        out[pre + "temp"] = temp.copy()
        out[pre + "H0g"] = H0g
        for v in VARIANTS:
            levels = (0, 1) if v.startswith("hybrid") else (0,)
            for level in levels:
                ns = rhs_ns[v]
                flags = np.full((ny, nx), -1, np.int32)

                def hook(loc, flags=flags):
                    flags[loc["j"] - if1, loc["i"] - if0] = loc["tag"]

                ns["_hooks"]["fn"] = hook
                KK = np.zeros((5, ny, nx))
                ns["rhs"](box[0], box[1], box[2], box[3], G, G, xlo, dx, w.T, H0.T, KK.T, pres.T,
                          temp.T, prm["alpha"], prm["kappa"], prm["mu"], prm["muB"], prm["R"],
                          prm["T_star_n"], prm["T_star_o"], prm["tau_n"], prm["tau_o"], tol, level,
                          prm["c"], c_lr, 5)
                out[pre + f"KK/{v}/L{level}"] = KK
                if v.startswith("hybrid"):
                    assert (flags >= 0).all()
                    out[pre + f"flags/{v}/L{level}"] = flags
                print(cname, v, level, "weno fraction",
                      flags.mean() if v.startswith("hybrid") else "-", flush=True)
        # runge_kutta on the hybrid_high_llf level-0 KK, SSP-RK3 stage 2 coefficients
        wn = w.copy()
        ww = np.ascontiguousarray(w[:, G:-G, G:-G] * 0.999)
        KK = out[pre + "KK/hybrid_high_llf/L0"]
        rk["runge_kutta"](box[0], box[1], box[2], box[3], G, G, 1.4577e-4, 0.75, 0.25, 0.25,
                          wn.T, ww.T, KK.T, 5)
        out[pre + "rk/ww"] = ww
        out[pre + "rk/w_n"] = wn
        # update_state on the result (interior only, ghosted arrays)
        p2 = pres.copy()
        t2 = temp.copy()
        us["update_state"](dx, xlo, box[0], box[1], box[2], box[3], G, G, wn.T, p2.T, t2.T,
                           prm["rho0"], prm["c"], prm["gamma1"], prm["c_p"], prm["p0"], prm["T0"],
                           c_lr, prm["c_v"], prm["R_tilde"], prm["M"], prm["R"], 5)
        out[pre + "us/pres"] = p2
        out[pre + "us/temp"] = t2
        tags = np.full((ny, nx), -7, np.int32)
        tg["tag_cells"](box[0], box[1], box[2], box[3], G, G, tags.T, w.T, H0g.T, 1, tol, 5)
        out[pre + "tags"] = tags
    out["params"] = np.array([prm[k] for k in PARAM_KEYS])
    np.savez_compressed(os.path.join(HERE, "enl_golden.npz"), **out)
    print("wrote", os.path.join(HERE, "enl_golden.npz"))


PARAM_KEYS = ("alpha", "kappa", "mu", "muB", "R", "T_star_n", "T_star_o", "tau_n", "tau_o", "c",
              "rho0", "gamma1", "c_p", "p0", "T0", "c_v", "R_tilde", "M")

if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <root of the reference tree>")
    main(sys.argv[1])
