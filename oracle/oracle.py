"""ctypes front end of the CPU oracle (test infrastructure only).

Loads ``oracle/_build/libenl_oracle.so`` (built from ``enl_oracle.cpp`` by
``build()``) and offers numpy-level wrappers whose argument meaning follows the
reference's F77 interface (enlightningfort.h:22-102).  Only the tests,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg import it, as
the checker of the CUDA library.

Array convention (SAMRAI CellData, depth-major): a ghosted field array of a
patch with interior ``nx x ny`` and ghost widths ``g0, g1`` is a C-contiguous
numpy array of shape ``(nfields, ny + 2*g1, nx + 2*g0)``; interior-only arrays
have shape ``(nfields, ny, nx)``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "enl_oracle.cpp")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libenl_oracle.so")

VARIANTS = [
    "hybrid_high_llf", "hybrid_high", "hybrid_low_llf", "hybrid_low",
    "weno_high_llf", "weno_high", "weno_low_llf", "weno_low", "drp",
]

REFLECT, ABSORB = 10, 20

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with strict IEEE evaluation (no FMA contraction)."""
    os.makedirs(BUILD, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
               "-fPIC", "-shared", "-o", tmp, SRC]
        subprocess.run(cmd, check=True)
        os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int)
        i, d = C.c_int, C.c_double
        L.ora_rhs.argtypes = [i, i, i, i, i, i, i, dp, dp, dp, dp, dp, dp, dp,
                              d, d, d, d, d, d, d, d, d, dp, i, d, d, i, ip, dp]
        L.ora_runge_kutta.argtypes = [i, i, i, i, i, i, d, d, d, d, dp, dp, dp, i]
        L.ora_update_state.argtypes = [dp, dp, i, i, i, i, i, i, dp, dp, dp,
                                       d, d, d, d, d, d, d, d, d, d, d, i]
        L.ora_tag_cells.argtypes = [i, i, i, i, i, i, ip, dp, dp, i, dp, i]
        L.ora_absorb.argtypes = [i, i, i, i, i, i, dp, dp, dp, dp, ip, d, d, d, d, dp, dp, dp]
        L.ora_phys_bc.argtypes = [i, i, i, i, i, i, ip, ip, i, i, dp, dp, dp, dp]
        L.ora_relaxation_times.argtypes = [d, d, d, dp, dp]
        L.ora_set_f32_literals.argtypes = [i]
        L.ora_set_threads.argtypes = [i]
        L.ora_get_threads.restype = i
        L.ora_paint_source.argtypes = [i, i, dp, dp, dp, i, i, d, d, dp, d, d, i, dp, d]
        _lib = L
    return _lib


def _dp(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_int))


def set_threads(n: int) -> None:
    lib().ora_set_threads(int(n))


def set_f32_literals(on: bool) -> None:
    lib().ora_set_f32_literals(1 if on else 0)


def relaxation_times(p0, T0, RH):
    a, b = C.c_double(), C.c_double()
    lib().ora_relaxation_times(p0, T0, RH, C.byref(a), C.byref(b))
    return a.value, b.value


def rhs(variant, box, g, xlo, dx, w_n, H0, pres, temp, prm, level, flags=False, opcounts=False):
    """KK for one patch.  ``box`` = (ifirst0, ilast0, ifirst1, ilast1), ``g`` = (g0, g1).

    ``prm`` holds alpha, kappa, mu, muB, R, T_star_n, T_star_o, tau_n, tau_o,
    tol (3), c, c_lr.  Returns KK (5, ny, nx) and optionally the switch flags
    and per-cell op counts.
    """
    v = VARIANTS.index(variant) if isinstance(variant, str) else int(variant)
    if0, il0, if1, il1 = box
    nx, ny = il0 - if0 + 1, il1 - if1 + 1
    KK = np.zeros((5, ny, nx))
    fl = np.zeros((ny, nx), np.int32) if flags else None
    oc = np.zeros((ny, nx, 5)) if opcounts else None
    tol = np.ascontiguousarray(prm["tol"], dtype=np.float64)
    lib().ora_rhs(v, if0, il0, if1, il1, g[0], g[1], _dp(np.asarray(xlo, np.float64)),
                  _dp(np.asarray(dx, np.float64)), _dp(w_n), _dp(H0), _dp(KK), _dp(pres), _dp(temp),
                  prm["alpha"], prm["kappa"], prm["mu"], prm["muB"], prm["R"], prm["T_star_n"],
                  prm["T_star_o"], prm["tau_n"], prm["tau_o"], _dp(tol), int(level), prm["c"],
                  prm["c_lr"], 5, _ip(fl), _dp(oc))
    out = [KK]
    if flags:
        out.append(fl)
    if opcounts:
        out.append(oc)
    return out[0] if len(out) == 1 else tuple(out)


def runge_kutta(box, g, dt, a1, a2, beta, w_n, ww, KK):
    if0, il0, if1, il1 = box
    lib().ora_runge_kutta(if0, il0, if1, il1, g[0], g[1], dt, a1, a2, beta, _dp(w_n), _dp(ww),
                          _dp(KK), 5)


def update_state(dx, xlo, box, g, w_n, pres, temp, prm):
    if0, il0, if1, il1 = box
    lib().ora_update_state(_dp(np.asarray(dx, np.float64)), _dp(np.asarray(xlo, np.float64)), if0,
                           il0, if1, il1, g[0], g[1], _dp(w_n), _dp(pres), _dp(temp), prm["rho0"],
                           prm["c"], prm["gamma1"], prm["c_p"], prm["p0"], prm["T0"], prm["c_lr"],
                           prm["c_v"], prm["R_tilde"], prm["M"], prm["R"], 5)


def tag_cells(box, g, w_n, H0g, tol, tag_val=1):
    if0, il0, if1, il1 = box
    tags = np.zeros((il1 - if1 + 1, il0 - if0 + 1), np.int32)
    lib().ora_tag_cells(if0, il0, if1, il1, g[0], g[1], _ip(tags), _dp(w_n), _dp(H0g), tag_val,
                        _dp(np.ascontiguousarray(tol, dtype=np.float64)), 5)
    return tags


def absorb(box, g, patch_xlo, dx, grid_xlo, grid_xhi, bc, width, prm, w_n, pres, temp):
    if0, il0, if1, il1 = box
    lib().ora_absorb(if0, il0, if1, il1, g[0], g[1], _dp(np.asarray(patch_xlo, np.float64)),
                     _dp(np.asarray(dx, np.float64)), _dp(np.asarray(grid_xlo, np.float64)),
                     _dp(np.asarray(grid_xhi, np.float64)), _ip(np.asarray(bc, np.int32)), width,
                     prm["p0"], prm["T0"], prm["rho0"], _dp(w_n), _dp(pres), _dp(temp))


def phys_bc(box, g, touches, bc, w_n, pres, temp, source, fill=None):
    if0, il0, if1, il1 = box
    fw = fill if fill is not None else g
    lib().ora_phys_bc(if0, il0, if1, il1, g[0], g[1], _ip(np.asarray(touches, np.int32)),
                      _ip(np.asarray(bc, np.int32)), fw[0], fw[1], _dp(w_n), _dp(pres), _dp(temp),
                      _dp(source))


def paint_source(nx, ny, xlo, dx, H, src_type, mode=10, amp=1.0, spread=1.0, pos=(0.0, 0.0),
                 sine_amp=0.0, sine_freq=0.0, segs=None, drive=1.0):
    """enlightning.C:2140-2307 on one patch (H interior (ny, nx), modified in place)."""
    sg = np.ascontiguousarray(np.asarray(segs if segs is not None else np.zeros((0, 4)), np.float64))
    lib().ora_paint_source(nx, ny, _dp(np.asarray(xlo, np.float64)), _dp(np.asarray(dx, np.float64)), _dp(H),
                           int(src_type), int(mode), float(amp), float(spread),
                           _dp(np.asarray(pos, np.float64)), float(sine_amp), float(sine_freq), sg.shape[0],
                           _dp(sg), float(drive))


class Patch:
    """Single-patch state for the oracle's stage driver (numpy, SAMRAI layout)."""

    def __init__(self, box, xlo, dx, level=0, touches=(1, 1, 1, 1), g=3):
        self.box, self.xlo, self.dx, self.level, self.touches, self.g = box, xlo, dx, level, touches, g
        nx, ny = box[1] - box[0] + 1, box[3] - box[2] + 1
        self.nx, self.ny = nx, ny
        NX, NY = nx + 2 * g, ny + 2 * g
        self.w_scr = np.zeros((5, NY, NX))
        self.w_cur = np.zeros((5, ny, nx))
        self.pres = np.zeros((NY, NX))
        self.temp = np.zeros((NY, NX))
        self.src = np.zeros((ny, nx))
        self.src_g = np.zeros((NY, NX))

    def interior(self, a):
        g = self.g
        return a[..., g:g + self.ny, g:g + self.nx]


def advance(P: Patch, prm, variant, dt, nsteps, bc=(REFLECT,) * 4, domain=((0, 0), (1, 1)),
            rk=((1.0, 0.75, 0.3333333333), (0.0, 0.25, 0.6666666667), (1.0, 0.25, 0.6666666667)),
            flags_out=None):
    """SAMRAI MOL loop for one patch with the reference's stage order
    (enlightning.C:459-583), the oracle's restatement of every call."""
    a1s, a2s, bs = rk
    g = P.g
    for _ in range(nsteps):
        P.interior(P.w_scr)[...] = P.w_cur
        for s in range(len(a1s)):
            phys_bc(P.box, (g, g), P.touches, bc, P.w_scr, P.pres, P.temp, P.src_g)
            res = rhs(variant, P.box, (g, g), P.xlo, P.dx, P.w_scr, P.src, P.pres, P.temp, prm, P.level,
                      flags=flags_out is not None)
            KK = res[0] if flags_out is not None else res
            if flags_out is not None:
                flags_out.append(res[1])
            runge_kutta(P.box, (g, g), dt, a1s[s], a2s[s], bs[s], P.w_scr, P.w_cur, KK)
            update_state(P.dx, P.xlo, P.box, (g, g), P.w_scr, P.pres, P.temp, prm)
            absorb(P.box, (g, g), P.xlo, P.dx, domain[0], domain[1], bc, prm["bc_absorb_width"], prm,
                   P.w_scr, P.pres, P.temp)
        P.w_cur[...] = P.interior(P.w_scr)
