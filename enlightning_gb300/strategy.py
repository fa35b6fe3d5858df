"""Host-side mirror of the reference's patch strategy (class enlightning).

Drives the drop-in entry points of libenlightning_gpu.so exactly the way
enlightning.C drives the Fortran: ``single_step`` is enlightning::singleStep
(enlightning.C:459-583: rhs -> runge_kutta -> update_state -> absorbing
envelope), ``set_physical_boundary_conditions`` is enlightning.C:790-1013,
``tag_gradient_detector_cells`` is enlightning.C:586-628 and
``compute_stable_dt`` is enlightning.C:433-456.  ``advance`` plays the role
of SAMRAI's MethodOfLinesIntegrator::advanceHierarchy for a single patch:
copy current -> scratch, per RK stage fill ghosts then singleStep, copy
scratch -> current.

Patch data lives on the device (torch CUDA tensors used as plain memory) in
SAMRAI CellData layout: ghosted arrays (nfields, ny + 2g, nx + 2g), interior
arrays (nfields, ny, nx).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import torch

from . import _lib
from .constants import ABSORB, CELLG, NEQU, REFLECT, RK3_ALPHA1, RK3_ALPHA2, RK3_BETA, VARIANTS


@dataclass
class Patch:
    """One patch: index box, geometry and device-resident CellData."""
    box: tuple  # (ifirst0, ilast0, ifirst1, ilast1)
    xlo: tuple  # lower corner of the patch interior (m)
    dx: tuple
    level: int = 0
    touches: tuple = (1, 1, 1, 1)  # patch side on the domain boundary: L, R, B, T
    g: int = CELLG
    w_scr: torch.Tensor = None    # scratch w_n, ghosted (5, NY, NX)
    w_cur: torch.Tensor = None    # current w, interior (5, ny, nx)
    pres: torch.Tensor = None     # ghosted (1, NY, NX)
    temp: torch.Tensor = None     # ghosted (1, NY, NX)
    src: torch.Tensor = None      # current source, interior (ny, nx)
    src_g: torch.Tensor = None    # scratch source, ghosted (1, NY, NX)
    K: torch.Tensor = None        # rhs scratch, interior (5, ny, nx)
    extra: dict = field(default_factory=dict)

    @property
    def nx(self):
        return self.box[1] - self.box[0] + 1

    @property
    def ny(self):
        return self.box[3] - self.box[2] + 1

    def allocate(self, device="cuda"):
        g, nx, ny = self.g, self.nx, self.ny
        NX, NY = nx + 2 * g, ny + 2 * g
        z = dict(dtype=torch.float64, device=device)
        self.w_scr = torch.zeros((NEQU, NY, NX), **z)
        self.w_cur = torch.zeros((NEQU, ny, nx), **z)
        self.pres = torch.zeros((1, NY, NX), **z)
        self.temp = torch.zeros((1, NY, NX), **z)
        self.src = torch.zeros((ny, nx), **z)
        self.src_g = torch.zeros((1, NY, NX), **z)
        self.K = torch.zeros((NEQU, ny, nx), **z)
        return self

    def interior(self, t):
        g = self.g
        return t[:, g:g + self.ny, g:g + self.nx]


def _ptr(t: torch.Tensor):
    assert t.is_contiguous()
    return C.c_void_p(t.data_ptr())


class Enlightning:
    """Patch strategy of the reference (enlightning.h:154-430), GPU-backed."""

    def __init__(self, params: dict, variant: str = "hybrid_high_llf", domain_xlo=(0.0, 0.0),
                 domain_xhi=(1.0, 1.0), bc=(REFLECT, REFLECT, REFLECT, REFLECT),
                 rk=(RK3_ALPHA1, RK3_ALPHA2, RK3_BETA)):
        self.p = dict(params)
        self.L = _lib.lib()
        self.variant = VARIANTS.index(variant) if isinstance(variant, str) else int(variant)
        self.domain_xlo = tuple(domain_xlo)
        self.domain_xhi = tuple(domain_xhi)
        self.bc = tuple(int(b) for b in bc)
        self.rk = rk
        _lib.check(self.L.enl_set_rhs_variant(self.variant), "enl_set_rhs_variant")
        self.set_stream(torch.cuda.current_stream())

    def set_stream(self, s):
        _lib.check(self.L.enl_set_stream(C.c_void_p(s.cuda_stream)), "enl_set_stream")

    # -- enlightning::initializeDataOnPatch (enlightning.C:382-430) ---------
    def initialize_ambient(self, P: Patch):
        p = self.p
        P.pres.fill_(p["p0"])
        P.temp.fill_(p["T0"])
        P.w_scr.zero_()
        P.w_scr[0].fill_(p["rho0"])
        P.w_scr[4].fill_(p["rho0"] * p["T0"])
        P.w_cur.copy_(P.interior(P.w_scr))
        P.src.zero_()
        P.src_g.zero_()

    # -- enlightning::computeStableDtOnPatch (enlightning.C:433-456) --------
    def compute_stable_dt(self, P: Patch) -> float:
        dx = P.dx
        dt = self.p["cfl"] * (dx[0] / self.p["c"]) if dx[0] <= dx[1] else self.p["cfl"] * (dx[1] / self.p["c"])
        if self.p.get("specific_dt", 0) > 0:
            dt = self.p["specific_dt"]
        return dt

    # -- enlightning::setPhysicalBoundaryConditions (enlightning.C:790-1013) -
    def set_physical_boundary_conditions(self, P: Patch, fill=None):
        fw = fill if fill is not None else (P.g, P.g)
        b = P.box
        _lib.check(self.L.enl_phys_bc(b[0], b[1], b[2], b[3], P.g, P.g, _lib.iarr(P.touches),
                                      _lib.iarr(self.bc), fw[0], fw[1], _ptr(P.w_scr), _ptr(P.pres),
                                      _ptr(P.temp), _ptr(P.src_g)), "enl_phys_bc")

    # -- enlightning::setAbsorbingBoundaryConditions (enlightning.C:634-786) -
    def set_absorbing_boundary_conditions(self, P: Patch):
        if ABSORB not in self.bc:
            return
        b, p = P.box, self.p
        _lib.check(self.L.enl_absorb(b[0], b[1], b[2], b[3], P.g, P.g, _lib.darr(P.xlo), _lib.darr(P.dx),
                                     _lib.darr(self.domain_xlo), _lib.darr(self.domain_xhi),
                                     _lib.iarr(self.bc), p["bc_absorb_width"], p["p0"], p["T0"], p["rho0"],
                                     _ptr(P.w_scr), _ptr(P.pres), _ptr(P.temp)), "enl_absorb")

    # -- enlightning::singleStep (enlightning.C:459-583) --------------------
    def single_step(self, P: Patch, dt: float, a1: float, a2: float, beta: float):
        L, p, b, g = self.L, self.p, P.box, P.g
        I = _lib.iref
        D = _lib.dref
        L.rhs_(I(b[0]), I(b[1]), I(b[2]), I(b[3]), I(g), I(g), _lib.darr(P.xlo), _lib.darr(P.dx),
               _ptr(P.w_scr), _ptr(P.src), _ptr(P.K), _ptr(P.pres), _ptr(P.temp), D(p["weno_alpha"]),
               D(p["kappa"]), D(p["mu"]), D(p["muB"]), D(p["R"]), D(p["T_star_n"]), D(p["T_star_o"]),
               D(p["tau_n"]), D(p["tau_o"]), _lib.darr(p["tol"]), I(P.level), D(p["c"]), D(p["c_lr"]),
               I(NEQU))
        L.runge_kutta_(I(b[0]), I(b[1]), I(b[2]), I(b[3]), I(g), I(g), D(dt), D(a1), D(a2), D(beta),
                       _ptr(P.w_scr), _ptr(P.w_cur), _ptr(P.K), I(NEQU))
        L.update_state_(_lib.darr(P.dx), _lib.darr(P.xlo), I(b[0]), I(b[1]), I(b[2]), I(b[3]), I(g), I(g),
                        _ptr(P.w_scr), _ptr(P.pres), _ptr(P.temp), D(p["rho0"]), D(p["c"]), D(p["gamma1"]),
                        D(p["c_p"]), D(p["p0"]), D(p["T0"]), D(p["c_lr"]), D(p["c_v"]), D(p["R_tilde"]),
                        D(p["M"]), D(p["R"]), I(NEQU))
        self.set_absorbing_boundary_conditions(P)
        _lib.check_sticky("single_step")

    # -- enlightning::tagGradientDetectorCells (enlightning.C:586-628) ------
    def tag_gradient_detector_cells(self, P: Patch, tags: torch.Tensor, tag_val: int = 1):
        b, g, I = P.box, P.g, _lib.iref
        self.L.tag_cells_(I(b[0]), I(b[1]), I(b[2]), I(b[3]), I(g), I(g), _ptr(tags), _ptr(P.w_scr),
                          _ptr(P.src_g), I(tag_val), _lib.darr(self.p["tol"]), I(NEQU))
        _lib.check_sticky("tag_cells")

    # -- one MOL step of a single-patch hierarchy ---------------------------
    def advance(self, P: Patch, dt: float, nsteps: int = 1):
        a1s, a2s, bs = self.rk
        for _ in range(nsteps):
            P.interior(P.w_scr).copy_(P.w_cur)          # copy current -> scratch
            for s in range(len(a1s)):
                self.set_physical_boundary_conditions(P)
                self.single_step(P, dt, a1s[s], a2s[s], bs[s])
            P.w_cur.copy_(P.interior(P.w_scr))          # copy scratch -> current
