"""Oracle of the multi-level time advance (test infrastructure only).

The reference leaves the hierarchy to SAMRAI (MethodOfLinesIntegrator with
LINEAR_REFINE / CONSERVATIVE_COARSEN, registered at enlightning.C:259-288),
which is not available.  This module is the written specification that the
GPU engine (enlightning_gb300/csrc/enl_engine.cu) follows, evaluated on the
CPU with the oracle's restated Fortran for every per-patch call:

* each level is one ghosted canvas (3 ghost cells) holding rho, rho*u,
  rho*v, rho*s, rho*T_n, p, T; patches are index boxes into it;
* one RK3 step: copy current -> scratch on the patch interiors; per stage:
  fill the ghosts of every level (coarse-fine cells = cells within Chebyshev
  distance 3 of a patch, inside the domain and not in a patch, interpolated
  bilinearly in cell centres from the coarser level; then the physical band
  by the rule of enlightning.C:790-1013), then rhs on every patch, then
  runge_kutta, update_state and the absorbing envelope on every patch
  (enlightning.C:459-583); copy scratch -> current; average fine cells onto
  the coarse cells under them, finest level first.
* order="samrai": the stage order of SAMRAI's MethodOfLinesIntegrator, which
  main.C:448 drives: per stage the levels go coarsest first, each filling
  its ghosts and then advancing its patches, so that a level's coarse-fine
  ghosts are interpolated from the coarser level's data after that level's
  update in the same stage (with the coarser level's own ghosts rebuilt
  around that data first, as SAMRAI's refine schedule does).
"""
from __future__ import annotations

import numpy as np

import oracle as ora

G = 3
RK = ((1.0, 0.75, 0.3333333333), (0.0, 0.25, 0.6666666667), (1.0, 0.25, 0.6666666667))


class OracleAMR:
    def __init__(self, prm, nx0, ny0, dx0, nlevels=1, ratio=2, xlo=(0.0, 0.0), bc=(ora.REFLECT,) * 4,
                 variant="hybrid_high_llf"):
        self.prm, self.nl, self.r, self.xlo, self.bc, self.variant = prm, nlevels, ratio, xlo, bc, variant
        self.shape = [(nx0 * ratio ** l, ny0 * ratio ** l) for l in range(nlevels)]
        self.dx = [(dx0[0] / ratio ** l, dx0[1] / ratio ** l) for l in range(nlevels)]
        self.cur = [np.zeros((7, ny + 2 * G, nx + 2 * G)) for nx, ny in self.shape]
        self.scr = [np.zeros_like(c) for c in self.cur]
        self.patches = [[] for _ in range(nlevels)]
        self.domain_hi = (xlo[0] + nx0 * dx0[0], xlo[1] + ny0 * dx0[1])

    def interior(self, a, l):
        nx, ny = self.shape[l]
        return a[:, G:G + ny, G:G + nx]

    # -- ghost fill ---------------------------------------------------------
    def halo_mask(self, l):
        from scipy.ndimage import binary_dilation
        nx, ny = self.shape[l]
        m = np.zeros((ny, nx), bool)
        for b in self.patches[l]:
            m[b[2]:b[3] + 1, b[0]:b[1] + 1] = True
        grown = binary_dilation(m, structure=np.ones((3, 3), bool), iterations=3)
        return grown & ~m

    def interp_cells(self, dst, src, l, cells_j, cells_i):
        r = self.r
        xc = (cells_i + 0.5) / r - 0.5
        yc = (cells_j + 0.5) / r - 0.5
        ic, jc = np.floor(xc).astype(int), np.floor(yc).astype(int)
        fx, fy = xc - ic, yc - jc
        for k in range(7):
            C = src[k]
            c00 = C[jc + G, ic + G]
            c10 = C[jc + G, ic + 1 + G]
            c01 = C[jc + 1 + G, ic + G]
            c11 = C[jc + 1 + G, ic + 1 + G]
            lo = (1.0 - fx) * c00 + fx * c10
            hi = (1.0 - fx) * c01 + fx * c11
            dst[k][cells_j + G, cells_i + G] = (1.0 - fy) * lo + fy * hi

    def physbc(self, a, l):
        nx, ny = self.shape[l]
        bcL, bcR, bcB, bcT = self.bc
        R = ora.REFLECT
        for d in range(G):
            a[:, G:G + ny, G - 1 - d] = a[:, G:G + ny, G]
            a[:, G:G + ny, G + nx + d] = a[:, G:G + ny, G + nx - 1]
            if bcL == R:
                a[1, G:G + ny, G - 1 - d] *= -1
            if bcR == R:
                a[1, G:G + ny, G + nx + d] *= -1
        for d in range(G):
            a[:, G - 1 - d, G:G + nx] = a[:, G, G:G + nx]
            a[:, G + ny + d, G:G + nx] = a[:, G + ny - 1, G:G + nx]
            if bcB == R:
                a[2, G - 1 - d, G:G + nx] *= -1
            if bcT == R:
                a[2, G + ny + d, G:G + nx] *= -1
        for xs in (0, 1):
            for ys in (0, 1):
                si = G + nx - 1 if xs else G
                sj = G + ny - 1 if ys else G
                rows = slice(G + ny, G + ny + G) if ys else slice(0, G)
                cols = slice(G + nx, G + nx + G) if xs else slice(0, G)
                v = a[:, sj, si].copy()
                if (bcR if xs else bcL) == R:
                    v[1] = -v[1]
                if (bcT if ys else bcB) == R:
                    v[2] = -v[2]
                a[:, rows, cols] = v[:, None, None]

    def fill(self, bufs, levels=None):
        for l in (range(self.nl) if levels is None else levels):
            if l > 0:
                jj, ii = np.nonzero(self.halo_mask(l))
                self.interp_cells(bufs[l], bufs[l - 1], l, jj, ii)
            self.physbc(bufs[l], l)

    # -- stepping -----------------------------------------------------------
    def _patch_view(self, a, b):
        return a[:, b[2]:b[3] + 1 + 2 * G, b[0]:b[1] + 1 + 2 * G]

    def step(self, dt, order="engine"):
        for l in range(self.nl):
            for b in self.patches[l]:
                self._patch_view(self.scr[l], b)[:, G:-G, G:-G] = self._patch_view(self.cur[l], b)[:, G:-G, G:-G]
        for s in range(3):
            if order == "samrai":
                for l in range(self.nl):
                    if l > 0:
                        # the coarser level's ghosts again, around its
                        # advanced data (SAMRAI's refine schedule rebuilds
                        # the coarse data it interpolates from)
                        self.fill(self.scr, levels=[l - 1])
                    self.fill(self.scr, levels=[l])
                    self._stage(dt, s, [l])
            else:
                self.fill(self.scr)
                self._stage(dt, s, range(self.nl))
        for l in range(self.nl):
            for b in self.patches[l]:
                self._patch_view(self.cur[l], b)[:, G:-G, G:-G] = self._patch_view(self.scr[l], b)[:, G:-G, G:-G]
        self.coarsen()

    def _stage(self, dt, s, levels):
        """Stage s on the patches of `levels`: rhs on every patch first, then
        runge_kutta, update_state and the envelope, in place in the scratch data."""
        prm = self.prm
        KK = {}
        for l in levels:
            for n, b in enumerate(self.patches[l]):
                v = self._patch_view(self.scr[l], b)
                w = np.ascontiguousarray(v[0:5])
                p = np.ascontiguousarray(v[5])
                t = np.ascontiguousarray(v[6])
                nx, ny = b[1] - b[0] + 1, b[3] - b[2] + 1
                xlo = (self.xlo[0] + self.dx[l][0] * b[0], self.xlo[1] + self.dx[l][1] * b[2])
                KK[(l, n)] = ora.rhs(self.variant, b, (G, G), xlo, self.dx[l], w, np.zeros((ny, nx)), p, t, prm, l)
        for l in levels:
            for n, b in enumerate(self.patches[l]):
                v = self._patch_view(self.scr[l], b)
                w = np.ascontiguousarray(v[0:5])
                p = np.ascontiguousarray(v[5])
                t = np.ascontiguousarray(v[6])
                ww = np.ascontiguousarray(self._patch_view(self.cur[l], b)[0:5, G:-G, G:-G])
                ora.runge_kutta(b, (G, G), dt, RK[0][s], RK[1][s], RK[2][s], w, ww, KK[(l, n)])
                xlo = (self.xlo[0] + self.dx[l][0] * b[0], self.xlo[1] + self.dx[l][1] * b[2])
                ora.update_state(self.dx[l], xlo, b, (G, G), w, p, t, prm)
                ora.absorb(b, (G, G), xlo, self.dx[l], self.xlo, self.level_hi(l), self.bc,
                           prm["bc_absorb_width"], prm, w, p, t)
                v[0:5, G:-G, G:-G] = w[:, G:-G, G:-G]
                v[5, G:-G, G:-G] = p[G:-G, G:-G]
                v[6, G:-G, G:-G] = t[G:-G, G:-G]

    def level_hi(self, l):
        nx, ny = self.shape[l]
        return (self.xlo[0] + self.dx[l][0] * nx, self.xlo[1] + self.dx[l][1] * ny)

    def coarsen(self):
        r = self.r
        for l in range(self.nl - 1, 0, -1):
            F, Cc = self.cur[l], self.cur[l - 1]
            for b in self.patches[l]:
                I0, I1, J0, J1 = b[0] // r, (b[1] + 1) // r - 1, b[2] // r, (b[3] + 1) // r - 1
                for J in range(J0, J1 + 1):
                    for I in range(I0, I1 + 1):
                        s = np.zeros(7)
                        for bb in range(r):
                            for aa in range(r):
                                s = s + F[:, J * r + bb + G, I * r + aa + G]
                        Cc[:, J + G, I + G] = s * (1.0 / (r * r))

    def refine_init(self, l, boxes):
        for b in boxes:
            jj, ii = np.mgrid[b[2]:b[3] + 1, b[0]:b[1] + 1]
            self.interp_cells(self.cur[l], self.cur[l - 1], l, jj.ravel(), ii.ravel())
