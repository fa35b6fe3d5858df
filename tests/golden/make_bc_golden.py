"""Generate tests/golden/enl_bc_golden.npz from the reference's own C++.

Builds the reference's enlightning::setAbsorbingBoundaryConditions
(enlightning.C:634-786) and enlightning::setPhysicalBoundaryConditions
(enlightning.C:790-1013) from its enlightning.C with oracle/ref_bc.py (the
routines' text compiled unchanged against stand-ins for the SAMRAI types), runs
them on the seeded cases of ``cases()`` and stores a SHA-256 digest of every
output array of every case, and the full output arrays of the named cases.

Run it where the reference tree is checked out, giving its root:

    python tests/golden/make_bc_golden.py <reference root>

The fixtures are committed; the tests never read the reference tree.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "enl_bc_golden.npz")

P0, T0, RHO0 = 101325.0, 293.15, 1.2
REFLECT, ABSORB = 10, 20

# Named cases (kept in full): the behaviours the boundary routines are known
# for.  Each is (name, kind, kwargs); kind "absorb" or "phys".
NAMED = [
    # envelope covering part of each row: the row loop stops where the
    # envelope reaches 1 and the `tmp = 0` reset restarts the next row
    ("absorb_left_partial", "absorb", dict(nx=24, ny=6, g=(3, 3), bc=(ABSORB, REFLECT, REFLECT, REFLECT),
                                           width=0.2, dx=(0.1, 0.1), offset=(0.0, 0.0))),
    ("absorb_right_partial", "absorb", dict(nx=24, ny=6, g=(3, 2), bc=(REFLECT, ABSORB, REFLECT, REFLECT),
                                            width=0.2, dx=(0.1, 0.1), offset=(0.0, 0.0))),
    ("absorb_bottom_top", "absorb", dict(nx=7, ny=30, g=(2, 3), bc=(REFLECT, REFLECT, ABSORB, ABSORB),
                                         width=0.2, dx=(0.1, 0.1), offset=(0.0, 0.0))),
    ("absorb_all_sides", "absorb", dict(nx=30, ny=28, g=(3, 3), bc=(ABSORB,) * 4, width=0.2,
                                        dx=(0.1, 0.1), offset=(0.0, 0.0))),
    # a patch away from the absorbing side: the envelope is 1 at its first
    # cell and nothing changes
    ("absorb_far_patch", "absorb", dict(nx=10, ny=8, g=(3, 3), bc=(ABSORB, REFLECT, REFLECT, REFLECT),
                                        width=0.3, dx=(0.1, 0.1), offset=(5.0, 0.0))),
    # one physical side only: the node boxes at both of its corners are filled
    ("phys_left_only", "phys", dict(nx=9, ny=7, g=(3, 3), touches=(1, 0, 0, 0), bc=(REFLECT,) * 4, fw=(3, 3))),
    ("phys_bottom_only", "phys", dict(nx=9, ny=7, g=(3, 3), touches=(0, 0, 1, 0), bc=(REFLECT,) * 4, fw=(3, 3))),
    ("phys_all_sides", "phys", dict(nx=9, ny=7, g=(3, 3), touches=(1, 1, 1, 1), bc=(REFLECT,) * 4, fw=(3, 3))),
    # an absorbing side is filled by copying without the sign change
    ("phys_mixed_types", "phys", dict(nx=8, ny=8, g=(3, 3), touches=(1, 1, 1, 1),
                                      bc=(ABSORB, REFLECT, ABSORB, REFLECT), fw=(3, 3))),
    # filling fewer ghosts than the patch holds
    ("phys_narrow_fill", "phys", dict(nx=6, ny=5, g=(3, 3), touches=(1, 0, 0, 1), bc=(REFLECT,) * 4, fw=(2, 1))),
]
N_RANDOM = 64


def _arrays(rng, nx, ny, g, with_source):
    NX, NY = nx + 2 * g[0], ny + 2 * g[1]
    w = np.empty((5, NY, NX))
    w[0] = RHO0 * (1 + 0.1 * rng.normal(size=(NY, NX)))
    w[1:4] = rng.normal(size=(3, NY, NX)) * np.array([40.0, 40.0, 5.0])[:, None, None]
    w[4] = w[0] * T0 * (1 + 0.01 * rng.normal(size=(NY, NX)))
    pres = P0 * (1 + 0.1 * rng.normal(size=(NY, NX)))
    temp = T0 * (1 + 0.01 * rng.normal(size=(NY, NX)))
    out = [w, pres, temp]
    if with_source:
        out.append(rng.normal(size=(NY, NX)))
    return out


def cases():
    """(name, kind, args, arrays) of every case, inputs regenerated from seeds.

    args for "absorb": (box, g, patch_xlo, dx, grid_xlo, grid_xhi, bc, width);
    for "phys": (box, g, touches, bc, fw)."""
    out = []
    for k, (name, kind, kw) in enumerate(NAMED):
        rng = np.random.default_rng(1000 + k)
        nx, ny, g = kw["nx"], kw["ny"], kw["g"]
        if kind == "absorb":
            dx = np.array(kw["dx"])
            grid_xlo = np.array([0.0, 0.0])
            patch_xlo = grid_xlo + np.array(kw["offset"])
            grid_xhi = patch_xlo + dx * np.array([nx, ny])
            box = (4, 4 + nx - 1, 2, 2 + ny - 1)
            args = (box, g, patch_xlo, dx, grid_xlo, grid_xhi, kw["bc"], kw["width"])
            out.append((name, kind, args, _arrays(rng, nx, ny, g, False)))
        else:
            box = (-3, -3 + nx - 1, 5, 5 + ny - 1)
            args = (box, g, kw["touches"], kw["bc"], kw["fw"])
            out.append((name, kind, args, _arrays(rng, nx, ny, g, True)))
    for k in range(N_RANDOM):
        rng = np.random.default_rng(5000 + k)
        nx, ny = (int(v) for v in rng.integers(1, 20, 2))
        g = tuple(int(v) for v in rng.integers(1, 4, 2))
        i0, j0 = (int(v) for v in rng.integers(-5, 40, 2))
        box = (i0, i0 + nx - 1, j0, j0 + ny - 1)
        bc = tuple(int(v) for v in rng.choice([REFLECT, ABSORB], 4))
        if k % 2 == 0:
            dx = rng.uniform(0.05, 1.0, 2)
            grid_xlo = rng.uniform(-3, 3, 2)
            patch_xlo = grid_xlo + rng.uniform(0, 8, 2) * rng.integers(0, 2, 2)
            grid_xhi = patch_xlo + dx * np.array([nx, ny]) + rng.uniform(0, 8, 2) * rng.integers(0, 2, 2)
            width = float(rng.choice([0.0, 0.5, 2.0, 5.0, 40.0]))
            args = (box, g, patch_xlo, dx, grid_xlo, grid_xhi, bc, width)
            out.append((f"random{k}", "absorb", args, _arrays(rng, nx, ny, g, False)))
        else:
            touches = tuple(int(v) for v in rng.integers(0, 2, 4))
            fw = (int(rng.integers(0, g[0] + 1)), int(rng.integers(0, g[1] + 1)))
            args = (box, g, touches, bc, fw)
            out.append((f"random{k}", "phys", args, _arrays(rng, nx, ny, g, True)))
    return out


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    a = np.ascontiguousarray(a, np.int32)
    return a.ctypes.data_as(C.POINTER(C.c_int)), a


def run(lib, prefix, kind, args, arrays):
    """Run `prefix`_absorb / `prefix`_phys_bc of a ctypes library (the
    reference build "ref" or the oracle "ora") on copies of the arrays."""
    arrs = [np.ascontiguousarray(a.copy()) for a in arrays]
    box, g = args[0], args[1]
    if kind == "absorb":
        _, _, pxlo, dx, gxlo, gxhi, bc, width = args
        bcp, keep = _ip(bc)
        getattr(lib, prefix + "_absorb")(*box, g[0], g[1], _dp(np.asarray(pxlo, np.float64)),
                                         _dp(np.asarray(dx, np.float64)), _dp(np.asarray(gxlo, np.float64)),
                                         _dp(np.asarray(gxhi, np.float64)), bcp, float(width), P0, T0, RHO0,
                                         _dp(arrs[0]), _dp(arrs[1]), _dp(arrs[2]))
    else:
        _, _, touches, bc, fw = args
        tp, keep1 = _ip(touches)
        bcp, keep2 = _ip(bc)
        getattr(lib, prefix + "_phys_bc")(*box, g[0], g[1], tp, bcp, fw[0], fw[1], _dp(arrs[0]), _dp(arrs[1]),
                                          _dp(arrs[2]), _dp(arrs[3]))
    return arrs


def digest(arrs):
    h = hashlib.sha256()
    for a in arrs:
        h.update(np.ascontiguousarray(a, np.float64).tobytes())
    return h.hexdigest()


def main(reference_root):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref_bc
    lib = ref_bc.load(ref_bc.build(reference_root))
    named = {n for n, _, _ in NAMED}
    data = {}
    changed = 0
    for name, kind, args, arrays in cases():
        out = run(lib, "ref", kind, args, arrays)
        changed += any(not np.array_equal(a, b) for a, b in zip(out, arrays))
        data[f"{name}/sha256"] = np.array(digest(out))
        if name in named:
            for k, a in enumerate(out):
                data[f"{name}/out{k}"] = a
    np.savez_compressed(OUT, **data)
    print(f"wrote {OUT}: {len(data)} entries, {changed} cases changed by the routines")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_bc_golden.py <reference root>")
    main(sys.argv[1])
