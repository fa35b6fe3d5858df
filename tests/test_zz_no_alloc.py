"""The allocation-free time-step entry point (enl_cfl_dt_static) against the
engine's device CFL reduction, through the C-ABI.

enl_cfl_dt_static is for callers that cannot allocate device memory when they
need a time step (device memory owned by a pool allocator or held to a fixed
budget during a step, or code that must not call cudaMalloc/cudaFree because
those can synchronise the device).  It keeps its partial maxima in a static
device array, so this test checks it on two calls in a row, each against the
dt the engine computes with its own cudaMalloc'd scratch for the same state.
The results are compared exactly: both are a maximum over the same cells and
the same final division.  The file sorts last so that a run stopping at the
first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from enlightning_gb300 import _lib, workloads  # noqa: E402
from enlightning_gb300.constants import REFLECT, default_params  # noqa: E402
from enlightning_gb300.engine import PREC_FP64, Engine  # noqa: E402


def _static_dt(L, box, g, w, dx, c, cfl, dt_max, g1=None):
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    fn = L.enl_cfl_dt_static
    fn.restype = C.c_int
    fn.argtypes = [C.c_int] * 6 + [C.c_void_p, C.POINTER(C.c_double), C.c_double, C.c_double, C.c_double,
                                   C.c_void_p]
    st = fn(box[0], box[1], box[2], box[3], g, g if g1 is None else g1, C.c_void_p(w.data_ptr()), _lib.darr(dx),
            c, cfl, dt_max, C.c_void_p(out.data_ptr()))
    _lib.check(st, "enl_cfl_dt_static")
    torch.cuda.synchronize()
    return float(out.item())


def test_static_dt_matches_engine_twice():
    prm = default_params()
    L = _lib.lib()
    nx, ny, dx = 160, 96, (0.1, 0.1)
    E = Engine(prm, nx, ny, dx, nlevels=1, bc=(REFLECT,) * 4, precision=PREC_FP64)
    E.set_patches(0, [(0, nx - 1, 0, ny - 1)])
    dp = workloads.gaussian_dp(nx, ny, 0.3 * prm["p0"], 6.0)
    w = workloads.state_from_dp(dp, prm)
    rng = np.random.default_rng(0)
    w[1] = w[0] * rng.normal(0.0, 40.0, (ny, nx))
    w[2] = w[0] * rng.normal(0.0, 30.0, (ny, nx))
    k = (prm["gamma1"] - 1.0) / (2.0 * prm["rho0"])
    p = prm["c"] ** 2 * ((w[0] - prm["rho0"]) + k * (w[0] - prm["rho0"]) ** 2) + prm["p0"]
    E.set_level_state(0, w, p, w[4] / w[0])
    E.set_adaptive_dt(True, 0.5)
    dt_max = 1.0
    for call in range(2):
        # the patch in SAMRAI layout (3 ghosts), copied from the engine's current state
        buf = E.buffer(0, 0)
        patch = buf[0:5].contiguous()
        torch.cuda.synchronize()
        dt_static = _static_dt(L, (0, nx - 1, 0, ny - 1), 3, patch, dx, prm["c"], 0.5, dt_max)
        E.step(dt_max)
        dt_engine, _ = E.time()
        assert dt_static == dt_engine, (call, dt_static, dt_engine)
        assert 0.0 < dt_static < 0.5 * 0.1 / prm["c"]
    assert E.health() == 0
    E.close()


def test_static_dt_rejects_patches_beyond_its_scratch():
    L = _lib.lib()
    w = torch.zeros((5, 10, 10), dtype=torch.float64, device="cuda")
    fn = L.enl_cfl_dt_static
    fn.restype = C.c_int
    fn.argtypes = [C.c_int] * 6 + [C.c_void_p, C.POINTER(C.c_double), C.c_double, C.c_double, C.c_double,
                                   C.c_void_p]
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    # 2048 x 1024 interior cells = 8192 tiles > 4096: refused before any launch
    st = fn(0, 2047, 0, 1023, 3, 3, C.c_void_p(w.data_ptr()), _lib.darr((0.1, 0.1)), 343.0, 0.5, 1.0,
            C.c_void_p(out.data_ptr()))
    assert st == 1  # ENL_ERR_ARG
    assert L.enl_get_last_error() == 1


def _samrai_patch(nx, ny, g0, g1, seed):
    """A random conserved state in SAMRAI layout (5 fields, ghosts g0 x g1;
    ghost values are garbage the call must not read)."""
    rng = np.random.default_rng(seed)
    w = rng.normal(0.0, 1e3, (5, ny + 2 * g1, nx + 2 * g0))
    rho = 1.2 * (1.0 + 0.3 * rng.random((ny, nx)))
    w[0, g1:g1 + ny, g0:g0 + nx] = rho
    w[1, g1:g1 + ny, g0:g0 + nx] = rho * rng.normal(0.0, 50.0, (ny, nx))
    w[2, g1:g1 + ny, g0:g0 + nx] = rho * rng.normal(0.0, 50.0, (ny, nx))
    return w


def _numpy_dt(w, nx, ny, g0, g1, dx, c, cfl, dt_max):
    r = w[0, g1:g1 + ny, g0:g0 + nx]
    u = np.abs(w[1, g1:g1 + ny, g0:g0 + nx] / r)
    v = np.abs(w[2, g1:g1 + ny, g0:g0 + nx] / r)
    m = float(np.max(np.maximum(u, v) + c))
    return min((cfl * min(dx)) / m, dt_max)


@pytest.mark.parametrize("nx,ny,g0,g1", [(157, 91, 3, 2), (2048, 512, 3, 3), (33, 9, 0, 4)])
def test_static_dt_ragged_tiles_and_uneven_ghosts(nx, ny, g0, g1):
    """Partial tiles, unequal ghost widths and a patch of exactly 4096 tiles
    (2048 x 512), against the same maximum and division in numpy, twice."""
    L = _lib.lib()
    c, cfl, dx, dt_max = 343.0, 0.5, (0.1, 0.07), 1.0
    for call in range(2):
        w = _samrai_patch(nx, ny, g0, g1, seed=call)
        wd = torch.from_numpy(w).cuda()
        got = _static_dt(L, (5, 5 + nx - 1, -2, -2 + ny - 1), g0, wd, dx, c, cfl, dt_max, g1=g1)
        assert got == _numpy_dt(w, nx, ny, g0, g1, dx, c, cfl, dt_max), (call, got)


def test_static_dt_nonfinite_density_gives_nan():
    """A NaN or non-positive density in the interior makes the step NaN; a
    clean state right after gives the exact step again (the shared scratch
    carries nothing over)."""
    L = _lib.lib()
    nx, ny, g, dx = 96, 40, 3, (0.1, 0.1)
    for bad in (float("nan"), 0.0, -1.0):
        w = _samrai_patch(nx, ny, g, g, seed=5)
        w[0, g + 17, g + 60] = bad
        got = _static_dt(L, (0, nx - 1, 0, ny - 1), g, torch.from_numpy(w).cuda(), dx, 343.0, 0.5, 1.0)
        assert np.isnan(got), (bad, got)
        w = _samrai_patch(nx, ny, g, g, seed=6)
        got = _static_dt(L, (0, nx - 1, 0, ny - 1), g, torch.from_numpy(w).cuda(), dx, 343.0, 0.5, 1.0)
        assert got == _numpy_dt(w, nx, ny, g, g, dx, 343.0, 0.5, 1.0)
