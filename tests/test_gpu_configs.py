"""Parity at the workloads' stated sizes and step counts (GPU).

* The single 512x512 pulse (0.1 p0, sigma 8 cells, dx 0.1 m, reflecting
  walls, CFL 0.5, 200 RK3 steps, hybrid WENO5/DRP with LLF splitting) through
  the drop-in rhs_/runge_kutta_/update_state_ entry points and through the
  batched FP64 engine, each against the oracle (the reference's Fortran
  restated, all host cores): relative L2 <= 1e-12 per conserved field and on
  rho - rho0 and rho T_n - rho0 T0, or ten times the oracle's own
  sensitivity to a one-ulp change of its initial state where that is larger.
* The 64 independent pulses (500 steps), the Mach-1.5 shock (2 levels, 400
  steps) and the 3-level line source (4096 x 2048 base, 1000 steps, regrid
  every 10 steps): the FP64 engine with the
  learned switch, and the FP32-perturbation-storage engine with the learned
  switch, against the FP64 engine with the reference's switch on the same
  cadence: relative L2 <= 1e-3 per field and on the perturbation fields.
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from enlightning_gb300 import sensor, workloads  # noqa: E402
from enlightning_gb300.constants import REFLECT, default_params  # noqa: E402
from enlightning_gb300.engine import PREC_FP32_STATE, PREC_FP64, Engine  # noqa: E402

G = 3
TOL = 1e-12
BUDGET = 1e-3
FIELDS = ("rho", "rho_u", "rho_v", "rho_s", "rho_Tn")


def relL2(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    d = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (d if d > 0 else 1.0))


def field_errors(a, b, prm, mask=None):
    """Relative L2 of state a against b (7 fields), per conserved field and
    on the perturbation fields rho - rho0, rho T_n - rho0 T0, p - p0."""
    if mask is not None:
        a, b = a[:, mask], b[:, mask]
    out = {n: relL2(a[k], b[k]) for k, n in enumerate(FIELDS)}
    out["rho-rho0"] = relL2(a[0] - prm["rho0"], b[0] - prm["rho0"])
    out["rhoTn-rho0T0"] = relL2(a[4] - prm["rho0"] * prm["T0"], b[4] - prm["rho0"] * prm["T0"])
    if a.shape[0] > 5:
        out["p-p0"] = relL2(a[5] - prm["p0"], b[5] - prm["p0"])
    return out


@pytest.fixture(scope="module")
def pulse512(ora):
    """Config-1 initial state and the oracle's state after 200 steps."""
    ora.set_threads(os.cpu_count() or 1)
    prm = default_params()
    n, dx, nsteps = 512, (0.1, 0.1), 200
    dt = workloads.pulse_dt(prm, dx)
    w0 = workloads.pulse_patch_state(n, n, prm, amp_frac=0.1, sigma_cells=8.0)
    box = (0, n - 1, 0, n - 1)
    op = ora.Patch(box, (0.0, 0.0), dx)
    op.w_scr[...] = w0
    op.w_cur[...] = op.interior(w0)
    ora.update_state(dx, (0, 0), box, (G, G), op.w_scr, op.pres, op.temp, prm)
    p0, t0 = op.pres.copy(), op.temp.copy()
    dom = ((0, 0), (n * dx[0], n * dx[1]))
    ora.advance(op, prm, "hybrid_high_llf", dt, nsteps, domain=dom)
    # the reference's own conditioning: the oracle again from an initial state
    # moved by one unit in the last place
    pp = ora.Patch(box, (0.0, 0.0), dx)
    pp.w_scr[...] = np.nextafter(w0, np.inf)
    pp.w_cur[...] = pp.interior(pp.w_scr)
    ora.update_state(dx, (0, 0), box, (G, G), pp.w_scr, pp.pres, pp.temp, prm)
    ora.advance(pp, prm, "hybrid_high_llf", dt, nsteps, domain=dom)
    sens = field_errors(pp.w_cur, op.w_cur, prm)
    return dict(prm=prm, n=n, dx=dx, dt=dt, nsteps=nsteps, w0=w0, p0=p0, t0=t0, ref=op.w_cur.copy(), sens=sens)


def check_against_oracle(errs, sens, what):
    """1e-12 per field, or ten times the reference's own sensitivity to a
    one-ulp change of the initial state where that is larger (rho s: its
    right-hand side is dominated by the conduction term kappa lap(T) / T, and
    T comes from exp and log, whose last-place results differ between any two
    math libraries)."""
    print(what, "errors:", errs)
    print(what, "oracle's own one-ulp sensitivity:", sens)
    for k, e in errs.items():
        assert e <= max(TOL, 10.0 * sens[k]), (k, e, sens[k])


def test_config1_dropin_path_200_steps_matches_oracle(pulse512):
    from enlightning_gb300.strategy import Enlightning, Patch
    c = pulse512
    n, dx, prm = c["n"], c["dx"], c["prm"]
    box = (0, n - 1, 0, n - 1)
    gp = Patch(box, (0.0, 0.0), dx).allocate()
    gp.w_scr.copy_(torch.from_numpy(c["w0"]))
    gp.w_cur.copy_(gp.interior(gp.w_scr))
    gp.pres[0].copy_(torch.from_numpy(c["p0"]))
    gp.temp[0].copy_(torch.from_numpy(c["t0"]))
    Enlightning(prm, domain_xhi=(n * dx[0], n * dx[1])).advance(gp, c["dt"], c["nsteps"])
    torch.cuda.synchronize()
    errs = field_errors(gp.w_cur.cpu().numpy(), c["ref"], prm)
    check_against_oracle(errs, c["sens"], "config 1 drop-in path vs oracle")


def test_config1_fp64_engine_200_steps_matches_oracle(pulse512):
    c = pulse512
    n, dx, prm = c["n"], c["dx"], c["prm"]
    E = Engine(prm, n, n, dx, nlevels=1, bc=(REFLECT,) * 4, precision=PREC_FP64)
    E.set_level_state(0, c["w0"][:, G:-G, G:-G], c["p0"][G:-G, G:-G], c["t0"][G:-G, G:-G])
    E.set_patches(0, [(0, n - 1, 0, n - 1)])
    for _ in range(c["nsteps"]):
        E.step(c["dt"])
    torch.cuda.synchronize()
    assert E.health() == 0
    errs = field_errors(E.level_state(0).cpu().numpy()[0:5], c["ref"], prm)
    E.close()
    check_against_oracle(errs, c["sens"], "config 1 FP64 engine vs oracle")


def _run(E, H, nsteps, dt, regrid_every):
    for s in range(nsteps):
        if H is not None and regrid_every and s and s % regrid_every == 0:
            H.regrid()
        E.step(dt)
    torch.cuda.synchronize()
    assert E.health() == 0


def test_config5_pulses_500_steps_learned_and_fp32_storage_within_budget():
    prm = default_params()
    net = sensor.load_weights()
    states, mask = {}, None
    lv = sensor.weights_levels()
    for key, prec, learned in (("plain", PREC_FP64, False), ("learned", PREC_FP64, lv),
                               ("fp32", PREC_FP32_STATE, lv)):
        E, boxes, info = workloads.pulse_batch(prm, seed=7, n=64, precision=prec, learned=learned)
        if learned:
            E.set_mlp(*net)
        _run(E, None, 500, info["dt"], 0)
        states[key] = E.level_state(0).cpu().numpy()
        if mask is None:
            mask = np.zeros(states[key].shape[1:], bool)
            for b in boxes:
                mask[b[2]:b[3] + 1, b[0]:b[1] + 1] = True
        E.close()
    for key in ("learned", "fp32"):
        errs = field_errors(states[key], states["plain"], prm, mask)
        print("config 5, 500 steps,", key, "vs FP64 reference switch:", errs)
        assert max(errs.values()) <= BUDGET, (key, errs)


def test_config3_line_source_1000_steps_learned_and_fp32_storage_within_budget():
    prm = default_params()
    net = sensor.load_weights()
    states = {}
    lv = sensor.weights_levels()
    for key, prec, learned in (("plain", PREC_FP64, False), ("learned", PREC_FP64, lv),
                               ("fp32", PREC_FP32_STATE, lv)):
        E, H, _ = workloads.line_source(prm, precision=prec, learned=learned)
        if learned:
            E.set_mlp(*net)
        _run(E, H, 1000, 1.0, 10)
        states[key] = E.level_state(0).cpu().numpy()
        E.close()
    for key in ("learned", "fp32"):
        errs = field_errors(states[key], states["plain"], prm)
        print("config 3, 1000 steps,", key, "vs FP64 reference switch:", errs)
        assert max(errs.values()) <= BUDGET, (key, errs)


def test_config2_mach_shock_400_steps_learned_and_fp32_storage_within_budget():
    """The Mach-1.5 shock into 1 % density noise (1024x512 base, 2 levels,
    regrid every 10 steps, device CFL time step) for its 400 steps."""
    prm = default_params()
    net = sensor.load_weights()
    lv = sensor.weights_levels()
    states = {}
    for key, prec, learned in (("plain", PREC_FP64, False), ("learned", PREC_FP64, lv),
                               ("fp32", PREC_FP32_STATE, lv)):
        E, H = workloads.mach_shock(prm, seed=0, precision=prec, learned=learned)
        if learned:
            E.set_mlp(*net)
        _run(E, H, 400, 1.0, 10)
        states[key] = E.level_state(0).cpu().numpy()
        E.close()
    for key in ("learned", "fp32"):
        errs = field_errors(states[key], states["plain"], prm)
        print("config 2, 400 steps,", key, "vs FP64 reference switch:", errs)
        assert max(errs.values()) <= BUDGET, (key, errs)
