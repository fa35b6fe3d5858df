"""The CPU oracle against golden vectors produced from the reference's Fortran.

tests/golden/enl_golden.npz was generated by tests/golden/make_golden.py, which
executes fortran/rhs_*.m4, runge_kutta.m4, update_state.m4 and tag_cells.m4 of
the reference through a Fortran-77 subset interpreter.  Every comparison here is
bit-exact.
"""
import numpy as np
import pytest

from enlightning_gb300.constants import VARIANTS, default_params

CASES = ("ambient", "smooth", "shock", "random")
G = 3


def _case(golden, name):
    pre = name + "/"
    box = tuple(int(x) for x in golden[pre + "box"])
    return dict(box=box, xlo=golden[pre + "xlo"], dx=golden[pre + "dx"],
                c_lr=float(golden[pre + "c_lr"]), w=golden[pre + "w"],
                pres=np.ascontiguousarray(golden[pre + "pres"]),
                temp=np.ascontiguousarray(golden[pre + "temp"]), H0g=golden[pre + "H0g"])


def _prm(c_lr):
    return default_params(c_lr=c_lr)


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("variant", VARIANTS)
def test_rhs_bit_exact(golden, ora, case, variant):
    c = _case(golden, case)
    prm = _prm(c["c_lr"])
    H0 = np.ascontiguousarray(c["H0g"][G:-G, G:-G])
    levels = (0, 1) if variant.startswith("hybrid") else (0,)
    for level in levels:
        KK, flags = ora.rhs(variant, c["box"], (G, G), c["xlo"], c["dx"], c["w"], H0, c["pres"],
                            c["temp"], prm, level, flags=True)
        ref = golden[f"{case}/KK/{variant}/L{level}"]
        assert np.array_equal(KK.view(np.uint64), ref.view(np.uint64)), (
            f"{variant} L{level}: {np.sum(KK != ref)} cells differ")
        if variant.startswith("hybrid"):
            assert np.array_equal(flags, golden[f"{case}/flags/{variant}/L{level}"])


@pytest.mark.parametrize("case", CASES)
def test_runge_kutta_update_state_tag_cells_bit_exact(golden, ora, case):
    c = _case(golden, case)
    prm = _prm(c["c_lr"])
    wn = c["w"].copy()
    ww = golden[f"{case}/rk/ww"]
    KK = np.ascontiguousarray(golden[f"{case}/KK/hybrid_high_llf/L0"])
    ora.runge_kutta(c["box"], (G, G), 1.4577e-4, 0.75, 0.25, 0.25, wn, ww, KK)
    assert np.array_equal(wn, golden[f"{case}/rk/w_n"])
    p2, t2 = c["pres"].copy(), c["temp"].copy()
    ora.update_state(c["dx"], c["xlo"], c["box"], (G, G), wn, p2, t2, prm)
    assert np.array_equal(p2, golden[f"{case}/us/pres"])
    assert np.array_equal(t2, golden[f"{case}/us/temp"])
    tags = ora.tag_cells(c["box"], (G, G), c["w"], np.ascontiguousarray(c["H0g"]), prm["tol"])
    assert np.array_equal(tags, golden[f"{case}/tags"])


def test_golden_has_both_switch_outcomes(golden):
    f = golden["shock/flags/hybrid_high_llf/L0"]
    assert 0 < f.mean() < 1
    f = golden["smooth/flags/hybrid_high_llf/L0"]
    assert 0 < f.mean() < 1


def test_f32_literal_switch_changes_results(golden, ora):
    """The REAL*4-literal convention is load-bearing: double literals differ."""
    c = _case(golden, "smooth")
    prm = _prm(c["c_lr"])
    H0 = np.ascontiguousarray(c["H0g"][G:-G, G:-G])
    ora.set_f32_literals(False)
    try:
        KK = ora.rhs("hybrid_high_llf", c["box"], (G, G), c["xlo"], c["dx"], c["w"], H0,
                     c["pres"], c["temp"], prm, 0)
    finally:
        ora.set_f32_literals(True)
    assert not np.array_equal(KK, golden["smooth/KK/hybrid_high_llf/L0"])
