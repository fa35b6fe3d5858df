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


# ---------------------------------------------------------------------------
# The absorbing envelope and the physical-boundary ghost fill against the
# reference's own C++ (enlightning.C:634-1013, compiled unchanged against
# stand-ins for the SAMRAI types by oracle/ref_bc.py; fixtures made by
# tests/golden/make_bc_golden.py).
# ---------------------------------------------------------------------------
def _bc_cases():
    import make_bc_golden
    return make_bc_golden, make_bc_golden.cases()


@pytest.fixture(scope="module")
def bc_golden():
    import os
    return np.load(os.path.join(os.path.dirname(__file__), "golden", "enl_bc_golden.npz"))


def test_absorb_and_phys_bc_bit_exact_against_reference_code(bc_golden, ora):
    mk, cases = _bc_cases()
    L = ora.lib()
    named = {n for n, _, _ in mk.NAMED}
    for name, kind, args, arrays in cases:
        out = mk.run(L, "ora", kind, args, arrays)
        assert mk.digest(out) == str(bc_golden[f"{name}/sha256"]), name
        if name in named:
            for k, a in enumerate(out):
                assert np.array_equal(a.view(np.int64), bc_golden[f"{name}/out{k}"].view(np.int64)), (name, k)


def test_bc_fixture_cases_exercise_the_routines(bc_golden):
    """The named cases change what they are meant to change: the partial
    envelope touches only some columns (the row loop's early stop and the
    `tmp = 0` reset), the far patch is untouched, a one-sided physical patch
    fills both of its corners."""
    mk, cases = _bc_cases()
    by = {n: (k, a, arr) for n, k, a, arr in cases}
    _, args, arr = by["absorb_left_partial"]
    g0, g1 = args[1]
    d = bc_golden["absorb_left_partial/out1"] != arr[1]
    cols = np.nonzero(d.any(axis=0))[0]
    rows = np.nonzero(d.any(axis=1))[0]
    nx = args[0][1] - args[0][0] + 1
    ny = args[0][3] - args[0][2] + 1
    assert cols.min() == g0 and cols.max() < g0 + nx - 1  # stops before the far side
    assert len(rows) == ny                                 # every row restarted
    _, args, arr = by["absorb_far_patch"]
    assert all(np.array_equal(bc_golden[f"absorb_far_patch/out{k}"], arr[k]) for k in range(3))
    _, args, arr = by["phys_left_only"]
    g0, g1 = args[1]
    out = bc_golden["phys_left_only/out1"]
    assert not np.array_equal(out[:g1, :g0], arr[1][:g1, :g0])    # lower-left corner filled
    assert not np.array_equal(out[-g1:, :g0], arr[1][-g1:, :g0])  # upper-left corner filled
    assert np.array_equal(out[:g1, g0:], arr[1][:g1, g0:])        # bottom side untouched


def test_reference_build_matches_oracle_on_fresh_cases(ora):
    """Where the reference's routines were built here (oracle/_ref), run them
    and the oracle on new random cases."""
    import os
    import ref_bc
    if not os.path.exists(ref_bc.LIB):
        pytest.skip("reference boundary routines not built on this machine")
    try:
        R = ref_bc.load()
    except OSError as e:
        pytest.skip(f"reference build not loadable here: {e}")
    mk, _ = _bc_cases()
    L = ora.lib()
    rng = np.random.default_rng(77)
    for k in range(200):
        nx, ny = (int(v) for v in rng.integers(1, 24, 2))
        g = tuple(int(v) for v in rng.integers(1, 4, 2))
        i0, j0 = (int(v) for v in rng.integers(-8, 64, 2))
        box = (i0, i0 + nx - 1, j0, j0 + ny - 1)
        bc = tuple(int(v) for v in rng.choice([10, 20], 4))
        arrays = mk._arrays(rng, nx, ny, g, True)
        if k % 2:
            dx = rng.uniform(0.02, 2.0, 2)
            gxlo = rng.uniform(-5, 5, 2)
            pxlo = gxlo + rng.uniform(0, 10, 2) * rng.integers(0, 2, 2)
            gxhi = pxlo + dx * np.array([nx, ny]) + rng.uniform(0, 10, 2) * rng.integers(0, 2, 2)
            args = (box, g, pxlo, dx, gxlo, gxhi, bc, float(rng.uniform(0.1, 20.0)))
            kind, arrays = "absorb", arrays[:3]
        else:
            touches = tuple(int(v) for v in rng.integers(0, 2, 4))
            fw = (int(rng.integers(0, g[0] + 1)), int(rng.integers(0, g[1] + 1)))
            args, kind = (box, g, touches, bc, fw), "phys"
        a = mk.run(R, "ref", kind, args, arrays)
        b = mk.run(L, "ora", kind, args, arrays)
        assert mk.digest(a) == mk.digest(b), (k, kind, args)


def test_fp64_roofline_operation_counts_match_the_oracle(golden, ora):
    """The FP64 roofline counts the reference algorithm's operations per cell
    (profiles/stage_fp64_flops.json, "algorithmic"): the rhs part must be
    what the oracle's instrumented restatement counts on WENO and DRP cells."""
    import json
    import os
    with open(os.path.join(os.path.dirname(os.path.dirname(__file__)), "profiles", "stage_fp64_flops.json")) as f:
        alg = json.load(f)["algorithmic"]
    seen = {0: set(), 1: set()}
    for case in ("shock", "smooth", "random"):
        c = _case(golden, case)
        prm = _prm(c["c_lr"])
        H0 = np.ascontiguousarray(c["H0g"][G:-G, G:-G])
        _, flags, oc = ora.rhs("hybrid_high_llf", c["box"], (G, G), c["xlo"], c["dx"], c["w"], H0, c["pres"],
                               c["temp"], prm, 0, flags=True, opcounts=True)
        flags = np.asarray(flags).reshape(oc.shape[0], oc.shape[1])
        for f in (0, 1):
            for v in oc[flags == f]:
                seen[f].add(int(v[0] + v[1] + v[2]))
    assert seen[1] == {alg["rhs_weno"]} and seen[0] == {alg["rhs_drp"]}, seen
    assert alg["weno_ops_per_cell"] == alg["rhs_weno"] + alg["runge_kutta"] + alg["update_state"]
    assert alg["drp_ops_per_cell"] == alg["rhs_drp"] + alg["runge_kutta"] + alg["update_state"]
