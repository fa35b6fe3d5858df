"""Batched multi-level engine (GPU) against the oracle's written specification.

* FP64 fused path and plain per-patch path: relative L2 <= 1e-12 per field
  after several RK3 steps, on a single patch (the reference's own
  single-patch semantics) and on a two-level hierarchy (oracle/amr.py);
* graph replay is bit-identical to direct launches;
* the FP32 perturbation-form paths (FP32 right-hand side on FP64 state, and
  FP32 perturbation state throughout) stay within 1e-3 relative L2 of FP64,
  also on the perturbation fields;
* tag_cells over the level canvas is bit-exact.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from enlightning_gb300 import workloads  # noqa: E402
from enlightning_gb300.constants import ABSORB, REFLECT, default_params  # noqa: E402
from enlightning_gb300 import _lib  # noqa: E402
from enlightning_gb300._lib import EnlightningError  # noqa: E402
from enlightning_gb300.engine import PREC_FP32, PREC_FP32_STATE, PREC_FP64, Engine  # noqa: E402

G = 3


def relL2(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    d = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (d if d > 0 else 1.0)


def pulse_level(nx, ny, prm, amp=0.1, sigma=4.0, cx=None, cy=None):
    dp = workloads.gaussian_dp(nx, ny, amp * prm["p0"], sigma, cx, cy)
    w = workloads.state_from_dp(dp, prm)
    import oracle as ora
    pres, temp = np.zeros((ny + 2 * G, nx + 2 * G)), np.zeros((ny + 2 * G, nx + 2 * G))
    wg = np.zeros((5, ny + 2 * G, nx + 2 * G))
    wg[:, G:-G, G:-G] = w
    wg[0][wg[0] == 0] = prm["rho0"]
    ora.update_state((1.0, 1.0), (0.0, 0.0), (0, nx - 1, 0, ny - 1), (G, G), wg, pres, temp, prm)
    return w, pres[G:-G, G:-G].copy(), temp[G:-G, G:-G].copy()


def make_pair(prm, nx, ny, dx, nlevels, patches, bc, variant, precision=PREC_FP64):
    from amr import OracleAMR
    E = Engine(prm, nx, ny, dx, nlevels=nlevels, bc=bc, variant=variant, precision=precision)
    O = OracleAMR(prm, nx, ny, dx, nlevels=nlevels, bc=bc, variant=variant)
    w, p, t = pulse_level(nx, ny, prm, amp=0.2, sigma=3.0, cx=nx * 0.45, cy=ny * 0.5)
    E.set_level_state(0, w, p, t)
    O.cur[0][0:5, G:-G, G:-G] = w
    O.cur[0][5, G:-G, G:-G] = p
    O.cur[0][6, G:-G, G:-G] = t
    for l, boxes in enumerate(patches):
        E.set_patches(l, boxes)
        O.patches[l] = list(boxes)
        if l > 0:
            O.refine_init(l, boxes)
            E.refine_init(l, boxes)
    return E, O


def compare(E, O, l, tol):
    got = E.level_state(l).cpu().numpy()
    ref = O.interior(O.cur[l], l)
    prm = O.prm
    mask = np.zeros(ref.shape[1:], bool)
    for b in O.patches[l]:
        mask[b[2]:b[3] + 1, b[0]:b[1] + 1] = True
    errs = []
    for k in range(7):
        errs.append(relL2(got[k][mask], ref[k][mask]))
    errs.append(relL2(got[0][mask] - prm["rho0"], ref[0][mask] - prm["rho0"]))
    errs.append(relL2(got[5][mask] - prm["p0"], ref[5][mask] - prm["p0"]))
    assert max(errs) <= tol, errs
    return max(errs)


@pytest.mark.parametrize("plain", [False, True])
@pytest.mark.parametrize("variant", ["hybrid_high_llf", "weno_high", "drp"])
def test_single_level_fp64_matches_oracle(ora, variant, plain):
    prm = default_params()
    nx, ny = 64, 48
    E, O = make_pair(prm, nx, ny, (0.1, 0.1), 1, [[(0, 31, 0, 47), (32, 63, 0, 23), (32, 63, 24, 47)]],
                     (REFLECT,) * 4, variant)
    dt = workloads.pulse_dt(prm, (0.1, 0.1))
    for _ in range(8):
        E.step(dt, plain=plain)
        O.step(dt)
    torch.cuda.synchronize()
    assert E.health() == 0
    compare(E, O, 0, 1e-12)


# fine patches away from the sides (the fused step leaves the fine level's
# physical band unfilled: nothing reads it) and touching them (it is filled)
FINE_SETS = {"inside": [(24, 55, 20, 51), (56, 71, 28, 43)],
             "at_sides": [(0, 23, 0, 31), (56, 95, 48, 79)]}


@pytest.mark.parametrize("fine_set", sorted(FINE_SETS))
@pytest.mark.parametrize("plain", [False, True])
def test_two_level_fp64_matches_oracle(ora, plain, fine_set):
    prm = default_params(bc_absorb_width=0.5)
    nx, ny = 48, 40
    fine = FINE_SETS[fine_set]
    E, O = make_pair(prm, nx, ny, (0.1, 0.1), 2, [[(0, 23, 0, 39), (24, 47, 0, 39)], fine],
                     (ABSORB, REFLECT, REFLECT, ABSORB), "hybrid_high_llf")
    dt = workloads.pulse_dt(prm, (0.05, 0.05))
    for _ in range(5):
        E.step(dt, plain=plain)
        O.step(dt)
    torch.cuda.synchronize()
    assert E.health() == 0
    compare(E, O, 0, 1e-12)
    compare(E, O, 1, 1e-12)


def test_graph_replay_bit_identical(ora):
    prm = default_params()
    nx, ny = 64, 64
    res = []
    for use_graph in (False, True):
        E, _ = make_pair(prm, nx, ny, (0.1, 0.1), 2, [[(0, 63, 0, 63)], [(40, 87, 40, 87)]], (REFLECT,) * 4,
                         "hybrid_high_llf")
        dt = workloads.pulse_dt(prm, (0.05, 0.05))
        torch.cuda.synchronize()
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            E.L.enl_set_stream(__import__("ctypes").c_void_p(s.cuda_stream))
            if use_graph:
                E.capture(dt)
                E.replay(6)
            else:
                for _ in range(6):
                    E.step(dt)
        torch.cuda.synchronize()
        res.append([E.level_state(l).cpu().numpy().copy() for l in range(2)])
        E.L.enl_set_stream(__import__("ctypes").c_void_p(torch.cuda.current_stream().cuda_stream))
    for a, b in zip(res[0], res[1]):
        assert np.array_equal(a, b)


def test_fp32_fast_path_within_budget(ora):
    prm = default_params()
    nx, ny = 96, 64
    boxes = [[(0, 47, 0, 63), (48, 95, 0, 63)], [(48, 143, 32, 95)]]
    out = {}
    for prec in (PREC_FP64, PREC_FP32, PREC_FP32_STATE):
        E, O = make_pair(prm, nx, ny, (0.1, 0.1), 2, boxes, (REFLECT,) * 4, "hybrid_high_llf", precision=prec)
        dt = workloads.pulse_dt(prm, (0.05, 0.05))
        for _ in range(20):
            E.step(dt)
        torch.cuda.synchronize()
        assert E.health() == 0
        out[prec] = [E.level_state(l).cpu().numpy().copy() for l in range(2)]
    for prec in (PREC_FP32, PREC_FP32_STATE):
        for l in range(2):
            a, b = out[prec][l], out[PREC_FP64][l]
            m = np.zeros(a.shape[1:], bool)
            for bx in boxes[l]:
                m[bx[2]:bx[3] + 1, bx[0]:bx[1] + 1] = True
            for k in (0, 1, 2, 4):
                assert relL2(a[k][m], b[k][m]) <= 1e-3, (prec, l, k)
            assert relL2(a[0][m] - prm["rho0"], b[0][m] - prm["rho0"]) <= 1e-3, (prec, l)
            assert relL2(a[5][m] - prm["p0"], b[5][m] - prm["p0"]) <= 1e-3, (prec, l)
            assert relL2(a[6][m] - prm["T0"], b[6][m] - prm["T0"]) <= 1e-3, (prec, l)


def test_engine_tag_bit_exact(ora):
    prm = default_params()
    nx, ny = 64, 48
    E, O = make_pair(prm, nx, ny, (0.1, 0.1), 1, [[(0, 63, 0, 47)]], (REFLECT,) * 4, "hybrid_high_llf")
    dt = workloads.pulse_dt(prm, (0.1, 0.1))
    for _ in range(3):
        E.step(dt)
    tags = E.tag(0).cpu().numpy()
    st = E.level_state(0).cpu().numpy()
    buf = E.buffer(0, 0).cpu().numpy()
    h0 = E.buffer(0, 3).cpu().numpy()[0]
    w = np.ascontiguousarray(buf[0:5])
    ref = ora.tag_cells((0, nx - 1, 0, ny - 1), (G, G), w, np.ascontiguousarray(h0), prm["tol"])
    assert np.array_equal(tags, ref)
    assert tags.sum() > 0
    assert st.shape == (7, ny, nx)


def test_engine_tag_bit_exact_near_threshold(ora):
    """The regrid tagging decides each density ratio as the reference's
    division would (tag_cells.m4:58-108) while dividing only ratios near the
    0.9999 threshold: rows of sawtooth densities whose differences (t, k t)
    put the ratio within a few 1e-14 of the threshold on both sides (the
    estimate's window is 2^-44), random rows, and flat rows (zero
    differences), against the oracle."""
    prm = default_params()
    nx, ny = 96, 48
    f32 = lambda x: float(np.float32(x))
    tol = prm["tol"]
    c = f32(0.9999)
    ep1 = ((f32(0.9) * tol[1]) * 1.0) / (1.0 - f32(0.9) * (tol[1] * tol[1]))

    def ratio(t1, t2):
        return (2.0 * abs(t1 * t2) + ep1) / ((t1 * t1 + t2 * t2) + ep1)

    t = 0.05
    lo, hi = 0.5, 1.0  # ratio(t, k t) rises to 1 at k = 1
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        lo, hi = (mid, hi) if ratio(t, mid * t) < c else (lo, mid)
    kstar = 0.5 * (lo + hi)
    rng = np.random.default_rng(5)
    rho = np.empty((ny, nx))
    for j in range(ny):
        if j < 36:
            k = kstar * (1.0 + (j - 18) * 2e-15)
            d = np.where(np.arange(nx) % 2 == 0, t, k * t)
            rho[j] = prm["rho0"] + np.cumsum(d) - d.sum() / 2
        elif j < 44:
            rho[j] = prm["rho0"] * (1.0 + 0.01 * rng.normal(size=nx))
        else:
            rho[j] = prm["rho0"]
    z = np.zeros_like(rho)
    w = np.stack([rho, z, z, z, rho * prm["T0"]])
    E = Engine(prm, nx, ny, (0.1, 0.1), nlevels=1, bc=(REFLECT,) * 4, precision=PREC_FP64)
    E.set_level_state(0, w, np.full_like(rho, prm["p0"]), np.full_like(rho, prm["T0"]))
    E.set_patches(0, [(0, nx - 1, 0, ny - 1)])
    tags = E.tag(0).cpu().numpy()
    buf = E.buffer(0, 0).cpu().numpy()
    h0 = E.buffer(0, 3).cpu().numpy()[0]
    E.close()
    ref = ora.tag_cells((0, nx - 1, 0, ny - 1), (G, G), np.ascontiguousarray(buf[0:5]),
                        np.ascontiguousarray(h0), prm["tol"])
    assert np.array_equal(tags, ref)
    # the rows straddle the threshold: ratios on both sides, many inside the
    # window where only the division decides
    r = buf[0, G:-G, :]
    t1, t2 = r[:, 1:-1] - r[:, :-2], r[:, 2:] - r[:, 1:-1]
    q = (2.0 * np.abs(t1 * t2) + ep1) / ((t1 * t1 + t2 * t2) + ep1)
    near = np.abs(q[:36] / c - 1.0) < 2.0 ** -44
    assert near.sum() > 100
    assert (q[:36][near] < c).any() and (q[:36][near] >= c).any()
    assert 0 < tags[:36].sum() < tags[:36].size


def test_paint_source_matches_oracle(ora):
    """Device source painting (POINT, SINE, LIGHTNING, DRIVEN) vs the oracle
    restatement of enlightning.C:2140-2307."""
    prm = default_params()
    nx, ny, dx = 96, 64, (0.25, 0.25)
    E = Engine(prm, nx, ny, dx, nlevels=1)
    E.set_patches(0, [(0, 47, 0, 63), (48, 95, 0, 63)])
    rng = np.random.default_rng(3)
    segs = workloads.random_walk_channel(rng, nseg=30, start=(12.0, 14.0), heading_deg=-90.0)
    cases = [dict(src_type=10, amp=5e5, spread=0.6, pos=(7.0, 9.0)),
             dict(src_type=10, mode=20, amp=5e5, spread=0.6, pos=(7.0, 9.0), drive=0.37),
             dict(src_type=20, amp=2e5, spread=0.4, pos=(12.0, 8.0), sine_amp=1.5, sine_freq=0.8),
             dict(src_type=30, amp=10 * prm["p0"], spread=workloads.gaussian_spread(0.5), segs=segs)]
    for kw in cases:
        E.buffer(0, 3).zero_()
        E.paint_source(0, **kw)
        torch.cuda.synchronize()
        got = E.buffer(0, 3).cpu().numpy()[0, 3:3 + ny, 3:3 + nx]
        ref = np.zeros((ny, nx))
        ora.paint_source(nx, ny, (0.0, 0.0), dx, ref, **kw)
        assert relL2(got, ref) <= 1e-12, kw["src_type"]
        assert np.abs(ref).max() > 0


def test_pack_roundtrip_and_adaptive_dt(ora):
    prm = default_params()
    nx, ny = 64, 48
    E, _ = make_pair(prm, nx, ny, (0.1, 0.1), 2, [[(0, 63, 0, 47)], [(32, 95, 24, 71)]], (REFLECT,) * 4,
                     "hybrid_high_llf")
    n = E.packed_size()
    host = torch.empty(n, dtype=torch.float64).pin_memory()
    E.download(host)
    torch.cuda.synchronize()
    before = [E.level_state(l).cpu().numpy().copy() for l in range(2)]
    E.buffer(0, 0).zero_()
    E.buffer(1, 0).zero_()
    E.upload(host)
    torch.cuda.synchronize()
    for l in range(2):
        after = E.level_state(l).cpu().numpy()
        for b in E.patches[l]:
            sl = (slice(None), slice(b[2], b[3] + 1), slice(b[0], b[1] + 1))
            assert np.array_equal(after[sl], before[l][sl])
    # device CFL reduction: dt = cfl * finest dx / max(|u|,|v|) + c
    E.buffer(0, 0)[1, 3:3 + ny, 3:3 + nx] += 3.0  # give the flow a speed
    torch.cuda.synchronize()
    st = [E.level_state(l).cpu().numpy() for l in range(2)]
    smax = 0.0
    for l in range(2):
        for b in E.patches[l]:
            r = st[l][0, b[2]:b[3] + 1, b[0]:b[1] + 1]
            u = np.abs(st[l][1, b[2]:b[3] + 1, b[0]:b[1] + 1] / r)
            v = np.abs(st[l][2, b[2]:b[3] + 1, b[0]:b[1] + 1] / r)
            smax = max(smax, max(u.max(), v.max()) + prm["c"])
    E.set_adaptive_dt(True, 0.5)
    E.step(1.0)
    dt, t = E.time()
    assert dt == pytest.approx(0.5 * 0.05 / smax, rel=1e-14)
    assert t == pytest.approx(dt, rel=1e-14)
    assert E.health() == 0


def test_line_source_hierarchy_small():
    """A reduced line-source run: painting, tagging, clustering into three
    levels, regrids, FP32 batched vs FP64 plain within 1e-3."""
    prm = default_params()
    out = {}
    for prec, plain in ((PREC_FP32, False), (PREC_FP32_STATE, False), (PREC_FP64, True)):
        E, H, segs = workloads.line_source(prm, nx0=256, ny0=128, dx0=0.5, nlevels=3, nseg=20, precision=prec,
                                           base_patch=64)
        assert len(E.patches[1]) > 0 and len(E.patches[2]) > 0
        for s in range(12):
            if s and s % 5 == 0:
                H.regrid()
            E.step(1.0, plain=plain)
        torch.cuda.synchronize()
        assert E.health() == 0
        out[prec] = E.level_state(0).cpu().numpy().copy()
    for prec in (PREC_FP32, PREC_FP32_STATE):
        a, b = out[prec], out[PREC_FP64]
        for k in (0, 1, 2, 4, 5):
            assert relL2(a[k], b[k]) <= 1e-3, (prec, k)
        assert relL2(a[0] - prm["rho0"], b[0] - prm["rho0"]) <= 1e-3, prec
        assert relL2(a[5] - prm["p0"], b[5] - prm["p0"]) <= 1e-3, prec


def test_independent_problems_match_single_patch_oracle(ora):
    """Batched independent pulse problems (one engine, one persistent launch
    per stage) equal separate single-patch oracle runs (FP64, 1e-12)."""
    prm = default_params()
    E, boxes, info = workloads.pulse_batch(prm, seed=3, n=3, side_range=(32, 96), precision=PREC_FP64, width=512)
    st0 = E.level_state(0).cpu().numpy().copy()
    for _ in range(6):
        E.step(info["dt"])
    torch.cuda.synchronize()
    assert E.health() == 0
    got = E.level_state(0).cpu().numpy()
    for b in boxes:
        s = b[1] - b[0] + 1
        P = ora.Patch((0, s - 1, 0, s - 1), (0.0, 0.0), (0.1, 0.1))
        v = st0[:, b[2]:b[3] + 1, b[0]:b[1] + 1]
        P.w_scr[:, G:-G, G:-G] = v[0:5]
        P.w_cur[...] = v[0:5]
        P.pres[G:-G, G:-G] = v[5]
        P.temp[G:-G, G:-G] = v[6]
        ora.advance(P, prm, "hybrid_high_llf", info["dt"], 6, domain=((0, 0), (s * 0.1, s * 0.1)))
        for k in range(5):
            assert relL2(got[k, b[2]:b[3] + 1, b[0]:b[1] + 1], P.w_cur[k]) <= 1e-12


def test_fp32_state_storage_roundtrip_and_graph(ora):
    """FP32 perturbation storage: the canvases hold float32 values about the
    ambient state, state I/O converts exactly, the packed exchange moves
    float32, and graph replay equals direct launches bit for bit."""
    prm = default_params()
    nx, ny = 64, 48
    res = []
    for use_graph in (False, True):
        E, _ = make_pair(prm, nx, ny, (0.1, 0.1), 2, [[(0, 63, 0, 47)], [(32, 95, 24, 71)]], (REFLECT,) * 4,
                         "hybrid_high_llf", precision=PREC_FP32_STATE)
        assert E.dtype == torch.float32
        assert E.offsets[0] == prm["rho0"] and E.offsets[5] == prm["p0"] and E.offsets[6] == prm["T0"]
        raw = E.buffer(0, 0)
        st = E.level_state(0)
        assert raw.dtype == torch.float32 and st.dtype == torch.float64
        assert torch.equal(st[0], raw[0, 3:3 + ny, 3:3 + nx].double() + prm["rho0"])
        dt = workloads.pulse_dt(prm, (0.05, 0.05))
        s = torch.cuda.Stream()
        torch.cuda.synchronize()
        with torch.cuda.stream(s):
            E.L.enl_set_stream(__import__("ctypes").c_void_p(s.cuda_stream))
            if use_graph:
                E.capture(dt)
                E.replay(5)
            else:
                for _ in range(5):
                    E.step(dt)
        torch.cuda.synchronize()
        E.L.enl_set_stream(__import__("ctypes").c_void_p(torch.cuda.current_stream().cuda_stream))
        assert E.health() == 0
        res.append([E.buffer(l, 0).cpu().numpy().copy() for l in range(2)])
        # packed exchange in float32
        host = E.packed_host(pin=True)
        assert host.dtype == torch.float32 and host.numel() == E.packed_size()
        E.download(host)
        torch.cuda.synchronize()
        before = [E.level_state(l).cpu().numpy().copy() for l in range(2)]
        E.buffer(0, 0).zero_()
        E.buffer(1, 0).zero_()
        E.upload(host)
        torch.cuda.synchronize()
        for l in range(2):
            after = E.level_state(l).cpu().numpy()
            for b in E.patches[l]:
                sl = (slice(None), slice(b[2], b[3] + 1), slice(b[0], b[1] + 1))
                assert np.array_equal(after[sl], before[l][sl])
        with pytest.raises(EnlightningError):
            E.step(dt, plain=True)  # the plain path needs FP64 storage
        assert _lib.lib().enl_get_last_error() == 5  # ENL_ERR_STATE, consumed here
    for a, b in zip(res[0], res[1]):
        assert np.array_equal(a, b)


def test_fp32_state_refuses_unaligned_patches():
    prm = default_params()
    E = Engine(prm, 64, 32, (0.1, 0.1), nlevels=1, precision=PREC_FP32_STATE)
    with pytest.raises(EnlightningError):
        E.set_patches(0, [(2, 33, 0, 31)])  # x origin not a multiple of 4
    assert _lib.lib().enl_get_last_error() == 1  # ENL_ERR_ARG, consumed here
    E.set_patches(0, [(4, 35, 0, 31)])
    E.close()


def _expected_mics(E, mics, it):
    """The reference's recordAudio rule (enlightning.C:2392-2506) on the
    engine's current state: (iteration, mic, level, patch, p) rows."""
    rows, base = [], 0
    for l in range(E.nlevels):
        st = E.level_state(l).cpu().numpy()
        dx, dy = E.dx(l)
        for q, b in enumerate(E.patches[l]):
            xl, xh = E.xlo[0] + dx * b[0], E.xlo[0] + dx * (b[1] + 1)
            yl, yh = E.xlo[1] + dy * b[2], E.xlo[1] + dy * (b[3] + 1)
            nx, ny = b[1] - b[0] + 1, b[3] - b[2] + 1
            for k, (x, y) in enumerate(mics):
                if x >= xl and x <= xh and y >= yl and y <= yh:
                    i, j = int((x - xl) / dx), int((y - yl) / dy)
                    idx = j * nx + i
                    p = st[5, b[2] + idx // nx, b[0] + idx % nx] if idx < nx * ny else np.nan
                    rows.append((it, k, l, base + q, p))
        base += len(E.patches[l])
    return sorted(rows, key=lambda r: (r[0], r[1], r[2], r[3]))


@pytest.mark.parametrize("precision", [PREC_FP64, PREC_FP32_STATE])
def test_microphones_follow_record_audio(ora, precision):
    prm = default_params()
    nx, ny = 64, 48
    E, _ = make_pair(prm, nx, ny, (0.1, 0.1), 2, [[(0, 31, 0, 47), (32, 63, 0, 47)], [(32, 95, 24, 71)]],
                     (REFLECT,) * 4, "hybrid_high_llf", precision=precision)
    mics = [(1.234, 2.71),   # level 0 only
            (2.5, 3.05),     # inside the fine patch: recorded on both levels
            (3.2, 1.0),      # on the boundary shared by the two level-0 patches
            (6.4, 4.8),      # upper corner of the domain: reads past the patch (NaN)
            (9.0, 9.0)]      # outside every patch
    E.set_mics(mics, capacity=4096, iteration=0)
    dt = workloads.pulse_dt(prm, (0.05, 0.05))
    want = []
    for it in range(1, 4):
        E.step(dt)
        torch.cuda.synchronize()
        want += _expected_mics(E, mics, it)
    got, dropped = E.mic_records()
    assert dropped == 0
    assert len(got) == len(want)
    for g, w in zip(got, want):
        assert (int(g["iteration"]), int(g["mic"]), int(g["level"]), int(g["patch"])) == w[:4]
        if np.isnan(w[4]):
            assert np.isnan(g["p"])
        else:
            assert g["p"] == w[4]
    assert sum(1 for w in want if w[1] == 1) == 2 * 3   # the fine-patch microphone, two levels per step
    assert sum(1 for w in want if w[1] == 2) == 2 * 3   # the shared boundary, two patches per step
    assert not any(w[1] == 4 for w in want)
    # the same sampling inside a captured graph; iterations continue at 4
    s = torch.cuda.Stream()
    torch.cuda.synchronize()
    with torch.cuda.stream(s):
        E.L.enl_set_stream(__import__("ctypes").c_void_p(s.cuda_stream))
        E.capture(dt)
        E.replay(2)
    torch.cuda.synchronize()
    E.L.enl_set_stream(__import__("ctypes").c_void_p(torch.cuda.current_stream().cuda_stream))
    got, _ = E.mic_records()
    assert sorted(set(int(v) for v in got["iteration"])) == [4, 5]  # capture records, replay runs two steps
    E.set_mics([])
    assert E.health() == 0


def test_mic_files_in_reference_format(tmp_path):
    from enlightning_gb300.engine import Engine as _E
    from enlightning_gb300.record import write_mic_files
    rec = np.zeros(3, _E.MIC_DTYPE)
    rec["iteration"] = [1, 1, 2]
    rec["mic"] = [0, 0, 0]
    rec["level"] = [0, 1, 0]
    rec["p"] = [101325.0, 101330.5, np.nan]
    write_mic_files(rec, str(tmp_path), [(0.7, 0.1)], 101325.0, 44100, first_pulse_time=2)
    assert (tmp_path / "mic-1.txt").read_text() == "1 0 1.013250e+05\n1 1 1.013305e+05\n2 0 nan\n"
    assert (tmp_path / "mic-1-info.txt").read_text() == (
        "1\n44100\n(0.7,0.1)\n1 0 1.013250e+05 1.013250e+05\n"
        "1\n44100\n(0.7,0.1)\n1 1 1.013250e+05 1.013305e+05\n")


def _exchange_engine(prm, precision):
    E, _ = make_pair(prm, 96, 64, (0.1, 0.1), 2, [[(0, 47, 0, 63), (48, 95, 0, 63)], [(64, 127, 32, 95)]],
                     (REFLECT,) * 4, "hybrid_high_llf", precision=precision)
    E.set_adaptive_dt(True, 0.5)
    return E


@pytest.mark.parametrize("precision", [PREC_FP64, PREC_FP32_STATE])
def test_pipelined_exchange_matches_sequential(ora, precision):
    """Uploads and downloads run on the engine's copy streams and overlap the
    steps around them.  Alternating two host inputs and two host outputs with
    no synchronisation in between gives, per output, exactly the state that a
    fully synchronised upload -> step -> download of its input gives."""
    prm = default_params()
    E = _exchange_engine(prm, precision)
    ins = [E.state_host(), E.state_host()]
    E.download_state(ins[0])
    E.step(1.0)
    E.download_state(ins[1])
    E.sync()
    expect = []
    for h in ins:
        o = E.state_host()
        E.upload_state(h)
        E.sync()
        E.step(1.0)
        E.download_state(o)
        E.sync()
        expect.append(o.clone())
    assert not torch.equal(expect[0], expect[1])
    outs = [E.state_host(), E.state_host()]
    for k in range(6):
        E.upload_state(ins[k % 2])
        E.step(1.0)
        E.download_state(outs[k % 2])
    E.sync()
    assert E.health() == 0
    for o, x in zip(outs, expect):
        assert torch.equal(o, x)
    E.close()


@pytest.mark.parametrize("precision", [PREC_FP64, PREC_FP32_STATE])
def test_round_trip_through_one_host_buffer(ora, precision):
    """download -> upload of the same host buffer every step (no
    synchronisation): the upload waits for the download it overlaps, so the
    run equals one that never leaves the device.  (The full 7-field state:
    on coarse cells under a fine patch, p and T are averages of the fine
    ones, which the 5-field exchange would recompute from the averaged state.)"""
    prm = default_params()
    E, F = _exchange_engine(prm, precision), _exchange_engine(prm, precision)
    h = E.packed_host()
    for _ in range(4):
        E.step(1.0)
        E.download(h)
        E.upload(h)
        F.step(1.0)
    E.sync()
    F.sync()
    for l in range(2):
        a, b = E.level_state(l).cpu().numpy(), F.level_state(l).cpu().numpy()
        for bx in E.patches[l]:
            sl = (slice(None), slice(bx[2], bx[3] + 1), slice(bx[0], bx[1] + 1))
            assert np.array_equal(a[sl], b[sl])
    E.close()
    F.close()


def test_exchange_refuses_a_small_host_buffer():
    prm = default_params()
    E = _exchange_engine(prm, PREC_FP32_STATE)
    small = torch.empty(E.state_host().numel() - 1, dtype=E.dtype).pin_memory()
    for fn in (E.download_state, E.upload_state):
        with pytest.raises(EnlightningError):
            fn(small)
        assert _lib.lib().enl_get_last_error() == 1  # ENL_ERR_ARG, consumed here
    E.close()


@pytest.mark.parametrize("precision", [PREC_FP64, PREC_FP32_STATE])
def test_state_exchange_recomputes_p_and_t(ora, precision):
    """download_state/upload_state move the 5 conserved fields; p and T come
    back from update_state on the device, equal bit for bit to what a stage
    wrote (single level, reflecting walls: every p, T is update_state of w)."""
    prm = default_params()
    nx, ny = 64, 48
    E, _ = make_pair(prm, nx, ny, (0.1, 0.1), 1, [[(0, 31, 0, 47), (32, 63, 0, 47)]], (REFLECT,) * 4,
                     "hybrid_high_llf", precision=precision)
    for _ in range(2):
        E.step(workloads.pulse_dt(prm, (0.1, 0.1)))
    host = E.state_host()
    assert host.numel() * 7 == E.packed_size() * 5
    E.download_state(host)
    torch.cuda.synchronize()
    before = E.level_state(0).cpu().numpy().copy()
    E.buffer(0, 0).zero_()
    E.upload_state(host)
    torch.cuda.synchronize()
    after = E.level_state(0).cpu().numpy()
    assert np.array_equal(after, before)
    assert E.health() == 0


@pytest.mark.parametrize("variant", ["hybrid_high_llf", "hybrid_high", "hybrid_low_llf", "hybrid_low",
                                     "weno_high_llf", "weno_high", "weno_low_llf", "weno_low", "drp"])
def test_fp32_state_every_variant_within_budget(ora, variant):
    """The FP32 perturbation-storage stage kernel of every scheme against the
    FP64 engine (itself held to the oracle at 1e-12), two levels, 6 steps."""
    prm = default_params()
    nx, ny = 96, 64
    boxes = [[(0, 47, 0, 63), (48, 95, 0, 63)], [(48, 143, 32, 95)]]
    out = {}
    for prec in (PREC_FP64, PREC_FP32_STATE):
        E, _ = make_pair(prm, nx, ny, (0.1, 0.1), 2, boxes, (REFLECT,) * 4, variant, precision=prec)
        dt = workloads.pulse_dt(prm, (0.05, 0.05))
        for _ in range(6):
            E.step(dt)
        torch.cuda.synchronize()
        assert E.health() == 0
        out[prec] = [E.level_state(l).cpu().numpy().copy() for l in range(2)]
        E.close()
    for l in range(2):
        a, b = out[PREC_FP32_STATE][l], out[PREC_FP64][l]
        m = np.zeros(a.shape[1:], bool)
        for bx in boxes[l]:
            m[bx[2]:bx[3] + 1, bx[0]:bx[1] + 1] = True
        assert relL2(a[0][m] - prm["rho0"], b[0][m] - prm["rho0"]) <= 1e-3, (variant, l)
        assert relL2(a[5][m] - prm["p0"], b[5][m] - prm["p0"]) <= 1e-3, (variant, l)
        for k in (1, 2):
            assert relL2(a[k][m], b[k][m]) <= 1e-3, (variant, l, k)


@pytest.mark.parametrize("precision", [PREC_FP64, PREC_FP32_STATE])
def test_restart_roundtrip(ora, tmp_path, precision):
    """save() / load(): a restarted engine continues exactly like the original."""
    prm = default_params()
    nx, ny = 64, 48
    E, _ = make_pair(prm, nx, ny, (0.1, 0.1), 2, [[(0, 31, 0, 47), (32, 63, 0, 47)], [(32, 95, 24, 71)]],
                     (REFLECT,) * 4, "hybrid_high_llf", precision=precision)
    E.set_adaptive_dt(True, 0.5)
    for _ in range(2):
        E.step(1.0)
    path = str(tmp_path / "restart.npz")
    E.save(path, iteration=2)
    F, it = Engine.load(path)
    assert it == 2 and F.patches == E.patches and F.dtype == E.dtype
    F.set_adaptive_dt(True, 0.5)
    for X in (E, F):
        for _ in range(2):
            X.step(1.0)
    torch.cuda.synchronize()
    for l in range(2):
        a, b = E.level_state(l).cpu().numpy(), F.level_state(l).cpu().numpy()
        for bx in E.patches[l]:
            sl = (slice(None), slice(bx[2], bx[3] + 1), slice(bx[0], bx[1] + 1))
            assert np.array_equal(a[sl], b[sl])
    assert E.time() == F.time()
    F.close()


@pytest.mark.parametrize("precision", [PREC_FP64, PREC_FP32_STATE])
def test_native_regrid_equals_host_regrid(precision):
    """enl_engine_regrid (one library call per level) builds the same
    hierarchy, and the same new fine data, as the host-side steps of
    Hierarchy (tag map, nesting, clustering, box difference, refine)."""
    prm = default_params()
    res = []
    for native in (False, True):
        E, H, _ = workloads.line_source(prm, nx0=256, ny0=128, dx0=0.5, nlevels=3, nseg=20, precision=precision,
                                        base_patch=64, native_regrid=native)
        for s in range(8):
            if s and s % 3 == 0:
                H.regrid()
            E.step(1.0)
        torch.cuda.synchronize()
        assert E.health() == 0
        res.append(([list(b) for b in E.patches], [E.level_state(l).cpu().numpy().copy() for l in range(3)]))
        E.close()
    assert res[0][0] == res[1][0]
    assert len(res[0][0][2]) > 0
    for a, b in zip(res[0][1], res[1][1]):
        assert np.array_equal(a, b)


def _block_map(tags, B, buf):
    """Block (bx, by) is set when a tag lies in its cells grown by buf cells
    (clipped to the level): the block map the regrid clusters."""
    ny, nx = tags.shape
    nbx, nby = -(-nx // B), -(-ny // B)
    out = np.zeros((nby, nbx), bool)
    for by in range(nby):
        for bx in range(nbx):
            i0, i1 = max(0, bx * B - buf), min(nx, (bx + 1) * B + buf)
            j0, j1 = max(0, by * B - buf), min(ny, (by + 1) * B + buf)
            out[by, bx] = tags[j0:j1, i0:i1].any()
    return out


@pytest.mark.parametrize("precision", [PREC_FP64, PREC_FP32_STATE])
def test_block_map_matches_tag_map(precision):
    """enl_engine_tag_blocks (two passes, bit masks of blocks up to 8x8 and a
    buffer up to the block size; one windowed scan otherwise) gives the map
    of the level's tag map, ragged edge blocks included."""
    prm = default_params()
    E, H, _ = workloads.line_source(prm, nx0=200, ny0=100, dx0=0.5, nlevels=2, nseg=20, precision=precision,
                                    base_patch=64)
    for _ in range(3):
        E.step(1.0)
    for level in range(2):
        tags = E.tag(level).cpu().numpy() != 0
        assert tags.any() and not tags.all()
        for B, buf in [(4, 2), (4, 0), (4, 4), (2, 1), (8, 3), (8, 8), (3, 2), (1, 1), (16, 2), (4, 5)]:
            got = E.tag_blocks(level, B, buf)
            assert np.array_equal(got, _block_map(tags, B, buf)), (level, B, buf)
    E.close()


@pytest.mark.parametrize("precision", [PREC_FP64, PREC_FP32_STATE])
def test_tables_after_regrids_match_a_fresh_engine(precision):
    """A regrid rebuilds only the tables of the levels it changed and copies
    only those to the device.  After a run with regrids of every level, a
    second engine given the same patches in one pass and the same state steps
    bit-identically, so the kept and rebuilt table entries are exact."""
    import ctypes as C
    prm = default_params()
    kw = dict(nx0=256, ny0=128, dx0=0.5, nlevels=3, nseg=20, precision=precision, base_patch=64,
              native_regrid=True)
    E, H, _ = workloads.line_source(prm, **kw)
    F, _, _ = workloads.line_source(prm, **kw)  # same sources painted on the same first patches
    for s in range(9):
        if s and s % 2 == 0:
            H.regrid()
        E.step(1.0)
    H.regrid()
    for l in range(3):
        F.set_patches(l, E.patches[l])
    assert F.patches == E.patches and all(len(b) > 0 for b in E.patches)
    host = E.packed_host(pin=False)
    E.download(host)
    torch.cuda.synchronize()
    F.upload(host)
    dt, t = E.time()
    _lib.check(F.L.enl_engine_set_time(F.h, C.c_double(dt), C.c_double(t)), "enl_engine_set_time")
    for X in (E, F):
        for _ in range(2):
            X.step(1.0)
    torch.cuda.synchronize()
    assert E.health() == 0 and F.health() == 0
    for l in range(3):
        a, b = E.level_state(l).cpu().numpy(), F.level_state(l).cpu().numpy()
        for bx in E.patches[l]:
            sl = (slice(None), slice(bx[2], bx[3] + 1), slice(bx[0], bx[1] + 1))
            assert np.array_equal(a[sl], b[sl])
    F.close()
    E.close()


def test_line_source_1000_steps_fp32_state_within_budget():
    """Long horizon: the reduced line source (1024x512 base, 3 levels, regrid
    every 10 steps) advanced 1000 RK3 steps in FP32 perturbation storage
    stays within 1e-3 relative L2 of the FP64 engine on the composite level
    0, on every field and on the perturbations rho - rho0 and p - p0, although
    the two runs' finest patches come to differ (their tags differ in the
    last bits)."""
    prm = default_params()
    kw = dict(nx0=1024, ny0=512, nseg=50)
    out = {}
    for prec in (PREC_FP32_STATE, PREC_FP64):
        E, H, _ = workloads.line_source(prm, precision=prec, **kw)
        for s in range(1000):
            if s and s % 10 == 0:
                H.regrid()
            E.step(1.0)
        torch.cuda.synchronize()
        assert E.health() == 0
        out[prec] = E.level_state(0).cpu().numpy().copy()
        E.close()
    a, b = out[PREC_FP32_STATE], out[PREC_FP64]
    for k in range(7):
        assert relL2(a[k], b[k]) <= 1e-3, k
    assert relL2(a[0] - prm["rho0"], b[0] - prm["rho0"]) <= 1e-3
    assert relL2(a[5] - prm["p0"], b[5] - prm["p0"]) <= 1e-3


def test_four_levels_fp32_state_within_budget(ora):
    """The deepest hierarchy the engine takes (ENL_MAX_LEVELS = 4) in FP32
    storage against FP64, with a regrid between steps."""
    prm = default_params()
    out = {}
    for prec in (PREC_FP64, PREC_FP32_STATE):
        E, H, _ = workloads.line_source(prm, nx0=128, ny0=64, dx0=1.0, nlevels=4, nseg=12, precision=prec,
                                        base_patch=64)
        assert all(len(E.patches[l]) > 0 for l in range(4))
        for s in range(6):
            if s == 3:
                H.regrid()
            E.step(1.0)
        torch.cuda.synchronize()
        assert E.health() == 0
        out[prec] = E.level_state(0).cpu().numpy().copy()
        E.close()
    a, b = out[PREC_FP32_STATE], out[PREC_FP64]
    assert relL2(a[0] - prm["rho0"], b[0] - prm["rho0"]) <= 1e-3
    assert relL2(a[5] - prm["p0"], b[5] - prm["p0"]) <= 1e-3


def test_independent_problems_fp32_state_within_budget(ora):
    """Batched independent pulses in FP32 storage against the FP64 engine."""
    prm = default_params()
    out = {}
    for prec in (PREC_FP64, PREC_FP32_STATE):
        E, boxes, info = workloads.pulse_batch(prm, seed=5, n=4, side_range=(32, 128), precision=prec, width=640)
        for _ in range(8):
            E.step(info["dt"])
        torch.cuda.synchronize()
        assert E.health() == 0
        out[prec] = E.level_state(0).cpu().numpy().copy()
        E.close()
    a, b = out[PREC_FP32_STATE], out[PREC_FP64]
    for bx in boxes:
        sl = (slice(bx[2], bx[3] + 1), slice(bx[0], bx[1] + 1))
        assert relL2(a[0][sl] - prm["rho0"], b[0][sl] - prm["rho0"]) <= 1e-3
        assert relL2(a[1][sl], b[1][sl]) <= 1e-3


@pytest.mark.parametrize("precision", [PREC_FP64, PREC_FP32_STATE])
def test_samrai_level_order_matches_oracle(ora, precision):
    """SAMRAI's stage order (each level's coarse-fine ghosts from the coarser
    level already advanced in the same stage, main.C:448) against the
    oracle's restatement of it: FP64 within 1e-12, FP32 storage within 1e-3;
    graph replay bit-identical to direct steps; and the order matters (the
    default order gives other states)."""
    prm = default_params(bc_absorb_width=0.5)
    nx, ny = 48, 40
    fine = FINE_SETS["inside"]
    levels = [[(0, 23, 0, 39), (24, 47, 0, 39)], fine]
    bc = (ABSORB, REFLECT, REFLECT, ABSORB)
    dt = workloads.pulse_dt(prm, (0.05, 0.05))
    E, O = make_pair(prm, nx, ny, (0.1, 0.1), 2, levels, bc, "hybrid_high_llf", precision=precision)
    E.set_level_order(True)
    for _ in range(5):
        E.step(dt)
        O.step(dt, order="samrai")
    torch.cuda.synchronize()
    assert E.health() == 0
    tol = 1e-12 if precision == PREC_FP64 else 1e-3
    compare(E, O, 0, tol)
    compare(E, O, 1, tol)
    if precision != PREC_FP64:
        return
    # graph replay of the per-level launches equals direct steps
    E2, _ = make_pair(prm, nx, ny, (0.1, 0.1), 2, levels, bc, "hybrid_high_llf", precision=precision)
    E2.set_level_order(True)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        E2.L.enl_set_stream(__import__("ctypes").c_void_p(s.cuda_stream))
        E2.capture(dt)
        E2.replay(5)
    torch.cuda.synchronize()
    for l in range(2):
        assert np.array_equal(E2.level_state(l).cpu().numpy(), E.level_state(l).cpu().numpy())
    # the default order differs from SAMRAI's
    E3, O3 = make_pair(prm, nx, ny, (0.1, 0.1), 2, levels, bc, "hybrid_high_llf", precision=precision)
    for _ in range(5):
        E3.step(dt)
    torch.cuda.synchronize()
    a, b = E3.level_state(1).cpu().numpy(), E.level_state(1).cpu().numpy()
    assert relL2(a[0] - prm["rho0"], b[0] - prm["rho0"]) > 1e-10


@pytest.mark.parametrize("case", ["mixed", "tiny"])
def test_cfl_speed_reduction_is_exact(case):
    """The FP64 CFL reduction divides only where a single-precision estimate
    allows the block maximum, and takes c for quotients its exponents show to
    be below a quarter ulp of c; dt must still be the double that dividing
    every cell gives.  "mixed": quotients tied to within 1e-9 at the top,
    zero, tiny and subnormal velocities, both signs; "tiny": every velocity
    at most 1e-12 (zero, subnormal, and around the quarter-ulp bound), so
    the maximum is c plus at most a few ulps.  Two levels each."""
    prm = default_params()
    nx, ny = 160, 96
    rng = np.random.default_rng(11)
    E = Engine(prm, nx, ny, (0.1, 0.1), nlevels=2, bc=(REFLECT,) * 4, precision=PREC_FP64)
    rho = prm["rho0"] * (1.0 + 0.05 * rng.uniform(-1, 1, (ny, nx)))
    tiny = np.array([0.0, 5e-324, 1e-310, 1e-300, 1e-40, 1e-20, 3e-15, 1e-14, 2e-14, 1e-13, 1e-12])
    if case == "mixed":
        u = 40.0 * (1.0 + 1e-9 * rng.uniform(-1, 1, (ny, nx))) * rng.choice([-1.0, 1.0], (ny, nx))
        v = 39.99999 * rng.uniform(-1, 1, (ny, nx))
        u[:, : nx // 3] = 0.0
        v[:, : nx // 3] = 0.0
        u[:, nx // 3: nx // 2] = rng.choice(tiny, (ny, nx // 2 - nx // 3)) * rng.choice([-1.0, 1.0], (ny, nx // 2 - nx // 3))
        v[:, nx // 3: nx // 2] = rng.choice(tiny, (ny, nx // 2 - nx // 3))
    else:
        u = rng.choice(tiny, (ny, nx)) * rng.choice([-1.0, 1.0], (ny, nx)) * rng.uniform(0.5, 1.0, (ny, nx))
        v = rng.choice(tiny, (ny, nx)) * rng.uniform(0.5, 1.0, (ny, nx))
    w = np.stack([rho, rho * u, rho * v, np.zeros_like(rho), rho * prm["T0"]])
    p = np.full_like(rho, prm["p0"])
    T = np.full_like(rho, prm["T0"])
    E.set_level_state(0, w, p, T)
    E.set_patches(0, [(0, 79, 0, 95), (80, 159, 0, 95)])
    fine = [(64, 191, 32, 127)]
    E.set_patches(1, fine)
    E.refine_init(1, fine)
    torch.cuda.synchronize()
    smax = 0.0
    for l in range(2):
        st = E.level_state(l).cpu().numpy()
        for b in E.patches[l]:
            sl = (slice(b[2], b[3] + 1), slice(b[0], b[1] + 1))
            q = np.maximum(np.abs(st[1][sl]), np.abs(st[2][sl])) / np.abs(st[0][sl])
            smax = max(smax, float((q + prm["c"]).max()))
    E.set_adaptive_dt(True, 0.5)
    E.step(1.0)
    dt, _ = E.time()
    assert dt == (0.5 * 0.05) / smax
    E.close()


@pytest.mark.parametrize("precision", [PREC_FP64, PREC_FP32_STATE])
def test_kernel_class_profile(precision):
    """Profile mode 2 times every other kernel of the step by class and
    leaves the results bit for bit as an untimed run; its algorithmic bytes
    follow the hierarchy (coarsening: 7 fields x (4 reads + 1 write) per
    covered coarse cell; CFL maximum: 3 fields per patch cell)."""
    prm = default_params()
    runs = {}
    for mode in (0, 2):
        E, H, _ = workloads.line_source(prm, nx0=256, ny0=128, dx0=0.5, nlevels=3, nseg=20, precision=precision,
                                        base_patch=64)
        E.profile(mode)
        for _ in range(3):
            E.step(1.0)
        torch.cuda.synchronize()
        cls = E.profile_kernels()
        E.profile(False)
        assert E.health() == 0
        runs[mode] = ([E.canvas_state(l) for l in range(3)], cls, [list(p) for p in E.patches],
                      4 if E.dtype == torch.float32 else 8)
        E.close()
    for a, b in zip(runs[0][0], runs[2][0]):
        assert np.array_equal(a, b)
    cls, patches, es = runs[2][1], runs[2][2], runs[2][3]
    assert all(v == (0.0, 0.0, 0) for v in runs[0][1].values())
    cells = [sum((b[1] - b[0] + 1) * (b[3] - b[2] + 1) for b in lv) for lv in patches]
    assert cls["interp"][2] == 3 * 3 * 2 and cls["coarsen"][2] == 3 * 2 and cls["cfl"][2] == 3
    assert cls["physbc"][2] >= 3 * 3
    assert cls["coarsen"][1] == 3 * 7 * es * 5 * (cells[1] + cells[2]) // 4
    assert cls["cfl"][1] == 3 * 3 * es * sum(cells)
    # level 0 covers the domain: its whole band is filled every stage
    assert cls["physbc"][1] >= 3 * 3 * 2 * 7 * es * (6 * (256 + 128) + 36)
    assert cls["interp"][1] > 0
    for k in ("interp", "physbc", "coarsen", "cfl"):
        assert cls[k][0] > 0, k
