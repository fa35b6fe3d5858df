"""Benchmark: RK3 cell-updates/s of Enlightning's per-patch time advance on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload pulse512]

Prints one JSON line (rank 0).  A "step" is one SSP-RK3 time step of the whole
workload (three stages, each: ghost fill, RHS, RK update, update_state,
absorbing envelope).  value = cell-updates/s = advanced interior cells x K /
max-over-ranks device time of the K timed steps.  Inputs are synthetic (see
enlightning_gb300/workloads.py).

--impl reference times the reference's CPU path on this machine's host cores:
the oracle's line-by-line restatement of the Fortran (no Fortran compiler
exists on the GPU machine), all host threads, on a bounded sample of the same
workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "RK3 cell-updates/s on 1 GB300: batched+learned vs plain at <=1e-3 rel L2"
UNIT = "cell-updates/s"
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM = 6800.0
# Algorithmic bytes of the RHS kernel per cell and stage: read w_n (5 fields),
# pressure, temperature, source (8 B each) and write KK (5 fields).
RHS_BYTES_PER_CELL = (5 + 3 + 5) * 8
# Algorithmic bytes per RK3 cell-update with ideal fusion (5 FP64 fields):
# stage 1 reads u^n and writes w1 (80 B), stages 2 and 3 read w, u^n and write
# (120 B each).
STEP_BYTES_PER_CELL = 320
# engine storage/arithmetic modes (include/enlightning_gpu.h ENL_PREC_*)
PREC_NAMES = {0: "fp64", 1: "fp32rhs_fp64state", 2: "fp32state"}
PREC_DTYPE = {0: "f64", 1: "f32 rhs / f64 state", 2: "f32 (perturbation state and rhs)"}
PREC_PATH = {0: "FP64 RHS", 1: "FP32 perturbation RHS on FP64 state",
             2: "FP32 perturbation state and RHS"}


def peaks():
    try:
        with open(PEAKS_FILE) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM, "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------


class Pulse512Plain:
    """Single pulse: one 512x512 patch, Gaussian overpressure 0.1 p0, sigma 8 cells,
    dx = 0.1 m, reflective walls, CFL 0.5, hybrid WENO5/DRP with LLF splitting,
    advanced through the drop-in F77 entry points (plain FP64 path)."""

    name = "pulse512: 1 patch 512x512, hybrid_high_llf, reflect, CFL 0.5"

    def __init__(self, n=512):
        import torch

        from enlightning_gb300 import workloads
        from enlightning_gb300.constants import default_params
        from enlightning_gb300.strategy import Enlightning, Patch

        self.torch = torch
        self.prm = default_params()
        self.n = n
        self.dx = (0.1, 0.1)
        self.dt = workloads.pulse_dt(self.prm, self.dx)
        self.box = (0, n - 1, 0, n - 1)
        self.w0 = workloads.pulse_patch_state(n, n, self.prm, amp_frac=0.1, sigma_cells=8.0)
        self.patch = Patch(self.box, (0.0, 0.0), self.dx).allocate()
        self.strat = Enlightning(self.prm, domain_xhi=(n * self.dx[0], n * self.dx[1]))
        self.reset()
        self.cells = n * n
        self.rhs_events = []

    def reset(self):
        P = self.patch
        P.w_scr.copy_(self.torch.from_numpy(self.w0))
        P.w_cur.copy_(P.interior(P.w_scr))
        # p, T of the initial state (update_state over the interior; the
        # ghosts are filled by the boundary fill of every stage)
        P.pres.fill_(self.prm["p0"])
        P.temp.fill_(self.prm["T0"])
        self._eos()

    def _eos(self):
        from enlightning_gb300 import _lib
        P, p, L = self.patch, self.prm, self.strat.L
        I, D = _lib.iref, _lib.dref
        b = self.box
        L.update_state_(_lib.darr(P.dx), _lib.darr(P.xlo), I(b[0]), I(b[1]), I(b[2]), I(b[3]), I(3), I(3),
                        self.strat_ptr(P.w_scr), self.strat_ptr(P.pres), self.strat_ptr(P.temp), D(p["rho0"]),
                        D(p["c"]), D(p["gamma1"]), D(p["c_p"]), D(p["p0"]), D(p["T0"]), D(p["c_lr"]),
                        D(p["c_v"]), D(p["R_tilde"]), D(p["M"]), D(p["R"]), I(5))

    @staticmethod
    def strat_ptr(t):
        import ctypes as C
        return C.c_void_p(t.data_ptr())

    def launches_per_step(self):
        # per stage: 4 edge + 4 node BC fills, rhs, runge_kutta, update_state
        return 3 * (8 + 3)

    def step(self, timed_rhs=False):
        P, s = self.patch, self.strat
        a1s, a2s, bs = s.rk
        P.interior(P.w_scr).copy_(P.w_cur)
        for st in range(3):
            s.set_physical_boundary_conditions(P)
            self._single_step(P, a1s[st], a2s[st], bs[st], timed_rhs)
        P.w_cur.copy_(P.interior(P.w_scr))

    def _single_step(self, P, a1, a2, beta, timed_rhs):
        torch = self.torch
        s = self.strat
        if not timed_rhs:
            s.single_step(P, self.dt, a1, a2, beta)
            return
        # identical call sequence; the rhs_ launch is bracketed by events
        from enlightning_gb300 import _lib
        L, p, b, g = s.L, s.p, P.box, P.g
        I, D = _lib.iref, _lib.dref
        ptr = self.strat_ptr
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        L.rhs_(I(b[0]), I(b[1]), I(b[2]), I(b[3]), I(g), I(g), _lib.darr(P.xlo), _lib.darr(P.dx),
               ptr(P.w_scr), ptr(P.src), ptr(P.K), ptr(P.pres), ptr(P.temp), D(p["weno_alpha"]), D(p["kappa"]),
               D(p["mu"]), D(p["muB"]), D(p["R"]), D(p["T_star_n"]), D(p["T_star_o"]), D(p["tau_n"]),
               D(p["tau_o"]), _lib.darr(p["tol"]), I(P.level), D(p["c"]), D(p["c_lr"]), I(5))
        e1.record()
        self.rhs_events.append((e0, e1))
        L.runge_kutta_(I(b[0]), I(b[1]), I(b[2]), I(b[3]), I(g), I(g), D(self.dt), D(a1), D(a2), D(beta),
                       ptr(P.w_scr), ptr(P.w_cur), ptr(P.K), I(5))
        L.update_state_(_lib.darr(P.dx), _lib.darr(P.xlo), I(b[0]), I(b[1]), I(b[2]), I(b[3]), I(g), I(g),
                        ptr(P.w_scr), ptr(P.pres), ptr(P.temp), D(p["rho0"]), D(p["c"]), D(p["gamma1"]),
                        D(p["c_p"]), D(p["p0"]), D(p["T0"]), D(p["c_lr"]), D(p["c_v"]), D(p["R_tilde"]),
                        D(p["M"]), D(p["R"]), I(5))
        s.set_absorbing_boundary_conditions(P)

    # host-buffer path: state in pinned host memory, copied in and out each step
    def e2e_setup(self):
        torch = self.torch
        P = self.patch
        self.h_w = torch.empty_like(P.w_cur, device="cpu").pin_memory()
        self.h_p = torch.empty_like(P.pres, device="cpu").pin_memory()
        self.h_t = torch.empty_like(P.temp, device="cpu").pin_memory()
        self.h_w.copy_(P.w_cur)
        self.h_p.copy_(P.pres)
        self.h_t.copy_(P.temp)
        torch.cuda.synchronize()
        return (self.h_w.numel() + self.h_p.numel() + self.h_t.numel()) * 8

    def e2e_step(self):
        P = self.patch
        P.w_cur.copy_(self.h_w, non_blocking=True)
        P.pres.copy_(self.h_p, non_blocking=True)
        P.temp.copy_(self.h_t, non_blocking=True)
        self.step()
        self.h_w.copy_(P.w_cur, non_blocking=True)
        self.h_p.copy_(P.pres, non_blocking=True)
        self.h_t.copy_(P.temp, non_blocking=True)

    def cpu_baseline(self, budget_s=12.0, threads=None):
        """The oracle (restated Fortran) on this host, all threads, whole patch."""
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as ora
        threads = threads or os.cpu_count() or 1
        ora.set_threads(threads)
        n, dx, prm = self.n, self.dx, self.prm
        op = ora.Patch(self.box, (0.0, 0.0), dx)
        op.w_scr[...] = self.w0
        op.w_cur[...] = op.interior(self.w0)
        ora.update_state(dx, (0, 0), self.box, (3, 3), op.w_scr, op.pres, op.temp, prm)
        dom = ((0.0, 0.0), (n * dx[0], n * dx[1]))
        ora.advance(op, prm, "hybrid_high_llf", self.dt, 1, domain=dom)  # warm-up
        steps, t0 = 0, time.perf_counter()
        while True:
            ora.advance(op, prm, "hybrid_high_llf", self.dt, 1, domain=dom)
            steps += 1
            el = time.perf_counter() - t0
            if el >= budget_s or steps >= 400:
                break
        return {"value": self.cells * steps / el, "unit": UNIT, "cores": threads, "kind": "port",
                "sample": f"{steps} RK3 steps of the full 512x512 patch ({el:.1f} s)"}


class LineSource:
    """Thunder-like line source on a 3-level hierarchy.

    4096x2048 base cells, dx = 0.5 m, refinement ratio 2 (finest dx 0.125 m),
    200-segment seeded random-walk channel depositing 10 p0 with sigma 2 base
    cells, ABSORB left/right/top and REFLECT ground, patches of 16..256 cells,
    regrid every 10 steps.  The headline arm is the batched engine (all
    patches of all levels in one persistent FP32-perturbation stage kernel,
    CUDA graph); the plain arm advances the same hierarchy with per-patch
    FP64 rhs / runge_kutta / update_state launches (the drop-in path)."""

    name = ("linesource3L: 4096x2048 base, dx 0.5 m, 3 levels ratio 2, 200-segment channel 10 p0 "
            "sigma 2 cells, hybrid_high_llf, regrid every 10 steps")
    REGRID = 10

    def __init__(self, seed=100, learned=False, scale=1, with_plain=True, precision=2, dense=False, tile_order=0):
        import torch

        from enlightning_gb300 import workloads
        from enlightning_gb300.constants import default_params
        from enlightning_gb300.engine import PREC_FP64

        self.torch = torch
        self.prm = default_params()
        self.learned = learned
        self.precision = precision
        # scale > 1 shrinks the base grid (same dx, smaller domain) for profiling captures
        kw = dict(nx0=4096 // scale, ny0=2048 // scale, nseg=max(20, 200 // scale)) if scale > 1 else {}
        if scale > 1:
            self.name = self.name.replace("4096x2048", f"{4096 // scale}x{2048 // scale}")
        self.fast, self.fast_h, self.segs = workloads.line_source(self.prm, seed=seed, precision=precision,
                                                                  learned=learned, dense=dense, tile_order=tile_order, **kw)
        if learned:
            from enlightning_gb300 import sensor
            P, margin = sensor.load_weights()
            self.fast.set_mlp(P, margin)
        self.plain, self.plain_h = None, None
        if with_plain:
            self.plain, self.plain_h, _ = workloads.line_source(self.prm, seed=seed, precision=PREC_FP64, **kw)
        self.steps_done = {"fast": 0, "plain": 0}
        self.regrid_s = {"fast": 0.0, "plain": 0.0}
        self.regrids = {"fast": 0, "plain": 0}
        self.captures = 0
        self.graph_ok = False
        self.dt_cap = 1.0

    def cells(self, E):
        return E.cells()

    def advance(self, which, nsteps, use_graph=False):
        """nsteps RK3 steps with regrids every REGRID steps; returns cell-updates."""
        E = self.fast if which == "fast" else self.plain
        H = self.fast_h if which == "fast" else self.plain_h
        done = 0
        for _ in range(nsteps):
            if self.REGRID and self.steps_done[which] > 0 and self.steps_done[which] % self.REGRID == 0:
                t0 = time.perf_counter()
                H.regrid()
                self.regrid_s[which] += time.perf_counter() - t0
                self.regrids[which] += 1
                if which == "fast" and not E.graph_valid():
                    self.graph_ok = False
            done += E.cells()
            if which == "fast" and use_graph:
                if not self.graph_ok:
                    E.capture(self.dt_cap)
                    self.captures += 1
                    self.graph_ok = True
                E.replay(1)
            else:
                E.step(self.dt_cap, plain=(which == "plain"))
            self.steps_done[which] += 1
        return done

    def compare(self, a_engine=None, b_engine=None):
        """rel-L2 of the fast arm (or a_engine) against the plain FP64 arm (or
        b_engine) on level 0 (composite)."""
        a = (a_engine or self.fast).level_state(0).cpu().numpy()
        b = (b_engine or self.plain).level_state(0).cpu().numpy()
        p = self.prm
        out = {}
        names = ["rho", "rho_u", "rho_v", "rho_s", "rho_Tn", "p", "T"]
        for k, n in enumerate(names):
            out[n] = float(np.linalg.norm(a[k] - b[k]) / max(np.linalg.norm(b[k]), 1e-300))
        out["rho-rho0"] = float(np.linalg.norm(a[0] - b[0]) / np.linalg.norm(b[0] - p["rho0"]))
        out["p-p0"] = float(np.linalg.norm(a[5] - b[5]) / np.linalg.norm(b[5] - p["p0"]))
        return out

    def cpu_baseline(self, budget_s=12.0, threads=None):
        """The oracle's restated Fortran on a sample of this hierarchy's patches
        (one RK3 step each, all host threads); patches drawn across levels in
        proportion to the levels' cell counts."""
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as ora
        threads = threads or os.cpu_count() or 1
        ora.set_threads(threads)
        E = self.fast
        rng = np.random.default_rng(0)
        cells_l = [sum((b[1] - b[0] + 1) * (b[3] - b[2] + 1) for b in E.patches[l]) for l in range(E.nlevels)]
        tot = float(sum(cells_l))
        sample = []
        for l in range(E.nlevels):
            k = max(1, int(round(12 * cells_l[l] / tot))) if E.patches[l] else 0
            idx = rng.choice(len(E.patches[l]), size=min(k, len(E.patches[l])), replace=False) if k else []
            buf = E.canvas_state(l)
            for q in idx:
                b = E.patches[l][q]
                v = np.ascontiguousarray(buf[:, b[2]:b[3] + 7, b[0]:b[1] + 7])
                sample.append((l, b, v))
        ncell, steps, t0 = 0, 0, time.perf_counter()
        while True:
            for l, b, v in sample:
                dx = E.dx(l)
                P = ora.Patch(b, (E.xlo[0] + dx[0] * b[0], E.xlo[1] + dx[1] * b[2]), dx, level=l,
                              touches=(0, 0, 0, 0))
                P.w_scr[...] = v[0:5]
                P.w_cur[...] = P.interior(v[0:5])
                P.pres[...] = v[5]
                P.temp[...] = v[6]
                ora.advance(P, self.prm, "hybrid_high_llf", 1e-5, 1, bc=(20, 20, 10, 20))
                ncell += P.nx * P.ny
            steps += 1
            el = time.perf_counter() - t0
            if el >= budget_s or steps >= 50:
                break
        return {"value": ncell / el, "unit": UNIT, "cores": threads, "kind": "port",
                "sample": f"{len(sample)} patches ({ncell // steps} cells) across the {E.nlevels} levels x {steps} RK3 "
                          f"steps ({el:.1f} s)"}


class PulseBatch(LineSource):
    """64 independent Gaussian-pulse problems (square sides uniform
    in 128..1024, multiples of 32; amplitude U(0.01, 0.5) p0; sigma U(4, 16)
    cells; dx 0.1 m; reflective walls; dt = cfl dx / c) advanced together: one
    persistent launch per RK stage covers every tile of every problem."""

    name = ("pulses64: 64 independent pulse problems, sides U{128..1024}/32, amp U(0.01,0.5) p0, "
            "sigma U(4,16) cells, dx 0.1 m, reflect, hybrid_high_llf")
    REGRID = 0

    def __init__(self, seed=7, learned=False, scale=1, with_plain=True, precision=2, dense=False, tile_order=0):
        import torch

        from enlightning_gb300 import workloads
        from enlightning_gb300.constants import default_params
        from enlightning_gb300.engine import PREC_FP64

        self.torch = torch
        self.prm = default_params()
        self.learned = learned
        self.precision = precision
        n = 64 // scale
        self.fast, self.boxes, self.info = workloads.pulse_batch(self.prm, seed=seed, n=n, precision=precision,
                                                                 learned=learned, dense=dense, tile_order=tile_order)
        if learned:
            from enlightning_gb300 import sensor
            P, margin = sensor.load_weights()
            self.fast.set_mlp(P, margin)
        self.plain = None
        if with_plain:
            self.plain, _, _ = workloads.pulse_batch(self.prm, seed=seed, n=n, precision=PREC_FP64)
        self.fast_h = self.plain_h = None
        self.steps_done = {"fast": 0, "plain": 0}
        self.regrid_s = {"fast": 0.0, "plain": 0.0}
        self.regrids = {"fast": 0, "plain": 0}
        self.captures = 0
        self.graph_ok = False
        self.dt_cap = self.info["dt"]

    def compare(self, a_engine=None, b_engine=None):
        a = (a_engine or self.fast).level_state(0).cpu().numpy()
        b = (b_engine or self.plain).level_state(0).cpu().numpy()
        m = np.zeros(a.shape[1:], bool)
        for bx in self.boxes:
            m[bx[2]:bx[3] + 1, bx[0]:bx[1] + 1] = True
        p = self.prm
        out = {}
        for k, nme in enumerate(["rho", "rho_u", "rho_v", "rho_s", "rho_Tn", "p", "T"]):
            out[nme] = float(np.linalg.norm(a[k][m] - b[k][m]) / max(np.linalg.norm(b[k][m]), 1e-300))
        out["rho-rho0"] = float(np.linalg.norm(a[0][m] - b[0][m]) / np.linalg.norm(b[0][m] - p["rho0"]))
        out["p-p0"] = float(np.linalg.norm(a[5][m] - b[5][m]) / np.linalg.norm(b[5][m] - p["p0"]))
        return out

    def cpu_baseline(self, budget_s=12.0, threads=None):
        """The oracle on four of the problems (one RK3 step each, all threads)."""
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as ora
        threads = threads or os.cpu_count() or 1
        ora.set_threads(threads)
        buf = self.fast.canvas_state(0)
        sample = []
        for bx in self.boxes[:4]:
            s = bx[1] - bx[0] + 1
            sample.append((s, np.ascontiguousarray(buf[:, bx[2]:bx[3] + 7, bx[0]:bx[1] + 7])))
        ncell, steps, t0 = 0, 0, time.perf_counter()
        while True:
            for s, v in sample:
                P = ora.Patch((0, s - 1, 0, s - 1), (0.0, 0.0), (0.1, 0.1))
                P.w_scr[...] = v[0:5]
                P.w_cur[...] = P.interior(v[0:5])
                P.pres[...] = v[5]
                P.temp[...] = v[6]
                ora.advance(P, self.prm, "hybrid_high_llf", self.dt_cap, 1,
                            domain=((0, 0), (s * 0.1, s * 0.1)))
                ncell += s * s
            steps += 1
            el = time.perf_counter() - t0
            if el >= budget_s or steps >= 50:
                break
        return {"value": ncell / el, "unit": UNIT, "cores": threads, "kind": "port",
                "sample": f"4 of the 64 problems ({ncell // steps} cells) x {steps} RK3 steps ({el:.1f} s)"}


class MachShock(LineSource):
    """Planar Mach 1.5 shock into air with 1 % i.i.d. density noise, 1024x512
    base grid (dx 0.1 m), 2 levels of ratio 2 by tag_cells gradient tagging,
    patches of 32 to 128 cells, regrid every 10 steps, device CFL time step
    (workloads.mach_shock).  The plain switch sends most noisy level-0 cells to
    WENO: the workload on which a learned switch can save work."""

    name = ("mach2L: Mach 1.5 shock into 1% density noise, 1024x512 base, dx 0.1 m, 2 levels ratio 2, "
            "patches 32-128, hybrid_high_llf, regrid every 10 steps")
    REGRID = 10

    def __init__(self, seed=0, learned=False, scale=1, with_plain=True, precision=2, dense=False, tile_order=0):
        import torch

        from enlightning_gb300 import workloads
        from enlightning_gb300.constants import default_params
        from enlightning_gb300.engine import PREC_FP64

        self.torch = torch
        self.prm = default_params()
        self.learned = learned
        self.precision = precision
        kw = dict(nx0=1024 // scale, ny0=512 // scale) if scale > 1 else {}
        self.fast, self.fast_h = workloads.mach_shock(self.prm, seed=seed, precision=precision, learned=learned,
                                                      dense=dense, tile_order=tile_order, **kw)
        if learned:
            from enlightning_gb300 import sensor
            P, margin = sensor.load_weights()
            self.fast.set_mlp(P, margin)
        self.plain, self.plain_h = None, None
        if with_plain:
            self.plain, self.plain_h = workloads.mach_shock(self.prm, seed=seed, precision=PREC_FP64, **kw)
        self.segs = None
        self.steps_done = {"fast": 0, "plain": 0}
        self.regrid_s = {"fast": 0.0, "plain": 0.0}
        self.regrids = {"fast": 0, "plain": 0}
        self.captures = 0
        self.graph_ok = False
        self.dt_cap = 1.0


WORKLOADS = {"pulse512": Pulse512Plain, "linesource": LineSource, "pulses64": PulseBatch, "mach": MachShock}


# ---------------------------------------------------------------------------


def host_cpu_model():
    """The host CPU's model name (/proc/cpuinfo, else lscpu), or the machine type."""
    import platform
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return platform.machine()


def cpu_baseline_with_single_core(wl):
    """The workload's CPU baseline with every host thread, plus the same
    sample on one thread (a shorter window) and the CPU model."""
    cb = wl.cpu_baseline()
    one = wl.cpu_baseline(budget_s=3.0, threads=1)
    cb["value_1core"] = one["value"]
    cb["sample_1core"] = one["sample"]
    cb["cpu_model"] = host_cpu_model()
    return cb


def max_over_ranks(ms, ws, device=None):
    """The slowest rank's time: replicas run the same work, and the job is
    done when the last one is."""
    if ws <= 1:
        return float(ms)
    import torch
    import torch.distributed as dist
    if device is None:
        device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank, ws, ms):
    """Whole-job throughput: every rank processed units_per_rank in ms (the max over ranks)."""
    return units_per_rank * ws / (ms * 1e-3)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def linesource_cpu_sample(seed=100, patch=128):
    """Patches of the line-source initial state built on the CPU (oracle
    painter, enlightning.C:2214-2281): per level (dx 0.5, 0.25, 0.125 m)
    patches centred on the channel, plus ambient level-0 patches, in the mix
    of cells the GPU hierarchy holds (level 0 : 1 : 2 ~ 2 : 1 : 1)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as ora
    from enlightning_gb300 import workloads
    from enlightning_gb300.constants import default_params
    prm = default_params()
    rng = np.random.default_rng(seed)
    nx0, ny0, dx0 = 4096, 2048, 0.5
    segs = workloads.random_walk_channel(rng, nseg=200, start=(0.5 * nx0 * dx0, 0.85 * ny0 * dx0),
                                         heading_deg=-90.0)
    amp, spread = 10.0 * prm["p0"], workloads.gaussian_spread(2.0 * dx0)
    out = []
    plan = [(0, 3, True), (0, 3, False), (1, 3, True), (2, 3, True)]
    for level, count, on_channel in plan:
        dx = dx0 / 2 ** level
        for q in range(count):
            if on_channel:
                sgm = segs[(q + 1) * len(segs) // (count + 1)]
                cx, cy = 0.5 * (sgm[0] + sgm[2]), 0.5 * (sgm[1] + sgm[3])
            else:
                cx, cy = 200.0 + 300.0 * q, 200.0
            i0 = int(cx / dx) - patch // 2
            j0 = int(cy / dx) - patch // 2
            n = patch + 6
            xlo = (dx * (i0 - 3), dx * (j0 - 3))
            H = np.zeros((n, n))
            ora.paint_source(n, n, xlo, (dx, dx), H, 30, amp=amp, spread=spread, segs=segs)
            w = workloads.state_from_dp(H, prm)
            out.append((level, (i0, i0 + patch - 1, j0, j0 + patch - 1), (dx, dx), np.ascontiguousarray(w)))
    return prm, out


def linesource_reference_rate(steps, warmup, threads):
    """The reference's CPU path (the oracle's restated Fortran) on the
    line-source sample, one RK3 step per pass over its patches: the median
    rate of `steps` passes after `warmup`.  The reference arm and the bench
    line's cpu_baseline both report this measurement."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as ora
    ora.set_threads(threads)
    prm, sample = linesource_cpu_sample()
    patches = []
    for level, box, dx, w in sample:
        P = ora.Patch(box, (box[0] * dx[0], box[2] * dx[1]), dx, level=level, touches=(0, 0, 0, 0))
        P.w_scr[...] = w
        P.w_cur[...] = P.interior(w)
        ora.update_state(dx, (0, 0), (box[0] - 3, box[1] + 3, box[2] - 3, box[3] + 3), (0, 0), P.w_scr, P.pres,
                         P.temp, prm)
        patches.append(P)
    dt = 0.5 * 0.125 / 733.0

    def one_pass():
        t0 = time.perf_counter()
        nc = 0
        for P in patches:
            ora.advance(P, prm, "hybrid_high_llf", dt, 1, bc=(20, 20, 10, 20))
            nc += P.nx * P.ny
        return nc, time.perf_counter() - t0

    for _ in range(max(1, warmup)):
        one_pass()
    vals = []
    for _ in range(max(1, steps)):
        nc, el = one_pass()
        vals.append(nc / el)
    cells = sum(P.nx * P.ny for P in patches)
    return {"value": float(np.median(vals)), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{len(patches)} patches of 128x128 ({cells} cells) of the line-source initial state across "
                      f"the 3 levels' resolutions, one RK3 step per pass, median of {max(1, steps)} passes after "
                      f"{max(1, warmup)}"}


def run_reference_linesource(args):
    cb = linesource_reference_rate(args.steps, args.warmup, os.cpu_count() or 1)
    v = cb["value"]
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": dist_env()[0],
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": {"workload": LineSource.name},
            "cpu_baseline": cb, "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    if args.workload == "linesource":
        run_reference_linesource(args)
        return
    wl = WORKLOADS[args.workload]
    # the reference arm needs no GPU: build the workload description only
    obj = wl.__new__(wl)
    from enlightning_gb300 import workloads
    from enlightning_gb300.constants import default_params
    obj.prm = default_params()
    obj.n = 512
    obj.dx = (0.1, 0.1)
    obj.dt = workloads.pulse_dt(obj.prm, obj.dx)
    obj.box = (0, 511, 0, 511)
    obj.w0 = workloads.pulse_patch_state(512, 512, obj.prm, amp_frac=0.1, sigma_cells=8.0)
    obj.cells = 512 * 512
    vals = []
    for _ in range(args.warmup):
        obj.cpu_baseline(budget_s=2.0)
    for _ in range(args.steps):
        vals.append(obj.cpu_baseline(budget_s=6.0))
    v = float(np.median([x["value"] for x in vals]))
    cb = dict(vals[-1])
    cb["value"] = v
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "config": {"workload": obj.name}, "cpu_baseline": cb,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    wl = WORKLOADS[args.workload]()
    hbm_peak, peak_kind = peaks()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()

    for _ in range(max(3, args.warmup)):
        wl.step()
    barrier()
    # timed region: per-step CUDA events, L2 flushed between steps (outside the events)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    wl.rhs_events = []
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            flush.zero_()
            ev[k][0].record()
            wl.step(timed_rhs=True)
            ev[k][1].record()
        barrier()
    ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in ev), ws)
    value = aggregate_rate(wl.cells * args.steps, ws, ms)
    rhs_ms = float(np.mean([a.elapsed_time(b) for a, b in wl.rhs_events]))
    achieved = wl.cells * RHS_BYTES_PER_CELL / (rhs_ms * 1e-3) / 1e9

    # e2e: host buffers in pinned memory, copies inside the timed region
    nbytes = wl.e2e_setup()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    e0.record()
    for _ in range(args.steps):
        wl.e2e_step()
    e1.record()
    barrier()
    e2e_ms = e0.elapsed_time(e1)
    e2e = {"value": wl.cells * args.steps * ws / (e2e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": nbytes,
           "d2h_bytes_per_step": nbytes}
    if rank != 0:
        return
    cb = cpu_baseline_with_single_core(wl) if not args.no_cpu_baseline else None
    traffic = None
    tf = os.path.join(ROOT, "profiles", "rhs_traffic.json")
    if os.path.exists(tf):
        try:
            with open(tf) as f:
                traffic = json.load(f).get(args.workload)
        except Exception:
            traffic = None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": wl.name, "path": "plain FP64, drop-in F77 ABI", "cells": wl.cells,
                   "l2": "flushed between timed steps (512 MB write)", "parallelism": "replicas" if ws > 1 else "1 GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": traffic, "kernel": "rhs_plain_kernel",
                     "peak_kind": peak_kind, "bytes_per_cell": RHS_BYTES_PER_CELL, "kernel_ms": rhs_ms},
        "step_roofline": {"bytes_per_cell_update": STEP_BYTES_PER_CELL,
                          "frac": value * STEP_BYTES_PER_CELL / (hbm_peak * 1e9)},
        "cpu_baseline": cb, "e2e": e2e, "clocks": clk.summary(),
        "gpu_launches": wl.launches_per_step() * args.steps,
    }
    print(json.dumps(line), flush=True)


def fp_peaks():
    """FP64 FMA (TFLOP/s), FP64 division (G/s) and FP32 FMA (TFLOP/s) rates of
    this GPU, measured now by the library (enl_measure_fp_peaks)."""
    import ctypes as C
    from enlightning_gb300 import _lib
    o = (C.c_double * 3)()
    _lib.check(_lib.lib().enl_measure_fp_peaks(o, 3), "enl_measure_fp_peaks")
    return {"fp64_fma_tflops": o[0], "fp64_div_per_s": o[1] * 1e9, "fp32_fma_tflops": o[2]}


def fp64_flops_per_cell(kind="algorithmic"):
    """FP64 operations per computed cell and stage by branch (WENO, DRP):
    "algorithmic" = the reference algorithm's operations (oracle-counted
    rhs plus runge_kutta and update_state, one per + - * /); "implementation"
    = what the stage kernel issues (ncu: 2 per FMA, 1 per add or multiply).
    From profiles/stage_fp64_flops.json."""
    try:
        with open(os.path.join(ROOT, "profiles", "stage_fp64_flops.json")) as f:
            d = json.load(f)
        if kind == "algorithmic":
            a = d["algorithmic"]
            return float(a["weno_ops_per_cell"]), float(a["drp_ops_per_cell"])
        return float(d["weno_flops_per_cell"]), float(d["drp_flops_per_cell"])
    except Exception:
        return None, None


KERNEL_NOTES = {
    "interp": "coarse-fine halo interpolation (bilinear, 7 fields): halo cells written + distinct coarse "
              "cells under their 2x2 stencils read",
    "physbc": "physical ghost band fill (sides a stencil reads): one read and one write per band cell",
    "coarsen": "fine-to-coarse averaging: ratio^2 fine reads + one coarse write per covered coarse cell",
    "cfl": "CFL maximum (speed_kernel + dt_kernel): rho, rho u, rho v of every patch cell read",
}


def other_kernels(cls, steps, hbm_peak, peak_kind):
    """Roofline of every other kernel class of the step from profile mode 2:
    algorithmic bytes per launch over its event-timed duration."""
    out = {}
    for k, (ms, by, n) in cls.items():
        if n == 0 or k not in KERNEL_NOTES:
            continue
        gbs = by / (ms * 1e-3) / 1e9 if ms > 0 else None
        out[k] = {"launches_per_step": n / steps, "ms_per_step": ms / steps, "ms_per_launch": ms / n,
                  "bytes_per_launch": by / n, "achieved": gbs, "peak": hbm_peak, "unit": "GB/s",
                  "frac": None if gbs is None else gbs / hbm_peak, "bound": "hbm", "peak_kind": peak_kind,
                  "bytes": KERNEL_NOTES[k]}
    return out


def host_copy_rates(nbytes, reps=3):
    """GB/s of one pinned-host <-> device copy of `nbytes` on a side stream
    (best of `reps`), each direction alone and both at once: what the e2e
    leg's exchange has to hide behind the steps on this machine."""
    import torch
    h_in = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    h_out = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    d_in = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    d_out = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    s_up, s_down = torch.cuda.Stream(), torch.cuda.Stream()

    def timed(h2d, d2h):
        best = None
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            if h2d:
                with torch.cuda.stream(s_up):
                    d_in.copy_(h_in, non_blocking=True)
            if d2h:
                with torch.cuda.stream(s_down):
                    h_out.copy_(d_out, non_blocking=True)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
        return best

    out = {"bytes": nbytes, "h2d": nbytes / timed(True, False) / 1e9, "d2h": nbytes / timed(False, True) / 1e9}
    both = timed(True, True)
    out["both_directions_each"] = nbytes / both / 1e9
    del h_in, h_out, d_in, d_out
    return out


def stage_timing(wl, which="fast", steps=3):
    """Stage-kernel launches of `steps` direct steps timed with CUDA events on
    the engine's stream: (ms per launch, cells per launch, counters,
    launches, {kernel class: (ms, algorithmic bytes, launches)} of the other
    kernels of those steps)."""
    E = wl.fast if which == "fast" else wl.plain
    E.stats()
    E.profile(2)
    wl.advance(which, steps, use_graph=False)
    cls = E.profile_kernels()
    kms, kl, kcells = E.profile(False)
    st = E.stats()
    return kms / max(1, kl), kcells / max(1, kl), st, max(1, kl), cls


def run_stats_only(args):
    """`args.steps` direct steps of the batched engine (no timing, no other
    arm), then the engine's counters summed over those steps: the companion
    of an ncu capture of the same command (FP64 instruction counts per cell
    in profiles/)."""
    import torch
    torch.cuda.set_device(0)
    torch.cuda.set_stream(torch.cuda.Stream())
    wl = WORKLOADS[args.workload](learned=args.learned, scale=args.scale, with_plain=False,
                                  precision=args.precision, dense=args.dense, tile_order=args.tile_order)
    wl.fast.stats()
    wl.advance("fast", args.steps, use_graph=False)
    torch.cuda.synchronize()
    st = wl.fast.stats()
    print(json.dumps({"workload": wl.name, "precision": PREC_NAMES[args.precision], "dense": bool(args.dense),
                      "steps": args.steps, "stage_launches": 3 * args.steps,
                      "weno_cells": int(st[:, 0].sum()), "cells": int(st[:, 1].sum()),
                      "uniform_cells": int(st[:, 3].sum())}), flush=True)


def extra_records(args, fpk):
    """Short runs of the other workloads, reported beside the line source:
    the 64 independent pulses and the Mach-1.5 shock (FP64 batched engine
    with the metric's switch, against the plain per-patch FP64 arm from the
    same state) and the single 512x512 pulse through the drop-in entry
    points.  Each: rate over `steps` graph-replayed steps, the stage kernel's
    FP64 roofline, and the relative L2 difference from the plain arm after
    a few matched steps (the full-horizon parity of these workloads is in the
    GPU tests)."""
    import torch
    out = {}
    f_weno, f_drp = fp64_flops_per_cell("algorithmic")
    steps, ncmp = 10, 4
    for name in ("pulses64", "mach"):
        t0 = time.perf_counter()
        wl = WORKLOADS[name](learned=args.learned, precision=0)
        tune = tune_schedule(wl, args.schedule_cache)
        wl.advance("fast", ncmp, use_graph=True)
        wl.advance("plain", ncmp)
        torch.cuda.synchronize()
        err = wl.compare()
        wl.advance("fast", 3, use_graph=True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        cu = wl.advance("fast", steps, use_graph=True)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        kms, kcells, kst, nl, _ = stage_timing(wl)
        dense = float(kst[:, 1].sum() - kst[:, 3].sum()) / nl
        weno = float(kst[:, 0].sum()) / nl
        flops = weno * f_weno + max(0.0, dense - weno) * f_drp if f_weno else None
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record()
        cup = wl.advance("plain", 2)
        p1.record()
        torch.cuda.synchronize()
        st_w = kst[:, 0].sum() / max(1, kst[:, 1].sum())
        out[name] = {"workload": wl.name, "dtype": "f64", "value": cu / (ms * 1e-3), "unit": UNIT,
                     "ms_per_step": ms / steps, "steps": steps, "cells_per_step": cu / steps,
                     "plain_value": cup / (p0.elapsed_time(p1) * 1e-3),
                     "rel_l2_vs_plain_fp64": err, "compare_steps": ncmp,
                     "weno_fraction": float(st_w), "schedule": tune["chosen"],
                     "stage_kernel_ms": kms,
                     "fp64_roofline": {"achieved": None if flops is None else flops / (kms * 1e-3) / 1e12,
                                       "peak": fpk["fp64_fma_tflops"], "unit": "TFLOP/s",
                                       "frac": None if flops is None else flops / (kms * 1e-3) / 1e12
                                       / fpk["fp64_fma_tflops"]},
                     "wall_s": time.perf_counter() - t0}
        wl.fast.close()
        wl.plain.close()
        del wl
    # the single pulse through the drop-in rhs_ / runge_kutta_ / update_state_
    wl = Pulse512Plain()
    for _ in range(3):
        wl.step()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(steps):
        wl.step()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    out["pulse512"] = {"workload": wl.name, "dtype": "f64", "path": "drop-in F77 entry points, per patch",
                       "value": wl.cells * steps / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms / steps,
                       "steps": steps,
                       "parity": "200 steps within 1e-12 of the oracle (rho s within ten times the oracle's own "
                                 "one-ulp sensitivity), tests/test_gpu_configs.py"}
    return out


def tune_schedule(wl, cache):
    """Autotune the stage kernel's schedule of a workload's fast engine
    (cached by workload signature); returns what the bench line reports."""
    t0 = time.perf_counter()
    res = wl.fast.autotune(wl.dt_cap, steps=3, cache=cache)
    wl.graph_ok = False  # a new schedule needs a new graph
    out = {"chosen": {k: res["schedule"][k] for k in wl.fast.SCHEDULE_KEYS}, "source": res["source"],
           "signature": res["signature"], "tune_s": time.perf_counter() - t0}
    if res["table"]:
        ms = sorted(res["table"], key=lambda r: r[1])
        out["candidates"] = len(ms)
        out["fastest_ms_per_step"] = ms[0][1]
        out["slowest_ms_per_step"] = ms[-1][1]
        dflt = [t for sc, t in ms if sc["tile_order"] == 0 and sc["reuse"] == 2 and sc["run"] == 1
                and sc["blocks_per_sm"] == res["schedule"]["max_blocks_per_sm"]]
        out["default_ms_per_step"] = dflt[0] if dflt else None
    return out


def run_linesource(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    # one non-default stream for torch and the library (graph capture needs it)
    torch.cuda.set_stream(torch.cuda.Stream())
    hbm_peak, peak_kind = peaks()
    t_build = time.perf_counter()
    cls = WORKLOADS[args.workload]
    wl = cls(learned=args.learned, scale=args.scale, with_plain=not args.no_plain, precision=args.precision,
             dense=args.dense, tile_order=args.tile_order)
    # the FP32-perturbation-storage engine on the same workload, reported beside
    # the FP64 headline (same switch, its own error against the plain arm)
    wl32 = None
    if args.precision == 0 and not args.no_secondary:
        wl32 = cls(learned=args.learned, scale=args.scale, with_plain=False, precision=2, dense=args.dense,
                   tile_order=args.tile_order)
    for w_ in (wl, wl32):
        if w_ is not None and args.regrid_every is not None and w_.REGRID:
            w_.REGRID = args.regrid_every
    esize = 4 if args.precision == 2 else 8
    t_build = time.perf_counter() - t_build

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()

    # accuracy: every arm from the same initial state, same regrid cadence
    ncmp = args.compare_steps
    err, err32, err32_fp64 = None, None, None
    if wl.plain is not None or wl32 is not None:
        wl.advance("fast", ncmp, use_graph=True)
        if wl32 is not None:
            wl32.advance("fast", ncmp, use_graph=True)
            barrier()
            err32_fp64 = wl.compare(wl32.fast, wl.fast)
        if wl.plain is not None:
            wl.advance("plain", ncmp)
            barrier()
            err = wl.compare()
            if wl32 is not None:
                err32 = wl.compare(wl32.fast, wl.plain)
    # the stage kernel's schedule for this workload: stored under the
    # workload's signature, or picked by the library's tuner (which leaves the
    # state where it was); untimed
    tune, tune32 = None, None
    if not args.no_autotune:
        tune = tune_schedule(wl, args.schedule_cache)
        if wl32 is not None:
            tune32 = tune_schedule(wl32, args.schedule_cache)
    # warm-up, then the timed region (graph replay, regrids included)
    wl.advance("fast", max(3, args.warmup), use_graph=True)
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    wl.fast.stats()
    rg0, rn0, cap0 = wl.regrid_s["fast"], wl.regrids["fast"], wl.captures
    ph0 = dict(wl.fast_h.timing) if wl.fast_h is not None else {}
    with ClockSampler(local) as clk:
        e0.record()
        cu = wl.advance("fast", args.steps, use_graph=True)
        e1.record()
        barrier()
    ms = max_over_ranks(e0.elapsed_time(e1), ws)
    value = aggregate_rate(cu, ws, ms)
    regrid_info = {"regrids": wl.regrids["fast"] - rn0, "host_ms": 1e3 * (wl.regrid_s["fast"] - rg0),
                   "graph_captures": wl.captures - cap0}
    if wl.fast_h is not None:
        regrid_info["phases_ms"] = {k: 1e3 * (v - ph0.get(k, 0.0)) for k, v in wl.fast_h.timing.items()}
    st = wl.fast.stats()
    weno_frac = {f"L{l}": float(st[l, 0] / max(1, st[l, 1])) for l in range(st.shape[0])}
    weno_frac["all"] = float(st[:, 0].sum() / max(1, st[:, 1].sum()))
    uniform_frac = float(st[:, 3].sum() / max(1, st[:, 1].sum()))
    launches = wl.fast.launches_per_step() * args.steps
    # plain arm (per-patch FP64 launches, same hierarchy logic)
    kp = max(1, min(args.steps, args.plain_steps))
    plain_value = None
    if wl.plain is not None:
        barrier()
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record()
        cup = wl.advance("plain", kp)
        p1.record()
        barrier()
        plain_value = cup / (p0.elapsed_time(p1) * 1e-3)
    # dominant kernel: the stage kernel, timed with events around each launch
    per_launch_ms, cells_per_launch, kst, nl, kcls = stage_timing(wl)
    # 320 B per RK3 cell-update of 5 FP64 fields (106.7 B per stage launch);
    # FP32 storage moves half of it
    bytes_per_cell_launch = STEP_BYTES_PER_CELL / 3.0 * esize / 8.0
    hbm_achieved = cells_per_launch * bytes_per_cell_launch / (per_launch_ms * 1e-3) / 1e9
    traffic = None
    tf = os.path.join(ROOT, "profiles", "stage_traffic.json")
    if os.path.exists(tf):
        try:
            with open(tf) as f:
                rec = json.load(f).get(PREC_NAMES[args.precision])
            if rec:
                traffic = rec["dram_bytes_per_cell_launch"] * cells_per_launch
        except Exception:
            traffic = None
    hbm = {"achieved": hbm_achieved, "peak": hbm_peak, "unit": "GB/s", "frac": hbm_achieved / hbm_peak,
           "peak_kind": peak_kind, "bytes_per_cell_launch": bytes_per_cell_launch, "traffic": traffic}
    fpk = fp_peaks()
    roof = {"kernel": "stage_kernel (" + PREC_NAMES[args.precision] + ")", "kernel_ms": per_launch_ms,
            "cells_per_launch": cells_per_launch}
    if args.precision == 0:
        f_weno, f_drp = fp64_flops_per_cell("algorithmic")
        i_weno, i_drp = fp64_flops_per_cell("implementation")
        dense_cells = float(kst[:, 1].sum() - kst[:, 3].sum()) / nl
        weno_cells = float(kst[:, 0].sum()) / nl
        flops = None if f_weno is None else weno_cells * f_weno + max(0.0, dense_cells - weno_cells) * f_drp
        iflops = None if i_weno is None else weno_cells * i_weno + max(0.0, dense_cells - weno_cells) * i_drp
        fp64_achieved = None if flops is None else flops / (per_launch_ms * 1e-3) / 1e12
        fp64_peak = fpk["fp64_fma_tflops"]
        roof.update({"bound": "fp64", "achieved": fp64_achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                     "frac": None if fp64_achieved is None else fp64_achieved / fp64_peak,
                     "peak_kind": "measured in this run (FP64 FMA chains on every SM, enl_measure_fp_peaks)",
                     "traffic": traffic,
                     "flops_per_launch": flops, "dense_cells_per_launch": dense_cells,
                     "weno_cells_per_launch": weno_cells,
                     "flops_per_cell": {"weno": f_weno, "drp": f_drp,
                                        "counting": "algorithmic: the reference algorithm's FP64 operations per "
                                                    "computed cell (oracle-counted rhs, runge_kutta, update_state; "
                                                    "profiles/stage_fp64_flops.json); cells of uniform tiles, whose "
                                                    "shared result is computed once per block, are not counted"},
                     "implementation": {"flops_per_cell": {"weno": i_weno, "drp": i_drp},
                                        "achieved": None if iflops is None else iflops / (per_launch_ms * 1e-3) / 1e12,
                                        "frac": None if iflops is None else iflops / (per_launch_ms * 1e-3) / 1e12
                                        / fp64_peak,
                                        "counting": "FP64 instructions the kernel issues (ncu: 2 per FMA, 1 per "
                                                    "add or multiply)"},
                     "hbm": hbm})
    else:
        roof.update({"bound": "hbm", "achieved": hbm_achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": hbm_achieved / hbm_peak, "peak_kind": peak_kind,
                     "bytes_per_cell_launch": bytes_per_cell_launch, "traffic": traffic})
    # e2e: every step takes its input state (the patch state of every patch
    # interior: the 5 conserved fields and p, T, as the reference's patches
    # hold them) from pinned host memory and returns its result state to
    # pinned host memory, through the public API.  Inputs alternate between
    # two host states and results between two host buffers, so an upload or a
    # download runs on the engine's copy streams while the neighbouring step
    # computes.  The hierarchy is held fixed (a regrid would change the
    # exchanged layout).  The same with the 5 conserved fields only (p and T
    # then recomputed on the device after each upload, by update_state) is
    # reported beside it.
    E = wl.fast

    def one_step():
        if not wl.graph_ok:
            E.capture(wl.dt_cap)
            wl.captures += 1
            wl.graph_ok = True
        E.replay(1)

    def e2e_leg(alloc, down, up, ke):
        ins = [alloc(pin=True), alloc(pin=True)]
        outs = [alloc(pin=True), alloc(pin=True)]
        down(ins[0])
        one_step()
        down(ins[1])
        for k in range(2):  # warm-up of the exchange path
            up(ins[k])
            one_step()
            down(outs[k])
        # two timed windows of ke steps (the host's copies vary between
        # boxes and between windows of a run): both are reported, the better
        # one is the figure
        wins = []
        for _ in range(2):
            E.sync()
            barrier()
            t_e2e = time.perf_counter()
            for k in range(ke):
                up(ins[k % 2])
                one_step()
                down(outs[k % 2])
            E.sync()
            wins.append(max_over_ranks(1e3 * (time.perf_counter() - t_e2e), ws))
            barrier()
        return min(wins), ins[0].numel(), wins

    ke = max(1, args.steps)  # as many steps as the timed region: pipeline fill and drain amortised alike
    e2e_ms, n, e2e_wins = e2e_leg(E.packed_host, E.download, E.upload, ke)
    cue = E.cells() * ke
    e2e_value = aggregate_rate(cue, ws, e2e_ms)
    nbytes = int(n * esize)
    copy_rates = host_copy_rates(nbytes)
    e2e5_ms, n5, e2e5_wins = e2e_leg(E.state_host, E.download_state, E.upload_state, ke)
    e2e_conserved = {"value": aggregate_rate(cue, ws, e2e5_ms), "ms_per_step": e2e5_ms / ke,
                     "windows_ms_per_step": [w / ke for w in e2e5_wins],
                     "h2d_bytes_per_step": int(n5 * esize), "d2h_bytes_per_step": int(n5 * esize),
                     "pattern": "the 5 conserved fields only; p and T recomputed on the device after each "
                                "upload (update_state, FP64 exp and log per cell)"}
    # the same engine with every tile computed cell by cell (no uniform-tile
    # reuse; identical states), a few steps after the e2e leg: what the reuse
    # is worth
    dense_value, dense_steps = None, max(2, min(args.steps, 6))
    if not args.dense:
        keep = wl.fast.schedule()
        wl.fast.set_schedule(keep["blocks_per_sm"], keep["tile_order"], 0, keep["run"])
        wl.graph_ok = False
        wl.advance("fast", 1, use_graph=True)
        barrier()
        d0, d1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        d0.record()
        cud = wl.advance("fast", dense_steps, use_graph=True)
        d1.record()
        barrier()
        dense_value = aggregate_rate(cud, ws, max_over_ranks(d0.elapsed_time(d1), ws))
        wl.fast.set_schedule(keep["blocks_per_sm"], keep["tile_order"], keep["reuse"], keep["run"])
        wl.graph_ok = False
    # the step's other kernels, timed with events around each launch over the
    # same three direct steps
    roof["other_kernels"] = other_kernels(kcls, 3, hbm_peak, peak_kind)
    roof["skip_kernels"] = {k: {"ms_per_step": kcls[k][0] / 3, "launches_per_step": kcls[k][2] / 3}
                            for k in ("skip_lists", "stage_rest") if kcls.get(k, (0, 0, 0))[2]}
    # the FP32-storage engine: its own timed region (graph replay, regrids)
    secondary = None
    if wl32 is not None:
        wl32.advance("fast", max(3, args.warmup), use_graph=True)
        barrier()
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record()
        cu32 = wl32.advance("fast", args.steps, use_graph=True)
        s1.record()
        barrier()
        ms32 = s0.elapsed_time(s1)
        k32, c32, _, _, kcls32 = stage_timing(wl32)
        a32 = c32 * (STEP_BYTES_PER_CELL / 6.0) / (k32 * 1e-3) / 1e9
        secondary = {"dtype": "f32 (perturbation state and rhs)", "value": aggregate_rate(cu32, ws, ms32),
                     "ms_per_step": ms32 / args.steps,
                     "rel_l2_vs_plain_fp64": err32, "rel_l2_vs_fp64_same_switch": err32_fp64,
                     "compare_steps": ncmp, "stage_kernel_ms": k32, "schedule": tune32,
                     "roofline": {"bound": "hbm", "achieved": a32, "peak": hbm_peak, "unit": "GB/s",
                                  "frac": a32 / hbm_peak, "bytes_per_cell_launch": STEP_BYTES_PER_CELL / 6.0},
                     "other_kernels": other_kernels(kcls32, 3, hbm_peak, peak_kind)}
    if rank != 0:
        return
    health = wl.fast.health()
    cb = None
    if not args.no_cpu_baseline:
        if args.workload == "linesource":
            cb = linesource_reference_rate(args.steps, args.warmup, os.cpu_count() or 1)
            one = linesource_reference_rate(max(2, args.steps // 4), 1, 1)
            cb["value_1core"] = one["value"]
            cb["sample_1core"] = one["sample"]
            cb["cpu_model"] = host_cpu_model()
        else:
            cb = cpu_baseline_with_single_core(wl)
    dt_last, sim_t = wl.fast.time()
    sched_info = tune or wl.fast.schedule()
    extra = None
    if not args.no_extra and args.workload == "linesource" and ws == 1:
        for w_ in (wl32,):
            if w_ is not None:
                w_.fast.close()
        wl.fast.close()
        if wl.plain is not None:
            wl.plain.close()
        extra = extra_records(args, fpk)
    path = ("batched: persistent fused stage kernel over all levels, " + PREC_PATH[args.precision]
            + ", CUDA graph" + ((", learned sensor on every level" if wl.learned == 2 else ", learned sensor on level 0")
                                if wl.learned else ", plain sensor")
            + ("" if args.dense else ", uniform tiles reuse a block-cached cell result"))
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": PREC_DTYPE[args.precision], "data": "synthetic",
        "config": {"workload": wl.name, "path": path,
                   "cells_per_step": cu / args.steps, "patches": [len(p) for p in wl.fast.patches],
                   "l2": "inputs larger than L2 (state of every level, > 1 GB)", "regrid_every": wl.REGRID,
                   "timed_regrids": regrid_info,
                   "dt": ("device CFL reduction, cfl 0.5 on max(|u|+c)" if wl.REGRID else "cfl*dx/c (reference)"),
                   "dt_last": dt_last, "sim_time": sim_t,
                   "plain_value": plain_value, "plain_steps": kp,
                   "plain_path": "per-patch FP64 rhs / runge_kutta / update_state launches, plain sensor",
                   "speedup_vs_plain": (value / plain_value) if plain_value else None,
                   "rel_l2_vs_plain_fp64": err, "compare_steps": ncmp, "weno_fraction": weno_frac,
                   "uniform_tile_fraction": uniform_frac, "schedule": sched_info,
                   "dense_value": dense_value, "dense_steps": dense_steps if dense_value else None,
                   "dense_note": "the same engine and schedule with every tile computed cell by cell "
                                 "(uniform-tile reuse off; identical states): every cell's update is "
                                 "computed and stored in both, the reuse computes a bitwise-uniform "
                                 "tile's shared result once per block",
                   "health": health, "build_s": t_build, "parallelism": "replicas" if ws > 1 else "1 GPU",
                   "fp_peaks": fpk},
        "fp32_state": secondary,
        "other_workloads": extra,
        "roofline": roof,
        "cpu_baseline": cb,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                "steps": ke, "ms_per_step": e2e_ms / ke, "windows_ms_per_step": [w / ke for w in e2e_wins],
                "windows": "two timed windows of `steps` steps each after the same warm-up; value from the "
                           "faster (the host copies' rate varies between boxes and windows)",
                "pattern": "per step: input patch state (rho, rho u, rho v, rho s, rho T_n, p, T of every patch "
                           "interior) host->device, one RK3 step, result state device->host (pinned; two "
                           "alternating inputs and outputs; copies on the engine's copy streams overlap the "
                           "neighbouring steps; wall clock)",
                "conserved_fields_only": e2e_conserved, "host_copy_gbs": copy_rates},
        "clocks": clk.summary(), "gpu_launches": launches,
        "gpu_launches_counted": "kernels of the timed steps (graph replays); the regrids inside the timed "
                                "region launch more (tagging, tag blocks, refine) and are not counted",
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="linesource", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--learned", type=int, default=-1, choices=[-1, 0, 1, 2],
                    help="learned switch: 1 on level 0, 2 on every level, 0 off, -1 (default) as the trained "
                         "network was made for, when it is present")
    ap.add_argument("--plain-steps", type=int, default=10)
    ap.add_argument("--compare-steps", type=int, default=20)
    ap.add_argument("--scale", type=int, default=1, help="shrink the line-source base grid (profiling)")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 arm (profiling)")
    ap.add_argument("--regrid-every", type=int, default=None,
                    help="regrid interval of the multi-level workloads (default: the workload's, 10)")
    ap.add_argument("--tile-order", type=int, default=0, choices=[0, 1, 2, 3],
                    help="stage-kernel tile order: 0 finest level first, 1 level 0 first, 2 alternately, "
                         "3 two streams by block")
    ap.add_argument("--dense", action="store_true",
                    help="compute every stage tile cell by cell (no uniform-tile reuse; same states)")
    ap.add_argument("--precision", type=int, default=0, choices=[0, 1, 2],
                    help="engine mode: 0 FP64 (default), 1 FP32 RHS on FP64 state, 2 FP32 perturbation state")
    ap.add_argument("--stats-only", action="store_true",
                    help="run --steps direct steps of the batched engine and print its counters (profiling)")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default stage-kernel schedule")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the short runs of the pulse batch, the Mach shock and the single pulse")
    ap.add_argument("--schedule-cache", default=os.path.join(tempfile.gettempdir(), "enlightning_gb300_schedules.json"),
                    help="JSON file of tuned schedules by workload signature")
    ap.add_argument("--no-secondary", action="store_true",
                    help="skip the FP32-storage engine reported beside the FP64 line")
    args = ap.parse_args()
    if args.learned < 0:  # the metric's configuration: batched + learned switch
        from enlightning_gb300 import sensor
        args.learned = sensor.weights_levels() if os.path.exists(sensor.WEIGHTS) else 0
    if args.stats_only:
        run_stats_only(args)
    elif args.impl == "reference":
        run_reference(args)
    elif args.workload in ("linesource", "pulses64", "mach"):
        run_linesource(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
