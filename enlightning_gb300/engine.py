"""Host side of the batched multi-level engine (include/enlightning_gpu.h, part 3).

``Engine`` owns one enl_engine handle: level canvases in device memory, the
patch boxes of every level, and the step entry points (fused batched path,
plain per-patch path, CUDA-graph capture/replay).  ``Hierarchy`` adds the AMR
host logic that SAMRAI provides to the reference (main.C:253-312,489-502):
tagging with tag_cells on the device, buffering of tags, clustering of tagged
cells into patches, proper nesting, and initialisation of new fine cells.

Canvas convention: field k of level cell (i, j) is at
``base[k*fstride + (j+3)*pitch + (i+3)]``; fields are rho, rho*u, rho*v,
rho*s, rho*T_n, p, T.  With PREC_FP32_STATE the canvases hold float32
perturbations about the ambient state (``offsets`` per field);
``level_state`` and ``set_level_state`` always speak absolute float64.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np
import torch

from . import _lib
from .constants import REFLECT, RK3_ALPHA1, RK3_ALPHA2, RK3_BETA, VARIANTS
from .cluster import cluster_tags_native

MAX_LEVELS = 4
PREC_FP64, PREC_FP32, PREC_FP32_STATE = 0, 1, 2


from ._lib import ENGINE_SIGNATURES, EngineConfig  # noqa: E402


def _boxes_arg(boxes):
    flat = np.ascontiguousarray(np.asarray(boxes, dtype=np.int32).reshape(-1))
    return flat, flat.ctypes.data_as(C.POINTER(C.c_int))


class Engine:
    """One multi-level canvas engine on the current CUDA device."""

    def __init__(self, params: dict, nx0: int, ny0: int, dx0, nlevels=1, ratio=2, xlo=(0.0, 0.0),
                 bc=(REFLECT,) * 4, variant="hybrid_high_llf", precision=PREC_FP64, learned=False,
                 independent=False, dense=False, tile_order=0):
        self.L = _lib.lib()
        p = params
        cfg = EngineConfig()
        cfg.nlevels, cfg.ratio, cfg.nx0, cfg.ny0 = nlevels, ratio, nx0, ny0
        cfg.xlo[:] = list(xlo)
        cfg.dx0[:] = list(dx0)
        cfg.bc[:] = list(bc)
        cfg.variant = VARIANTS.index(variant) if isinstance(variant, str) else int(variant)
        # learned: False/0 off, True/1 the learned switch on level 0, 2 or
        # "all" on every level
        lv = 2 if learned in (2, "all") else int(bool(learned))
        cfg.precision, cfg.learned = int(precision), lv
        for k in ("weno_alpha", "kappa", "mu", "muB", "R", "T_star_n", "tau_n", "c", "c_lr", "rho0", "gamma1",
                  "c_p", "p0", "T0", "c_v"):
            setattr(cfg, k, float(p[k]))
        cfg.tol[:] = list(p["tol"])
        cfg.absorb_width = float(p["bc_absorb_width"])
        cfg.rk_alpha1[:] = list(RK3_ALPHA1)
        cfg.rk_alpha2[:] = list(RK3_ALPHA2)
        cfg.rk_beta[:] = list(RK3_BETA)
        cfg.independent = int(bool(independent))
        cfg.dense = int(bool(dense))
        cfg.tile_order = int(tile_order)
        self.cfg = cfg
        self.params = dict(p)
        self._init_args = dict(nx0=nx0, ny0=ny0, dx0=tuple(dx0), nlevels=nlevels, ratio=ratio, xlo=tuple(xlo),
                               bc=tuple(bc), variant=variant, precision=int(precision), learned=lv,
                               independent=bool(independent), dense=bool(dense), tile_order=int(tile_order))
        self.nlevels, self.ratio = nlevels, ratio
        self.dx0 = tuple(dx0)
        self.xlo = tuple(xlo)
        _lib.check(self.L.enl_set_stream(C.c_void_p(torch.cuda.current_stream().cuda_stream)), "enl_set_stream")
        h = C.c_void_p()
        _lib.check(self.L.enl_engine_create(C.byref(cfg), C.byref(h)), "enl_engine_create")
        self.h = h
        self.patches = [[] for _ in range(nlevels)]
        eb = C.c_int()
        off = (C.c_double * 7)()
        _lib.check(self.L.enl_engine_storage(h, C.byref(eb), off), "enl_engine_storage")
        self.dtype = torch.float32 if eb.value == 4 else torch.float64
        self.offsets = np.array(off[:], np.float64)

    def close(self):
        if self.h:
            self.L.enl_engine_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- geometry -----------------------------------------------------------
    def level_shape(self, level):
        nx, ny = C.c_int(), C.c_int()
        _lib.check(self.L.enl_engine_buffer(self.h, level, 0, None, None, None, C.byref(nx), C.byref(ny)))
        return nx.value, ny.value

    def dx(self, level):
        r = self.ratio ** level
        return (self.dx0[0] / r, self.dx0[1] / r)

    def buffer(self, level, which=0):
        """torch view (nfields, ny+6, nx+6) of a level canvas (no copy)."""
        base, pitch, fstride = C.c_void_p(), C.c_long(), C.c_long()
        nx, ny = C.c_int(), C.c_int()
        _lib.check(self.L.enl_engine_buffer(self.h, level, which, C.byref(base), C.byref(pitch), C.byref(fstride),
                                            C.byref(nx), C.byref(ny)), "enl_engine_buffer")
        nf = 1 if which == 3 else 7
        n = fstride.value * nf
        storage = _DeviceMemory(base.value, n, "<f4" if self.dtype == torch.float32 else "<f8")
        t = torch.as_tensor(storage, device="cuda")
        t = t.as_strided((nf, ny.value + 6, nx.value + 6), (fstride.value, pitch.value, 1))
        return t

    # -- patches ------------------------------------------------------------
    def set_patches(self, level, boxes):
        boxes = [tuple(int(v) for v in b) for b in boxes]
        flat, ptr = _boxes_arg(boxes if boxes else np.zeros((0, 4)))
        _lib.check(self.L.enl_engine_set_patches(self.h, level, len(boxes), ptr), "enl_engine_set_patches")
        self.patches[level] = boxes

    def refine_init(self, level, boxes):
        if not boxes:
            return
        flat, ptr = _boxes_arg(boxes)
        _lib.check(self.L.enl_engine_refine_init(self.h, level, len(boxes), ptr), "enl_engine_refine_init")

    def cells(self):
        return sum((b[1] - b[0] + 1) * (b[3] - b[2] + 1) for lv in self.patches for b in lv)

    def set_level_order(self, samrai=True):
        """Stage order across levels: SAMRAI's (each level filled from the
        coarser level already advanced in the same stage) or the default
        (every level from the same stage input, one launch per stage)."""
        _lib.check(self.L.enl_engine_set_level_order(self.h, int(bool(samrai))), "enl_engine_set_level_order")

    # -- schedule and autotuner ---------------------------------------------
    SCHEDULE_KEYS = ("blocks_per_sm", "tile_order", "reuse", "run")

    def schedule(self):
        """The stage kernel's schedule in force (enl_engine_get_schedule)."""
        v = (C.c_int * 5)()
        _lib.check(self.L.enl_engine_get_schedule(self.h, v, 5), "enl_engine_get_schedule")
        out = dict(zip(self.SCHEDULE_KEYS, v[:4]))
        out["max_blocks_per_sm"] = v[4]
        return out

    def set_schedule(self, blocks_per_sm=0, tile_order=0, reuse=2, run=1):
        v = (C.c_int * 4)(int(blocks_per_sm), int(tile_order), int(reuse), int(run))
        _lib.check(self.L.enl_engine_set_schedule(self.h, v, 4), "enl_engine_set_schedule")

    def signature(self):
        """Workload signature the tuned schedule is kept under: device, storage
        precision, scheme, learned switch, and per level the patch count and
        cell count (two significant digits)."""
        props = torch.cuda.get_device_properties(torch.cuda.current_device())
        parts = [props.name.replace(" ", "_"), f"sm{props.multi_processor_count}",
                 f"p{self.cfg.precision}", f"v{self.cfg.variant}", f"l{self.cfg.learned}", f"i{self.cfg.independent}",
                 f"clr{int(self.params.get('c_lr', 0.0) != 0.0)}"]
        for lv, boxes in enumerate(self.patches):
            cells = sum((b[1] - b[0] + 1) * (b[3] - b[2] + 1) for b in boxes)
            parts.append(f"L{lv}:{len(boxes)}:{float(f'{cells:.2g}'):.0f}")
        return "/".join(parts)

    def autotune(self, dt, steps=3, cache=None):
        """Pick the stage kernel's schedule for this workload.

        With `cache` (a JSON file path), a schedule stored under this engine's
        signature() is applied without timing; otherwise the library's tuner
        (enl_engine_autotune) times the candidates on the current state, which
        it leaves unchanged, applies the fastest and, with `cache`, stores it.
        Returns dict(schedule, signature, source "cache"|"tuned", table of
        (schedule, ms per step) rows when tuned)."""
        import json
        import os
        sig = self.signature()
        store = {}
        if cache and os.path.exists(cache):
            with open(cache) as f:
                store = json.load(f)
            if sig in store:
                self.set_schedule(**{k: store[sig][k] for k in self.SCHEDULE_KEYS})
                return dict(schedule=self.schedule(), signature=sig, source="cache", table=[])
        cap = 64
        tried = (C.c_int * (4 * cap))()
        ms = (C.c_float * cap)()
        n = C.c_int()
        _lib.check(self.L.enl_engine_autotune(self.h, float(dt), int(steps), cap, tried, ms, C.byref(n)),
                   "enl_engine_autotune")
        table = [(dict(zip(self.SCHEDULE_KEYS, tried[4 * k:4 * k + 4])), float(ms[k])) for k in range(min(cap, n.value))]
        sched = self.schedule()
        if cache:
            store[sig] = {k: sched[k] for k in self.SCHEDULE_KEYS}
            d = os.path.dirname(os.path.abspath(cache))
            os.makedirs(d, exist_ok=True)
            tmp = cache + ".tmp%d" % os.getpid()
            with open(tmp, "w") as f:
                json.dump(store, f, indent=1, sort_keys=True)
            os.replace(tmp, cache)
        return dict(schedule=sched, signature=sig, source="tuned", table=table)

    # -- stepping -----------------------------------------------------------
    def fill(self, which=0):
        _lib.check(self.L.enl_engine_fill(self.h, which), "enl_engine_fill")

    def step(self, dt, plain=False):
        fn = self.L.enl_engine_step_plain if plain else self.L.enl_engine_step
        _lib.check(fn(self.h, float(dt)), "enl_engine_step")

    def capture(self, dt):
        _lib.check(self.L.enl_engine_graph_capture(self.h, float(dt)), "enl_engine_graph_capture")

    def graph_valid(self):
        """True while the captured graph can be replayed (it survives regrids
        unless a device table had to grow)."""
        return bool(self.L.enl_engine_graph_valid(self.h))

    def replay(self, nsteps):
        _lib.check(self.L.enl_engine_graph_replay(self.h, int(nsteps)), "enl_engine_graph_replay")

    def launches_per_step(self, plain=False):
        return int(self.L.enl_engine_launches_per_step(self.h, int(plain)))

    def stats(self):
        """Per level: [WENO cells, cells, cells decided by the plain fallback, cells of uniform
        tiles stored from the cache] since the last call."""
        arr = (C.c_longlong * (4 * MAX_LEVELS))()
        _lib.check(self.L.enl_engine_stats(self.h, arr), "enl_engine_stats")
        a = np.array(arr[:], dtype=np.int64).reshape(MAX_LEVELS, 4)
        return a[: self.nlevels]

    def skipped_tiles(self):
        """(tiles the last step's stage 3 flagged as uniform from the records,
        of those stored without loading their halo box, tiles)."""
        f, w, n = C.c_longlong(), C.c_longlong(), C.c_longlong()
        _lib.check(self.L.enl_engine_skipped_tiles(self.h, C.byref(f), C.byref(w), C.byref(n)),
                   "enl_engine_skipped_tiles")
        return f.value, w.value, n.value

    def health(self):
        return int(self.L.enl_engine_health(self.h))

    def tag(self, level):
        nx, ny = self.level_shape(level)
        tags = torch.zeros((ny, nx), dtype=torch.int32, device="cuda")
        _lib.check(self.L.enl_engine_tag(self.h, level, C.c_void_p(tags.data_ptr())), "enl_engine_tag")
        return tags

    def set_mlp(self, params, margin):
        """Install the learned switch (FP32 parameter vector) in an engine created with learned=True."""
        P = np.ascontiguousarray(np.asarray(params, np.float32))
        _lib.check(self.L.enl_engine_set_mlp(self.h, P.ctypes.data_as(C.c_void_p), float(margin)),
                   "enl_engine_set_mlp")

    def profile(self, on=True):
        """Switch event timing (True or 1: stage kernels; 2: also the other
        kernels of the step); returns (ms, launches, cells) of the stage
        kernels since the last call and resets every profile figure."""
        ms, n, c = C.c_double(), C.c_longlong(), C.c_longlong()
        _lib.check(self.L.enl_engine_profile(self.h, int(on), C.byref(ms), C.byref(n), C.byref(c)),
                   "enl_engine_profile")
        return ms.value, n.value, c.value

    KERNEL_CLASSES = ("interp", "physbc", "coarsen", "cfl", "skip_lists", "stage_rest")

    def profile_kernels(self):
        """{class: (ms, algorithmic bytes, launches)} of the step's other
        kernels under profile(2), since the last profile() call (the two
        skip classes are part of the stage figures; bytes 0)."""
        ms, by, n = (C.c_double * 6)(), (C.c_double * 6)(), (C.c_longlong * 6)()
        _lib.check(self.L.enl_engine_profile_kernels(self.h, ms, by, n), "enl_engine_profile_kernels")
        return {k: (ms[i], by[i], n[i]) for i, k in enumerate(self.KERNEL_CLASSES)}

    def packed_size(self):
        n = C.c_longlong()
        _lib.check(self.L.enl_engine_packed_size(self.h, C.byref(n)), "enl_engine_packed_size")
        return n.value

    def packed_host(self, pin=True):
        """Host tensor sized for download/upload (storage dtype)."""
        t = torch.empty(self.packed_size(), dtype=self.dtype)
        return t.pin_memory() if pin else t

    @staticmethod
    def _host_arg(host: torch.Tensor):
        assert host.device.type == "cpu" and host.is_contiguous()
        return C.c_void_p(host.data_ptr()), host.numel() * host.element_size()

    def download(self, host: torch.Tensor):
        """Packed 7-field state to host memory (asynchronous: sync() before reading)."""
        assert host.dtype == self.dtype
        _lib.check(self.L.enl_engine_download(self.h, *self._host_arg(host)), "enl_engine_download")

    def upload(self, host: torch.Tensor):
        """Packed 7-field state from host memory (asynchronous: keep it unchanged until sync())."""
        assert host.dtype == self.dtype
        _lib.check(self.L.enl_engine_upload(self.h, *self._host_arg(host)), "enl_engine_upload")

    def state_host(self, pin=True):
        """Host tensor sized for download_state/upload_state (5 fields)."""
        t = torch.empty(self.packed_size() // 7 * 5, dtype=self.dtype)
        return t.pin_memory() if pin else t

    def download_state(self, host: torch.Tensor):
        """Conserved state (5 fields) of every patch interior to host memory
        (asynchronous: sync() before reading)."""
        assert host.dtype == self.dtype
        _lib.check(self.L.enl_engine_download_state(self.h, *self._host_arg(host)), "enl_engine_download_state")

    def upload_state(self, host: torch.Tensor):
        """Conserved state from host memory; p and T follow on the device
        (asynchronous: keep the host data unchanged until sync())."""
        assert host.dtype == self.dtype
        _lib.check(self.L.enl_engine_upload_state(self.h, *self._host_arg(host)), "enl_engine_upload_state")

    def sync(self):
        """Wait for the engine's host copies and the library stream."""
        _lib.check(self.L.enl_engine_sync(self.h), "enl_engine_sync")

    def set_adaptive_dt(self, on=True, cfl=0.5):
        _lib.check(self.L.enl_engine_set_adaptive_dt(self.h, int(on), float(cfl)), "enl_engine_set_adaptive_dt")

    def time(self):
        dt, t = C.c_double(), C.c_double()
        _lib.check(self.L.enl_engine_time(self.h, C.byref(dt), C.byref(t)), "enl_engine_time")
        return dt.value, t.value

    # -- restart (the role of enlightning.C:1859-2060 for this engine) ------------
    def save(self, path, iteration=0):
        """Restart file (.npz): construction arguments, parameters, patch boxes
        of every level, the packed state of every patch interior (7 fields,
        storage type), the CFL state and the iteration number."""
        host = self.packed_host(pin=False)
        self.download(host)
        self.sync()
        dt, t = self.time()
        boxes = np.full((self.nlevels, max(1, max(len(b) for b in self.patches)), 4), -1, np.int64)
        for l, bl in enumerate(self.patches):
            if bl:
                boxes[l, :len(bl)] = np.asarray(bl, np.int64)
        np.savez(path, state=host.numpy(), boxes=boxes, npatch=np.array([len(b) for b in self.patches]),
                 dt=dt, time=t, iteration=int(iteration),
                 init=np.array(repr(self._init_args)), params=np.array(repr(self.params)))

    @classmethod
    def load(cls, path):
        """Engine, iteration from a restart file written by save()."""
        import ast
        d = np.load(path)
        params = ast.literal_eval(str(d["params"]))
        init = ast.literal_eval(str(d["init"]))
        E = cls(params, init.pop("nx0"), init.pop("ny0"), init.pop("dx0"), **init)
        for l in range(E.nlevels):
            n = int(d["npatch"][l])
            E.set_patches(l, [tuple(int(v) for v in b) for b in d["boxes"][l, :n]])
        host = torch.from_numpy(np.ascontiguousarray(d["state"]))
        assert host.numel() == E.packed_size() and host.dtype == E.dtype
        E.upload(host)
        _lib.check(E.L.enl_engine_set_time(E.h, float(d["dt"]), float(d["time"])), "enl_engine_set_time")
        E.sync()
        return E, int(d["iteration"])

    def paint_source(self, level, src_type, mode=10, amp=1.0, spread=1.0, pos=(0.0, 0.0), sine_amp=0.0,
                     sine_freq=0.0, segs=None, drive=1.0):
        """enlightning::addSource on one level (types 10 POINT, 20 SINE, 30 LIGHTNING)."""
        segarr = np.ascontiguousarray(np.asarray(segs if segs is not None else np.zeros((0, 4)), np.float64))
        nseg = segarr.shape[0]
        _lib.check(self.L.enl_engine_paint_source(
            self.h, level, int(src_type), int(mode), float(amp), float(spread), _lib.darr(pos), float(sine_amp),
            float(sine_freq), nseg, segarr.ctypes.data_as(C.POINTER(C.c_double)), float(drive)),
            "enl_engine_paint_source")

    # -- microphones (enlightning.C:2392-2506) ---------------------------------
    MIC_DTYPE = np.dtype([("iteration", "<i4"), ("mic", "<i4"), ("level", "<i4"), ("patch", "<i4"), ("p", "<f8")])

    def set_mics(self, positions, capacity=1 << 20, iteration=0):
        """Sample the pressure at these (x, y) positions after every step."""
        xy = np.ascontiguousarray(np.asarray(positions, np.float64).reshape(-1))
        _lib.check(self.L.enl_engine_set_mics(self.h, xy.size // 2, xy.ctypes.data_as(C.c_void_p) if xy.size else None,
                                              int(capacity), int(iteration)), "enl_engine_set_mics")
        self.nmics = xy.size // 2

    def mic_records(self, max_records=1 << 20):
        """Drain the device record buffer: structured array in the reference's
        file order (iteration, microphone, level, patch) and the dropped count."""
        out = np.zeros(max_records, self.MIC_DTYPE)
        n, dropped = C.c_longlong(), C.c_longlong()
        _lib.check(self.L.enl_engine_mic_records(self.h, out.ctypes.data_as(C.c_void_p), int(max_records),
                                                 C.byref(n), C.byref(dropped)), "enl_engine_mic_records")
        rec = out[: n.value]
        order = np.lexsort((rec["patch"], rec["level"], rec["mic"], rec["iteration"]))
        return rec[order], dropped.value

    def state_from_overpressure(self, level):
        _lib.check(self.L.enl_engine_state_from_overpressure(self.h, level), "enl_engine_state_from_overpressure")

    def tag_blocks(self, level, block, buffer):
        nbx, nby = C.c_int(), C.c_int()
        _lib.check(self.L.enl_engine_tag_blocks(self.h, level, block, buffer, None, C.byref(nbx), C.byref(nby)))
        m = np.zeros((nby.value, nbx.value), np.uint8)
        _lib.check(self.L.enl_engine_tag_blocks(self.h, level, block, buffer, m.ctypes.data_as(C.c_void_p),
                                                C.byref(nbx), C.byref(nby)), "enl_engine_tag_blocks")
        return m.astype(bool)

    # -- state I/O ----------------------------------------------------------
    def set_level_state(self, level, w, pres, temp, which=0):
        """Write interior (5, ny, nx) state and p, T (ny, nx) of a level (absolute values)."""
        buf = self.buffer(level, which)
        ny, nx = pres.shape
        full = torch.empty((7, ny, nx), dtype=torch.float64, device="cuda")
        full[0:5] = torch.as_tensor(w, device="cuda")
        full[5] = torch.as_tensor(pres, device="cuda")
        full[6] = torch.as_tensor(temp, device="cuda")
        if self.dtype == torch.float32:
            full -= torch.as_tensor(self.offsets, device="cuda")[:, None, None]
        buf[:, 3:3 + ny, 3:3 + nx].copy_(full)

    def set_box_state(self, level, i0, j0, w, pres, temp, which=0):
        """Write absolute state (5, h, w) and p, T (h, w) into the cells
        starting at level cell (i0, j0)."""
        buf = self.buffer(level, which)
        h, wd = pres.shape
        full = torch.empty((7, h, wd), dtype=torch.float64, device="cuda")
        full[0:5] = torch.as_tensor(w, device="cuda")
        full[5] = torch.as_tensor(pres, device="cuda")
        full[6] = torch.as_tensor(temp, device="cuda")
        if self.dtype == torch.float32:
            full -= torch.as_tensor(self.offsets, device="cuda")[:, None, None]
        buf[:, 3 + j0:3 + j0 + h, 3 + i0:3 + i0 + wd].copy_(full)

    def canvas_state(self, level, which=0):
        """Whole canvas (7, ny+6, nx+6) with ghosts as absolute float64 (host numpy)."""
        v = self.buffer(level, which).double()
        if self.dtype == torch.float32:
            v = v + torch.as_tensor(self.offsets, device="cuda")[:, None, None]
        return v.cpu().numpy()

    def level_state(self, level, which=0):
        """Interior (7, ny, nx) of a level: a view of the canvas with FP64
        storage, an absolute float64 copy with FP32 perturbation storage."""
        buf = self.buffer(level, which)
        nx, ny = self.level_shape(level)
        v = buf[:, 3:3 + ny, 3:3 + nx]
        if self.dtype == torch.float32:
            return v.double() + torch.as_tensor(self.offsets, device="cuda")[:, None, None]
        return v


class _DeviceMemory:
    """__cuda_array_interface__ wrapper of library-owned device memory."""

    def __init__(self, ptr, n, typestr="<f8"):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False), "version": 3,
                                         "strides": None}


# ---------------------------------------------------------------------------
# AMR hierarchy (host metadata, as SAMRAI keeps it)
# ---------------------------------------------------------------------------

class Hierarchy:
    """Patch hierarchy over an Engine: tagging, clustering, nesting, regrid.

    Follows the reference's gridding loop (main.C:489-502 with
    StandardTagAndInitialize + BergerRigoutsos, input.txt:103-127): tag cells
    of level l with tag_cells (fortran/tag_cells.m4, on the device), grow the
    tags by tag_buffer cells, cluster them into boxes of efficiency >= 0.7 with
    sides between min_size and max_size (level l+1 cells), refine the boxes by
    the ratio and keep them properly nested inside level l.  Tags reach the
    host as a map of block x block cells (the device folds the tag buffer into
    that reduction), so clustering works on 1/block^2 of the cells and patch
    corners fall on block boundaries.
    """

    def __init__(self, engine: Engine, min_size=16, max_size=256, tag_buffer=2, efficiency=0.7, block=4,
                 nest_blocks=1, native=True):
        self.E = engine
        self.native = native  # one library call per level (enl_engine_regrid) instead of the steps below
        self.min_size, self.max_size = min_size, max_size
        self.tag_buffer, self.efficiency = tag_buffer, efficiency
        self.block, self.nest_blocks = block, nest_blocks
        # host seconds spent per regrid phase (tag map, clustering, tables, new fine data)
        self.timing = {"tag": 0.0, "cluster": 0.0, "tables": 0.0, "refine": 0.0}

    def base_patches(self, size=256):
        nx, ny = self.E.level_shape(0)
        boxes = []
        for j in range(0, ny, size):
            for i in range(0, nx, size):
                boxes.append((i, min(nx, i + size) - 1, j, min(ny, j + size) - 1))
        self.E.set_patches(0, boxes)
        return boxes

    def _nesting_blocks(self, level, nbx, nby):
        """Blocks fully inside the patches of `level` (before the erosion by
        nest_blocks that _nest_erode gives for fine levels)."""
        B = self.block
        m = np.zeros((nby, nbx), bool)
        for b in self.E.patches[level]:
            bx0, bx1 = -(-b[0] // B), (b[1] + 1) // B - 1
            by0, by1 = -(-b[2] // B), (b[3] + 1) // B - 1
            if bx1 >= bx0 and by1 >= by0:
                m[by0:by1 + 1, bx0:bx1 + 1] = True
        return m

    def _nest_erode(self, level):
        return self.nest_blocks if (self.nest_blocks > 0 and level > 0) else 0

    def propose(self, level):
        """Fine boxes (level+1 index space) from the current tags of `level`."""
        E, B, r = self.E, self.block, self.E.ratio
        t0 = time.perf_counter()
        bmap = E.tag_blocks(level, B, self.tag_buffer)
        t1 = time.perf_counter()
        self.timing["tag"] += t1 - t0
        nest = self._nesting_blocks(level, bmap.shape[1], bmap.shape[0])
        cell = B * r  # level+1 cells per block side
        cboxes = cluster_tags_native(bmap, efficiency=self.efficiency, min_size=max(1, self.min_size // cell),
                                     max_size=max(1, self.max_size // cell), allowed=nest,
                                     nest_erode=self._nest_erode(level))
        nxf, nyf = E.level_shape(level + 1)
        fine = []
        for b in cboxes:
            fb = (b[0] * cell, min(nxf, (b[1] + 1) * cell) - 1, b[2] * cell, min(nyf, (b[3] + 1) * cell) - 1)
            if fb[1] >= fb[0] and fb[3] >= fb[2]:
                fine.append(fb)
        self.timing["cluster"] += time.perf_counter() - t1
        return fine

    def regrid_level(self, level):
        """Rebuild level+1 from the tags of `level`; returns the new boxes."""
        E = self.E
        if level + 1 >= E.nlevels:
            return []
        if self.native:
            return self._regrid_native(level)
        fine = self.propose(level)
        old = list(E.patches[level + 1])
        t0 = time.perf_counter()
        new_regions = box_difference(fine, old)
        E.set_patches(level + 1, fine)
        t1 = time.perf_counter()
        E.refine_init(level + 1, new_regions)
        t2 = time.perf_counter()
        self.timing["tables"] += t1 - t0
        self.timing["refine"] += t2 - t1
        return fine

    def _regrid_native(self, level):
        """The same regrid in one library call (enl_engine_regrid)."""
        E = self.E
        t0 = time.perf_counter()
        _lib.check(E.L.enl_engine_regrid(E.h, level, self.block, self.tag_buffer, self.nest_blocks,
                                         float(self.efficiency), self.min_size, self.max_size), "enl_engine_regrid")
        n = C.c_int()
        E.L.enl_engine_get_patches(E.h, level + 1, None, 0, C.byref(n))
        out = np.zeros((max(1, n.value), 4), np.int32)
        _lib.check(E.L.enl_engine_get_patches(E.h, level + 1, out.ctypes.data_as(C.c_void_p), n.value, C.byref(n)),
                   "enl_engine_get_patches")
        E.patches[level + 1] = [tuple(int(v) for v in b) for b in out[: n.value]]
        self.timing["native"] = self.timing.get("native", 0.0) + time.perf_counter() - t0
        ph = (C.c_double * 5)()
        E.L.enl_engine_regrid_timing(E.h, ph)
        for k, v in zip(("queue_wait", "tag", "cluster", "tables", "refine"), ph):
            self.timing["native_" + k] = self.timing.get("native_" + k, 0.0) + v * 1e-3
        return E.patches[level + 1]

    def regrid(self):
        """Regrid every finer level, coarse to fine (regridAllFinerLevels)."""
        return [self.regrid_level(l) for l in range(self.E.nlevels - 1)]


def box_difference(boxes, remove):
    """Rectangles covering the union of `boxes` minus the union of `remove`."""
    out = []
    for b in boxes:
        pieces = [b]
        for r in remove:
            nxt = []
            for p in pieces:
                nxt.extend(_subtract(p, r))
            pieces = nxt
        out.extend(pieces)
    return out


def _subtract(a, r):
    ilo, ihi, jlo, jhi = a
    if r[1] < ilo or r[0] > ihi or r[3] < jlo or r[2] > jhi:
        return [a]
    res = []
    if jlo < r[2]:
        res.append((ilo, ihi, jlo, r[2] - 1))
    if jhi > r[3]:
        res.append((ilo, ihi, r[3] + 1, jhi))
    j0, j1 = max(jlo, r[2]), min(jhi, r[3])
    if ilo < r[0]:
        res.append((ilo, r[0] - 1, j0, j1))
    if ihi > r[1]:
        res.append((r[1] + 1, ihi, j0, j1))
    return res
