"""Stage-kernel schedules and the autotuner (GPU).

The reference balances its patches over MPI ranks with SAMRAI's load balancer
(main.C:268-301); here every patch of every level shares one persistent grid
and a schedule decides how the grid's blocks take tiles (blocks per SM, tile
order, uniform-tile reuse, tiles claimed per run).  Checked here:

* every schedule advances the state bit for bit like the default one, on a
  three-level line source in FP64 and in FP32 perturbation storage;
* the tuner leaves the simulation where it was (canvases of every level,
  simulated time) and applies a schedule no slower than the default;
* a stored choice is found again under the workload's signature.
"""
import json

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from enlightning_gb300 import workloads  # noqa: E402
from enlightning_gb300.constants import default_params  # noqa: E402
from enlightning_gb300.engine import PREC_FP32_STATE, PREC_FP64  # noqa: E402


def small_line_source(precision):
    prm = default_params()
    return workloads.line_source(prm, nx0=512, ny0=256, dx0=0.5, nseg=40, seed=3, precision=precision,
                                 base_patch=128, max_size=128)


def states(E):
    return [E.canvas_state(l) for l in range(E.nlevels)]


@pytest.mark.parametrize("precision", [PREC_FP64, PREC_FP32_STATE])
def test_every_schedule_gives_the_same_states(precision):
    results = {}
    scheds = [None, dict(blocks_per_sm=1, tile_order=1, reuse=0, run=4), dict(blocks_per_sm=0, tile_order=0, reuse=1, run=2),
              dict(blocks_per_sm=0, tile_order=1, reuse=1, run=3), dict(blocks_per_sm=0, tile_order=2, reuse=1, run=1),
              dict(blocks_per_sm=0, tile_order=2, reuse=0, run=4), dict(blocks_per_sm=0, tile_order=3, reuse=1, run=1),
              dict(blocks_per_sm=1, tile_order=3, reuse=0, run=1)]
    for k, sc in enumerate(scheds):
        E, H, _ = small_line_source(precision)
        if sc is not None:
            E.set_schedule(**sc)
        for _ in range(4):
            E.step(1.0)
        torch.cuda.synchronize()
        assert E.health() == 0
        results[k] = (states(E), E.time())
        E.close()
    for k in range(1, len(scheds)):
        assert results[k][1] == results[0][1], k
        for l, (a, b) in enumerate(zip(results[k][0], results[0][0])):
            assert np.array_equal(a.view(np.int64) if a.dtype == np.float64 else a,
                                  b.view(np.int64) if b.dtype == np.float64 else b), (k, l)


def test_autotune_leaves_the_state_and_is_no_slower_than_default(tmp_path):
    E, H, _ = small_line_source(PREC_FP64)
    for _ in range(2):
        E.step(1.0)
    torch.cuda.synchronize()
    before, t_before = states(E), E.time()
    default = E.schedule()
    cache = str(tmp_path / "schedules.json")
    res = E.autotune(1.0, steps=3, cache=cache)
    torch.cuda.synchronize()
    after, t_after = states(E), E.time()
    assert t_after == t_before
    for a, b in zip(after, before):
        assert np.array_equal(a, b)
    assert res["source"] == "tuned" and len(res["table"]) >= 8
    ms = {tuple(s[k] for k in E.SCHEDULE_KEYS): t for s, t in res["table"]}
    chosen = tuple(res["schedule"][k] for k in E.SCHEDULE_KEYS)
    dflt = tuple(default[k] for k in E.SCHEDULE_KEYS)
    print("tuner table (ms/step):", sorted(ms.items(), key=lambda kv: kv[1])[:6], "default", dflt, ms[dflt])
    assert ms[chosen] <= ms[dflt]
    # the choice is stored under the workload's signature and found again
    with open(cache) as f:
        assert E.signature() in json.load(f)
    E.set_schedule(**{k: default[k] for k in E.SCHEDULE_KEYS})
    again = E.autotune(1.0, steps=3, cache=cache)
    assert again["source"] == "cache"
    assert tuple(again["schedule"][k] for k in E.SCHEDULE_KEYS) == chosen
    # and the tuned run continues exactly as an untuned one would
    for _ in range(3):
        E.step(1.0)
    torch.cuda.synchronize()
    tuned_state = states(E)
    E.close()
    E2, _, _ = small_line_source(PREC_FP64)
    for _ in range(5):
        E2.step(1.0)
    torch.cuda.synchronize()
    for a, b in zip(tuned_state, states(E2)):
        assert np.array_equal(a, b)
    E2.close()


@pytest.mark.parametrize("precision", [PREC_FP64, PREC_FP32_STATE])
def test_skipping_uniform_tiles_changes_nothing(precision):
    """Reuse 2 takes the tiles that the previous stage's records prove
    uniform without loading their halo boxes (or, when no block has computed
    their key yet, in a second launch over the full path); a line source run
    with a regrid steps bit for bit as with reuse 1 and 0, and flags tiles."""
    results = {}
    for reuse in (2, 1, 0):
        E, H, _ = small_line_source(precision)
        E.set_schedule(blocks_per_sm=0, tile_order=3, reuse=reuse, run=1)
        for s in range(6):
            if s == 3:
                H.regrid()
            E.step(1.0)
        torch.cuda.synchronize()
        assert E.health() == 0
        flagged, written, tiles = E.skipped_tiles()
        assert 0 <= written <= flagged <= tiles
        results[reuse] = (states(E), E.time(), E.stats(), flagged, tiles, written)
        E.close()
    for reuse in (1, 0):
        assert results[reuse][1] == results[2][1]
        for a, b in zip(results[reuse][0], results[2][0]):
            assert np.array_equal(a.view(np.int64) if a.dtype == np.float64 else a,
                                  b.view(np.int64) if b.dtype == np.float64 else b), reuse
    assert results[1][3] == 0 and results[0][3] == 0
    print("line source: stage 3 flagged", results[2][3], "of", results[2][4], "tiles,", results[2][5],
          "stored without their box")
    assert results[2][3] > 0
