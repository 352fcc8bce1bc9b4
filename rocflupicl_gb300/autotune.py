"""Launch-configuration autotuner.

The engine's passes walk tile lists; what a launch looks like is a choice the
results do not depend on (every per-cell sum keeps its order), so it is made
by timing real steps on the device:

* the device numbering of cells and faces (locality order or the host's),
  chosen at registration (`tune_order`);
* per pass, its block size: the gradient + limiter pass (`gradBlock`), the
  interior-face flux pass (`faceBlock`, with `facesPerThread` faces per
  thread) and the residual gather + update pass (`cellBlock`), 64 / 128 / 256;
* the persistent grid (`gridCap`): one block per tile, or a grid of a few
  blocks per SM walking the tiles (multiples of the SM count the device
  reports);
* one cooperative launch per RK stage (`persistentStage`) against one launch
  per pass, on whole steps.

The search is coordinate descent from the default shape: each knob in turn
takes its candidates with the others fixed, judged by the CUDA-event time of
the pass it shapes (the engine's per-kernel profiler, on the handle's stream)
or, for the grid, of the whole step; the best is kept.  The steps taken while
tuning advance the solution like any other step.
"""
from __future__ import annotations

from typing import Dict, Sequence

from . import engine as E

BLOCKS = (64, 128, 256)
KNOB_KERNEL = {"gradBlock": "gradient", "faceBlock": "face_flux", "facesPerThread": "face_flux",
               "cellBlock": "gather_update", "gridCap": None}


def sm_count() -> int:
    """The current GPU's SM count (cudaDevAttrMultiProcessorCount)."""
    return E.sm_count()


def _measure(h, shape: Dict[str, int], step, steps: int, kernel) -> float:
    """ms per step of the whole step (kernel None) or of one pass."""
    h.set_tuning(**shape)
    step()                                  # settle (first launch of a shape)
    h.sync()
    h.profile(True)
    h.timer_start()
    for _ in range(steps):
        step()
    ms = h.timer_stop()
    prof = h.profile_read()
    h.profile(False)
    if kernel is None:
        return ms / steps
    t, n = prof.get(kernel, (0.0, 0))
    return t / max(n, 1) if n else ms / steps


def _descend(h, step, steps: int, knobs: Dict[str, Sequence[int]],
             persistent: bool = False) -> Dict[str, object]:
    shape = {k: 0 for k in E.TUNING_KEYS}
    timings: Dict[str, Dict[int, float]] = {}
    taken = 0
    for knob, cands in knobs.items():
        kernel = KNOB_KERNEL[knob]
        res = {}
        for v in cands:
            trial = dict(shape, **{knob: v})
            res[v] = _measure(h, trial, step, steps, kernel)
            taken += steps + 1
        best = min(res, key=res.get)
        shape[knob] = best
        timings[knob] = res
    if persistent:
        # one cooperative launch per stage (default block shapes, the chosen
        # grid cap) against the best per-pass shape, whole steps
        res = {0: _measure(h, shape, step, steps, None)}
        coop = {k: 0 for k in E.TUNING_KEYS}
        coop.update(gridCap=shape["gridCap"], persistentStage=1)
        res[1] = _measure(h, coop, step, steps, None)
        taken += 2 * (steps + 1)
        timings["persistentStage"] = res
        if res[1] < res[0]:
            shape = coop
    h.set_tuning(**shape)
    return {"shape": shape, "ms": timings, "steps_taken": taken}


def tune_region(region: "E.Region", cfl: float, dt_imposed: float, end_time: float = 0.0,
                steps: int = 3, grid_caps: Sequence[int] = None) -> Dict[str, object]:
    """Tune one region's launch shapes on rfgpu_step.  Returns the shape kept
    and the per-candidate milliseconds (per launch of the pass a knob shapes,
    per step for the grid)."""
    sms = sm_count()
    if grid_caps is None:
        grid_caps = [0] + [sms * k for k in (4, 8, 16)]
    knobs = {"gradBlock": BLOCKS, "faceBlock": BLOCKS, "facesPerThread": (1, 2),
             "cellBlock": BLOCKS, "gridCap": grid_caps}
    out = _descend(region, lambda: region.step(cfl, dt_imposed, 0.0, end_time), steps, knobs,
                   persistent=True)
    out["sms"] = sms
    return out


def tune_batch(batch: "E.Batch", cfl: float, dt_imposed: float = 1.0, end_time: float = 0.0,
               candidates: Sequence[int] = None, steps: int = 2,
               blocks: bool = True) -> Dict[str, object]:
    """Tune a batch's launch shapes on rfgpu_batch_step (the grid cap first:
    for many uneven meshes it matters most)."""
    sms = sm_count()
    if candidates is None:
        candidates = [0] + [sms * k for k in (2, 4, 8, 16, 32)]
    knobs = {"gridCap": candidates}
    if blocks:
        knobs.update({"gradBlock": BLOCKS, "faceBlock": BLOCKS, "facesPerThread": (1, 2),
                      "cellBlock": BLOCKS})
    out = _descend(batch, lambda: batch.step(cfl, dt_imposed, 0.0, end_time), steps, knobs,
                   persistent=True)
    out["sms"] = sms
    out["grid_cap"] = out["shape"]["gridCap"]
    out["ms_per_step"] = out["ms"]["gridCap"]
    return out


def tune_order(case, steps: int = 3) -> Dict[str, object]:
    """Register the case in both device numberings, time rfgpu_step on each,
    and return the faster order (E.ORDER_LOCALITY or E.ORDER_HOST) with the
    milliseconds per step of both."""
    res = {}
    for order in (E.ORDER_LOCALITY, E.ORDER_HOST):
        r = E.Region(case, cell_order=order)
        cfl = case.numerics.cfl
        dti = r.time_step(cfl, 1.0, 0.0, 1.0)
        r.set_time(0.0)
        r.step(cfl, dti)
        r.sync()
        r.timer_start()
        for _ in range(steps):
            r.step(cfl, dti)
        res[order] = r.timer_stop() / steps
        r.close()
    best = min(res, key=res.get)
    return {"order": best, "ms_per_step": {"locality": res[E.ORDER_LOCALITY],
                                           "host": res[E.ORDER_HOST]}}
