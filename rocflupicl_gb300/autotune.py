"""Launch-configuration autotuner.

The engine's kernels walk a tile list; a launch either gives every tile its
own block or runs a persistent grid that strides over the tiles.  For a batch
of many uneven meshes the best grid size depends on the mix, so it is chosen
by timing real steps (CUDA events on the batch's stream) over candidate grid
sizes in multiples of the SM count, and the fastest is kept.  The steps taken
while tuning advance the solution like any other step.
"""
from __future__ import annotations

import ctypes as C
from typing import Dict, Sequence

from . import engine as E


def sm_count() -> int:
    """The current GPU's SM count (cudaDevAttrMultiProcessorCount)."""
    return E.sm_count()


def tune_batch(batch: "E.Batch", cfl: float, dt_imposed: float = 1.0, end_time: float = 0.0,
               candidates: Sequence[int] = None, steps: int = 2) -> Dict[str, object]:
    sms = sm_count()
    if candidates is None:
        candidates = [0] + [sms * k for k in (2, 4, 8, 16, 32)]
    timings = {}
    for g in candidates:
        batch.set_grid_cap(g)
        batch.step(cfl, dt_imposed, 0.0, end_time)   # settle
        batch.timer_start()
        for _ in range(steps):
            batch.step(cfl, dt_imposed, 0.0, end_time)
        timings[g] = batch.timer_stop() / steps
    best = min(timings, key=timings.get)
    batch.set_grid_cap(best)
    return {"grid_cap": best, "ms_per_step": timings, "sms": sms,
            "steps_taken": (steps + 1) * len(candidates)}
