"""Continuous-batching serving loop for solve requests.

Requests (jittered-tet shock boxes of seeded size, Mach number and flux
scheme) arrive as a Poisson stream.  Each is prepared by a thread pool as soon
as it arrives (mesh, face list and geometry on the host; c2c stencils and
moments on the GPU; initial state), admitted to
the GPU when its device footprint fits the HBM budget, takes its first
(dtImposed) step alone, and then joins the batch: every iteration advances all
active solves by one time step with one launch per pass over all of them
(rfgpu_batch_step).  A solve that reaches the end time is retired (state read
back, device memory freed) and its slot goes to the next ready request.

Each solve's arithmetic is independent of its batch mates (per-region tiles,
time step and end-time clip), so its result is the same alone and in any mix.
"""
from __future__ import annotations

import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from . import case as K
from . import engine as E

SCHEMES = [K.DISCR_UPW_AUSMPLUS, K.DISCR_UPW_ROE, K.DISCR_UPW_HLLC]


@dataclass
class Request:
    rid: int
    arrival: float      # seconds after the stream starts
    n: int              # base hexes per direction (cells = 6 n^3)
    Ms: float
    scheme: int
    seed: int

    @property
    def cells(self) -> int:
        return 6 * self.n ** 3


@dataclass
class Result:
    rid: int
    cells: int
    steps: int
    face_evals: int
    latency: float       # arrival -> state read back
    queue: float         # arrival -> admission
    t_final: float
    cv: Optional[np.ndarray] = None
    dv: Optional[np.ndarray] = None


def poisson_requests(count: int, lam: float, seed: int, cells_min: int = 10_000,
                     cells_max: int = 4_000_000) -> List[Request]:
    """Seeded Poisson arrivals (rate lam per second); cell counts log-uniform
    in [cells_min, cells_max] quantised to 6 k^3, k = round((Nc/6)^(1/3));
    Ms uniform in [1.2, 3]; flux scheme uniform over AUSM+/Roe/HLLC."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / lam, count))
    nc = np.exp(rng.uniform(np.log(cells_min), np.log(cells_max), count))
    ks = np.maximum(2, np.round((nc / 6.0) ** (1.0 / 3.0)).astype(int))
    ms = rng.uniform(1.2, 3.0, count)
    sch = rng.integers(0, 3, count)
    return [Request(i, float(t[i]), int(ks[i]), float(ms[i]), SCHEMES[int(sch[i])],
                    int(seed * 100003 + i)) for i in range(count)]


def build_case(req: Request, precision: int = K.PREC_MIXED, threads: int = 4,
               stencils: str = "all-device") -> K.Case:
    """The request's mesh and initial state.  stencils="all-device" builds the
    face list, geometry, vertex-to-cell lists, c2c stencils and WLSQ moments
    on the GPU (identical to the host builder's), leaving the vertex and cell
    generation on the host; "device" builds only the stencils and moments
    there."""
    num = K.Numerics(spaceDiscr=req.scheme, precision=precision, venkatGuard=1)
    return K.tet_shock_box(req.n, seed=req.seed, Ms=req.Ms, numerics=num, threads=threads,
                           stencils=stencils)


@dataclass
class _Active:
    req: Request
    case: K.Case
    region: E.Region
    admitted: float
    steps: int = 0


class Server:
    """Admission by HBM footprint, device-resident state per solve,
    continuous batching of all active solves."""

    def __init__(self, t_end: float, hbm_budget: Optional[int] = None,
                 precision: int = K.PREC_MIXED, prepare_workers: int = 4,
                 mesh_threads: int = 4, keep_state: bool = False,
                 bytes_per_cell: float = 800.0, max_steps: int = 100000,
                 stencils: str = "all-device"):
        self.t_end = t_end
        self.stencils = stencils
        self.max_steps = max_steps
        self.precision = precision
        self.keep_state = keep_state
        self.prepare_workers = prepare_workers
        self.mesh_threads = mesh_threads
        self.bytes_per_cell = bytes_per_cell
        if hbm_budget is None:
            free, _ = E.mem_info()
            hbm_budget = int(free * 0.85)
        self.hbm_budget = hbm_budget
        self.max_active = 0
        self.iterations = 0
        self.batch_launches = 0

    @staticmethod
    def _open(c: K.Case):
        """Register a prepared case (host-side layout build, device upload) and
        take its initial CFL time step; runs on a pool thread so the batch
        keeps stepping meanwhile."""
        reg = E.Region(c)
        dti = reg.time_step(c.numerics.cfl, 1.0, 0.0, 1.0)
        reg.set_time(0.0)
        return reg, dti

    def run(self, requests: List[Request]) -> Dict[int, Result]:
        reqs = sorted(requests, key=lambda r: r.arrival)
        pool = ThreadPoolExecutor(self.prepare_workers)
        preparing = {}
        opening = {}
        ready: List = []
        active: List[_Active] = []
        results: Dict[int, Result] = {}
        used = 0
        batch = None
        dirty = False
        nxt = 0
        t0 = time.perf_counter()
        cfl = 0.5
        try:
            while len(results) < len(reqs):
                now = time.perf_counter() - t0
                while nxt < len(reqs) and reqs[nxt].arrival <= now:
                    r = reqs[nxt]
                    preparing[r.rid] = (r, pool.submit(build_case, r, self.precision,
                                                       self.mesh_threads, self.stencils))
                    nxt += 1
                for rid in [k for k, (_, f) in preparing.items() if f.done()]:
                    r, f = preparing.pop(rid)
                    ready.append((r, f.result()))
                ready.sort(key=lambda x: x[0].arrival)
                # admission: first come first served while the footprint fits; the
                # footprint is reserved and the region is opened on a pool thread
                while ready:
                    r, c = ready[0]
                    need = int(self.bytes_per_cell * c.mesh.nCells)
                    if (active or opening) and used + need > self.hbm_budget:
                        break
                    ready.pop(0)
                    used += need
                    opening[r.rid] = (r, c, need, pool.submit(self._open, c))
                for rid in [k for k, v in opening.items() if v[3].done()]:
                    r, c, need, f = opening.pop(rid)
                    reg, dti = f.result()
                    cfl = c.numerics.cfl
                    reg.step(cfl, dti, 0.0, self.t_end)   # first step: its own dtImposed
                    reg.sync()
                    used += reg.device_bytes - need
                    active.append(_Active(r, c, reg, time.perf_counter() - t0, 1))
                    dirty = True
                if active:
                    if dirty:
                        if batch is not None:
                            batch.close()
                        batch = E.Batch([a.region for a in active])
                        dirty = False
                    batch.step(cfl, 1.0, 0.0, self.t_end)
                    batch.sync()
                    self.iterations += 1
                    self.max_active = max(self.max_active, len(active))
                    keep = []
                    for a in active:
                        a.steps += 1
                        t, _ = a.region.time()
                        if not np.isfinite(t) or a.steps > self.max_steps:
                            raise RuntimeError(f"request {a.req.rid}: time {t} after {a.steps} "
                                               f"steps (status {a.region.status()})")
                        if t >= self.t_end:
                            self._retire(a, results, t0)
                            used -= a.region.device_bytes
                            a.region.close()
                            dirty = True
                        else:
                            keep.append(a)
                    active = keep
                    if not active and batch is not None:
                        batch.close()
                        batch = None
                else:
                    time.sleep(0.0005)
        finally:
            pool.shutdown(wait=True)
            for _, _, _, f in opening.values():
                if f.done() and f.exception() is None:
                    f.result()[0].close()
            if batch is not None:
                batch.close()
            for a in active:
                a.region.close()
        return results

    def _retire(self, a: _Active, results, t0):
        m = a.case.mesh
        # steps actually advancing time: the counted ones minus trailing no-op
        # steps cannot occur (a solve retires on the step that reaches t_end)
        cv = dv = None
        if self.keep_state:
            cv, dv = a.region.download()
        else:
            a.region.sync()
        t, _ = a.region.time()
        done = time.perf_counter() - t0
        results[a.req.rid] = Result(a.req.rid, m.nCells, a.steps,
                                    3 * (m.nFaces + m.nBFaces) * a.steps,
                                    done - a.req.arrival, a.admitted - a.req.arrival, t, cv, dv)


def solve_alone(req: Request, t_end: float, precision: int = K.PREC_MIXED,
                max_steps: int = 100000, stencils: str = "all-device"):
    """The same request run by itself: first step with its own dtImposed, then
    device steps to the end time."""
    c = build_case(req, precision, stencils=stencils)
    r = E.Region(c)
    cfl = c.numerics.cfl
    dti = r.time_step(cfl, 1.0, 0.0, 1.0)
    r.set_time(0.0)
    steps = 0
    while True:
        r.step(cfl, dti, 0.0, t_end)
        steps += 1
        t, _ = r.time()
        if not np.isfinite(t) or steps > max_steps:
            raise RuntimeError(f"request {req.rid}: time {t} after {steps} steps")
        if t >= t_end:
            break
    cv, dv = r.download()
    r.close()
    return cv, dv, steps


def summarize(results: Dict[int, Result], wall: float) -> dict:
    lat = np.array([r.latency for r in results.values()])
    evals = sum(r.face_evals for r in results.values())
    slow = sorted(results.values(), key=lambda r: -r.latency)[:3]
    return {"requests": len(results), "p50_s": float(np.percentile(lat, 50)),
            "p99_s": float(np.percentile(lat, 99)), "mean_s": float(lat.mean()),
            "slowest": [{"cells": r.cells, "latency_s": r.latency, "admitted_after_s": r.queue,
                         "steps": r.steps} for r in slow],
            "face_evals": int(evals), "wall_s": wall, "face_evals_per_s": evals / wall,
            "cells_total": int(sum(r.cells for r in results.values()))}
