"""Runners for the secondary benchmark workloads (bench.py --workload ...).

  sod    1000x2x2 Sod tube, FP64, AUSM+, Wray RK3, CFL 0.5 to t = 0.2
  mixed  96^3 mixed hex/prism/tet/pyramid box, single residual repeated,
         all three flux schemes, FP64 and mixed precision
  tubes  256 independent n x 2 x 2 shock tubes (n log-uniform in
         [500, 125000]), mixed precision, one batched launch per pass over all
         tubes, CUDA-graph replay of whole steps, autotuned persistent grid
  partitioned
         the n^3 x 6 tet shock box cut into 2, 4 and 8 slab regions with
         virtual cells, advanced as one coupled batch (one device time step,
         the halo exchange after every stage), against the same mesh as one
         region

Every runner times on the device with the engine's CUDA-event timers and
returns a dict; face-flux evaluations count interior + boundary faces per
stage (per residual for `mixed`).
"""
from __future__ import annotations

import time

import numpy as np

from . import autotune
from . import case as K
from . import engine as E
from . import perfmodel


def _evals(m, stages):
    return (m.nFaces + m.nBFaces) * stages


def run_sod(steps_cap: int = 5000) -> dict:
    c = K.shock_tube(1000, numerics=K.Numerics(venkatGuard=1))
    r = E.Region(c)
    dti = r.time_step(c.numerics.cfl, 1.0, 0.0, 1.0)
    r.set_time(0.0)
    r.step(c.numerics.cfl, dti, 0.0, 0.2)    # first step (warm)
    r.sync()
    r.set_time(0.0)
    r.upload(c.cv, c.dv)
    r.timer_start()
    steps = 0
    chunk = 100
    while steps < steps_cap:
        r.steps_graph(chunk, c.numerics.cfl, dti, 0.0, 0.2)
        steps += chunk
        t, _ = r.time()
        if t >= 0.2:
            break
    ms = r.timer_stop()
    cv, dv = r.download()
    st = r.status()
    r.close()
    # steps that advanced time: the clip makes later ones no-ops
    return {"workload": "sod 1000x2x2 FP64 AUSM+ Venkat(guarded) Wray CFL 0.5 to t=0.2",
            "cells": c.mesh.nCells, "time_to_solution_ms": ms, "graph_steps": steps,
            "status": st, "t_final": t}


def run_mixed_residual(repeats: int = 1000, n: int = 96) -> dict:
    c0 = K.mixed_box(n)
    m = c0.mesh
    out = {"workload": f"mixed-element box {n}^3: hex/prism/tet/pyramid, single residual x{repeats}",
           "cells": m.nCells, "faces": m.nFaces, "bfaces": m.nBFaces, "members": m.nMembs,
           "types": {"tet": m.n_of_type[0], "hex": m.n_of_type[1], "prism": m.n_of_type[2],
                     "pyramid": m.n_of_type[3]}, "runs": {}}
    for prec, pname in ((K.PREC_MIXED, "mixed"), (K.PREC_FP64, "fp64")):
        for scheme, sname in ((K.DISCR_UPW_AUSMPLUS, "ausm+"), (K.DISCR_UPW_ROE, "roe"),
                              (K.DISCR_UPW_HLLC, "hllc")):
            c = c0.with_numerics(precision=prec, spaceDiscr=scheme, venkatGuard=1)
            r = E.Region(c)
            reps = repeats if prec == K.PREC_MIXED else max(10, repeats // 20)
            for _ in range(3):
                r.residual(to_host=False)
            r.timer_start()
            for _ in range(reps):
                r.residual(to_host=False)
            ms = r.timer_stop()
            r.close()
            s = 4 if prec == K.PREC_MIXED else 8
            b = perfmodel.residual_bytes(m.nCells, m.nFaces, m.nBFaces, m.nMembs, s)
            out["runs"][f"{pname}/{sname}"] = {
                "repeats": reps, "ms_per_residual": ms / reps,
                "face_flux_evals_per_s": _evals(m, reps) / (ms * 1e-3),
                "algorithmic_gbs": b / (ms / reps * 1e-3) / 1e9}
    return out


def run_tubes(steps: int = 300, count: int = 256, seed: int = 11, cross: int = 2) -> dict:
    t0 = time.perf_counter()
    cases = K.tube_ensemble(count=count, seed=seed, cross=cross, n_steps=steps,
                            numerics=K.Numerics(precision=K.PREC_MIXED, venkatGuard=1))
    build_s = time.perf_counter() - t0
    regs = [E.Region(c) for c in cases]
    cfl = cases[0].numerics.cfl
    for r in regs:
        dti = r.time_step(cfl, 1.0, 0.0, 1.0)
        r.set_time(0.0)
        r.step(cfl, dti)                 # each tube's first (dtImposed) step
        r.sync()
    b = E.Batch(regs)
    tune = autotune.tune_batch(b, cfl)
    done = 1 + tune["steps_taken"]
    todo = max(steps - done, 1)
    b.steps_graph(1, cfl, 1.0)        # build the graph
    b.sync()
    b.timer_start()
    b.steps_graph(todo, cfl, 1.0)
    ms = b.timer_stop()
    cells = sum(c.mesh.nCells for c in cases)
    evals = sum(_evals(c.mesh, 3) for c in cases) * todo
    stats = [r.status() for r in regs]
    dev = sum(r.device_bytes for r in regs)
    b.close()
    for r in regs:
        r.close()
    return {"workload": f"{count} shock tubes n x {cross} x {cross}, n log-uniform [500,125000], "
                        f"mixed, batched persistent launch + CUDA graph",
            "tubes": count, "cells": cells, "cells_min": min(c.mesh.nCells for c in cases),
            "cells_max": max(c.mesh.nCells for c in cases), "steps_total": steps,
            "timed_steps": todo, "ms_per_step": ms / todo, "face_flux_evals_per_s": evals / (ms * 1e-3),
            "autotune": tune, "status_any": int(np.bitwise_or.reduce(stats)),
            "device_bytes": dev, "host_build_s": build_s}


def run_partitioned(n: int = 64, parts=(2, 4, 8), steps: int = 50,
                    precision: int = K.PREC_MIXED) -> dict:
    from . import partition as P
    num = K.Numerics(spaceDiscr=K.DISCR_UPW_ROE, venkatGuard=1, precision=precision)
    c = K.tet_shock_box(n, numerics=num)
    m = c.mesh
    cfl = num.cfl
    whole_evals = _evals(m, 3) * steps
    out = {"workload": f"tet_shock_box {n}^3x6 Kuhn tets, Roe, WLSQ+Venkatakrishnan, Wray RK3, "
                       f"{'mixed' if precision == K.PREC_MIXED else 'fp64'}; slab regions as one "
                       f"coupled batch vs one region",
           "cells": m.nCells, "faces": m.nFaces, "steps": steps, "runs": {}}
    r = E.Region(c)
    d0 = r.time_step(cfl, 1.0, 0.0, 1.0)
    r.set_time(0.0)
    r.steps_graph(1, cfl, d0)
    r.sync()
    r.timer_start()
    r.steps_graph(steps, cfl, d0)
    ms1 = r.timer_stop()
    cv1, _ = r.download()
    r.close()
    out["runs"]["1"] = {"ms_per_step": ms1 / steps,
                        "face_flux_evals_per_s": whole_evals / (ms1 * 1e-3)}
    for np_ in parts:
        t0 = time.perf_counter()
        cases = P.partition_case(c, np_)
        part_s = time.perf_counter() - t0
        regs = [E.Region(p) for p in cases]
        d0 = min(x.time_step(cfl, 1.0, 0.0, 1.0) for x in regs)
        for x in regs:
            x.set_time(0.0)
            x.sync()
        b = E.Batch(regs, coupled=True)
        b.steps_graph(1, cfl, d0)
        b.sync()
        b.profile(True)
        b.step(cfl, d0)
        prof = b.profile_read()
        b.profile(False)
        b.timer_start()
        b.steps_graph(steps, cfl, d0)
        ms = b.timer_stop()
        for x, p in zip(regs, cases):
            p.cv[:], _ = x.download()
        st = int(np.bitwise_or.reduce([x.status() for x in regs]))
        g = P.gather(cases, "cv")
        b.close()
        for x in regs:
            x.close()
        tot = sum(p.mesh.nTot for p in cases)
        out["runs"][str(np_)] = {
            "ms_per_step": ms / steps, "face_flux_evals_per_s": whole_evals / (ms * 1e-3),
            "cells_with_virtual": tot, "virtual_fraction": tot / m.nCells - 1.0,
            "faces_computed": sum(p.mesh.nFaces for p in cases),
            "halo_cells": sum(sum(len(bd.icgRecv) for bd in p.mesh.borders) for p in cases),
            "halo_ms_per_stage": prof["halo"][0] / max(1, prof["halo"][1]),
            "status": st, "partition_host_s": part_s,
            "l1_rho_vs_one_region": float(np.abs(g[:, 0] - cv1[:, 0]).sum() / np.abs(cv1[:, 0]).sum()),
        }
    return out
