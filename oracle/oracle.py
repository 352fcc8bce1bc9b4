"""ctypes front end of the CPU oracle (rflu_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by the
benchmark's CPU-baseline / reference leg as the checker.  The engine package
never imports it.  Parity against reference outputs is unpinned (no runnable
reference, no golden vectors for this path); the oracle is pinned to the
reference-defined known answers in tests/test_oracle_kats.py.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "liborc.so"
MAXP = 16

_lib = None


def build(force: bool = False) -> Path:
    src = HERE / "rflu_oracle.cpp"
    hdr = HERE / "rflu_oracle.h"
    BUILD.mkdir(exist_ok=True)
    if force or not LIB.exists() or max(src.stat().st_mtime, hdr.stat().st_mtime) > LIB.stat().st_mtime:
        cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
               "-fno-fast-math", str(src), "-o", str(LIB)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


class OrcPatch(C.Structure):
    _fields_ = [("bcType", C.c_int), ("spaceOrder", C.c_int), ("bcOptType", C.c_int),
                ("nBFaces", C.c_int), ("bf2c", C.POINTER(C.c_int)), ("fn", C.POINTER(C.c_double)),
                ("fc", C.POINTER(C.c_double)), ("vals", C.POINTER(C.c_double)),
                ("distrib", C.c_int), ("nData", C.c_int),
                ("bcOptFixed", C.c_int), ("nBFacesTot", C.c_int)]


class OrcRegion(C.Structure):
    _fields_ = [("nCells", C.c_int), ("nFaces", C.c_int), ("nPatches", C.c_int),
                ("f2c", C.POINTER(C.c_int)), ("fn", C.POINTER(C.c_double)),
                ("fc", C.POINTER(C.c_double)), ("cofg", C.POINTER(C.c_double)),
                ("vol", C.POINTER(C.c_double)), ("csOff", C.POINTER(C.c_int)),
                ("csMem", C.POINTER(C.c_int)), ("xyzMoms", C.POINTER(C.c_double)),
                ("patches", OrcPatch * MAXP),
                ("spaceDiscr", C.c_int), ("spaceOrder", C.c_int), ("reconst", C.c_int),
                ("rkScheme", C.c_int), ("refCp", C.c_double), ("refGamma", C.c_double),
                ("gvCp", C.c_double), ("gvMol", C.c_double), ("epsentr", C.c_double),
                ("dissFact", C.c_double), ("venkatGuard", C.c_int),
                ("ausmSigma", C.c_double), ("ausmKp", C.c_double), ("ausmKu", C.c_double),
                ("ausmMInf", C.c_double), ("nCellsTot", C.c_int), ("nFacesAll", C.c_int)]


def _load():
    global _lib
    if _lib is None:
        lib = C.CDLL(str(build()))
        R = C.POINTER(OrcRegion)
        dp = C.POINTER(C.c_double)
        lib.orc_rk_stage.argtypes = [R, C.c_int, C.c_double] + [dp] * 6
        lib.orc_rk_stage.restype = C.c_int
        lib.orc_rk_stage_omp.argtypes = [R, C.c_int, C.c_double] + [dp] * 6 + [C.c_int]
        lib.orc_rk_stage_omp.restype = C.c_int
        lib.orc_residual.argtypes = [R, dp, dp, dp, dp]
        lib.orc_dt.argtypes = [R, dp, dp, C.c_double, C.c_double, C.c_double, C.c_double]
        lib.orc_dt.restype = C.c_double
        lib.orc_omp_plan_create.argtypes = [R]
        lib.orc_omp_plan_create.restype = C.c_void_p
        lib.orc_omp_plan_destroy.argtypes = [C.c_void_p]
        lib.orc_rk_stage_omp_plan.argtypes = [R, C.c_void_p, C.c_int, C.c_double] + [dp] * 6 + [C.c_int]
        lib.orc_rk_stage_omp_plan.restype = C.c_int
        lib.orc_dt_omp.argtypes = [R, C.c_void_p, dp, dp, C.c_double, C.c_double, C.c_double,
                                   C.c_double, C.c_int]
        lib.orc_dt_omp.restype = C.c_double
        lib.orc_set_dv.argtypes = [R, dp, dp]
        lib.orc_set_dv_range.argtypes = [R, dp, dp, C.c_long, C.c_long]
        lib.orc_face_flux.argtypes = [R, dp, dp, dp, dp]
        _lib = lib
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


class Oracle:
    """The oracle bound to one case's mesh, boundary conditions and numerics."""

    def __init__(self, case):
        self.lib = _load()
        m, num = case.mesh, case.numerics
        self._keep = []

        def keep(a, dt):
            a = np.ascontiguousarray(a, dtype=dt)
            self._keep.append(a)
            return a

        reg = OrcRegion()
        reg.nCells, reg.nFaces = m.nCells, m.nFaces
        reg.nCellsTot = m.nTot
        f2c, fn, fc = m.all_faces()   # flux faces, then a region's VV / VX faces
        reg.nFacesAll = m.nFacesAll
        reg.f2c = _ip(keep(f2c, np.int32))
        reg.fn = _dp(keep(fn, np.float64))
        reg.fc = _dp(keep(fc, np.float64))
        reg.cofg = _dp(keep(m.cofg, np.float64))
        reg.vol = _dp(keep(m.vol, np.float64))
        reg.csOff = _ip(keep(m.c2cs_off, np.int32))
        reg.csMem = _ip(keep(m.c2cs_mem, np.int32))
        reg.xyzMoms = _dp(keep(m.xyzmoms, np.float64))
        np_ = 0
        for p, bc in zip(m.patches, case.bcs):
            if p.n == 0 and p.n_vb == 0:
                continue
            P = reg.patches[np_]
            P.bcType, P.spaceOrder, P.bcOptType, P.nBFaces = bc.bcType, bc.spaceOrder, bc.bcOptType, p.n
            bf2c, bfn, bfc = p.all_faces()   # a region's VB faces after the actual ones
            P.nBFacesTot = p.n + p.n_vb
            P.bf2c = _ip(keep(bf2c, np.int32))
            P.fn = _dp(keep(bfn, np.float64))
            P.fc = _dp(keep(bfc, np.float64))
            vals, nd, dist = bc.vals_array(p.n)
            P.vals = _dp(keep(vals, np.float64))
            P.distrib, P.nData = dist, nd
            P.bcOptFixed = bc.bcOptFixed
            np_ += 1
        reg.nPatches = np_
        reg.spaceDiscr, reg.spaceOrder, reg.reconst, reg.rkScheme = (
            num.spaceDiscr, num.spaceOrder, num.reconst, num.rkScheme)
        reg.refCp, reg.refGamma = num.refCp, num.refGamma
        reg.gvCp, reg.gvMol = num.gv
        reg.epsentr, reg.dissFact = num.epsentr, num.dissFact
        reg.venkatGuard = num.venkatGuard
        reg.ausmSigma, reg.ausmKp, reg.ausmKu, reg.ausmMInf = (
            num.ausmSigma, num.ausmKp, num.ausmKu, num.ausmMInf)
        self.reg = reg
        self.nCells = m.nTot      # rows of every per-cell array (actual + virtual)
        self.nAct = m.nCells
        self.num = num
        n = m.nTot
        self.cvOld = np.zeros((n, 5))
        self.rhs = np.zeros((n, 5))
        self.rhsSum = np.zeros((n, 5))
        self.grad = np.zeros((n, 5, 3))

    def _omp_plan(self):
        """The OpenMP path's cell -> face lists, built on first use."""
        if getattr(self, "_plan", None) is None:
            self._plan = self.lib.orc_omp_plan_create(C.byref(self.reg))
        return self._plan

    def __del__(self):
        plan = getattr(self, "_plan", None)
        if plan is not None:
            self.lib.orc_omp_plan_destroy(plan)
            self._plan = None

    def stage(self, cv, dv, istage, dtMin, threads: int = 0) -> int:
        """One RK stage in place on cv, dv (C-contiguous float64); threads > 0
        runs the OpenMP form (bit-identical)."""
        bufs = (_dp(cv), _dp(dv), _dp(self.cvOld), _dp(self.rhs), _dp(self.rhsSum),
                _dp(self.grad))
        if threads:
            return self.lib.orc_rk_stage_omp_plan(C.byref(self.reg), self._omp_plan(), istage,
                                                  dtMin, *bufs, threads)
        return self.lib.orc_rk_stage(C.byref(self.reg), istage, dtMin, *bufs)

    def residual(self, cv, dv):
        rhs = np.zeros((self.nCells, 5))
        grad = np.zeros((self.nCells, 5, 3))
        self.lib.orc_residual(C.byref(self.reg), _dp(np.ascontiguousarray(cv)),
                              _dp(np.ascontiguousarray(dv)), _dp(rhs), _dp(grad))
        return rhs, grad

    def dt(self, cv, dv, cfl, dtImposed, dtMinLimit=0.0, currentTime=1.0, threads: int = 0):
        if threads:
            return self.lib.orc_dt_omp(C.byref(self.reg), self._omp_plan(), _dp(cv), _dp(dv),
                                       cfl, dtImposed, dtMinLimit, currentTime, threads)
        return self.lib.orc_dt(C.byref(self.reg), _dp(cv), _dp(dv), cfl, dtImposed, dtMinLimit,
                               currentTime)

    def set_dv(self, cv):
        dv = np.zeros((self.nCells, 3))
        self.lib.orc_set_dv(C.byref(self.reg), _dp(np.ascontiguousarray(cv)), _dp(dv))
        return dv

    def set_dv_range(self, cv, dv, first, last):
        """dv(first:last) from cv in place (RFLU_SetVarsContWrapper over a range)."""
        self.lib.orc_set_dv_range(C.byref(self.reg), _dp(cv), _dp(dv), first, last)

    def face_flux(self, left, right, n):
        f = np.zeros(5)
        self.lib.orc_face_flux(C.byref(self.reg), _dp(np.asarray(left, np.float64)),
                               _dp(np.asarray(right, np.float64)), _dp(np.asarray(n, np.float64)),
                               _dp(f))
        return f

    def run(self, cv, dv, n_steps=None, t_end=None, dt_imposed=None, threads=0, stages=None):
        """Time loop of rocflu/RFLU_TimeStepping.F90:453-494: dt from
        RFLU_TimeStepInviscid/MinimumTimeStep, clipped to the end time, then
        nrkSteps stages.  Returns (time, steps, status)."""
        nst = {1: 4, 2: 3, 3: 1}[self.num.rkScheme]
        t, k, st = 0.0, 0, 0
        if dt_imposed is None:
            dt_imposed = self.dt(cv, dv, self.num.cfl, 1.0, 0.0, 1.0)
        while True:
            if n_steps is not None and k >= n_steps:
                break
            if t_end is not None and t >= t_end:
                break
            dtm = self.dt(cv, dv, self.num.cfl, dt_imposed, 0.0, t, threads)
            finished = False
            if t_end is not None and t + dtm > t_end:  # RFLU_TimeStepping.F90:490-493
                dtm = t_end - t
                finished = True
            for s in range(1, nst + 1):
                st |= self.stage(cv, dv, s, dtm, threads)
            t += dtm
            k += 1
            if finished:
                break
        return t, k, st


class MultiOracle:
    """The oracle over the regions of one partitioned case
    (libfloflu/RungeKuttaMP.F90:190-396 with nRegionsLocal regions): every
    region's stage, then the halo exchange of every border
    (RFLU_MPI_CopyWrapper: cv of the send cells into the neighbour's receive
    cells) and the dependent variables of the received virtual cells
    (RFLU_SetVarsContWrapper(nCells+1,nCellsTot)); one time step, the minimum
    over the regions (RFLU_MinimumTimeStep)."""

    def __init__(self, cases):
        self.cases = list(cases)
        self.orcs = [Oracle(c) for c in self.cases]
        self.num = self.cases[0].numerics
        ids = [c.mesh.iRegionGlobal for c in self.cases]
        self.index = {g: i for i, g in enumerate(ids)}

    def exchange(self, cvs, dvs):
        for r, c in enumerate(self.cases):
            for b in c.mesh.borders:
                s = self.index[b.iRegionGlobal]
                b2 = self.cases[s].mesh.borders[b.iBorder - 1]
                cvs[s][b2.icgRecv - 1] = cvs[r][b.icgSend - 1]
        for s, o in enumerate(self.orcs):
            o.set_dv_range(cvs[s], dvs[s], o.nAct, o.nCells)

    def dt(self, cvs, dvs, cfl, dtImposed, dtMinLimit=0.0, currentTime=1.0):
        return min(o.dt(cv, dv, cfl, dtImposed, dtMinLimit, currentTime)
                   for o, cv, dv in zip(self.orcs, cvs, dvs))

    def stage(self, cvs, dvs, istage, dtMin) -> int:
        st = 0
        for o, cv, dv in zip(self.orcs, cvs, dvs):
            st |= o.stage(cv, dv, istage, dtMin)
        self.exchange(cvs, dvs)
        return st

    def run(self, cvs, dvs, n_steps=None, t_end=None, dt_imposed=None):
        """Time loop as Oracle.run over all regions.  Returns (time, steps, status)."""
        nst = {1: 4, 2: 3, 3: 1}[self.num.rkScheme]
        t, k, st = 0.0, 0, 0
        if dt_imposed is None:
            dt_imposed = self.dt(cvs, dvs, self.num.cfl, 1.0, 0.0, 1.0)
        while True:
            if n_steps is not None and k >= n_steps:
                break
            if t_end is not None and t >= t_end:
                break
            dtm = self.dt(cvs, dvs, self.num.cfl, dt_imposed, 0.0, t)
            finished = False
            if t_end is not None and t + dtm > t_end:
                dtm = t_end - t
                finished = True
            for s in range(1, nst + 1):
                st |= self.stage(cvs, dvs, s, dtm)
            t += dtm
            k += 1
            if finished:
                break
        return t, k, st
