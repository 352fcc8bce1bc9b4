"""Python front end of the residual engine (include/rfgpu.h).

Mirrors the reference's operator interface for the hot path:

  Region.rk_stage(istage, dtMin)   libfloflu/RungeKuttaMP.F90 per-region stage body
  Region.time_step(...)            RFLU_TimeStepInviscid + RFLU_MinimumTimeStep
  Region.residual()                CellGradientsMP + ConvectiveFluxesMP
  Region.step(...)                 one time step (dt + all stages) on the device
  Region.solve(...)                the RFLU_TimeStepping loop to an end time / step count

Errors raise `EngineError` carrying the C-ABI code, as the Fortran shim maps
them onto ErrorStop.  There is no CPU fallback: without the CUDA library or a
GPU every call fails.
"""
from __future__ import annotations

import ctypes as C
from typing import List, Optional, Sequence

import numpy as np

from . import _build
from .case import Case, PREC_FP64, PREC_MIXED, PREC_SPLIT  # noqa: F401

OK, ERR_ARG, ERR_UNSUPPORTED, ERR_CUDA, ERR_NOMEM, ERR_STATE, ERR_TIMEOUT, ERR_NOALLOC_LIMIT = range(8)
NOALLOC_SCRATCH_BYTES = 32 << 20
ST_NAN, ST_NEGPOS, ST_PFLOOR, ST_PCLAMP = 1, 2, 4, 8
_NAMES = {1: "RFGPU_ERR_ARG", 2: "RFGPU_ERR_UNSUPPORTED", 3: "RFGPU_ERR_CUDA",
          4: "RFGPU_ERR_NOMEM", 5: "RFGPU_ERR_STATE", 6: "RFGPU_ERR_TIMEOUT",
          7: "RFGPU_ERR_NOALLOC_LIMIT"}


class EngineError(RuntimeError):
    def __init__(self, code: int, where: str):
        super().__init__(f"{where}: {_NAMES.get(code, code)}")
        self.code = code


class PatchT(C.Structure):
    _fields_ = [("bcType", C.c_int), ("spaceOrder", C.c_int), ("bcOptType", C.c_int),
                ("nBFaces", C.c_int), ("bf2c", C.POINTER(C.c_int)), ("fn", C.POINTER(C.c_double)),
                ("fc", C.POINTER(C.c_double)), ("vals", C.POINTER(C.c_double)),
                ("distrib", C.c_int), ("nData", C.c_int),
                ("bcOptFixed", C.c_int), ("nBFacesTot", C.c_int)]


class BorderT(C.Structure):
    _fields_ = [("iRegionGlobal", C.c_int), ("iBorder", C.c_int), ("nCellsSend", C.c_int),
                ("icgSend", C.POINTER(C.c_int)), ("nCellsRecv", C.c_int),
                ("icgRecv", C.POINTER(C.c_int))]


class RegionDescT(C.Structure):
    _fields_ = [("nCells", C.c_int), ("nFaces", C.c_int), ("f2cLd", C.c_int),
                ("f2c", C.POINTER(C.c_int)), ("fn", C.POINTER(C.c_double)),
                ("fc", C.POINTER(C.c_double)), ("cofg", C.POINTER(C.c_double)),
                ("vol", C.POINTER(C.c_double)), ("c2csOffsets", C.POINTER(C.c_int)),
                ("c2csMembers", C.POINTER(C.c_int)), ("xyzMoms", C.POINTER(C.c_double)),
                ("nPatches", C.c_int), ("patches", C.POINTER(PatchT)),
                ("cv", C.POINTER(C.c_double)), ("dv", C.POINTER(C.c_double)),
                ("gasModel", C.c_int), ("flowModel", C.c_int),
                ("spaceDiscr", C.c_int), ("spaceOrder", C.c_int), ("reconst", C.c_int),
                ("rkScheme", C.c_int), ("refCp", C.c_double), ("refGamma", C.c_double),
                ("gvCp", C.c_double), ("gvMol", C.c_double), ("epsentr", C.c_double),
                ("dissFact", C.c_double), ("precision", C.c_int), ("venkatGuard", C.c_int),
                ("cellOrder", C.c_int), ("ausmSigma", C.c_double), ("ausmKp", C.c_double),
                ("ausmKu", C.c_double), ("ausmMInf", C.c_double), ("nCellsTot", C.c_int),
                ("iRegionGlobal", C.c_int), ("nBorders", C.c_int),
                ("borders", C.POINTER(BorderT)), ("nFacesAll", C.c_int)]


class TuningT(C.Structure):
    """rfgpu_tuning_t: launch shapes of the stage passes (0 = default)."""
    _fields_ = [("gridCap", C.c_int), ("gradBlock", C.c_int), ("faceBlock", C.c_int),
                ("facesPerThread", C.c_int), ("cellBlock", C.c_int),
                ("persistentStage", C.c_int)]


TUNING_KEYS = [f for f, _ in TuningT._fields_]


def _tuning(**kw) -> TuningT:
    t = TuningT()
    for k, v in kw.items():
        if k not in TUNING_KEYS:
            raise KeyError(k)
        setattr(t, k, int(v))
    return t


# device numbering of cells and faces (rfgpu.h RFGPU_ORDER_*)
ORDER_LOCALITY, ORDER_HOST = 0, 1


SYMBOLS = ["rfgpu_region_create", "rfgpu_region_destroy", "rfgpu_stage", "rfgpu_dt",
           "rfgpu_step", "rfgpu_steps_graph", "rfgpu_residual", "rfgpu_download",
           "rfgpu_upload", "rfgpu_step_host", "rfgpu_download_grad", "rfgpu_time",
           "rfgpu_set_time",
           "rfgpu_status", "rfgpu_sync", "rfgpu_stream", "rfgpu_device_bytes",
           "rfgpu_launch_count", "rfgpu_set_tuning", "rfgpu_batch_create",
           "rfgpu_batch_destroy", "rfgpu_batch_step", "rfgpu_batch_steps_graph",
           "rfgpu_batch_sync", "rfgpu_batch_stream", "rfgpu_profile", "rfgpu_profile_read",
           "rfgpu_batch_profile", "rfgpu_batch_profile_read", "rfgpu_batch_launch_count",
           "rfgpu_timer_start", "rfgpu_timer_stop", "rfgpu_batch_timer_start",
           "rfgpu_batch_timer_stop", "rfgpu_set_device", "rfgpu_host_alloc", "rfgpu_host_free",
           "rfgpu_mem_info", "rfgpu_sm_count", "rfgpu_residual_noalloc", "rfgpu_batch_set_tuning",
           "rfgpu_batch_test_barrier",
           "rfgpu_mesh_stencils", "rfgpu_border_copy", "rfgpu_border_pack",
           "rfgpu_border_unpack", "rfgpu_batch_create_ex", "rfgpu_mesh_build",
           "rfgpu_mesh_sizes", "rfgpu_mesh_faces", "rfgpu_mesh_cells", "rfgpu_mesh_patch",
           "rfgpu_mesh_destroy"]

BATCH_COUPLED = 1

KERNELS = ["gradient", "weno_xyz", "face_flux", "bface_flux", "gather_update", "dt_face",
           "dt_bface", "dt_cell", "dt_finalize", "halo", "stage_persistent"]

_lib = None


def load(path: Optional[str] = None):
    """Load (building if needed) librfgpu.so and declare the C signatures."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    lib = C.CDLL(str(path or _build.build_gpu()))
    vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int)
    d = C.c_double
    sig = {
        "rfgpu_region_create": ([C.POINTER(RegionDescT), C.POINTER(vp)], C.c_int),
        "rfgpu_region_destroy": ([vp], C.c_int),
        "rfgpu_stage": ([vp, C.c_int, d], C.c_int),
        "rfgpu_dt": ([vp, d, d, d, d, dp], C.c_int),
        "rfgpu_step": ([vp, d, d, d, d], C.c_int),
        "rfgpu_steps_graph": ([vp, C.c_int, d, d, d, d], C.c_int),
        "rfgpu_residual": ([vp, dp], C.c_int),
        "rfgpu_download": ([vp, dp, dp], C.c_int),
        "rfgpu_upload": ([vp, dp, dp], C.c_int),
        "rfgpu_step_host": ([vp, dp, dp, d, d, d, d], C.c_int),
        "rfgpu_download_grad": ([vp, dp], C.c_int),
        "rfgpu_time": ([vp, dp, dp], C.c_int),
        "rfgpu_set_time": ([vp, d], C.c_int),
        "rfgpu_status": ([vp, ip], C.c_int),
        "rfgpu_sync": ([vp], C.c_int),
        "rfgpu_stream": ([vp], vp),
        "rfgpu_device_bytes": ([vp], C.c_longlong),
        "rfgpu_launch_count": ([vp], C.c_longlong),
        "rfgpu_set_tuning": ([vp, C.POINTER(TuningT)], C.c_int),
        "rfgpu_batch_create": ([C.POINTER(vp), C.c_int, C.POINTER(vp)], C.c_int),
        "rfgpu_batch_destroy": ([vp], C.c_int),
        "rfgpu_batch_step": ([vp, d, d, d, d], C.c_int),
        "rfgpu_batch_steps_graph": ([vp, C.c_int, d, d, d, d], C.c_int),
        "rfgpu_batch_sync": ([vp], C.c_int),
        "rfgpu_batch_stream": ([vp], vp),
        "rfgpu_profile": ([vp, C.c_int], C.c_int),
        "rfgpu_profile_read": ([vp, dp, C.POINTER(C.c_longlong), C.c_int], C.c_int),
        "rfgpu_batch_profile": ([vp, C.c_int], C.c_int),
        "rfgpu_batch_profile_read": ([vp, dp, C.POINTER(C.c_longlong), C.c_int], C.c_int),
        "rfgpu_batch_launch_count": ([vp], C.c_longlong),
        "rfgpu_timer_start": ([vp], C.c_int),
        "rfgpu_timer_stop": ([vp, dp], C.c_int),
        "rfgpu_batch_timer_start": ([vp], C.c_int),
        "rfgpu_batch_timer_stop": ([vp, dp], C.c_int),
        "rfgpu_set_device": ([C.c_int], C.c_int),
        "rfgpu_host_alloc": ([C.c_longlong], vp),
        "rfgpu_host_free": ([vp], C.c_int),
        "rfgpu_mem_info": ([C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)], C.c_int),
        "rfgpu_sm_count": ([ip], C.c_int),
        "rfgpu_residual_noalloc": ([vp, dp], C.c_int),
        "rfgpu_batch_set_tuning": ([vp, C.POINTER(TuningT)], C.c_int),
        "rfgpu_batch_test_barrier": ([vp, C.c_int, C.c_longlong], C.c_int),
        "rfgpu_mesh_stencils": ([C.c_int, C.c_int, ip, ip, ip, ip, dp, ip, ip, dp], C.c_int),
        "rfgpu_border_copy": ([vp, C.c_int, vp], C.c_int),
        "rfgpu_border_pack": ([vp, C.c_int, dp], C.c_int),
        "rfgpu_border_unpack": ([vp, C.c_int, dp], C.c_int),
        "rfgpu_batch_create_ex": ([C.POINTER(vp), C.c_int, C.c_int, C.POINTER(vp)], C.c_int),
        "rfgpu_mesh_build": ([C.c_int, C.c_int, dp, ip, ip, ip, dp, dp, C.POINTER(vp)], C.c_int),
        "rfgpu_mesh_sizes": ([vp, C.POINTER(C.c_longlong)], C.c_int),
        "rfgpu_mesh_faces": ([vp, ip, dp, dp], C.c_int),
        "rfgpu_mesh_cells": ([vp, dp, dp, ip, ip, dp, ip, ip], C.c_int),
        "rfgpu_mesh_patch": ([vp, C.c_int, ip, dp, dp, ip], C.c_int),
        "rfgpu_mesh_destroy": ([vp], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    if path is None:
        _lib = lib
    return lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _check(rc: int, where: str):
    if rc != OK:
        raise EngineError(rc, where)


def _prof_read(fn, h):
    n = len(KERNELS)
    ms = (C.c_double * n)()
    cnt = (C.c_longlong * n)()
    _check(fn(h, ms, cnt, n), "rfgpu_profile_read")
    return {KERNELS[i]: (ms[i], cnt[i]) for i in range(n)}


def set_device(device: int):
    """Select the GPU for this host thread (one process per GPU)."""
    _check(load().rfgpu_set_device(device), "rfgpu_set_device")


def mem_info():
    """(free, total) device bytes of the current GPU."""
    f, t = C.c_longlong(), C.c_longlong()
    _check(load().rfgpu_mem_info(C.byref(f), C.byref(t)), "rfgpu_mem_info")
    return f.value, t.value


def sm_count() -> int:
    """Streaming multiprocessors of the current GPU, asked of the device."""
    n = C.c_int()
    _check(load().rfgpu_sm_count(C.byref(n)), "rfgpu_sm_count")
    return n.value


def mesh_stencils(n_cells: int, n_verts: int, cell_verts, cell_nverts, v2c_off, v2c, cofg):
    """rfgpu_mesh_stencils: c2c stencils and WLSQ moments of every cell built on
    the GPU with the host builder's per-cell routine.  Returns (offsets
    (n+1, 0-based), members (1-based), moments (n, 10))."""
    lib = load()
    cv = np.ascontiguousarray(cell_verts, np.int32)
    nv = np.ascontiguousarray(cell_nverts, np.int32)
    vo = np.ascontiguousarray(v2c_off, np.int32)
    vc = np.ascontiguousarray(v2c, np.int32)
    cg = np.ascontiguousarray(cofg, np.float64)
    off = np.empty(n_cells + 1, np.int32)
    mem = np.empty(40 * n_cells, np.int32)
    mom = np.empty((n_cells, 10), np.float64)
    _check(lib.rfgpu_mesh_stencils(n_cells, n_verts, _ip(cv), _ip(nv), _ip(vo), _ip(vc), _dp(cg),
                                   _ip(off), _ip(mem), _dp(mom)), "rfgpu_mesh_stencils")
    return off, mem[:off[-1]].copy(), mom


def mesh_build(n_verts: int, xyz, cell_verts, cell_nverts, cell_type, lo, hi):
    """rfgpu_mesh_build: face list, geometry, vertex-to-cell lists, stencils and
    moments of a box mesh on the GPU (rfmesh.h's host builder, bit for bit).
    Returns a dict of arrays in the host builder's layouts."""
    lib = load()
    xyz = np.ascontiguousarray(xyz, np.float64)
    cv = np.ascontiguousarray(cell_verts, np.int32)
    nv = np.ascontiguousarray(cell_nverts, np.int32)
    ct = np.ascontiguousarray(cell_type, np.int32)
    n = nv.shape[0]
    lo_a = (C.c_double * 3)(*lo)
    hi_a = (C.c_double * 3)(*hi)
    h = C.c_void_p()
    _check(lib.rfgpu_mesh_build(n, n_verts, _dp(xyz), _ip(cv), _ip(nv), _ip(ct), lo_a, hi_a,
                                C.byref(h)), "rfgpu_mesh_build")
    try:
        sz = (C.c_longlong * 8)()
        _check(lib.rfgpu_mesh_sizes(h, sz), "rfgpu_mesh_sizes")
        nF, nM = sz[0], sz[1]
        out = {"f2c": np.empty((nF, 2), np.int32), "fn": np.empty((nF, 4)),
               "fc": np.empty((nF, 3)), "vol": np.empty(n), "cofg": np.empty((n, 3)),
               "c2cs_off": np.empty(n + 1, np.int32), "c2cs_mem": np.empty(nM, np.int32),
               "xyzmoms": np.empty((n, 10)), "v2c_off": np.empty(n_verts + 1, np.int32)}
        _check(lib.rfgpu_mesh_faces(h, _ip(out["f2c"]), _dp(out["fn"]), _dp(out["fc"])),
               "rfgpu_mesh_faces")
        _check(lib.rfgpu_mesh_cells(h, _dp(out["vol"]), _dp(out["cofg"]), _ip(out["c2cs_off"]),
                                    _ip(out["c2cs_mem"]), _dp(out["xyzmoms"]),
                                    _ip(out["v2c_off"]), None), "rfgpu_mesh_cells")
        out["v2c"] = np.empty(int(out["v2c_off"][-1]), np.int32)
        _check(lib.rfgpu_mesh_cells(h, None, None, None, None, None, None, _ip(out["v2c"])),
               "rfgpu_mesh_cells")
        out["patches"] = []
        for ipt in range(6):
            nb = sz[2 + ipt]
            pa = {"bf2c": np.empty(nb, np.int32), "fn": np.empty((nb, 4)), "fc": np.empty((nb, 3)),
                  "bf2v": np.empty((nb, 4), np.int32)}
            _check(lib.rfgpu_mesh_patch(h, ipt, _ip(pa["bf2c"]), _dp(pa["fn"]), _dp(pa["fc"]),
                                        _ip(pa["bf2v"])), "rfgpu_mesh_patch")
            out["patches"].append(pa)
        return out
    finally:
        lib.rfgpu_mesh_destroy(h)


class PinnedArray:
    """A page-locked host buffer viewed as a float64 NumPy array."""

    def __init__(self, shape):
        self.lib = load()
        n = int(np.prod(shape))
        self.ptr = self.lib.rfgpu_host_alloc(8 * n)
        if not self.ptr:
            raise EngineError(ERR_NOMEM, "rfgpu_host_alloc")
        buf = (C.c_double * n).from_address(self.ptr)
        self.array = np.ctypeslib.as_array(buf).reshape(shape)

    def close(self):
        if getattr(self, "ptr", None):
            self.array = None
            self.lib.rfgpu_host_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Region:
    """One registered region on the GPU (device-resident state)."""

    def __init__(self, case: Case, precision: Optional[int] = None,
                 cell_order: int = ORDER_LOCALITY):
        self.lib = load()
        m, num = case.mesh, case.numerics
        self.case = case
        self.num = num
        self.nCells = m.nTot          # rows of every per-cell array crossing the ABI
        self.nAct = m.nCells
        self.precision = num.precision if precision is None else precision
        keep = []

        def k(a, dt):
            a = np.ascontiguousarray(a, dtype=dt)
            keep.append(a)
            return a

        patches = [(p, bc) for p, bc in zip(m.patches, case.bcs) if p.n + p.n_vb > 0]
        parr = (PatchT * max(1, len(patches)))()
        for i, (p, bc) in enumerate(patches):
            P = parr[i]
            P.bcType, P.spaceOrder, P.bcOptType, P.nBFaces = bc.bcType, bc.spaceOrder, bc.bcOptType, p.n
            bf2c, bfn, bfc = p.all_faces()   # a region's VB faces after the actual ones
            P.nBFacesTot = p.n + p.n_vb
            P.bf2c = _ip(k(bf2c, np.int32))
            P.fn = _dp(k(bfn, np.float64))
            P.fc = _dp(k(bfc, np.float64))
            vals, nd, dist = bc.vals_array(p.n)
            P.vals = _dp(k(vals, np.float64))
            P.distrib, P.nData = dist, nd
            P.bcOptFixed = bc.bcOptFixed
        d = RegionDescT()
        d.nCells, d.nFaces, d.f2cLd = m.nCells, m.nFaces, 2
        f2c, fn, fc = m.all_faces()   # flux faces, then a region's VV / VX faces
        d.nFacesAll = m.nFacesAll
        d.f2c = _ip(k(f2c, np.int32))
        d.fn = _dp(k(fn, np.float64))
        d.fc = _dp(k(fc, np.float64))
        d.cofg = _dp(k(m.cofg, np.float64))
        d.vol = _dp(k(m.vol, np.float64))
        d.c2csOffsets = _ip(k(m.c2cs_off, np.int32))
        d.c2csMembers = _ip(k(m.c2cs_mem, np.int32))
        d.xyzMoms = _dp(k(m.xyzmoms, np.float64))
        d.nPatches = len(patches)
        d.patches = parr
        d.cv = _dp(k(case.cv, np.float64))
        d.dv = _dp(k(case.dv, np.float64))
        d.gasModel, d.flowModel = 1, 0
        d.spaceDiscr, d.spaceOrder, d.reconst, d.rkScheme = (
            num.spaceDiscr, num.spaceOrder, num.reconst, num.rkScheme)
        d.refCp, d.refGamma = num.refCp, num.refGamma
        d.gvCp, d.gvMol = num.gv
        d.epsentr, d.dissFact = num.epsentr, num.dissFact
        d.precision = self.precision
        d.venkatGuard = num.venkatGuard
        d.cellOrder = cell_order
        d.ausmSigma, d.ausmKp, d.ausmKu, d.ausmMInf = (
            num.ausmSigma, num.ausmKp, num.ausmKu, num.ausmMInf)
        d.nCellsTot = m.nCellsTot
        d.iRegionGlobal = m.iRegionGlobal
        barr = (BorderT * max(1, len(m.borders)))()
        for i, b in enumerate(m.borders):
            B = barr[i]
            B.iRegionGlobal, B.iBorder = b.iRegionGlobal, b.iBorder
            B.nCellsSend, B.icgSend = len(b.icgSend), _ip(k(b.icgSend, np.int32))
            B.nCellsRecv, B.icgRecv = len(b.icgRecv), _ip(k(b.icgRecv, np.int32))
        d.nBorders = len(m.borders)
        d.borders = barr
        self.borders = m.borders
        self.iRegionGlobal = m.iRegionGlobal
        h = C.c_void_p()
        _check(self.lib.rfgpu_region_create(C.byref(d), C.byref(h)), "rfgpu_region_create")
        self.h = h
        self.nSteps = {1: 4, 2: 3, 3: 1}[num.rkScheme]

    def close(self):
        if getattr(self, "h", None):
            self.lib.rfgpu_region_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- reference-shaped operations -----------------------------------------
    def rk_stage(self, istage: int, dtMin: float):
        _check(self.lib.rfgpu_stage(self.h, istage, dtMin), "rfgpu_stage")

    def time_step(self, cfl: float, dtImposed: float, dtMinLimit: float = 0.0,
                  currentTime: float = 1.0) -> float:
        out = C.c_double()
        _check(self.lib.rfgpu_dt(self.h, cfl, dtImposed, dtMinLimit, currentTime, C.byref(out)),
               "rfgpu_dt")
        return out.value

    def step(self, cfl: float, dtImposed: float, dtMinLimit: float = 0.0, endTime: float = 0.0):
        _check(self.lib.rfgpu_step(self.h, cfl, dtImposed, dtMinLimit, endTime), "rfgpu_step")

    def steps_graph(self, n: int, cfl: float, dtImposed: float, dtMinLimit: float = 0.0,
                    endTime: float = 0.0):
        _check(self.lib.rfgpu_steps_graph(self.h, n, cfl, dtImposed, dtMinLimit, endTime),
               "rfgpu_steps_graph")

    def residual(self, to_host: bool = True):
        if not to_host:
            _check(self.lib.rfgpu_residual(self.h, None), "rfgpu_residual")
            return None
        rhs = np.empty((self.nCells, 5))
        _check(self.lib.rfgpu_residual(self.h, _dp(rhs)), "rfgpu_residual")
        return rhs

    def residual_noalloc(self):
        """rfgpu_residual_noalloc: the residual with no device allocation, its
        scratch in the library's fixed static device array (see include/rfgpu.h
        for who needs it and its size limit)."""
        rhs = np.empty((self.nCells, 5))
        _check(self.lib.rfgpu_residual_noalloc(self.h, _dp(rhs)), "rfgpu_residual_noalloc")
        return rhs

    def download(self):
        cv = np.empty((self.nCells, 5))
        dv = np.empty((self.nCells, 3))
        _check(self.lib.rfgpu_download(self.h, _dp(cv), _dp(dv)), "rfgpu_download")
        return cv, dv

    def download_into(self, cv: np.ndarray, dv: Optional[np.ndarray] = None):
        _check(self.lib.rfgpu_download(self.h, _dp(cv), _dp(dv) if dv is not None else None),
               "rfgpu_download")

    def upload(self, cv: np.ndarray, dv: Optional[np.ndarray] = None):
        cv = np.ascontiguousarray(cv, np.float64)
        dvp = None
        if dv is not None:
            dv = np.ascontiguousarray(dv, np.float64)
            dvp = _dp(dv)
        _check(self.lib.rfgpu_upload(self.h, _dp(cv), dvp), "rfgpu_upload")

    def step_host(self, cv: np.ndarray, dv: Optional[np.ndarray], cfl: float, dtImposed: float,
                  dtMinLimit: float = 0.0, endTime: float = 0.0):
        """rfgpu_step_host: one time step of the host state cv (nCells, 5), C-contiguous
        float64, overwritten in place; dv (nCells, 3) receives the dependent variables
        (or None).  Use pinned arrays (PinnedArray) for full copy rates."""
        for a, k in ((cv, 5), (dv, 3)):
            if a is not None and (a.dtype != np.float64 or not a.flags.c_contiguous
                                  or a.shape != (self.nCells, k)):
                raise ValueError(f"step_host needs a C-contiguous float64 ({self.nCells}, {k}) array")
        _check(self.lib.rfgpu_step_host(self.h, _dp(cv), _dp(dv) if dv is not None else None,
                                        cfl, dtImposed, dtMinLimit, endTime), "rfgpu_step_host")

    def gradients(self):
        g = np.empty((self.nCells, 5, 3))
        _check(self.lib.rfgpu_download_grad(self.h, _dp(g)), "rfgpu_download_grad")
        return g

    # --- halo exchange (RFLU_MPI_CopyWrapper / ISendWrapper / RecvWrapper) -----
    def border_copy(self, i_border: int, dst: "Region"):
        """cv of this region's border i_border (1-based) send cells into the
        receive cells of the matching border of dst, with their dv."""
        _check(self.lib.rfgpu_border_copy(self.h, i_border, dst.h), "rfgpu_border_copy")

    def border_pack(self, i_border: int) -> np.ndarray:
        """sendBuff(5,nCellsSend) of border i_border as (nCellsSend, 5)."""
        buf = np.empty((len(self.borders[i_border - 1].icgSend), 5))
        _check(self.lib.rfgpu_border_pack(self.h, i_border, _dp(buf)), "rfgpu_border_pack")
        return buf

    def border_unpack(self, i_border: int, buf: np.ndarray):
        """cv of border i_border's receive cells from recvBuff (nCellsRecv, 5)."""
        buf = np.ascontiguousarray(buf, np.float64)
        _check(self.lib.rfgpu_border_unpack(self.h, i_border, _dp(buf)), "rfgpu_border_unpack")

    def time(self):
        t, dt = C.c_double(), C.c_double()
        _check(self.lib.rfgpu_time(self.h, C.byref(t), C.byref(dt)), "rfgpu_time")
        return t.value, dt.value

    def set_time(self, t: float):
        _check(self.lib.rfgpu_set_time(self.h, t), "rfgpu_set_time")

    def status(self) -> int:
        fl = C.c_int()
        rc = self.lib.rfgpu_status(self.h, C.byref(fl))
        if rc not in (OK, ERR_STATE):
            raise EngineError(rc, "rfgpu_status")
        return fl.value

    def sync(self):
        _check(self.lib.rfgpu_sync(self.h), "rfgpu_sync")

    @property
    def stream(self) -> int:
        return self.lib.rfgpu_stream(self.h) or 0

    @property
    def device_bytes(self) -> int:
        return self.lib.rfgpu_device_bytes(self.h)

    @property
    def launches(self) -> int:
        return self.lib.rfgpu_launch_count(self.h)

    def timer_start(self):
        _check(self.lib.rfgpu_timer_start(self.h), "rfgpu_timer_start")

    def timer_stop(self) -> float:
        ms = C.c_double()
        _check(self.lib.rfgpu_timer_stop(self.h, C.byref(ms)), "rfgpu_timer_stop")
        return ms.value

    def profile(self, enable: bool = True):
        _check(self.lib.rfgpu_profile(self.h, int(enable)), "rfgpu_profile")

    def profile_read(self):
        """{kernel: (total ms, launches)} since profiling was enabled/read."""
        return _prof_read(self.lib.rfgpu_profile_read, self.h)

    def set_tuning(self, **kw):
        """rfgpu_set_tuning: gridCap, gradBlock, faceBlock, facesPerThread,
        cellBlock (omitted keys: the default)."""
        t = _tuning(**kw)
        _check(self.lib.rfgpu_set_tuning(self.h, C.byref(t)), "rfgpu_set_tuning")

    def set_grid_cap(self, blocks: int):
        self.set_tuning(gridCap=blocks)

    def solve(self, t_end: Optional[float] = None, n_steps: Optional[int] = None,
              dt_imposed: Optional[float] = None, graph: bool = False):
        """RFLU_TimeStepping loop: the first step uses dtImposed (the CFL step
        of the initial state unless given), later steps cfl*min(dt); the last
        step is clipped to t_end.  Returns (time, steps, status)."""
        cfl = self.num.cfl
        if dt_imposed is None:
            dt_imposed = self.time_step(cfl, 1.0, 0.0, 1.0)
        self.set_time(0.0)
        end = t_end if t_end is not None else 0.0
        k = 0
        if n_steps is not None:
            if graph:
                self.steps_graph(n_steps, cfl, dt_imposed, 0.0, end)
            else:
                for _ in range(n_steps):
                    self.step(cfl, dt_imposed, 0.0, end)
            k = n_steps
        else:
            chunk = 64
            while k < 10_000_000:
                if graph:
                    self.steps_graph(chunk, cfl, dt_imposed, 0.0, end)
                else:
                    for _ in range(chunk):
                        self.step(cfl, dt_imposed, 0.0, end)
                k += chunk
                t, _ = self.time()
                if not np.isfinite(t):
                    raise EngineError(ERR_STATE, "solve: non-finite time")
                if t >= end:
                    break
        t, _ = self.time()
        return t, k, self.status()


class Batch:
    """Many regions advanced together: one launch per pass over all regions."""

    def __init__(self, regions: Sequence[Region], coupled: bool = False):
        """coupled=True: the regions of one partitioned case (one time step, the
        minimum over them, and the halo exchange after every stage)."""
        self.lib = load()
        self.regions = list(regions)
        arr = (C.c_void_p * len(self.regions))(*[r.h for r in self.regions])
        h = C.c_void_p()
        _check(self.lib.rfgpu_batch_create_ex(arr, len(self.regions),
                                              BATCH_COUPLED if coupled else 0, C.byref(h)),
               "rfgpu_batch_create_ex")
        self.h = h

    def step(self, cfl, dtImposed, dtMinLimit=0.0, endTime=0.0):
        _check(self.lib.rfgpu_batch_step(self.h, cfl, dtImposed, dtMinLimit, endTime),
               "rfgpu_batch_step")

    def steps_graph(self, n, cfl, dtImposed, dtMinLimit=0.0, endTime=0.0):
        _check(self.lib.rfgpu_batch_steps_graph(self.h, n, cfl, dtImposed, dtMinLimit, endTime),
               "rfgpu_batch_steps_graph")

    def sync(self):
        _check(self.lib.rfgpu_batch_sync(self.h), "rfgpu_batch_sync")

    def timer_start(self):
        _check(self.lib.rfgpu_batch_timer_start(self.h), "rfgpu_batch_timer_start")

    def timer_stop(self) -> float:
        ms = C.c_double()
        _check(self.lib.rfgpu_batch_timer_stop(self.h, C.byref(ms)), "rfgpu_batch_timer_stop")
        return ms.value

    def set_tuning(self, **kw):
        t = _tuning(**kw)
        _check(self.lib.rfgpu_batch_set_tuning(self.h, C.byref(t)), "rfgpu_batch_set_tuning")

    def test_barrier(self, extra: int, spin_cycles: int = 0):
        """rfgpu_batch_test_barrier: make the persistent stage's grid-wide
        barrier wait for `extra` blocks that never arrive (0 restores)."""
        _check(self.lib.rfgpu_batch_test_barrier(self.h, extra, spin_cycles),
               "rfgpu_batch_test_barrier")

    def set_grid_cap(self, blocks: int):
        self.set_tuning(gridCap=blocks)

    def profile(self, enable: bool = True):
        _check(self.lib.rfgpu_batch_profile(self.h, int(enable)), "rfgpu_batch_profile")

    def profile_read(self):
        return _prof_read(self.lib.rfgpu_batch_profile_read, self.h)

    @property
    def launches(self) -> int:
        return self.lib.rfgpu_batch_launch_count(self.h)

    @property
    def stream(self) -> int:
        return self.lib.rfgpu_batch_stream(self.h) or 0

    def close(self):
        if getattr(self, "h", None):
            self.lib.rfgpu_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
