"""C-ABI libraries: they load, export every entry point the headers declare,
and the host-side validation answers without touching the GPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from rocflupicl_gb300 import case as K
from rocflupicl_gb300 import engine as E
from rocflupicl_gb300 import mesh as M

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    txt = open(os.path.join(ROOT, "include", header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(rf(?:gpu|mesh)_[a-z0-9_]+)\s*\(", txt)))


def test_engine_exports_every_declared_symbol():
    lib = E.load()
    names = declared("rfgpu.h")
    assert len(names) >= 30
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(E.SYMBOLS)


def test_mesh_exports_every_declared_symbol():
    lib = M._load()
    for n in declared("rfmesh.h"):
        assert hasattr(lib, n), n


def _desc(c, **over):
    """Descriptor through the same path Region uses, without creating it."""
    lib = E.load()
    m = c.mesh
    keep = []

    def k(a, dt):
        a = np.ascontiguousarray(a, dtype=dt)
        keep.append(a)
        return a

    d = E.RegionDescT()
    d.nCells, d.nFaces, d.f2cLd = m.nCells, m.nFaces, 2
    d.f2c = E._ip(k(m.f2c, np.int32))
    d.fn, d.fc = E._dp(k(m.fn, np.float64)), E._dp(k(m.fc, np.float64))
    d.cofg, d.vol = E._dp(k(m.cofg, np.float64)), E._dp(k(m.vol, np.float64))
    d.c2csOffsets = E._ip(k(m.c2cs_off, np.int32))
    d.c2csMembers = E._ip(k(m.c2cs_mem, np.int32))
    d.xyzMoms = E._dp(k(m.xyzmoms, np.float64))
    d.nPatches = 0
    d.cv = E._dp(k(c.cv, np.float64))
    d.dv = E._dp(k(c.dv, np.float64))
    d.gasModel, d.flowModel = 1, 0
    d.spaceDiscr, d.spaceOrder, d.reconst, d.rkScheme = 4, 2, 11, 2
    d.refCp, d.refGamma = 1004.5, 1.4
    d.gvCp, d.gvMol = c.numerics.gv
    d.epsentr, d.dissFact, d.precision = 0.05, 1.0, 0
    for key, val in over.items():
        setattr(d, key, val)
    return lib, d, keep


@pytest.mark.parametrize("field,value", [("spaceDiscr", 2), ("spaceOrder", 3), ("reconst", 1),
                                         ("rkScheme", 7), ("gasModel", 2), ("flowModel", 1),
                                         ("precision", 9)])
def test_unsupported_options_refused_before_any_cuda_call(field, value):
    c = K.shock_tube(6)
    lib, d, keep = _desc(c, **{field: value})
    h = C.c_void_p()
    assert lib.rfgpu_region_create(C.byref(d), C.byref(h)) == E.ERR_UNSUPPORTED
    assert not h.value


def test_bad_indices_refused():
    c = K.shock_tube(6)
    bad = c.mesh.f2c.copy()
    bad[3, 1] = c.mesh.nCells + 1
    lib, d, keep = _desc(c)
    keep.append(bad)
    d.f2c = E._ip(bad)
    h = C.c_void_p()
    assert lib.rfgpu_region_create(C.byref(d), C.byref(h)) == E.ERR_ARG
    lib2, d2, keep2 = _desc(c, nCells=0)
    assert lib2.rfgpu_region_create(C.byref(d2), C.byref(h)) == E.ERR_ARG
    assert lib.rfgpu_region_create(None, C.byref(h)) == E.ERR_ARG


def test_null_handles_are_errors():
    lib = E.load()
    assert lib.rfgpu_stage(None, 1, 1.0) == E.ERR_ARG
    assert lib.rfgpu_sync(None) == E.ERR_ARG
    assert lib.rfgpu_region_destroy(None) == E.ERR_ARG
    assert lib.rfgpu_launch_count(None) == -1
    cv = np.zeros(5)
    assert lib.rfgpu_step_host(None, E._dp(cv), None, 0.5, 0.0, 0.0, 0.0) == E.ERR_ARG


def test_perfmodel_matches_pass_totals():
    from rocflupicl_gb300 import perfmodel as P
    nc, nf, nb, m = 1000, 2000, 100, 40000
    assert P.stage_bytes(nc, nf, nb, m, 8) == 964 * nc + 4 * m + 112 * nf + 64 * nb
    assert P.stage_bytes(nc, nf, nb, m, 4) == 664 * nc + 4 * m + 112 * nf + 64 * nb


def test_mesh_stencils_validates_before_any_device_work():
    """rfgpu_mesh_stencils checks every index on the host: an out-of-range
    vertex or cell id is refused with RFGPU_ERR_ARG before any CUDA call, so
    this runs without a GPU."""
    from rocflupicl_gb300 import engine as E
    from rocflupicl_gb300 import mesh as M
    import ctypes as C
    lib = M._load()
    h = C.c_void_p()
    lo = (C.c_double * 3)(0.0, 0.0, 0.0)
    hi = (C.c_double * 3)(1.0, 1.0, 1.0)
    assert lib.rfmesh_create_box_ex(M.TET, 2, 2, 2, lo, hi, 0.0, 1, 0, M.RFMESH_DEFER_STENCILS,
                                    C.byref(h)) == 0
    try:
        s = (C.c_longlong * M._NSIZES)()
        lib.rfmesh_sizes(h, s)
        nV, nC = s[0], s[1]
        view = lambda p, n: np.ctypeslib.as_array(p, shape=(n,)).copy()
        cv = view(lib.rfmesh_cell_verts(h), 8 * nC)
        nv = view(lib.rfmesh_cell_nverts(h), nC)
        vo = view(lib.rfmesh_v2c_offsets(h), nV + 1)
        vc = view(lib.rfmesh_v2c(h), int(vo[-1]))
        cg = np.ctypeslib.as_array(lib.rfmesh_cofg_view(h), shape=(3 * nC,)).copy()
    finally:
        lib.rfmesh_destroy(h)
    for bad in ("vertex", "cell", "count"):
        cv2, vc2, nv2 = cv.copy(), vc.copy(), nv.copy()
        if bad == "vertex":
            cv2[2] = nV  # a used slot of cell 0 (4 vertices)
        elif bad == "cell":
            vc2[3] = nC
        else:
            nv2[0] = 9
        with pytest.raises(E.EngineError) as ei:
            E.mesh_stencils(nC, nV, cv2, nv2, vo, vc2, cg)
        assert ei.value.code == E.ERR_ARG


def test_mesh_build_validates_before_any_device_work():
    """rfgpu_mesh_build checks every index and cell type on the host first."""
    lib = E.load()
    xyz = np.zeros((5, 3))
    cv = np.full((1, 8), -1, np.int32)
    cv[0, :4] = [0, 1, 2, 3]
    nv = np.array([4], np.int32)
    ct = np.array([0], np.int32)
    lo = (C.c_double * 3)(0.0, 0.0, 0.0)
    hi = (C.c_double * 3)(1.0, 1.0, 1.0)
    h = C.c_void_p()
    for bad in ("vertex", "type", "count", "pad"):
        cv2, nv2, ct2 = cv.copy(), nv.copy(), ct.copy()
        if bad == "vertex":
            cv2[0, 1] = 5
        elif bad == "type":
            ct2[0] = 4
        elif bad == "count":
            nv2[0] = 8
        else:
            cv2[0, 5] = 2
        assert lib.rfgpu_mesh_build(1, 5, E._dp(xyz), E._ip(cv2), E._ip(nv2), E._ip(ct2), lo, hi,
                                    C.byref(h)) == E.ERR_ARG
        assert not h.value
