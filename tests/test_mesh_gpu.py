"""Device-side mesh preprocessing: rfgpu_mesh_stencils builds the c2c
stencils and WLSQ moments on the GPU with the host builder's per-cell routine;
members (including the unstable quicksort's tie-breaking on regular hex
meshes), their order and the moments must equal the host builder's bit for
bit, and a region built from them must give the same residual."""
import ctypes as C

import numpy as np
import pytest

from rocflupicl_gb300 import case as K
from rocflupicl_gb300 import engine as E
from rocflupicl_gb300 import mesh as M

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,n,jitter", [(M.HEX, 9, 0.0), (M.HEX, 7, 0.1), (M.TET, 8, 0.1),
                                           (M.TET, 6, 0.0), (M.MIXED, 10, 0.0)])
def test_device_stencils_equal_host(kind, n, jitter):
    a = M.box(kind, n, n + 1, n + 2, jitter=jitter, seed=4)
    b = M.box(kind, n, n + 1, n + 2, jitter=jitter, seed=4, stencils="device")
    assert np.array_equal(a.c2cs_off, b.c2cs_off)
    assert np.array_equal(a.c2cs_mem, b.c2cs_mem)
    assert np.array_equal(a.xyzmoms, b.xyzmoms)


def test_device_stencils_case_residual():
    num = K.Numerics(spaceDiscr=K.DISCR_UPW_HLLC, venkatGuard=1)
    a = K.tet_shock_box(5, seed=8, numerics=num)
    b = K.tet_shock_box(5, seed=8, numerics=num, stencils="device")
    ra, rb = E.Region(a), E.Region(b)
    assert np.array_equal(ra.residual(), rb.residual())
    ra.close()
    rb.close()


def _host_v2c(kind, n, jitter, seed):
    """Vertex-to-cell lists of the host builder (rfmesh.h views)."""
    lib = M._load()
    h = C.c_void_p()
    lo = (C.c_double * 3)(0.0, 0.0, 0.0)
    hi = (C.c_double * 3)(1.0, 1.0, 1.0)
    assert lib.rfmesh_create_box_ex(kind, n, n + 1, n + 2, lo, hi, jitter, seed, 0,
                                    M.RFMESH_DEFER_STENCILS, C.byref(h)) == 0
    try:
        s = (C.c_longlong * M._NSIZES)()
        lib.rfmesh_sizes(h, s)
        nV = s[0]
        vo = np.ctypeslib.as_array(lib.rfmesh_v2c_offsets(h), shape=(nV + 1,)).copy()
        vc = np.ctypeslib.as_array(lib.rfmesh_v2c(h), shape=(int(vo[-1]),)).copy()
    finally:
        lib.rfmesh_destroy(h)
    return vo, vc


@pytest.mark.parametrize("kind", [M.HEX, M.TET, M.MIXED])
def test_device_mesh_build_equals_host_builder(kind):
    """rfgpu_mesh_build (face list, geometry, vertex-to-cell lists, stencils,
    moments on the GPU) reproduces the host builder bit for bit."""
    n, jit, seed = 7, 0.1, 9
    a = M.box(kind, n, n + 1, n + 2, jitter=jit, seed=seed, stencils="host")
    b = M.box(kind, n, n + 1, n + 2, jitter=jit, seed=seed, stencils="all-device")
    assert a.nCells == b.nCells and a.nFaces == b.nFaces
    for f in ("xyz", "vol", "cofg", "f2c", "fn", "fc", "c2cs_off", "c2cs_mem", "xyzmoms",
              "cell_type"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f
    for pa, pb in zip(a.patches, b.patches):
        for f in ("bf2c", "fn", "fc", "bf2v"):
            assert np.array_equal(getattr(pa, f), getattr(pb, f)), f
    vo, vc = _host_v2c(kind, n, jit, seed)
    lib = M._load()
    h = C.c_void_p()
    lo = (C.c_double * 3)(0.0, 0.0, 0.0)
    hi = (C.c_double * 3)(1.0, 1.0, 1.0)
    assert lib.rfmesh_create_box_ex(kind, n, n + 1, n + 2, lo, hi, jit, seed, 0,
                                    M.RFMESH_CELLS_ONLY, C.byref(h)) == 0
    try:
        s = (C.c_longlong * M._NSIZES)()
        lib.rfmesh_sizes(h, s)
        nV, nC = s[0], s[1]
        view = lambda p, k, dt: np.ctypeslib.as_array(p, shape=(k,)).astype(dt)
        r = E.mesh_build(nV, view(lib.rfmesh_xyz(h), 3 * nV, np.float64),
                         view(lib.rfmesh_cell_verts(h), 8 * nC, np.int32),
                         view(lib.rfmesh_cell_nverts(h), nC, np.int32),
                         view(lib.rfmesh_cell_type(h), nC, np.int32), (0, 0, 0), (1, 1, 1))
    finally:
        lib.rfmesh_destroy(h)
    assert np.array_equal(r["v2c_off"], vo) and np.array_equal(r["v2c"], vc)


def test_device_mesh_build_large_tet_box_and_residual():
    """A larger jittered tet box through the device build registers and gives
    the same residual as the host-built mesh."""
    from rocflupicl_gb300 import case as K
    num = K.Numerics(spaceDiscr=K.DISCR_UPW_ROE, venkatGuard=1)
    ca = K.tet_shock_box(24, numerics=num, stencils="host")
    cb = K.tet_shock_box(24, numerics=num, stencils="all-device")
    assert np.array_equal(ca.mesh.f2c, cb.mesh.f2c)
    assert np.array_equal(ca.mesh.xyzmoms, cb.mesh.xyzmoms)
    ra, rb = E.Region(ca), E.Region(cb)
    assert np.array_equal(ra.residual(), rb.residual())
    ra.close()
    rb.close()
