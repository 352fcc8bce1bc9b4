"""Device-side mesh preprocessing: rfgpu_mesh_stencils builds the c2c
stencils and WLSQ moments on the GPU with the host builder's per-cell routine;
members (including the unstable quicksort's tie-breaking on regular hex
meshes), their order and the moments must equal the host builder's bit for
bit, and a region built from them must give the same residual."""
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
