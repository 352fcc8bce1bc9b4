"""Host transfers of the mixed path through the C ABI: DMA copies of the
Fortran images cv(5,N) / dv(3,N) into device staging buffers and one fused
conversion pass per direction.  Page-locked and pageable host buffers give
the same state bit for bit, in either device numbering, with and without a
host dv on upload."""
import numpy as np
import pytest

from rocflupicl_gb300 import case as K
from rocflupicl_gb300 import engine as E

pytestmark = pytest.mark.gpu


def _pinned(a):
    p = E.PinnedArray(a.shape)
    p.array[:] = a
    return p


@pytest.mark.parametrize("order", [E.ORDER_HOST, E.ORDER_LOCALITY])
@pytest.mark.parametrize("with_dv", [False, True])
def test_pinned_and_pageable_transfers_agree(order, with_dv):
    c = K.tet_shock_box(4, seed=3, numerics=K.Numerics(precision=K.PREC_MIXED, venkatGuard=1))
    direct = E.Region(c, cell_order=order)
    staged = E.Region(c, cell_order=order)
    cvp, dvp = _pinned(c.cv), _pinned(c.dv)
    direct.upload(cvp.array, dvp.array if with_dv else None)      # page-locked
    staged.upload(c.cv.copy(), c.dv.copy() if with_dv else None)   # pageable
    out = []
    for r in (direct, staged):
        r.solve(n_steps=3)
    ocv, odv = E.PinnedArray(c.cv.shape), E.PinnedArray(c.dv.shape)
    direct.download_into(ocv.array, odv.array)
    cv_s, dv_s = staged.download()
    assert np.array_equal(ocv.array, cv_s)
    assert np.array_equal(odv.array, dv_s)
    assert np.all(np.isfinite(cv_s)) and not np.array_equal(cv_s, c.cv)
    # a download of cv alone into page-locked memory
    only = E.PinnedArray(c.cv.shape)
    direct.download_into(only.array)
    assert np.array_equal(only.array, cv_s)
    for p in (cvp, dvp, ocv, odv, only):
        p.close()
    direct.close()
    staged.close()


@pytest.mark.parametrize("dims", [(1, 1, 1), (5, 3, 7), (40, 7, 3), (50, 9, 11)])
@pytest.mark.parametrize("order", [E.ORDER_HOST, E.ORDER_LOCALITY])
def test_chunked_upload_download_round_trip(dims, order):
    """Upload then download with no step between: the transfers run in up to 8
    chunks of cell tiles (a region smaller than 8 tiles in fewer, the last tile
    partial); cv comes back as the float-float split of the input joined again,
    bit for bit, for every cell."""
    nx, ny, nz = dims
    c = K.tet_shock_box(nx, ny=ny, nz=nz, seed=5,
                        numerics=K.Numerics(precision=K.PREC_MIXED, venkatGuard=1))
    r = E.Region(c, cell_order=order)
    q = np.ascontiguousarray(c.cv, np.float64)
    hi = q.astype(np.float32)
    lo = (q - hi.astype(np.float64)).astype(np.float32)
    want = hi.astype(np.float64) + lo.astype(np.float64)
    for pinned in (False, True):
        if pinned:
            src = E.PinnedArray(q.shape)
            src.array[:] = q
            r.upload(src.array)
        else:
            r.upload(q.copy())
        cv, dv = r.download()
        assert np.array_equal(cv, want)
        assert np.allclose(dv, K.eos_dv(c.numerics, want), rtol=1e-13, atol=0)
    r.close()
