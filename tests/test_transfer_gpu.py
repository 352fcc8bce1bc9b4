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


@pytest.mark.parametrize("prec", [K.PREC_MIXED, K.PREC_SPLIT], ids=["mixed", "split"])
@pytest.mark.parametrize("dims", [(1, 1, 1), (5, 3, 7), (40, 7, 3), (50, 9, 11)])
@pytest.mark.parametrize("order", [E.ORDER_HOST, E.ORDER_LOCALITY])
def test_chunked_upload_download_round_trip(dims, order, prec):
    """Upload then download with no step between: the transfers run in up to 8
    chunks of cell tiles (a region smaller than 8 tiles in fewer, the last tile
    partial); cv comes back, bit for bit for every cell, as the float-float
    split of the input joined again (mixed path) or as the input itself (split
    path, FP64 state)."""
    nx, ny, nz = dims
    c = K.tet_shock_box(nx, ny=ny, nz=nz, seed=5,
                        numerics=K.Numerics(precision=prec, venkatGuard=1))
    r = E.Region(c, cell_order=order)
    q = np.ascontiguousarray(c.cv, np.float64)
    if prec == K.PREC_MIXED:
        hi = q.astype(np.float32)
        lo = (q - hi.astype(np.float64)).astype(np.float32)
        want = hi.astype(np.float64) + lo.astype(np.float64)
    else:
        want = q
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


def _case(dims, prec, discr=K.DISCR_UPW_ROE, rk=K.RK_SCHEME_3_WRAY, order=2,
          reconst=K.RECONST_LIM_VENKAT):
    nx, ny, nz = dims
    num = K.Numerics(precision=prec, venkatGuard=1, spaceDiscr=discr, rkScheme=rk,
                     spaceOrder=order, reconst=reconst)
    return K.tet_shock_box(nx, ny=ny, nz=nz, seed=7, numerics=num)


@pytest.mark.parametrize("dims", [(3, 3, 3), (5, 3, 7), (24, 8, 8), (50, 9, 11)])
@pytest.mark.parametrize("variant", ["roe-wray", "hllc-rk4", "ausm+-euler", "first-order", "fp64",
                                     "split", "split-rk4", "ausm+up-unlimited"])
@pytest.mark.parametrize("order", [E.ORDER_HOST, E.ORDER_LOCALITY])
def test_step_host_equals_three_calls(dims, variant, order):
    """rfgpu_step_host against rfgpu_upload + rfgpu_step + rfgpu_download on the
    same host state, three steps: cv, dv and the device time agree bit for bit.
    On the mixed path at second order the copies and conversions run in up to
    8 chunks with the first stage's gradient pass split into phases by the
    chunks its records travel in and the last stage's update split by the
    chunks it hands back (regions smaller than 8 tiles in fewer chunks); the
    FP64 path and first order run the three calls in sequence.  With more than
    one stage and no WENO pass the whole last stage (gradient, faces, boundary
    faces, update) runs in the download's phases."""
    prec, discr, rk, sord = K.PREC_MIXED, K.DISCR_UPW_ROE, K.RK_SCHEME_3_WRAY, 2
    reconst = K.RECONST_LIM_VENKAT
    if variant == "hllc-rk4":
        discr, rk = K.DISCR_UPW_HLLC, K.RK_SCHEME_4_CLASSICAL
    elif variant == "ausm+-euler":
        discr, rk = K.DISCR_UPW_AUSMPLUS, K.RK_SCHEME_1_EULER
    elif variant == "first-order":
        sord = 1
    elif variant == "fp64":
        prec = K.PREC_FP64
    elif variant == "split":
        prec = K.PREC_SPLIT
    elif variant == "split-rk4":
        prec, discr, rk = K.PREC_SPLIT, K.DISCR_UPW_HLLC, K.RK_SCHEME_4_CLASSICAL
    elif variant == "ausm+up-unlimited":
        discr, reconst = K.DISCR_UPW_AUSMPLUSUP, K.RECONST_NONE
    c = _case(dims, prec, discr, rk, sord, reconst)
    cfl = 0.5
    a = E.Region(c, cell_order=order)
    b = E.Region(c, cell_order=order)
    cv_a, dv_a = E.PinnedArray(c.cv.shape), E.PinnedArray(c.dv.shape)
    cv_a.array[:] = c.cv
    cv_b = np.ascontiguousarray(c.cv, np.float64).copy()
    for _ in range(3):
        a.step_host(cv_a.array, dv_a.array, cfl, 0.0)
        b.upload(cv_b)
        b.step(cfl, 0.0)
        cv_b, dv_b = b.download()
    assert np.all(np.isfinite(cv_b)) and np.all(np.isfinite(dv_b))
    assert np.array_equal(cv_a.array, cv_b)
    assert np.array_equal(dv_a.array, dv_b)
    assert a.time() == b.time()
    assert a.status() == 0 and not np.array_equal(cv_b, c.cv)
    # dv is optional; pageable host memory works too
    cv_c = cv_b.copy()
    a.step_host(cv_c, None, cfl, 0.0)
    b.upload(cv_b)
    b.step(cfl, 0.0)
    assert np.array_equal(cv_c, b.download()[0])
    for p in (cv_a, dv_a):
        p.close()
    a.close()
    b.close()


def test_step_host_refuses_bad_arrays():
    c = _case((3, 3, 3), K.PREC_MIXED)
    r = E.Region(c)
    with pytest.raises(ValueError):
        r.step_host(np.zeros((r.nCells, 4)), None, 0.5, 1e-4)
    with pytest.raises(ValueError):
        r.step_host(np.zeros((r.nCells, 5), np.float32), None, 0.5, 1e-4)
    r.close()
