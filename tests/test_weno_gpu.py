"""RECONST 2 on the GPU through the C ABI: WLSQ gradients weighted by
RFLU_WENOGradCellsXYZFast_3D (modflu/RFLU_ModWENO.F90:1402-1588), then
RFLU_LimitGradCellsSimple (modflu/RFLU_ModLimiters.F90:793-921), as
CellGradientsMP calls them (libfloflu/CellGradientsMP.F90:217-222).  The FP64
path is bit-identical to the oracle (gradients, residuals, trajectories, a
batch mixing RECONST 2 and 11 regions); the mixed path stays within its
tolerance; the host-state step equals the three calls."""
import numpy as np
import pytest

from rocflupicl_gb300 import case as K
from rocflupicl_gb300 import engine as E
from test_parity_gpu import assert_same, _oracle

pytestmark = pytest.mark.gpu


def weno_case(kind, scheme=K.DISCR_UPW_ROE, prec=K.PREC_FP64, low_density=False, **kw):
    num = K.Numerics(spaceDiscr=scheme, reconst=K.RECONST_WENO_XYZ, precision=prec, **kw)
    if kind == "tet":
        c = K.tet_shock_box(4, seed=5, numerics=num)
    elif kind == "mixed":
        c = K.mixed_box(6, numerics=num)
    else:
        c = K.shock_tube(24, numerics=num)
    if low_density:  # density from 0.02 to about 1: the positivity check zeroes gradients
        x = c.mesh.cofg
        c.cv *= (0.02 + 4.0 * (x[:, 0] - 0.5) ** 2)[:, None]
        c.dv = K.eos_dv(c.numerics, c.cv)
    return c


@pytest.mark.parametrize("kind", ["tube", "tet", "mixed"])
@pytest.mark.parametrize("scheme", [K.DISCR_UPW_ROE, K.DISCR_UPW_HLLC, K.DISCR_UPW_AUSMPLUS])
@pytest.mark.parametrize("low", [False, True])
def test_weno_residual_bitwise(kind, scheme, low):
    c = weno_case(kind, scheme, low_density=low)
    rhs_o, grad_o = _oracle(c).residual(c.cv, c.dv)
    r = E.Region(c)
    rhs_g = r.residual()
    assert_same(r.gradients(), grad_o, "WENO-XYZ gradients")
    assert_same(rhs_g, rhs_o, "residual")
    r.close()


@pytest.mark.parametrize("kind", ["tet", "mixed"])
@pytest.mark.parametrize("order", [E.ORDER_LOCALITY, E.ORDER_HOST])
def test_weno_steps_bitwise(kind, order):
    c = weno_case(kind)
    o = _oracle(c)
    cv, dv = c.cv.copy(), c.dv.copy()
    t_o, _, st_o = o.run(cv, dv, n_steps=4)
    r = E.Region(c, cell_order=order)
    t_g, _, st_g = r.solve(n_steps=4)
    cvg, dvg = r.download()
    assert st_g == st_o and t_g == t_o
    assert_same(cvg, cv, "cv after 4 steps")
    assert_same(dvg, dv, "dv after 4 steps")
    r.close()


def test_weno_residual_noalloc_equals_residual():
    c = weno_case("tet")
    r = E.Region(c)
    assert np.array_equal(r.residual_noalloc(), r.residual())
    r.close()


def test_batch_mixing_weno_and_venkat_regions():
    """One batched launch per pass over a RECONST 2 region and a RECONST 11
    region: each equals the oracle's run of its own case."""
    from oracle.oracle import Oracle
    cw = weno_case("tet")
    cv_ = K.tet_shock_box(4, seed=6, numerics=K.Numerics(spaceDiscr=K.DISCR_UPW_ROE,
                                                         venkatGuard=1))
    cases = [cw, cv_]
    cfl = cw.numerics.cfl
    regs = [E.Region(c) for c in cases]
    for r in regs:
        r.set_time(0.0)
    b = E.Batch(regs)
    d0 = min(r.time_step(cfl, 1.0, 0.0, 1.0) for r in regs)
    b.steps_graph(3, cfl, d0)
    b.sync()
    for r, c in zip(regs, cases):
        cv, dv = c.cv.copy(), c.dv.copy()
        Oracle(c).run(cv, dv, n_steps=3, dt_imposed=d0)
        cvb, dvb = r.download()
        assert_same(cvb, cv, "batched cv")
        assert_same(dvb, dv, "batched dv")
    b.close()


def test_weno_mixed_precision_l1():
    c = weno_case("tet", prec=K.PREC_MIXED)
    o = _oracle(c)
    cv, dv = c.cv.copy(), c.dv.copy()
    dti = o.dt(cv, dv, c.numerics.cfl, 1.0, 0.0, 1.0)
    o.run(cv, dv, n_steps=5, dt_imposed=dti)
    r = E.Region(c)
    r.solve(n_steps=5, dt_imposed=dti)
    cvg, dvg = r.download()
    assert np.mean(np.abs(cvg[:, 0] / cv[:, 0] - 1.0)) <= 1e-5
    assert np.mean(np.abs(dvg[:, 0] / dv[:, 0] - 1.0)) <= 1e-5
    r.close()


def test_weno_step_host_equals_three_calls():
    c = K.tet_shock_box(24, ny=8, nz=8, seed=7, numerics=K.Numerics(
        precision=K.PREC_MIXED, reconst=K.RECONST_WENO_XYZ, spaceDiscr=K.DISCR_UPW_ROE))
    a, b = E.Region(c), E.Region(c)
    cva = E.PinnedArray(c.cv.shape)
    dva = E.PinnedArray(c.dv.shape)
    cva.array[:] = c.cv
    cvb = np.ascontiguousarray(c.cv, np.float64).copy()
    for _ in range(3):
        a.step_host(cva.array, dva.array, 0.5, 0.0)
        b.upload(cvb)
        b.step(0.5, 0.0)
        cvb, dvb = b.download()
    assert np.all(np.isfinite(cvb))
    assert np.array_equal(cva.array, cvb) and np.array_equal(dva.array, dvb)
    for p in (cva, dva):
        p.close()
    a.close()
    b.close()
