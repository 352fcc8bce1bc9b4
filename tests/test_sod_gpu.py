"""Config 1 end to end: the Sod shock tube 1000x2x2 hexes (4000 cells), AUSM+,
WLSQ + Venkatakrishnan, Wray RK3 at CFL 0.5 to t = 0.2 (about 2160 steps),
slip walls on y/z and supersonic outflow at the x ends.  The FP64 GPU
trajectory is bit-identical to the oracle's at t = 0.2, and both match the
exact Riemann solution with the reference's L1 definition.  The limiter uses
the signed guard: with the reference's verbatim guard this configuration
fails within 100 steps (see test_oracle_kats.py)."""
import numpy as np
import pytest

import exact_riemann as er
from rocflupicl_gb300 import case as K
from rocflupicl_gb300 import engine as E

pytestmark = pytest.mark.gpu


def test_sod_config1_to_t02():
    from oracle.oracle import Oracle
    c = K.shock_tube(1000, numerics=K.Numerics(venkatGuard=1))
    o = Oracle(c)
    cv, dv = c.cv.copy(), c.dv.copy()
    t_o, k_o, st_o = o.run(cv, dv, t_end=0.2)
    r = E.Region(c)
    dti = o.dt(c.cv.copy(), c.dv.copy(), 0.5, 1.0, 0.0, 1.0)
    r.set_time(0.0)
    steps = 0
    while True:
        r.step(0.5, dti, 0.0, 0.2)
        steps += 1
        t, _ = r.time()
        if t >= 0.2 or steps > 5000:
            break
    cvg, dvg = r.download()
    assert st_o == 0 and r.status() == 0
    assert steps == k_o and t == t_o == 0.2
    assert np.array_equal(cvg, cv) and np.array_equal(dvg, dv)
    ex = er.sample(c.mesh.cofg[:, 0], 0.2, 0.5, (1.0, 0.0, 1.0), (0.125, 0.0, 0.1),
                   c.numerics.gamma_gv)
    l1r = np.mean(np.abs(cvg[:, 0] / ex[:, 0] - 1.0))
    l1p = np.mean(np.abs(dvg[:, 0] / ex[:, 2] - 1.0))
    assert l1r < 0.01 and l1p < 0.006, (l1r, l1p)
    r.close()


def test_sod_mixed_precision_close_to_fp64():
    c64 = K.shock_tube(1000, numerics=K.Numerics(venkatGuard=1))
    cmx = K.shock_tube(1000, numerics=K.Numerics(venkatGuard=1, precision=K.PREC_MIXED))
    out = []
    for c in (c64, cmx):
        r = E.Region(c)
        r.solve(n_steps=300)
        out.append(r.download())
        r.close()
    (cva, dva), (cvb, dvb) = out
    assert np.mean(np.abs(cvb[:, 0] / cva[:, 0] - 1.0)) <= 1e-5
    assert np.mean(np.abs(dvb[:, 0] / dva[:, 0] - 1.0)) <= 1e-5


@pytest.mark.parametrize("precision,n", [(K.PREC_FP64, 200), (K.PREC_FP64, 400),
                                         (K.PREC_MIXED, 200), (K.PREC_SPLIT, 200),
                                         (K.PREC_MIXED, 400), (K.PREC_SPLIT, 400)])
def test_sod2_strong_tube(precision, n):
    """st_sod2 (density and pressure ratios of 100, the reference's
    RFLU_InitFlowHardCode.F90:4309-4340) on n x 2 x 2 hexes to t = 4e-4 s: the
    FP64 path equals the oracle bit for bit, status word included (at n = 400
    the run applies the reference's energy floor, CheckPositivity's p <= 0 ->
    e = 1e4, a warning bit, and the reduced-precision modes apply it too).
    Against FP64 the reduced-precision modes keep L1(p) near 1.2e-6, but
    L1(rho) is 7.8e-5 (mixed) / 7.3e-5 (split) at n = 200 and 3.0e-5 /
    1.9e-5 at n = 400: the FP32 gradients and limiter move a few cells at the
    hundredfold density jump of the contact by up to ~2e-3, so this stress case
    is held to 2e-4 in L1(rho) and 1e-5 in L1(p), not to the 1e-5 of the
    benchmark configuration (both modes share the FP32 flux path, so the FP64
    update of the split mode does not change this)."""
    from oracle.oracle import Oracle
    left, right = (1.0, 0.0, 1.0e5), (0.01, 0.0, 1.0e3)
    mk = lambda p: K.shock_tube(n, left=left, right=right, t_end=4e-4,
                                numerics=K.Numerics(venkatGuard=1, precision=p))
    c = mk(K.PREC_FP64)
    o = Oracle(c)
    cv, dv = c.cv.copy(), c.dv.copy()
    t_o, k_o, st_o = o.run(cv, dv, t_end=4e-4)
    assert st_o & 3 == 0 and (st_o != 0) == (n == 400), st_o
    cg = mk(precision)
    r = E.Region(cg)
    cfl = cg.numerics.cfl
    dti = r.time_step(cfl, 1.0, 0.0, 1.0)
    r.set_time(0.0)
    steps = 0
    while True:
        r.step(cfl, dti, 0.0, 4e-4)
        steps += 1
        t, _ = r.time()
        if t >= 4e-4 or steps > 5000:
            break
    cvg, dvg = r.download()
    assert t == t_o
    if precision == K.PREC_FP64:
        assert steps == k_o and r.status() == st_o
        assert np.array_equal(cvg, cv) and np.array_equal(dvg, dv)
    else:
        assert r.status() == st_o
        assert np.mean(np.abs(cvg[:, 0] / cv[:, 0] - 1.0)) <= 2e-4
        assert np.mean(np.abs(dvg[:, 0] / dv[:, 0] - 1.0)) <= 1e-5
    r.close()
