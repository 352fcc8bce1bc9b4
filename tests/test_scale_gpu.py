"""FP64 parity at the benchmarked sizes, through the C ABI.

The small-mesh tests of test_parity_gpu.py pin every option; these pin the
two full-size workloads the benchmark quotes, on the limiter variants it uses
and on the reference's literal one:

* the planar Ms = 2 shock over the 128^3 x 6 jittered Kuhn-tet box
  (12,582,912 cells): residual, limited gradients and one whole Wray RK3 step
  (device time step + 3 stages), bit for bit against the OpenMP oracle (which
  equals the serial oracle bit for bit), for Roe with the reference's
  Venkatakrishnan term (venkatGuard 0) and the signed guard (1), and for HLLC;
* the 96^3 mixed hex/prism/tet/pyramid box (2.48 M cells): the single
  residual of all three flux schemes, bit for bit; the reduced-precision
  modes' residuals within 1e-5 of the FP64 oracle's in the L1 sense,
  sum |R - R_ref| / sum |R_ref| per component (the largest single-cell
  difference, about 1e-3 of max |R_ref|, sits where the FP32 limiter picks a
  different face minimum than the FP64 one).

The oracle's stage-1 pass returns the residual of its input state (rhs) and
the limited gradients before it updates; those are what the GPU's residual
call returns.
"""
import os

import numpy as np
import pytest

from rocflupicl_gb300 import case as K
from rocflupicl_gb300 import engine as E

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def _same(a, b, what, finite=True):
    """Bit-identical; with finite=False the oracle may hold NaN or inf (the
    reference's literal limiter term breaks down on some cells of the full
    mesh) and the GPU must hold them in exactly the same entries."""
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape, what
    if finite:
        assert np.all(np.isfinite(b)), f"{what}: oracle not finite"
    elif np.array_equal(a, b, equal_nan=True):  # same NaN entries, same infinities
        return
    if not np.array_equal(a, b):
        d = np.abs(a - b)
        bad = int(np.count_nonzero(d))
        i = np.unravel_index(np.argmax(d), d.shape)
        raise AssertionError(f"{what}: {bad} entries differ; largest at {i}: gpu {a[i]!r} "
                             f"oracle {b[i]!r}")


@pytest.fixture(scope="module")
def tet128():
    # config 2's mesh and state (the benchmark's generator and seed)
    return K.tet_shock_box(128, numerics=K.Numerics(spaceDiscr=K.DISCR_UPW_ROE, venkatGuard=1))


@pytest.fixture(scope="module")
def mixed96():
    return K.mixed_box(96)


def _oracle_stage1(c):
    """Residual and limited gradients of c's state (oracle stage 1 with a zero
    time step leaves cv as it found it up to the update, which is not read)."""
    from oracle.oracle import Oracle
    o = Oracle(c)
    cv, dv = c.cv.copy(), c.dv.copy()
    o.stage(cv, dv, 1, 0.0, threads=THREADS)
    return o, o.rhs[:c.mesh.nCells].copy(), o.grad[:c.mesh.nCells].copy()


@pytest.mark.parametrize("scheme,guard", [(K.DISCR_UPW_ROE, 0), (K.DISCR_UPW_ROE, 1),
                                          (K.DISCR_UPW_HLLC, 1)],
                         ids=["roe-refguard", "roe-guard", "hllc-guard"])
def test_tet128_residual_and_step_bitwise(tet128, scheme, guard):
    c = tet128.with_numerics(spaceDiscr=scheme, venkatGuard=guard, precision=K.PREC_FP64)
    o, rhs_o, grad_o = _oracle_stage1(c)
    r = E.Region(c)
    if guard == 0:
        # the reference's literal term numer/(denom + 1e-12) cancels for some
        # d2 < 0 faces of this mesh (modflu/RFLU_ModLimiters.F90:482-504): the
        # limiter goes to -inf there and the oracle's residual is not finite;
        # the engine reproduces exactly those entries, and nothing is stepped
        nonfinite = int(np.count_nonzero(~np.isfinite(rhs_o)))
        assert nonfinite > 0
        _same(r.residual(), rhs_o, "residual", finite=False)
        _same(r.gradients(), grad_o, "limited gradients", finite=False)
        r.close()
        return
    _same(r.residual(), rhs_o, "residual")
    _same(r.gradients(), grad_o, "limited gradients")
    # one whole time step: dt (the first step takes dtImposed = the CFL step of
    # the initial state, rocflu/RFLU_TimeStepping.F90) and the three Wray stages
    cv, dv = c.cv.copy(), c.dv.copy()
    dti = o.dt(cv, dv, c.numerics.cfl, 1.0, 0.0, 1.0)
    assert r.time_step(c.numerics.cfl, 1.0, 0.0, 1.0) == dti
    t_o, _, st_o = o.run(cv, dv, n_steps=1, dt_imposed=dti, threads=THREADS)
    t_g, _, st_g = r.solve(n_steps=1, dt_imposed=dti)
    assert t_g == t_o and st_g == st_o
    cvg, dvg = r.download()
    _same(cvg, cv, "cv after one RK3 step")
    _same(dvg, dv, "dv after one RK3 step")
    r.close()


@pytest.mark.parametrize("scheme", [K.DISCR_UPW_AUSMPLUS, K.DISCR_UPW_ROE, K.DISCR_UPW_HLLC],
                         ids=["ausm+", "roe", "hllc"])
def test_mixed96_residual(mixed96, scheme):
    c = mixed96.with_numerics(spaceDiscr=scheme, venkatGuard=1)
    _, rhs_o, grad_o = _oracle_stage1(c)
    r = E.Region(c)
    _same(r.residual(), rhs_o, "residual (FP64)")
    _same(r.gradients(), grad_o, "limited gradients (FP64)")
    r.close()
    for prec in (K.PREC_MIXED, K.PREC_SPLIT):
        m = E.Region(c, precision=prec)
        rhs_m = m.residual()
        m.close()
        err = np.abs(rhs_m - rhs_o).sum(axis=0) / np.abs(rhs_o).sum(axis=0)
        worst = np.abs(rhs_m - rhs_o).max(axis=0) / np.abs(rhs_o).max(axis=0)
        assert np.all(err <= 1e-5), (prec, err, worst)
