"""Batched execution: many independent regions advanced by one launch per pass
(persistent grid over a tile work list), captured in a CUDA graph.  Each
region's arithmetic is independent of its batch mates, so a region gives the
same bits alone and in a batch."""
import numpy as np
import pytest

from rocflupicl_gb300 import case as K
from rocflupicl_gb300 import engine as E

pytestmark = pytest.mark.gpu


def tubes(prec, count=5):
    return K.tube_ensemble(count=count, seed=3, n_min=20, n_max=120, cross=2,
                           numerics=K.Numerics(precision=prec, venkatGuard=1))


@pytest.mark.parametrize("prec", [K.PREC_FP64, K.PREC_MIXED, K.PREC_SPLIT])
def test_batch_equals_individual_runs(prec):
    cases = tubes(prec)
    cfl = cases[0].numerics.cfl
    alone = []
    for c in cases:
        r = E.Region(c)
        dti = r.time_step(cfl, 1.0, 0.0, 1.0)
        r.set_time(0.0)
        for _ in range(7):
            r.step(cfl, dti)
        alone.append(r.download())
        r.close()
    regs = [E.Region(c) for c in cases]
    dtis = [r.time_step(cfl, 1.0, 0.0, 1.0) for r in regs]
    for r in regs:
        r.set_time(0.0)
    # all tubes share one imposed first step in a batch: use each tube's own by
    # running step 1 per region, then the rest batched
    for r, d in zip(regs, dtis):
        r.step(cfl, d)
        r.sync()
    b = E.Batch(regs)
    # after step 1 the device time is > 1e-8 so dtImposed is no longer used
    for _ in range(3):
        b.step(cfl, 1.0)
    b.steps_graph(3, cfl, 1.0)
    b.sync()
    for r, (cv, dv) in zip(regs, alone):
        cvb, dvb = r.download()
        assert np.array_equal(cvb, cv)
        assert np.array_equal(dvb, dv)
    assert b.launches > 0
    b.close()
    for r in regs:
        r.close()


def test_batch_fp64_matches_oracle():
    from oracle.oracle import Oracle
    cases = tubes(K.PREC_FP64, count=3)
    cfl = cases[0].numerics.cfl
    regs = [E.Region(c) for c in cases]
    for r, c in zip(regs, cases):
        r.set_time(0.0)
    b = E.Batch(regs)
    dti = [r.time_step(cfl, 1.0, 0.0, 1.0) for r in regs]
    # a common imposed first step for all members
    d0 = min(dti)
    b.steps_graph(4, cfl, d0)
    b.sync()
    for r, c in zip(regs, cases):
        o = Oracle(c)
        cv, dv = c.cv.copy(), c.dv.copy()
        o.run(cv, dv, n_steps=4, dt_imposed=d0)
        cvb, dvb = r.download()
        assert np.array_equal(cvb, cv) and np.array_equal(dvb, dv)
    b.close()
