"""Launch shapes (rfgpu_set_tuning) change where the work runs, never what it
computes: every shape the autotuner may pick gives the same state bit for
bit, on a region and on a batch, and shapes outside the documented values are
refused."""
import itertools

import numpy as np
import pytest

from rocflupicl_gb300 import autotune
from rocflupicl_gb300 import case as K
from rocflupicl_gb300 import engine as E

pytestmark = pytest.mark.gpu

SHAPES = [dict(gridCap=g, gradBlock=gb, faceBlock=fb, facesPerThread=fpt, cellBlock=cb)
          for g, gb, fb, fpt, cb in itertools.product((0, 152), (64, 256), (64, 128, 256), (1, 2),
                                                       (64, 256))]


def _run(c, shape, steps=3):
    r = E.Region(c)
    if shape is not None:
        r.set_tuning(**shape)
    r.solve(n_steps=steps)
    out = r.download()
    r.close()
    return out


@pytest.mark.parametrize("prec", [K.PREC_FP64, K.PREC_MIXED, K.PREC_SPLIT],
                         ids=["fp64", "mixed", "split"])
def test_every_shape_gives_the_same_state(prec):
    c = K.tet_shock_box(5, ny=3, nz=7, seed=4,
                        numerics=K.Numerics(spaceDiscr=K.DISCR_UPW_HLLC, venkatGuard=1,
                                            precision=prec))
    cv0, dv0 = _run(c, None)
    for shape in SHAPES[:: 3 if prec != K.PREC_FP64 else 6]:
        cv, dv = _run(c, shape)
        assert np.array_equal(cv, cv0) and np.array_equal(dv, dv0), shape


def test_batch_shapes_and_autotuner():
    cases = K.tube_ensemble(count=4, seed=3, n_min=20, n_max=300, cross=2,
                            numerics=K.Numerics(precision=K.PREC_MIXED, venkatGuard=1))
    cfl = cases[0].numerics.cfl

    def run(shape, steps=6):
        regs = [E.Region(c) for c in cases]
        for r in regs:
            r.set_time(0.0)
        b = E.Batch(regs)
        if shape is not None:
            b.set_tuning(**shape)
        for _ in range(steps):
            b.step(cfl, 1e-6)
        b.sync()
        out = [r.download() for r in regs]
        b.close()
        for r in regs:
            r.close()
        return out

    # the autotuner on its own batch: a valid shape, then that shape's run
    regs = [E.Region(c) for c in cases]
    for r in regs:
        r.set_time(0.0)
    b = E.Batch(regs)
    t = autotune.tune_batch(b, cfl, 1e-6, steps=1)
    assert set(t["shape"]) == set(E.TUNING_KEYS) and t["shape"]["gradBlock"] in (64, 128, 256)
    b.close()
    for r in regs:
        r.close()
    ref = run(None)
    for shape in (SHAPES[5], SHAPES[-1], t["shape"]):
        got = run(shape)
        for (cv, dv), (cv0, dv0) in zip(got, ref):
            assert np.array_equal(cv, cv0) and np.array_equal(dv, dv0), shape


def test_region_autotuner_keeps_a_valid_shape():
    c = K.tet_shock_box(6, seed=2, numerics=K.Numerics(spaceDiscr=K.DISCR_UPW_ROE, venkatGuard=1,
                                                        precision=K.PREC_MIXED))
    r = E.Region(c)
    cfl = c.numerics.cfl
    dti = r.time_step(cfl, 1.0, 0.0, 1.0)
    r.set_time(0.0)
    t = autotune.tune_region(r, cfl, dti, steps=1, grid_caps=[0, 2 * autotune.sm_count()])
    assert t["shape"]["gradBlock"] in (64, 128, 256)
    assert t["shape"]["facesPerThread"] in (1, 2)
    assert t["sms"] == E.sm_count() > 0
    r.step(cfl, dti)
    assert r.status() == 0
    r.close()


@pytest.mark.parametrize("bad", [dict(gradBlock=96), dict(faceBlock=512), dict(facesPerThread=3),
                                 dict(cellBlock=32), dict(gridCap=-1)])
def test_bad_shapes_refused(bad):
    r = E.Region(K.shock_tube(8, numerics=K.Numerics(venkatGuard=1)))
    with pytest.raises(E.EngineError) as ei:
        r.set_tuning(**bad)
    assert ei.value.code == E.ERR_ARG
    r.close()
