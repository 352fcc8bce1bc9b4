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
    # a chosen persistent stage keeps the default block shapes (0)
    assert set(t["shape"]) == set(E.TUNING_KEYS) and t["shape"]["gradBlock"] in (0, 64, 128, 256)
    assert t["shape"]["persistentStage"] in (0, 1)
    b.close()
    for r in regs:
        r.close()
    ref = run(None)
    for shape in (SHAPES[5], SHAPES[-1], t["shape"]):
        got = run(shape)
        for (cv, dv), (cv0, dv0) in zip(got, ref):
            if shape.get("persistentStage"):
                assert_fp32_close(cv, cv0) and assert_fp32_close(dv, dv0)
            else:
                assert np.array_equal(cv, cv0) and np.array_equal(dv, dv0), shape


def test_region_autotuner_keeps_a_valid_shape():
    c = K.tet_shock_box(6, seed=2, numerics=K.Numerics(spaceDiscr=K.DISCR_UPW_ROE, venkatGuard=1,
                                                        precision=K.PREC_MIXED))
    r = E.Region(c)
    cfl = c.numerics.cfl
    dti = r.time_step(cfl, 1.0, 0.0, 1.0)
    r.set_time(0.0)
    t = autotune.tune_region(r, cfl, dti, steps=1, grid_caps=[0, 2 * autotune.sm_count()])
    assert t["shape"]["gradBlock"] in (0, 64, 128, 256)   # 0: the persistent stage won
    assert t["shape"]["facesPerThread"] in (0, 1, 2)
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


def assert_fp32_close(a, b):
    """The persistent stage kernel inlines the per-pass kernels' device code in
    another kernel, where the mixed unit's FMA contraction may round a
    product differently.  Those FP32 rounding differences stay at FP32 level
    on average; where they tip the Venkatakrishnan limiter's minimum over a
    cell's faces a single cell can move further (up to ~4e-4 relative after
    three steps on the shock box), as between any two FP32 evaluations."""
    assert np.all(np.isfinite(a))
    rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-30)
    assert rel.max() <= 1e-3 and rel.mean() <= 1e-6, (rel.max(), rel.mean())
    return True


@pytest.mark.parametrize("prec", [K.PREC_FP64, K.PREC_MIXED, K.PREC_SPLIT],
                         ids=["fp64", "mixed", "split"])
@pytest.mark.parametrize("reconst", [K.RECONST_LIM_VENKAT, K.RECONST_WENO_XYZ])
def test_persistent_stage_equals_per_pass_launches(prec, reconst):
    """One cooperative launch per RK stage (grid-wide barriers between the
    passes) against one launch per pass, on a region (stream steps and graph
    replay): bit for bit on the FP64 path (compiled without contraction),
    within FP32 rounding on the reduced-precision paths."""
    c = K.tet_shock_box(6, ny=4, nz=5, seed=4,
                        numerics=K.Numerics(spaceDiscr=K.DISCR_UPW_ROE, venkatGuard=1,
                                            precision=prec, reconst=reconst))

    def same(a, b):
        if prec == K.PREC_FP64:
            assert np.array_equal(a, b)
        else:
            assert_fp32_close(a, b)

    cv0, dv0 = _run(c, None)
    for shape in (dict(persistentStage=1), dict(persistentStage=1, gridCap=40)):
        cv, dv = _run(c, shape)
        same(cv, cv0)
        same(dv, dv0)
    r = E.Region(c)
    r.set_tuning(persistentStage=1)
    r.solve(n_steps=3, graph=True)
    cvg, dvg = r.download()
    same(cvg, cv0)
    same(dvg, dv0)
    assert r.status() == 0
    r.close()


def test_persistent_stage_coupled_batch():
    """A coupled batch (halo exchange after every update) run with one
    launch per stage equals the per-pass launches bit for bit (FP64)."""
    from rocflupicl_gb300 import partition as P
    c = K.tet_shock_box(12, ny=4, nz=4, length=(3.0, 1.0, 1.0), x_shock=1.0,
                        numerics=K.Numerics(spaceDiscr=K.DISCR_UPW_HLLC, venkatGuard=1))
    parts = P.partition_case(c, 3)
    outs = []
    for coop in (0, 1):
        regs = [E.Region(p) for p in parts]
        cfl = parts[0].numerics.cfl
        d0 = min(r.time_step(cfl, 1.0, 0.0, 1.0) for r in regs)
        for r in regs:
            r.set_time(0.0)
            r.sync()
        b = E.Batch(regs, coupled=True)
        b.set_tuning(persistentStage=coop)
        b.steps_graph(4, cfl, d0)
        b.sync()
        outs.append([r.download() for r in regs])
        b.close()
        for r in regs:
            r.close()
    for (cv0, dv0), (cv1, dv1) in zip(*outs):
        assert np.array_equal(cv0, cv1) and np.array_equal(dv0, dv1)


def test_persistent_stage_barrier_wait_runs_out():
    """Failure detection without a GPU fault: the persistent stage's grid-wide
    barrier is made to wait for a block that never arrives; its bounded wait
    (a million SM cycles here) runs out, the launch ends, rfgpu_batch_sync
    reports RFGPU_ERR_TIMEOUT, and the context stays usable."""
    cases = K.tube_ensemble(count=3, seed=5, n_min=40, n_max=200, cross=2,
                            numerics=K.Numerics(precision=K.PREC_MIXED, venkatGuard=1))
    regs = [E.Region(c) for c in cases]
    for r in regs:
        r.set_time(0.0)
    b = E.Batch(regs)
    b.set_tuning(persistentStage=1)
    b.test_barrier(1, 1_000_000)
    b.step(cases[0].numerics.cfl, 1e-6)
    with pytest.raises(E.EngineError) as ei:
        b.sync()
    assert ei.value.code == E.ERR_TIMEOUT
    b.sync()                                  # the error word was cleared
    b.test_barrier(0)
    for r, c in zip(regs, cases):             # a fresh state, then normal steps
        r.upload(c.cv, c.dv)
        r.set_time(0.0)
    for _ in range(3):
        b.step(cases[0].numerics.cfl, 1e-6)
    b.sync()
    for r in regs:
        cv, _ = r.download()
        assert np.all(np.isfinite(cv)) and r.status() == 0
    b.close()
    for r in regs:
        r.close()


def test_persistent_stage_refuses_other_block_shapes():
    r = E.Region(K.shock_tube(8, numerics=K.Numerics(venkatGuard=1)))
    with pytest.raises(E.EngineError) as ei:
        r.set_tuning(persistentStage=1, faceBlock=256)
    assert ei.value.code == E.ERR_ARG
    r.close()
