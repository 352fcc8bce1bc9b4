"""Partitioned cases on one GPU: regions with virtual cells advanced by a
coupled batch (one time step for all regions, the halo exchange after every
stage's update in one launch) or by the per-region stage call plus the border
calls, against the oracle's multi-region loop (MultiOracle: every region's
stage, then RFLU_MPI_CopyWrapper and the virtual cells' dependent variables)."""
import numpy as np
import pytest

from rocflupicl_gb300 import case as K
from rocflupicl_gb300 import engine as E
from rocflupicl_gb300 import partition as P

pytestmark = pytest.mark.gpu

N_STEPS = 5


def tube(order=2, discr=K.DISCR_UPW_ROE, prec=K.PREC_FP64, n=24):
    num = K.Numerics(spaceDiscr=discr, spaceOrder=order, venkatGuard=1, precision=prec)
    return K.tet_shock_box(n, ny=4, nz=4, length=(6.0, 1.0, 1.0), x_shock=2.0, numerics=num)


def oracle_run(parts, n_steps=N_STEPS):
    from oracle.oracle import MultiOracle
    mo = MultiOracle(parts)
    cvs = [p.cv.copy() for p in parts]
    dvs = [p.dv.copy() for p in parts]
    t, _, st = mo.run(cvs, dvs, n_steps=n_steps)
    return t, cvs, dvs, st


def first_dt(regs, cfl):
    return min(r.time_step(cfl, 1.0, 0.0, 1.0) for r in regs)


def batch_run(parts, n_steps=N_STEPS, graph=False):
    regs = [E.Region(p) for p in parts]
    cfl = parts[0].numerics.cfl
    d0 = first_dt(regs, cfl)
    for r in regs:
        r.set_time(0.0)
        r.sync()
    b = E.Batch(regs, coupled=True)
    if graph:
        b.steps_graph(n_steps, cfl, d0)
    else:
        for _ in range(n_steps):
            b.step(cfl, d0)
    b.sync()
    out = [r.download() for r in regs]
    times = [r.time()[0] for r in regs]
    st = [r.status() for r in regs]
    b.close()
    for r in regs:
        r.close()
    return out, times, st


def stage_run(parts, n_steps=N_STEPS, mode="copy", prec=None, dts=None):
    """The reference's loop through the per-region API: dt = min over regions,
    every region's stage, then the border exchange (device copies, or
    pack/unpack through host buffers as an MPI neighbour would)."""
    regs = [E.Region(p, precision=prec) for p in parts]
    idx = {r.iRegionGlobal: i for i, r in enumerate(regs)}
    cfl = parts[0].numerics.cfl
    nst = regs[0].nSteps
    d0 = first_dt(regs, cfl)
    t, used = 0.0, []
    for k in range(n_steps):
        dt = dts[k] if dts is not None else min(r.time_step(cfl, d0, 0.0, t) for r in regs)
        used.append(dt)
        for s in range(1, nst + 1):
            for r in regs:
                r.rk_stage(s, dt)
            for r in regs:
                for ib, b in enumerate(r.borders, start=1):
                    dst = regs[idx[b.iRegionGlobal]]
                    if mode == "copy":
                        r.border_copy(ib, dst)
                    else:
                        dst.border_unpack(b.iBorder, r.border_pack(ib))
        t += dt
    for r in regs:
        r.sync()
    out = [r.download() for r in regs]
    for r in regs:
        r.close()
    return out, t, used


@pytest.mark.parametrize("discr", [K.DISCR_UPW_ROE, K.DISCR_UPW_HLLC])
@pytest.mark.parametrize("kind", ["tets", "mixed_dip"])
def test_weno_xyz_partitioned_fp64_bitwise_oracle(discr, kind):
    """RECONST 2 (the reference's default reconstruction) on partitioned
    regions: the virtual cells' positivity check walks all their faces (AV,
    VV, VX and the patches' faces on virtual cells), as
    RFLU_LimitGradCellsSimple does; the coupled batch and the stage API with
    border copies equal the oracle's multi-region loop bit for bit."""
    from test_partition import weno_dip_case
    num = K.Numerics(spaceDiscr=discr, reconst=K.RECONST_WENO_XYZ, venkatGuard=1)
    if kind == "tets":
        c = K.tet_shock_box(18, ny=4, nz=4, length=(4.5, 1.0, 1.0), x_shock=1.5, numerics=num)
    else:
        c = weno_dip_case(num)  # the virtual faces decide some virtual cells' gradients
    parts = P.partition_case(c, 3)
    assert all(p.mesh.nFacesAll > p.mesh.nFaces for p in parts)
    t, cvs, dvs, st = oracle_run(parts)
    assert st == 0
    out, times, sts = batch_run(parts)
    for (cv, dv), ocv, odv in zip(out, cvs, dvs):
        assert np.array_equal(cv, ocv) and np.array_equal(dv, odv)
    assert all(x == t for x in times) and sts == [0, 0, 0]
    out2, t2, _ = stage_run(parts, mode="copy")
    assert t2 == t
    for (cv, dv), ocv, odv in zip(out2, cvs, dvs):
        assert np.array_equal(cv, ocv) and np.array_equal(dv, odv)


@pytest.mark.parametrize("discr", [K.DISCR_UPW_ROE, K.DISCR_UPW_HLLC, K.DISCR_UPW_AUSMPLUS])
def test_coupled_batch_fp64_bitwise_oracle(discr):
    parts = P.partition_case(tube(discr=discr), 3)
    t, cvs, dvs, st = oracle_run(parts)
    assert st == 0
    out, times, sts = batch_run(parts)
    for (cv, dv), ocv, odv, p in zip(out, cvs, dvs, parts):
        assert np.array_equal(cv, ocv)
        assert np.array_equal(dv, odv)
    assert all(x == t for x in times) and sts == [0, 0, 0]


def test_coupled_batch_graph_equals_steps():
    parts = P.partition_case(tube(), 4)
    a, ta, _ = batch_run(parts, graph=False)
    b, tb, _ = batch_run(parts, graph=True)
    assert ta == tb
    for (x, _), (y, _) in zip(a, b):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("mode", ["copy", "pack"])
def test_stage_api_with_border_calls_bitwise_oracle(mode):
    parts = P.partition_case(tube(), 3)
    t, cvs, dvs, _ = oracle_run(parts)
    out, t2, _ = stage_run(parts, mode=mode)
    assert t2 == t
    for (cv, dv), ocv, odv in zip(out, cvs, dvs):
        assert np.array_equal(cv, ocv)
        assert np.array_equal(dv, odv)


def test_first_order_partition_equals_single_region():
    c = tube(order=1)
    parts = P.partition_case(c, 3)
    r = E.Region(c)
    cfl = c.numerics.cfl
    d0 = r.time_step(cfl, 1.0, 0.0, 1.0)
    r.set_time(0.0)
    for _ in range(N_STEPS):
        r.step(cfl, d0)
    cv1, dv1 = r.download()
    r.close()
    out, _, _ = batch_run(parts)
    for p, (cv, dv) in zip(parts, out):
        p.cv[:], p.dv[:] = cv, dv
    assert np.array_equal(P.gather(parts, "cv"), cv1)
    assert np.array_equal(P.gather(parts, "dv"), dv1)


def test_residual_and_gradients_with_virtual_cells_bitwise_oracle():
    from oracle.oracle import Oracle
    p = P.partition_case(tube(), 3)[1]
    r = E.Region(p)
    rhs = r.residual()
    g = r.gradients()
    orhs, og = Oracle(p).residual(p.cv, p.dv)
    r.close()
    assert np.array_equal(rhs, orhs)
    assert not np.any(rhs[p.mesh.nCells:])
    assert np.array_equal(g, og)


def test_mixed_partition_close_to_fp64_and_batch_equals_stage_api():
    parts64 = P.partition_case(tube(), 3)
    ref, _, dts = stage_run(parts64, n_steps=10)
    partsM = P.partition_case(tube(prec=K.PREC_MIXED), 3)
    mixed, _, _ = stage_run(partsM, n_steps=10, prec=K.PREC_MIXED, dts=dts)
    # L1 = (1/Nc) sum |q/q_ref - 1| over the actual cells
    # (utilities/post/RFLU_ComputeExactFlowError.F90:946-976)
    err = np.concatenate([np.abs(a[:p.mesh.nCells, 0] / b[:p.mesh.nCells, 0] - 1.0)
                          for (a, _), (b, _), p in zip(mixed, ref, parts64)])
    assert err.mean() <= 1e-5
    # the coupled batch (device time step, one exchange launch) against the
    # per-region path: the batch's first stage runs the gradient pass that also
    # reduces the time step, a separate instantiation whose FP32 contractions
    # may round differently, so the two agree to FP32 rounding, not bit for bit
    # (the FP64 unit, compiled without contraction, agrees exactly above)
    b1, _, sts = batch_run(partsM, n_steps=4)
    s1, _, _ = stage_run(partsM, n_steps=4, prec=K.PREC_MIXED)
    assert sts == [0, 0, 0]
    err = np.concatenate([np.abs(x[:p.mesh.nCells, 0] / y[:p.mesh.nCells, 0] - 1.0)
                          for (x, _), (y, _), p in zip(b1, s1, partsM)])
    assert err.mean() <= 1e-6


def test_border_refusals():
    parts = P.partition_case(tube(n=12), 2)
    regs = [E.Region(p) for p in parts]
    with pytest.raises(E.EngineError) as ei:
        regs[0].step(0.5, 1e-7)
    assert ei.value.code == E.ERR_UNSUPPORTED
    with pytest.raises(E.EngineError) as ei:
        E.Batch(regs)  # a plain batch does not exchange halos
    assert ei.value.code == E.ERR_UNSUPPORTED
    with pytest.raises(E.EngineError) as ei:
        E.Batch(regs[:1], coupled=True)  # the neighbour is missing
    assert ei.value.code == E.ERR_ARG
    with pytest.raises(E.EngineError) as ei:
        regs[0].border_copy(1, regs[0])
    assert ei.value.code == E.ERR_ARG
    with pytest.raises(E.EngineError) as ei:
        regs[0].border_copy(len(parts[0].mesh.borders) + 1, regs[1])
    assert ei.value.code == E.ERR_ARG
    for r in regs:
        r.close()


def test_halo_launches_profiled():
    parts = P.partition_case(tube(), 3)
    regs = [E.Region(p) for p in parts]
    cfl = parts[0].numerics.cfl
    d0 = first_dt(regs, cfl)
    b = E.Batch(regs, coupled=True)
    b.profile(True)
    b.step(cfl, d0)
    prof = b.profile_read()
    assert prof["halo"][1] == regs[0].nSteps
    assert prof["dt_finalize"][1] == 1
    b.close()
    for r in regs:
        r.close()


def _variant(name):
    if name == "mixed_elements":
        c = K.mixed_box(8, numerics=K.Numerics(spaceDiscr=K.DISCR_UPW_HLLC, venkatGuard=1))
        return c, 3
    disc = K.DISCR_UPW_AUSMPLUSUP if name == "ausmup" else K.DISCR_UPW_ROE
    rk = {"rk4": K.RK_SCHEME_4_CLASSICAL, "euler": K.RK_SCHEME_1_EULER}.get(name,
                                                                          K.RK_SCHEME_3_WRAY)
    num = K.Numerics(spaceDiscr=disc, venkatGuard=1, rkScheme=rk)
    c = K.tet_shock_box(24, ny=4, nz=4, length=(6.0, 1.0, 1.0), x_shock=2.0, numerics=num)
    if name == "farfield":
        for ip in (0, 1):
            c.bcs[ip] = K.PatchBC(K.BC_FARFIELD, 2, 0,
                                  vals=np.array([0.6, 0.1, 0.05, 1.0e5, 300.0]))
    elif name == "inject":
        n0 = c.mesh.patches[2].n   # YLO wall, cut by every region
        vals = np.stack([np.linspace(1.0, 3.0, n0), np.full(n0, 320.0)], axis=1)
        c.bcs[2] = K.PatchBC(K.BC_INJECTION, 2, 0, vals=vals)
    elif name == "inflow":
        g = c.numerics.gamma_gv
        R = 8314.3 / c.numerics.gv[1]
        r2, u2, p2 = K.rankine_hugoniot(2.0, g, 1.2, 1.0e5)
        T2 = p2 / (r2 * R)
        m2 = u2 / np.sqrt(g * R * T2)
        f = 1.0 + 0.5 * (g - 1.0) * m2 * m2
        c.bcs[0] = K.PatchBC(K.BC_INFLOW_TOTANG, 2, K.BCOPT_MIXED,
                             vals=np.array([p2 * f ** (g / (g - 1.0)), T2 * f, 0.1, 0.05, m2]))
    elif name == "order1_patches":
        for ip in range(6):
            c.bcs[ip] = K.PatchBC(c.bcs[ip].bcType, 1, c.bcs[ip].bcOptType)
    return c, 3


@pytest.mark.parametrize("name", ["mixed_elements", "rk4", "euler", "ausmup", "farfield",
                                  "inject", "inflow", "order1_patches"])
def test_partition_variants_bitwise_oracle(name):
    c, n = _variant(name)
    parts = P.partition_case(c, n)
    t, cvs, dvs, st = oracle_run(parts, n_steps=4)
    out, times, sts = batch_run(parts, n_steps=4)
    for (cv, dv), ocv, odv in zip(out, cvs, dvs):
        if name == "inflow":  # the subsonic total-condition inflow's run-time power: ulps
            assert np.allclose(cv, ocv, rtol=1e-12, atol=0)
            assert np.allclose(dv, odv, rtol=1e-12, atol=0)
        else:
            assert np.array_equal(cv, ocv)
            assert np.array_equal(dv, odv)
    if name != "inflow":
        assert all(x == t for x in times)
    assert st == 0 and sts == [0] * len(parts)


def test_residual_noalloc_with_virtual_cells():
    p = P.partition_case(tube(n=12), 2)[1]
    r = E.Region(p)
    a = r.residual()
    b = r.residual_noalloc()
    r.close()
    assert np.array_equal(a, b)
    assert not np.any(b[p.mesh.nCells:])
