"""Partitioned regions on the host: the partition's structure, the oracle's
multi-region stage loop against the whole mesh, and the C ABI's validation
of virtual cells and borders (no GPU)."""
import ctypes as C

import numpy as np
import pytest

from rocflupicl_gb300 import case as K
from rocflupicl_gb300 import engine as E
from rocflupicl_gb300 import partition as P


def tube(order=2, discr=K.DISCR_UPW_ROE, prec=K.PREC_FP64, n=24):
    num = K.Numerics(spaceDiscr=discr, spaceOrder=order, venkatGuard=1, precision=prec)
    return K.tet_shock_box(n, ny=4, nz=4, length=(6.0, 1.0, 1.0), x_shock=2.0, numerics=num)


def test_partition_structure():
    c = tube()
    m = c.mesh
    parts = P.partition_case(c, 3)
    own = np.concatenate([p.mesh.global_cells[:p.mesh.nCells] for p in parts])
    assert np.array_equal(np.sort(own), np.arange(m.nCells))  # every cell owned once
    mem0 = m.c2cs_mem - 1
    for p in parts:
        g = p.mesh
        loc = g.global_cells
        assert g.nCellsTot == loc.shape[0] > g.nCells
        act = set(loc[:g.nCells].tolist())
        present = set(loc.tolist())
        # the whole-mesh stencils and face neighbours of actual cells are present
        for c0 in loc[:g.nCells]:
            assert set(mem0[m.c2cs_off[c0]:m.c2cs_off[c0 + 1]].tolist()) <= present
        # every face with an actual cell, in the whole mesh's order
        fa = m.f2c - 1
        sel = np.flatnonzero(np.isin(fa[:, 0], list(act)) | np.isin(fa[:, 1], list(act)))
        assert g.nFaces == sel.shape[0]
        assert np.array_equal(loc[g.f2c - 1], fa[sel])
        # virtual cells in ascending whole-mesh id
        assert np.all(np.diff(loc[g.nCells:]) > 0)
        # every virtual cell is received exactly once
        rec = np.concatenate([b.icgRecv for b in g.borders])
        assert np.array_equal(np.sort(rec), np.arange(g.nCells + 1, g.nCellsTot + 1))
        for b in g.borders:
            nb = parts[b.iRegionGlobal - 1].mesh
            b2 = nb.borders[b.iBorder - 1]
            assert b2.iRegionGlobal == g.iRegionGlobal
            assert np.all(b.icgSend <= g.nCells)
            # send cell k here is receive cell k there: the same whole-mesh cell
            assert np.array_equal(loc[b.icgSend - 1], nb.global_cells[b2.icgRecv - 1])


def _run_multi(parts, n_steps):
    from oracle.oracle import MultiOracle
    mo = MultiOracle(parts)
    cvs = [p.cv.copy() for p in parts]
    dvs = [p.dv.copy() for p in parts]
    t, k, st = mo.run(cvs, dvs, n_steps=n_steps)
    return t, cvs, dvs, st


def test_oracle_first_order_partition_equals_whole_mesh():
    """First order: an actual cell's residual sums the same face fluxes in the
    same order in its region as in the whole mesh (faces keep the whole mesh's
    order, virtual cells carry their owners' state), and the global time step is
    the whole mesh's, so the partitioned run is bit-identical."""
    from oracle.oracle import Oracle
    c = tube(order=1)
    parts = P.partition_case(c, 3)
    cv, dv = c.cv.copy(), c.dv.copy()
    t0, _, _ = Oracle(c).run(cv, dv, n_steps=6)
    t1, cvs, dvs, st = _run_multi(parts, 6)
    assert st == 0 and t1 == t0
    for p, x, y in zip(parts, cvs, dvs):
        p.cv[:], p.dv[:] = x, y
    assert np.array_equal(P.gather(parts, "cv"), cv)
    assert np.array_equal(P.gather(parts, "dv"), dv)


def test_oracle_second_order_partition_close_to_whole_mesh():
    """Second order: a virtual cell's limiter sees only the faces its region
    holds (RFLU_ComputeLimiterVenkat runs over 1..nFaces) and its stencil is
    the region's own, so the partitioned run differs from the whole-mesh one
    near borders, as in the reference; it stays close."""
    from oracle.oracle import Oracle
    c = tube(order=2)
    parts = P.partition_case(c, 3)
    cv, dv = c.cv.copy(), c.dv.copy()
    Oracle(c).run(cv, dv, n_steps=6)
    _, cvs, _, st = _run_multi(parts, 6)
    assert st == 0
    for p, x in zip(parts, cvs):
        p.cv[:] = x
    g = P.gather(parts, "cv")
    l1 = np.abs(g[:, 0] - cv[:, 0]).sum() / np.abs(cv[:, 0]).sum()
    assert 0.0 < l1 < 2e-3


def test_oracle_omp_stage_equals_serial_with_virtual_cells():
    from oracle.oracle import Oracle
    parts = P.partition_case(tube(order=2), 3)
    p = parts[1]
    oa, ob = Oracle(p), Oracle(p)
    a_cv, a_dv, b_cv, b_dv = p.cv.copy(), p.dv.copy(), p.cv.copy(), p.dv.copy()
    for s in (1, 2, 3):
        oa.stage(a_cv, a_dv, s, 1e-7)
        ob.stage(b_cv, b_dv, s, 1e-7, threads=4)
    assert np.array_equal(a_cv, b_cv) and np.array_equal(a_dv, b_dv)
    assert np.array_equal(oa.rhs, ob.rhs)
    assert not np.any(oa.rhs[p.mesh.nCells:])  # ZeroDummyCellsMP


def _desc_of(case, **over):
    """A region descriptor through Region's field filling, without creating it."""
    from test_abi import _desc
    lib, d, keep = _desc(case)
    m = case.mesh
    d.nCellsTot = m.nTot
    d.iRegionGlobal = m.iRegionGlobal
    barr = (E.BorderT * max(1, len(m.borders)))()
    for i, b in enumerate(m.borders):
        s = np.ascontiguousarray(b.icgSend, np.int32)
        r = np.ascontiguousarray(b.icgRecv, np.int32)
        keep += [s, r]
        barr[i].iRegionGlobal, barr[i].iBorder = b.iRegionGlobal, b.iBorder
        barr[i].nCellsSend, barr[i].icgSend = s.shape[0], E._ip(s)
        barr[i].nCellsRecv, barr[i].icgRecv = r.shape[0], E._ip(r)
    d.nBorders = len(m.borders)
    d.borders = barr
    keep.append(barr)
    for key, val in over.items():
        setattr(d, key, val)
    return lib, d, keep


@pytest.mark.parametrize("bad", ["recv_actual", "send_virtual", "tot_small", "iborder"])
def test_border_indices_refused_before_any_cuda_call(bad):
    p = P.partition_case(tube(order=2, n=12), 2)[0]
    lib, d, keep = _desc_of(p)
    b = d.borders[0]
    if bad == "recv_actual":
        arr = np.array([1] * b.nCellsRecv, np.int32)
        keep.append(arr)
        b.icgRecv = E._ip(arr)
    elif bad == "send_virtual":
        arr = np.full(b.nCellsSend, p.mesh.nCells + 1, np.int32)
        keep.append(arr)
        b.icgSend = E._ip(arr)
    elif bad == "tot_small":
        d.nCellsTot = p.mesh.nCells - 1
    else:
        b.iBorder = 0
    h = C.c_void_p()
    assert lib.rfgpu_region_create(C.byref(d), C.byref(h)) == E.ERR_ARG
    assert not h.value


def test_border_calls_reject_null_handles():
    lib = E.load()
    assert lib.rfgpu_border_copy(None, 1, None) == E.ERR_ARG
    buf = np.zeros(5)
    assert lib.rfgpu_border_pack(None, 1, E._dp(buf)) == E.ERR_ARG
    assert lib.rfgpu_border_unpack(None, 1, E._dp(buf)) == E.ERR_ARG
    out = C.c_void_p()
    assert lib.rfgpu_batch_create_ex(None, 0, E.BATCH_COUPLED, C.byref(out)) == E.ERR_ARG


def test_partition_splits_per_face_patch_values():
    c = tube(order=2)
    n0 = c.mesh.patches[2].n
    vals = np.stack([np.arange(n0, dtype=float), np.full(n0, 320.0)], axis=1)
    c.bcs[2] = K.PatchBC(K.BC_INJECTION, 2, 0, vals=vals)
    parts = P.partition_case(c, 3)
    got = []
    for p in parts:
        pa = p.mesh.patches[2]
        assert p.bcs[2].vals.shape == (pa.n, 2)
        assert np.array_equal(p.bcs[2].vals[:, 0], pa.global_faces.astype(float))
        got.append(pa.global_faces)
    assert np.array_equal(np.sort(np.concatenate(got)), np.arange(n0))


def test_region_face_lists_cover_every_face_of_every_cell():
    """The flux faces (AA, AV), the virtual cells' VV and VX faces and the
    patches' faces on actual and virtual cells give every cell of a region,
    actual or virtual, exactly the faces of its type: RFLU_LimitGradCellsSimple
    (RECONST 2) walks all of them."""
    c = K.mixed_box(6, numerics=K.Numerics(reconst=K.RECONST_WENO_XYZ, venkatGuard=1))
    per_type = {0: 4, 1: 6, 2: 5, 3: 5}   # tet, hex, prism, pyramid
    for p in P.partition_case(c, 3):
        m = p.mesh
        f2c, fn, fc = m.all_faces()
        assert f2c.shape[0] == fn.shape[0] == fc.shape[0] == m.nFacesAll > m.nFaces
        extra = f2c[m.nFaces:]
        virt = (extra > m.nCells) & (extra <= m.nTot)
        assert np.all(virt.any(axis=1))                      # VV / VX: a virtual side
        assert np.all(virt | (extra == 0))                   # the other virtual or outside
        cnt = np.zeros(m.nTot + 1, int)
        for k in (0, 1):
            np.add.at(cnt, f2c[:, k], 1)
        for pa in m.patches:
            assert np.all(pa.bf2c <= m.nCells)
            if pa.n_vb:
                assert np.all(pa.vb_bf2c > m.nCells)
            np.add.at(cnt, pa.all_faces()[0], 1)
        assert np.array_equal(cnt[1:], [per_type[t] for t in m.cell_type])


@pytest.mark.parametrize("bad", ["vv_actual", "vb_actual", "all_small"])
def test_virtual_faces_refused_before_any_cuda_call(bad):
    """Faces past the flux faces must have a virtual side, a patch's faces past
    nBFaces must sit on virtual cells, nFacesAll may not undercut nFaces."""
    p = P.partition_case(tube(order=2, n=12), 2)[0].with_numerics(reconst=K.RECONST_WENO_XYZ)
    lib, d, keep = _desc_of(p)
    m = p.mesh
    f2c, fn, fc = (np.ascontiguousarray(a) for a in m.all_faces())
    f2c = f2c.astype(np.int32)
    keep += [f2c, fn, fc]
    d.f2c, d.fn, d.fc, d.nFacesAll = E._ip(f2c), E._dp(fn), E._dp(fc), m.nFacesAll
    if bad == "vv_actual":
        f2c[m.nFaces] = (1, 2)
    elif bad == "all_small":
        d.nFacesAll = m.nFaces - 1
    else:
        pa = next(x for x in m.patches if x.n > 0)
        bf = np.concatenate([pa.bf2c, [1]]).astype(np.int32)
        bfn = np.concatenate([pa.fn, pa.fn[:1]])
        bfc = np.concatenate([pa.fc, pa.fc[:1]])
        keep += [bf, bfn, bfc]
        parr = (E.PatchT * 1)()
        parr[0].bcType, parr[0].spaceOrder, parr[0].nBFaces = K.BC_SLIPWALL, 2, pa.n
        parr[0].nBFacesTot = pa.n + 1
        parr[0].bf2c, parr[0].fn, parr[0].fc = E._ip(bf), E._dp(bfn), E._dp(bfc)
        keep.append(parr)
        d.nPatches, d.patches = 1, parr
    h = C.c_void_p()
    assert lib.rfgpu_region_create(C.byref(d), C.byref(h)) == E.ERR_ARG
    assert not h.value


def weno_dip_case(num):
    """Mixed 8^3 box whose density dips to 0.02 at x = 0.65, inside the second
    slab of a 3-region partition: RECONST 2's positivity check fires there,
    and on some virtual cells only through a face between two virtual cells,
    to a cell outside the region or on a patch."""
    c = K.mixed_box(8, numerics=num)
    x = c.mesh.cofg[:, 0]
    c.cv *= (0.02 + 4.0 * (x - 0.65) ** 2)[:, None]
    c.dv = K.eos_dv(c.numerics, c.cv)
    return c


def test_virtual_faces_decide_some_virtual_gradients():
    """In the dip case the oracle's limited gradients of some virtual cells
    change when their VV / VX / VB faces are left out (and of no actual cell):
    those faces are on the tested path."""
    import dataclasses
    from oracle.oracle import Oracle
    num = K.Numerics(spaceDiscr=K.DISCR_UPW_ROE, reconst=K.RECONST_WENO_XYZ, venkatGuard=1)
    changed = 0
    for p in P.partition_case(weno_dip_case(num), 3):
        m = p.mesh
        bare = dataclasses.replace(m, vf2c=None, vfn=None, vfc=None, patches=[
            dataclasses.replace(pa, vb_bf2c=None, vb_fn=None, vb_fc=None) for pa in m.patches])
        _, g1 = Oracle(p).residual(p.cv, p.dv)
        _, g2 = Oracle(dataclasses.replace(p, mesh=bare)).residual(p.cv, p.dv)
        diff = np.flatnonzero(np.any(g1 != g2, axis=(1, 2)))
        assert np.all(diff >= m.nCells)
        changed += diff.size
    assert changed > 0
