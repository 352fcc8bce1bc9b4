"""Host mesh builder: geometry invariants, stencil construction, determinism."""
import numpy as np
import pytest

from rocflupicl_gb300 import mesh as M


def closure(m):
    """Sum of outward face vectors per cell (must vanish for closed cells)."""
    s = np.zeros((m.nCells, 3))
    S = m.fn[:, :3] * m.fn[:, 3:4]
    np.add.at(s, m.f2c[:, 0] - 1, S)
    np.add.at(s, m.f2c[:, 1] - 1, -S)
    for p in m.patches:
        np.add.at(s, p.bf2c - 1, p.fn[:, :3] * p.fn[:, 3:4])
    return s


@pytest.mark.parametrize("kind,dims,jit", [(M.HEX, (10, 2, 2), 0.0), (M.TET, (4, 3, 5), 0.1),
                                           (M.MIXED, (6, 6, 6), 0.0), (M.HEX, (5, 4, 3), 0.1)])
def test_geometry_closed_and_volume(kind, dims, jit):
    hi = (1.0, 0.5, 2.0)
    m = M.box(kind, *dims, hi=hi, jitter=jit, seed=3)
    assert np.all(m.vol > 0)
    assert abs(m.vol.sum() - 1.0) < 1e-12
    cl = closure(m)
    scale = np.abs(m.fn[:, 3]).max()
    assert np.abs(cl).max() < 1e-12 * scale
    # boundary faces lie on the box surface of their patch
    for ip, p in enumerate(m.patches):
        d, side = divmod(ip, 2)
        want = 0.0 if side == 0 else hi[d]
        assert np.allclose(p.fc[:, d], want)
        assert np.all(np.sign(p.fn[:, d]) == (-1 if side == 0 else 1))


def test_counts_hex_tube():
    m = M.box(M.HEX, 1000, 2, 2, hi=(1.0, 0.01, 0.01))
    assert m.nCells == 4000
    assert m.nFaces == 999 * 4 + 1000 * 2 * 2
    assert m.nBFaces == 2 * 4 + 4 * 2000
    # hex stencils are the full vertex-neighbour sets, never truncated
    sizes = np.diff(m.c2cs_off)
    assert set(sizes.tolist()) <= {7, 11}


def test_counts_kuhn_tets():
    m = M.box(M.TET, 8, 8, 8, jitter=0.1, seed=1)
    assert m.nCells == 6 * 512
    assert m.nFaces == (4 * 6 * 512 - 6 * 2 * 64) // 2
    sizes = np.diff(m.c2cs_off)
    assert sizes.max() == 40 and sizes.min() >= 4


def test_mixed_types_and_conformity():
    m = M.box(M.MIXED, 8, 8, 8)
    nt, nh, npr, npy = m.n_of_type
    assert nh == 4 * 8 * 4          # x<0.5, z<0.5
    assert npr == 2 * 4 * 8 * 8     # x>0.5 (prism precedence)
    assert npy > 0 and nt > 0
    # conforming: every face has exactly one or two cells and cells are closed
    assert np.abs(closure(m)).max() < 1e-13


def test_stencils_sorted_and_moments_spd():
    m = M.box(M.TET, 5, 5, 5, jitter=0.1, seed=2)
    for c in range(0, m.nCells, 37):
        memb = m.c2cs_mem[m.c2cs_off[c]:m.c2cs_off[c + 1]]
        assert np.all(np.diff(memb) > 0)           # first layer re-sorted by index
        assert c + 1 not in memb
    r = m.xyzmoms
    assert np.all(r[:, 0] > 0) and np.all(r[:, 2] > 0) and np.all(r[:, 5] > 0)


def test_wlsq_moments_match_definition():
    """xyzMoms = Cholesky factor of sum of unit direction outer products."""
    m = M.box(M.TET, 3, 3, 3, jitter=0.1, seed=9)
    for c in range(0, m.nCells, 11):
        memb = m.c2cs_mem[m.c2cs_off[c]:m.c2cs_off[c + 1]] - 1
        d = m.cofg[memb] - m.cofg[c]
        dh = d / np.linalg.norm(d, axis=1)[:, None]
        A = dh.T @ dh
        Lc = np.linalg.cholesky(A)
        r = m.xyzmoms[c]
        assert np.allclose([Lc[0, 0], Lc[1, 0], Lc[1, 1], Lc[2, 0], Lc[2, 1], Lc[2, 2]],
                           r[:6], rtol=1e-12)


def test_deterministic_across_thread_counts():
    a = M.box(M.TET, 6, 5, 4, jitter=0.1, seed=4, threads=1)
    b = M.box(M.TET, 6, 5, 4, jitter=0.1, seed=4, threads=4)
    for f in ("xyz", "vol", "cofg", "f2c", "fn", "fc", "c2cs_off", "c2cs_mem", "xyzmoms"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f


def test_bad_arguments_rejected():
    with pytest.raises(RuntimeError):
        M.box(M.HEX, 0, 2, 2)
    with pytest.raises(RuntimeError):
        M.box(7, 2, 2, 2)


def test_deferred_stencils_roundtrip():
    """A mesh built with its stencils deferred and then given the host
    builder's stencils and moments through rfmesh_set_stencils exports the
    same arrays as a mesh built in one go (the path the GPU builder uses)."""
    import ctypes as C
    from rocflupicl_gb300 import mesh as M
    ref = M.box(M.TET, 4, 3, 3, jitter=0.1, seed=9)
    lib = M._load()
    h = C.c_void_p()
    lo = (C.c_double * 3)(0.0, 0.0, 0.0)
    hi = (C.c_double * 3)(1.0, 1.0, 1.0)
    assert lib.rfmesh_create_box_ex(M.TET, 4, 3, 3, lo, hi, 0.1, 9, 0, M.RFMESH_DEFER_STENCILS,
                                    C.byref(h)) == 0
    try:
        off = np.ascontiguousarray(ref.c2cs_off, np.int32)
        mem = np.ascontiguousarray(ref.c2cs_mem, np.int32)
        mom = np.ascontiguousarray(ref.xyzmoms, np.float64)
        assert lib.rfmesh_set_stencils(h, off.ctypes.data_as(C.POINTER(C.c_int)),
                                       mem.ctypes.data_as(C.POINTER(C.c_int)),
                                       mom.ctypes.data_as(C.POINTER(C.c_double))) == 0
        n = ref.nCells
        got_off = np.ctypeslib.as_array(lib.rfmesh_c2cs_offsets(h), shape=(n + 1,))
        got_mem = np.ctypeslib.as_array(lib.rfmesh_c2cs_members(h), shape=(int(off[-1]),))
        got_mom = np.ctypeslib.as_array(lib.rfmesh_xyzmoms(h), shape=(10 * n,))
        assert np.array_equal(got_off, off) and np.array_equal(got_mem, mem)
        assert np.array_equal(got_mom, mom.ravel())
        cv = np.ctypeslib.as_array(lib.rfmesh_cell_verts(h), shape=(8 * n,)).reshape(n, 8)
        nv = np.ctypeslib.as_array(lib.rfmesh_cell_nverts(h), shape=(n,))
        assert np.all(nv == 4) and np.all(cv[:, 4:] == -1) and cv[:, :4].min() >= 0
        # members out of range are refused
        bad = mem.copy()
        bad[0] = n + 1
        assert lib.rfmesh_set_stencils(h, off.ctypes.data_as(C.POINTER(C.c_int)),
                                       bad.ctypes.data_as(C.POINTER(C.c_int)),
                                       mom.ctypes.data_as(C.POINTER(C.c_double))) != 0
    finally:
        lib.rfmesh_destroy(h)
