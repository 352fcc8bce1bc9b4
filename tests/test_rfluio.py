"""Grid and flow files in the reference's formats (rocflupicl_gb300/rfluio.py):
the Fortran edit descriptors, ASCII and binary round trips, and a mesh read
back from a grid file reproducing the mesh it was written from."""
import numpy as np
import pytest

from rocflupicl_gb300 import mesh as M
from rocflupicl_gb300 import rfluio as IO


def test_e23_16_known_answers():
    assert IO._e23_16(1.0) == " 0.1000000000000000E+01"
    assert IO._e23_16(-2.5e-10) == "-0.2500000000000000E-09"
    assert IO._e23_16(0.0) == " 0.0000000000000000E+00"
    assert IO._e23_16(1.0e100) == " 0.1000000000000000+101"
    assert IO._e23_16(1.0 / 3.0) == " 0.3333333333333333E+00"
    assert IO._e23_16(123456.789) == " 0.1234567890000000E+06"
    for s in (" 0.1000000000000000E+01", "-0.2500000000000000E-09", " 0.1000000000000000+101",
              "0.25D+02"):
        assert IO._read_e(s) == float(s.replace("D", "E").replace("0+101", "0E+101"))
    assert all(len(IO._e23_16(x)) == 23 for x in (1e-300, -7.0, 1e300, 5e-324 * 1e10))


def test_grid_ascii_text_of_one_tet(tmp_path):
    g = IO.Grid(np.array([[0.0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]]),
                np.array([[1, 2, 3, 4]], np.int32), np.zeros((0, 8), np.int32),
                np.zeros((0, 6), np.int32), np.zeros((0, 5), np.int32),
                [IO.GridPatch(np.array([[1, 3, 2], [1, 2, 4], [2, 3, 4], [1, 4, 3]], np.int32),
                              np.zeros((0, 4), np.int32))])
    p = tmp_path / "one.grda"
    IO.write_grid_ascii(str(p), g)
    t = p.read_text().splitlines()
    assert t[:6] == ["# ROCFLU grid file", "# Precision and range", "      15     307",
                     "# Physical time", " 0.0000000000000000E+00", "# Dimensions"]
    assert t[6] == "%16d%16d%16d%16d%16d" % (4, 1, 0, 0, 0)
    assert t[7] == "# Coordinates"
    assert t[8] == (" 0.0000000000000000E+00" + " 0.1000000000000000E+01" +
                    " 0.0000000000000000E+00" * 2)
    assert "# Tetrahedra" in t and "# Boundaries (v2)" in t and t[-1] == "# End"
    i = t.index("# Tetrahedra")
    assert t[i + 1:i + 5] == ["%16d" % v for v in (1, 2, 3, 4)]
    b = t.index("# Boundaries (v2)")
    assert t[b + 1] == "%16d" % 1 and t[b + 2] == "%16d%16d%16d" % (4, 0, 0)
    assert t[b + 3] == "".join("%16d" % v for v in (1, 1, 2, 1))


@pytest.mark.parametrize("kind", [M.HEX, M.TET, M.MIXED])
def test_grid_roundtrip_and_mesh_rebuild(tmp_path, kind):
    m = M.box(kind, 5, 4, 6, jitter=0.1 if kind == M.TET else 0.0, seed=3)
    g = IO.grid_of_mesh(m)
    pa, pb = tmp_path / "g.grda", tmp_path / "g.grd"
    IO.write_grid_ascii(str(pa), g)
    IO.write_grid_binary(str(pb), g, endian=">")
    ga, gb = IO.read_grid_ascii(str(pa)), IO.read_grid_binary(str(pb), endian=">")
    for h in (ga, gb):
        for k in IO._CELL_KEYS:
            assert np.array_equal(h.conn(k), g.conn(k))
        assert len(h.patches) == len(g.patches)
        for p, q in zip(h.patches, g.patches):
            assert np.array_equal(p.tri2v, q.tri2v) and np.array_equal(p.quad2v, q.quad2v)
    assert np.array_equal(gb.xyz, g.xyz)                       # binary: exact
    assert np.allclose(ga.xyz, g.xyz, rtol=1e-15, atol=1e-300)  # ASCII: 16 digits
    mb = IO.mesh_of_grid(gb)
    for f in ("cofg", "vol", "f2c", "fn", "c2cs_off", "c2cs_mem", "xyzmoms"):
        assert np.array_equal(getattr(mb, f), getattr(m, f)), f
    for p, q in zip(mb.patches, m.patches):
        assert sorted(p.bf2c.tolist()) == sorted(q.bf2c.tolist())
    # text written from the ASCII read equals the text written first
    pa2 = tmp_path / "g2.grda"
    IO.write_grid_ascii(str(pa2), ga)
    assert pa2.read_text() == pa.read_text()


def test_flow_roundtrip(tmp_path):
    rng = np.random.default_rng(5)
    cv = rng.standard_normal((37, 5)) * 10.0 ** rng.integers(-5, 6, (37, 5))
    fl = IO.Flow(cv, time=1.25e-3, res_init=0.5)
    pa, pb = tmp_path / "f.flo_ascii", tmp_path / "f.flo"
    IO.write_flow_ascii(str(pa), fl)
    IO.write_flow_binary(str(pb), fl)
    a, b = IO.read_flow_ascii(str(pa)), IO.read_flow_binary(str(pb))
    assert np.array_equal(b.cv, cv) and b.time == fl.time and b.res_init == fl.res_init
    assert np.allclose(a.cv, cv, rtol=1e-15, atol=0) and a.time == fl.time
    assert pa.read_text().splitlines()[-1] == "# End"
    assert "#  3" in pa.read_text().splitlines()


def test_grid_with_unmatched_boundary_face_is_refused():
    m = M.box(M.HEX, 2, 2, 2)
    g = IO.grid_of_mesh(m)
    g.patches[0] = IO.GridPatch(g.patches[0].tri2v, g.patches[0].quad2v[1:])
    with pytest.raises(RuntimeError):
        IO.mesh_of_grid(g)
