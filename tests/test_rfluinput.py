"""RocfluMP case input files (.inp sections, .bc sections): the reference's
reading rules, the mapping onto the engine's options and the report of
settings outside its envelope.  CPU only."""
import math
import os

import numpy as np
import pytest

from rocflupicl_gb300 import case as K
from rocflupicl_gb300 import rfluinput as RI

INP = """# FORMATS
GRID      0
#

# FLOWMODEL
MODEL    0
MOVEGRID 0
#

# NUMERICS
CFL      -0.8   ! the reference keeps |CFL|
DISCR    3
ORDER    2
ENTROPY  0.1
RECONST  11
CRECONSTC  0
CRECONSTCW 1    ! CRECONSTC is defined above, so this line is CRECONSTCW's
ORDERBF  2
SIGMA    0.9
#

# TIMESTEP
FLOWTYPE   1
ORDER      2    ! the time-stepping ORDER, not the space ORDER
TIMESTEP   2.5E-06
DTMINLIMIT 1.0D-11
MAXTIME    3.0E-03
RKSCHEME   2
#

# REFERENCE
GAMMA 1.3
CP    1100.0
!DENS 9.0
#

# MIXTURE
GASMODEL 1
#
"""

BC = """# BC_OUTFLOW
PATCH  2 2
TYPE   1
PRESS  9.5E4
#

# BC_FARF
PATCH  3 4
MACH   0.6
ATTACK 30.0
SLIP   0.0
PRESS  1.0E5
TEMP   300.0
ORDER  1
#

# BC_INFLOW_TOTANG
PATCH  1 1
TYPE   2
FIXED  1
PTOT   2.0E5
TTOT   350.0
BETAH  10.0
BETAV  -5.0
MACH   1.2
#

# BC_SLIPW
PATCH 5 6
#
"""


@pytest.fixture
def files(tmp_path):
    p = tmp_path / "case.inp"
    p.write_text(INP)
    b = tmp_path / "case.bc"
    b.write_text(BC)
    return str(p), str(b)


def test_inp_keys_sections_and_defaults(files):
    ci = RI.read_inp(files[0])
    n = ci.numerics
    assert n.cfl == 0.8 and n.spaceDiscr == K.DISCR_UPW_HLLC and n.spaceOrder == 2
    assert n.reconst == K.RECONST_LIM_VENKAT and n.epsentr == 0.1 and n.ausmSigma == 0.9
    assert n.ausmKp == 0.25 and n.dissFact == 1.0          # defaults
    assert n.rkScheme == K.RK_SCHEME_3_WRAY and n.refGamma == 1.3 and n.refCp == 1100.0
    assert ci.dt_imposed == 2.5e-6 and ci.dt_min_limit == 1.0e-11 and ci.max_time == 3.0e-3
    assert ci.order_bfaces == 2
    assert ci.raw["NUMERICS"]["CRECONSTC"] == 0 and ci.raw["NUMERICS"]["CRECONSTCW"] == 1
    assert "DENS" not in ci.raw["REFERENCE"]                 # a commented line
    assert ci.unsupported == []


def test_inp_envelope_reported(tmp_path):
    p = tmp_path / "bad.inp"
    p.write_text(INP.replace("RECONST  11", "RECONST  1").replace("CRECONSTC  0", "CRECONSTC  1")
                 .replace("FLOWTYPE   1", "FLOWTYPE   0").replace("MODEL    0", "MODEL    1"))
    bad = RI.read_inp(str(p)).unsupported
    assert any(b.startswith("RECONST 1") for b in bad)
    assert any(b.startswith("CRECONSTC 1") for b in bad)
    assert any(b.startswith("FLOWTYPE 0") for b in bad)
    assert any("Euler only" in b for b in bad)


def test_bc_sections(files):
    bcs, bad = RI.read_bc(files[1], 6, order_bfaces=2)
    assert bad == []
    assert [b.bcType for b in bcs] == [K.BC_INFLOW_TOTANG, K.BC_OUTFLOW, K.BC_FARFIELD,
                                       K.BC_FARFIELD, K.BC_SLIPWALL, K.BC_SLIPWALL]
    d2r = 1.0 / (180.0 / (4.0 * math.atan(1.0)))
    t = bcs[0]
    assert t.bcOptType == K.BCOPT_MIXED and t.bcOptFixed == 1 and t.spaceOrder == 2
    assert np.array_equal(t.vals, np.array([2.0e5, 350.0, 10.0 * d2r, -5.0 * d2r, 1.2]))
    assert bcs[1].bcOptType == K.BCOPT_SUBSONIC and bcs[1].pout[0] == 9.5e4
    assert bcs[2].spaceOrder == 1
    assert np.array_equal(bcs[2].vals, np.array([0.6, 30.0 * d2r, 0.0, 1.0e5, 300.0]))


def test_bc_unassigned_and_unsupported(tmp_path):
    b = tmp_path / "x.bc"
    b.write_text("# BC_NOSLIP\nPATCH 1 1\n#\n# BC_INJECT\nPATCH 2 2\nDISTRIB 1\nMFRATE 1.0\nTEMP 300\n#\n")
    bcs, bad = RI.read_bc(str(b), 3)
    assert any(s.startswith("BC_NOSLIP") for s in bad)
    assert any("DISTRIB 1" in s for s in bad)
    assert any(s.startswith("patch 1") for s in bad) and any(s.startswith("patch 3") for s in bad)
    assert bcs[1].bcType == K.BC_INJECTION


# The reference tree's root comes from RFLU_REFERENCE_ROOT; the test is skipped
# where it is not set or the deck is not there.
REF_INP = os.path.join(os.environ.get("RFLU_REFERENCE_ROOT", ""), "input_files", "AirShock",
                       "rectshktb.inp")


@pytest.mark.skipif(not os.environ.get("RFLU_REFERENCE_ROOT") or not os.path.exists(REF_INP),
                    reason="reference tree not present (set RFLU_REFERENCE_ROOT)")
def test_reference_airshock_input_read():
    """The reference's own AirShock deck: AUSM+up second order with RK3 and
    WENO-XYZ reconstruction (all in the envelope), with constrained
    reconstruction and particle coupling, which the engine reports as outside
    it."""
    ci = RI.read_inp(REF_INP)
    n = ci.numerics
    assert (n.spaceDiscr, n.spaceOrder, n.rkScheme, n.cfl) == (5, 2, 2, 0.5)
    assert (n.ausmSigma, n.ausmKp, n.ausmKu, n.ausmMInf) == (1.0, 0.25, 0.75, 0.1)
    assert ci.dt_min_limit == 2.0e-10 and n.refCp == 1004.64
    assert ci.numerics.reconst == K.RECONST_WENO_XYZ
    assert not any(b.startswith("RECONST") for b in ci.unsupported)
    assert any(b.startswith("CRECONSTC 1") for b in ci.unsupported)
    assert any(b.startswith("PICL USED") for b in ci.unsupported)
    # its INITFLOW section: the rectshktb planar shock (hard-coded, FLAG 3)
    v = ci.raw["INITFLOW"]
    assert v["FLAG"] == K.INITFLOW_FROMHARDCODE and v["RVAL1"] == -0.005
    assert (v["RVAL2"], v["RVAL3"], v["RVAL4"]) == (2.0725901075834, 304.1461483936438,
                                                    252082.2060022760706)
    assert (v["RVAL5"], v["RVAL6"]) == (0.9721771595969, 82700.0)
    xyz = np.array([[-0.01, 0.0, 0.0], [0.0, 0.0, 0.0]])
    r, u, _, _, p = K.hardcoded_prims("rectshktb", xyz, v)
    assert list(r) == [v["RVAL2"], v["RVAL5"]] and list(p) == [v["RVAL4"], v["RVAL6"]]


def test_case_files_round_trip_residual(tmp_path):
    """A case written as binary grid and flow files plus .inp and .bc files and
    read back with from_case_files gives the oracle the same residual, bit for
    bit (the ASCII forms hold 16 significant digits, E23.16, so they round a
    double's last bit)."""
    from oracle.oracle import Oracle
    from rocflupicl_gb300 import rfluio as IO
    num = K.Numerics(spaceDiscr=K.DISCR_UPW_ROE, spaceOrder=2, reconst=K.RECONST_LIM_VENKAT,
                     rkScheme=K.RK_SCHEME_3_WRAY, cfl=0.5, epsentr=0.05)
    c = K.tet_shock_box(4, seed=3, numerics=num)
    g = IO.grid_of_mesh(c.mesh)
    IO.write_grid_binary(str(tmp_path / "c.grda"), g)
    K.write_flow(str(tmp_path / "c.flo"), c.cv, binary=True)
    (tmp_path / "c.inp").write_text(
        "# FLOWMODEL\nMODEL 0\nMOVEGRID 0\n#\n# NUMERICS\nCFL 0.5\nDISCR 1\nORDER 2\n"
        "RECONST 11\nENTROPY 0.05\n#\n# TIMESTEP\nFLOWTYPE 1\nRKSCHEME 2\nMAXTIME 1.0E-3\n#\n"
        "# REFERENCE\nGAMMA 1.4\nCP 1004.5\n#\n# MIXTURE\nGASMODEL 1\n#\n")
    (tmp_path / "c.bc").write_text(
        "# BC_OUTFLOW\nPATCH 1 2\nTYPE 0\nORDER 2\n#\n# BC_SLIPW\nPATCH 3 6\nORDER 2\n#\n")
    c2, ci, bad = K.from_case_files(str(tmp_path / "c.grda"), str(tmp_path / "c.flo"),
                                    str(tmp_path / "c.inp"), str(tmp_path / "c.bc"), binary=True)
    assert bad == [] and c2.t_end == 1.0e-3
    r1, _ = Oracle(c).residual(c.cv, c.dv)
    r2, _ = Oracle(c2).residual(c2.cv, c2.dv)
    assert np.array_equal(r1, r2)


def test_case_files_strict_refuses(tmp_path):
    from rocflupicl_gb300 import rfluio as IO
    c = K.tet_shock_box(3, seed=3)
    IO.write_grid_ascii(str(tmp_path / "c.grda"), IO.grid_of_mesh(c.mesh))
    K.write_flow(str(tmp_path / "c.flo"), c.cv)
    (tmp_path / "c.inp").write_text("# NUMERICS\nDISCR 1\nORDER 2\nRECONST 1\n#\n"
                                    "# TIMESTEP\nFLOWTYPE 1\n#\n")
    (tmp_path / "c.bc").write_text("# BC_SLIPW\nPATCH 1 6\n#\n")
    with pytest.raises(ValueError, match="RECONST 1"):
        K.from_case_files(str(tmp_path / "c.grda"), str(tmp_path / "c.flo"),
                          str(tmp_path / "c.inp"), str(tmp_path / "c.bc"))


def test_a_line_defines_one_key(tmp_path):
    """ReadSection stops at the first undefined key a line matches: with RVAL1
    undefined, `RVAL10 5.0` defines RVAL1 (reading 0 from `0 5.0`), not RVAL10."""
    p = tmp_path / "keys.inp"
    p.write_text("# INITFLOW\nFLAG 3\nRVAL10 5.0\nRVAL1 7.0\nRVAL2 8.0\nRVAL20 9.0\n#\n")
    v = RI.read_inp(str(p)).raw["INITFLOW"]
    assert v["FLAG"] == 3 and v["RVAL1"] == 0.0 and "RVAL10" not in v
    assert v["RVAL2"] == 8.0 and v["RVAL20"] == 9.0


def test_initflow_states(tmp_path):
    """INITFLOW FLAG 1 (RFLU_InitFlowScratch) and FLAG 3 hard-coded states of
    RFLU_InitFlowHardCode at chosen centroids."""
    num = K.Numerics()
    xyz = np.array([[-0.1, 0.2, 0.0], [0.3, -0.4, 0.1], [0.7, 0.0, 0.0]])
    cv = K.initial_cv("any", xyz, num, {"FLAG": 1, "VELX": 10.0, "VELY": 0.0, "VELZ": -2.0,
                                         "PRESS": 9.0e4, "DENS": 1.1})
    assert np.array_equal(cv, K.prim_to_cv(num, *(np.full(3, a) for a in (1.1, 10.0, 0.0, -2.0,
                                                                          9.0e4))))
    shk = {"FLAG": 3, "RVAL1": 0.0, "RVAL2": 2.07, "RVAL3": 304.1, "RVAL4": 2.52e5,
           "RVAL5": 0.972, "RVAL6": 8.27e4}
    r, u, v, w, p = K.hardcoded_prims("rectshktb", xyz, shk)
    assert list(r) == [2.07, 0.972, 0.972] and list(u) == [304.1, 0.0, 0.0]
    assert list(p) == [2.52e5, 8.27e4, 8.27e4] and not v.any() and not w.any()
    r, u, v, w, p = K.hardcoded_prims("cylds", xyz, shk)     # radius 0.224, 0.5, 0.7
    assert list(r) == [0.972] * 3
    r, u, v, w, p = K.hardcoded_prims("cylds", xyz, dict(shk, RVAL1=0.6))
    assert list(r) == [2.07, 2.07, 0.972]
    assert np.isclose(u[1], 304.1 * 0.3 / 0.5) and np.isclose(v[1], -304.1 * 0.4 / 0.5)
    r, _, _, _, p = K.hardcoded_prims("st_sod2", xyz, {})
    assert list(r) == [1.0, 0.01, 0.01] and list(p) == [1e5, 1e3, 1e3]
    r, _, _, _, p = K.hardcoded_prims("st_sod1", xyz, {})
    assert list(r) == [1.0, 1.0, 0.125]
    stg = {"RVAL1": 0.0, "RVAL2": 1.0, "RVAL3": 1.0, "RVAL4": 1.0, "RVAL5": 2.0, "RVAL6": 2.0,
           "RVAL7": 2.0, "RVAL11": 0.5, "RVAL12": 3.0, "RVAL13": 3.0, "RVAL14": 3.0}
    r, u, _, _, p = K.hardcoded_prims("stg1d", xyz, stg)
    assert list(r) == [1.0, 2.0, 3.0] and list(u) == [1.0, 2.0, 3.0]
    r, u, v, w, p = K.hardcoded_prims("gtlin", xyz, {})
    x, y, z = xyz.T
    assert np.allclose(u, 3 * x + 4 * y + 5 * z) and np.allclose(w, 7 * x + 8 * y + 9 * z)
    dmin = x.min() + 2 * y.min() + 3 * z.min()
    assert np.allclose(r, x + 2 * y + 3 * z - 2 * dmin)
    r, u, _, _, p = K.hardcoded_prims("gttri", xyz, {"RVAL1": 1.0, "RVAL2": 1.0, "RVAL3": 1.0})
    assert np.allclose(u, np.cos(np.pi * x) * np.sin(np.pi * y) * np.cos(np.pi * z))
    assert np.allclose(r, u + 2.0) and np.allclose(p, u + 2.0)
    with pytest.raises(ValueError):
        K.hardcoded_prims("rectshktb", xyz, {"FLAG": 3})      # RVALs missing
    with pytest.raises(ValueError):
        K.initial_cv("wedge", xyz, num, {"FLAG": 3})          # not restated
    with pytest.raises(ValueError):
        K.initial_cv("any", xyz, num, {"FLAG": 2})            # from a flow file


def test_case_files_without_flow_file(tmp_path):
    """No flow file: rfluinit's state from the deck's INITFLOW section, named
    after the .inp file (st_sod1.inp -> the st_sod1 tube), or a uniform state
    (FLAG 1), on the grid file's centroids."""
    from rocflupicl_gb300 import rfluio as IO
    c = K.shock_tube(20, 2, 2, length=(1.0, 0.1, 0.1))
    IO.write_grid_ascii(str(tmp_path / "g.grda"), IO.grid_of_mesh(c.mesh))
    deck = ("# NUMERICS\nCFL 0.5\nDISCR 1\nORDER 2\nRECONST 11\n#\n# TIMESTEP\nFLOWTYPE 1\n"
            "RKSCHEME 2\nMAXTIME 2.0E-4\n#\n# INITFLOW\n{}#\n")
    (tmp_path / "st_sod1.inp").write_text(deck.format("FLAG 3\n"))
    (tmp_path / "uniform.inp").write_text(
        deck.format("FLAG 1\nVELX 5.0\nVELY 0.0\nVELZ 0.0\nPRESS 1.0E5\nDENS 1.2\n"))
    (tmp_path / "c.bc").write_text("# BC_OUTFLOW\nPATCH 1 2\nTYPE 0\n#\n# BC_SLIPW\nPATCH 3 6\n#\n")
    args = (str(tmp_path / "g.grda"), None)
    c1, _, bad = K.from_case_files(*args, str(tmp_path / "st_sod1.inp"), str(tmp_path / "c.bc"))
    x = c1.mesh.cofg[:c1.mesh.nCells, 0]
    assert bad == [] and c1.meta["casename"] == "st_sod1"
    assert np.array_equal(c1.cv[:, 0], np.where(x < 0.5, 1.0, 0.125))
    assert np.allclose(c1.dv[:, 0], np.where(x < 0.5, 1.0e5, 1.0e4), rtol=1e-14)
    c2, _, _ = K.from_case_files(*args, str(tmp_path / "uniform.inp"), str(tmp_path / "c.bc"))
    assert np.array_equal(c2.cv[:, 0], np.full(len(x), 1.2))
    assert np.allclose(c2.cv[:, 1], 6.0) and np.allclose(c2.dv[:, 0], 1.0e5, rtol=1e-14)
    with pytest.raises(ValueError, match="not restated"):
        K.from_case_files(*args, str(tmp_path / "st_sod1.inp"), str(tmp_path / "c.bc"),
                          casename="wedge")


def test_bc_key_given_twice_takes_the_later_value(tmp_path):
    """ReadPatchSection keeps no record of defined keys: the later line wins
    (the .inp sections' ReadSection keeps the first)."""
    b = tmp_path / "twice.bc"
    b.write_text("# BC_OUTFLOW\nPATCH 1 1\nTYPE 1\nPRESS 9.0E4\nPRESS 8.0E4\n#\n")
    bcs, _ = RI.read_bc(str(b), 1)
    assert bcs[0].pout[0] == 8.0e4
    p = tmp_path / "twice.inp"
    p.write_text("# NUMERICS\nCFL 0.5\nCFL 0.9\n#\n")
    assert RI.read_inp(str(p)).numerics.cfl == 0.5
