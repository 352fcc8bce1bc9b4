"""The C ABI seen from a compiled caller.

The Fortran binding module written out in the repository's integration notes
declares BIND(C) derived types for the structs of include/rfgpu.h; a BIND(C) type is laid out like the
C struct with the same fields in the same order.  The layout those Fortran
types imply (C_INT 4 bytes, C_DOUBLE and C_PTR 8, each field at its natural
alignment) is computed here from the text of those notes and checked three
ways: at compile time against the header (offsetof / sizeof static_asserts in
a C++ translation unit that includes include/rfgpu.h, built with g++), and at
run time against the Python front end's ctypes mirrors.  On a GPU the same
C++ program, linked against librfgpu.so, registers a region and runs the
time-step loop through rfgpu_dt / rfgpu_stage / rfgpu_status /
rfgpu_download, and its state equals the oracle's bit for bit.
"""
import ctypes as C
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from rocflupicl_gb300 import _build
from rocflupicl_gb300 import case as K
from rocflupicl_gb300 import engine as E

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c_abi", "rfgpu_abi_smoke.cpp")
KINDS = {"INTEGER(C_INT)": 4, "REAL(C_DOUBLE)": 8, "TYPE(C_PTR)": 8}


def bindc_types():
    """{type name: [(field, size)]} from the BIND(C) types of the integration notes."""
    txt = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    out = {}
    for name, body in re.findall(r"TYPE, BIND\(C\) :: (\w+)\n(.*?)\n\s*END TYPE \1", txt, re.S):
        fields = []
        for line in body.splitlines():
            m = re.match(r"\s*(INTEGER\(C_INT\)|REAL\(C_DOUBLE\)|TYPE\(C_PTR\))\s*::\s*(.+)", line)
            assert m, line
            for f in m.group(2).split(","):
                fields.append((f.strip(), KINDS[m.group(1)]))
        out[name] = fields
    return out


def layout(fields):
    """C layout of a field list: (offsets {field: offset}, size)."""
    off, pos, align = {}, 0, 1
    for f, sz in fields:
        pos = (pos + sz - 1) // sz * sz
        off[f] = pos
        pos += sz
        align = max(align, sz)
    return off, (pos + align - 1) // align * align


def layout_header(path):
    lines = ["#include <cstddef>"]
    for name, fields in bindc_types().items():
        off, size = layout(fields)
        for f, o in off.items():
            lines.append(f'static_assert(offsetof({name}, {f}) == {o}, "{name}.{f} at {o}");')
        lines.append(f'static_assert(sizeof({name}) == {size}, "sizeof({name}) == {size}");')
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def test_bindc_types_cover_the_header_structs():
    t = bindc_types()
    assert set(t) == {"rfgpu_patch_t", "rfgpu_border_t", "rfgpu_region_desc_t", "rfgpu_tuning_t"}
    hdr = open(os.path.join(ROOT, "include", "rfgpu.h")).read()
    for name, fields in t.items():
        body = re.search(r"typedef struct \{([^{}]*)\} " + name + ";", hdr).group(1)
        body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
        declared = re.findall(r"\**\s*(\w+)\s*(?:,|;)", body)
        assert [f for f, _ in fields] == declared, name


@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_header_layout_at_compile_time(tmp_path):
    hdr = tmp_path / "layout_expect.h"
    layout_header(hdr)
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", f"-I{ROOT}/include",
                        f'-DRFGPU_LAYOUT_H="{hdr}"', SRC], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_ctypes_mirrors_match_the_bindc_layout():
    mirrors = {"rfgpu_patch_t": E.PatchT, "rfgpu_border_t": E.BorderT,
               "rfgpu_region_desc_t": E.RegionDescT, "rfgpu_tuning_t": E.TuningT}
    for name, fields in bindc_types().items():
        off, size = layout(fields)
        S = mirrors[name]
        assert C.sizeof(S) == size, name
        assert [f for f, _ in S._fields_] == [f for f, _ in fields], name
        for f, o in off.items():
            assert getattr(S, f).offset == o, (name, f)


def _write_case(c, d, n_steps):
    m, num = c.mesh, c.numerics
    pats = [(p, bc) for p, bc in zip(m.patches, c.bcs) if p.n > 0]
    vals = [m.nCells, m.nFaces, m.nMembs, len(pats), num.spaceDiscr, num.spaceOrder, num.reconst,
            num.rkScheme, num.precision, num.venkatGuard, repr(num.refCp), repr(num.refGamma),
            repr(num.gv[0]), repr(num.gv[1]), repr(num.epsentr), repr(num.dissFact), repr(num.cfl),
            n_steps]
    for p, bc in pats:
        vals += [bc.bcType, bc.spaceOrder, bc.bcOptType, p.n]
    (d / "meta.txt").write_text(" ".join(str(v) for v in vals) + "\n")

    def put(name, a, dt):
        np.ascontiguousarray(a, dt).tofile(d / name)
    put("f2c.i32", m.f2c, np.int32)
    put("fn.f64", m.fn, np.float64)
    put("fc.f64", m.fc, np.float64)
    put("cofg.f64", m.cofg, np.float64)
    put("vol.f64", m.vol, np.float64)
    put("c2csoff.i32", m.c2cs_off, np.int32)
    put("c2csmem.i32", m.c2cs_mem, np.int32)
    put("xyzmoms.f64", m.xyzmoms, np.float64)
    put("cv.f64", c.cv, np.float64)
    put("dv.f64", c.dv, np.float64)
    for k, (p, bc) in enumerate(pats):
        put(f"p{k}_bf2c.i32", p.bf2c, np.int32)
        put(f"p{k}_fn.f64", p.fn, np.float64)
        put(f"p{k}_fc.f64", p.fc, np.float64)


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", [K.DISCR_UPW_ROE, K.DISCR_UPW_HLLC], ids=["roe", "hllc"])
def test_cpp_caller_runs_the_time_step_loop(tmp_path, scheme):
    from oracle.oracle import Oracle
    lib = _build.build_gpu()
    hdr = tmp_path / "layout_expect.h"
    layout_header(hdr)
    exe = tmp_path / "rfgpu_abi_smoke"
    r = subprocess.run(["g++", "-std=c++17", "-O2", f"-I{ROOT}/include", f'-DRFGPU_LAYOUT_H="{hdr}"',
                        SRC, "-o", str(exe), f"-L{lib.parent}", "-lrfgpu",
                        f"-Wl,-rpath,{lib.parent}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    c = K.tet_shock_box(5, seed=9, numerics=K.Numerics(spaceDiscr=scheme, venkatGuard=1))
    n_steps = 3
    _write_case(c, tmp_path, n_steps)
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    flags, t = (tmp_path / "out.txt").read_text().split()
    cvg = np.fromfile(tmp_path / "out_cv.f64").reshape(-1, 5)
    dvg = np.fromfile(tmp_path / "out_dv.f64").reshape(-1, 3)
    o = Oracle(c)
    cv, dv = c.cv.copy(), c.dv.copy()
    dti = o.dt(cv, dv, c.numerics.cfl, 1.0, 0.0, 1.0)
    t_o, _, st_o = o.run(cv, dv, n_steps=n_steps, dt_imposed=dti)
    assert int(flags) == st_o == 0
    assert float(t) == t_o
    assert np.array_equal(cvg, cv) and np.array_equal(dvg, dv)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [K.PREC_MIXED, K.PREC_SPLIT], ids=["mixed", "split"])
def test_cpp_caller_reduced_precision(tmp_path, prec):
    """The compiled caller on the reduced-precision paths: the same calls
    (rfgpu_dt, rfgpu_stage per stage, rfgpu_download) made through the Python
    front end give the same state bit for bit, and it stays within 1e-5 of the
    FP64 oracle in the reference's L1 sense."""
    from oracle.oracle import Oracle
    lib = _build.build_gpu()
    hdr = tmp_path / "layout_expect.h"
    layout_header(hdr)
    exe = tmp_path / "rfgpu_abi_smoke"
    r = subprocess.run(["g++", "-std=c++17", "-O2", f"-I{ROOT}/include", f'-DRFGPU_LAYOUT_H="{hdr}"',
                        SRC, "-o", str(exe), f"-L{lib.parent}", "-lrfgpu",
                        f"-Wl,-rpath,{lib.parent}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    c = K.tet_shock_box(6, seed=9, numerics=K.Numerics(spaceDiscr=K.DISCR_UPW_HLLC, venkatGuard=1,
                                                       precision=prec))
    n_steps = 3
    _write_case(c, tmp_path, n_steps)
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    flags, t = (tmp_path / "out.txt").read_text().split()
    cvg = np.fromfile(tmp_path / "out_cv.f64").reshape(-1, 5)
    dvg = np.fromfile(tmp_path / "out_dv.f64").reshape(-1, 3)
    # the caller registers in the locality order; so does this region
    reg = E.Region(c, cell_order=E.ORDER_LOCALITY)
    cfl = c.numerics.cfl
    dti = reg.time_step(cfl, 1.0, 0.0, 1.0)
    tp = 0.0
    for _ in range(n_steps):
        dtm = reg.time_step(cfl, dti, 0.0, tp)
        for s in (1, 2, 3):
            reg.rk_stage(s, dtm)
        tp += dtm
    cvp, dvp = reg.download()
    assert int(flags) == reg.status() == 0
    assert float(t) == tp
    reg.close()
    assert np.array_equal(cvg, cvp) and np.array_equal(dvg, dvp)
    o = Oracle(c.with_numerics(precision=K.PREC_FP64))
    cv, dv = c.cv.copy(), c.dv.copy()
    dto = o.dt(cv, dv, cfl, 1.0, 0.0, 1.0)
    o.run(cv, dv, n_steps=n_steps, dt_imposed=dto)
    assert np.mean(np.abs(cvg[:, 0] / cv[:, 0] - 1.0)) <= 1e-5
    assert np.mean(np.abs(dvg[:, 0] / dv[:, 0] - 1.0)) <= 1e-5
