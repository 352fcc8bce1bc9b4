"""The reference's grid and flow files, so real RocfluMP cases can be fed to
the engine and its results written back where the Fortran tools read them.

Grid files (modflu/RFLU_ModReadWriteGrid.F90): ASCII `.grda`
(RFLU_ReadGridASCII :124-594, RFLU_WriteGridASCII :1207-1452) and binary
`.grd` (RFLU_ReadGridBinary :620-1099, RFLU_WriteGridBinary :1475-1731).
Flow files (modflu/RFLU_ModReadWriteFlow.F90): the v2 layout, ASCII
(RFLU_ReadFlowV2ASCII :750-888, RFLU_WriteFlowASCII :2187-2367) and binary
(RFLU_ReadFlowV2Binary :912-1051, RFLU_WriteFlowBinary :2392-2559).

ASCII records use the reference's Fortran edit descriptors: section strings
'(A)', precision and range '(2(I8))', reals '(5(E23.16))' / '(E23.16)',
integers '(10(I16))' / '(5(I16))'.  Binary files are Fortran sequential
unformatted records (4-byte length markers before and after each record),
little- or big-endian as the reference's FORMAT_BINARY_L / _B options write
them; section strings are 80-character records (CHRLEN).

Layouts follow the reference's arrays: xyz(3,nVert) is written one
coordinate at a time, tet2v(4,nTets) one local vertex at a time, and so on;
here they are held as NumPy arrays (nVert,3), (nTets,4), ... with 1-based
vertex ids.
"""
from __future__ import annotations

import re
import struct
from dataclasses import dataclass, field
from typing import List, Optional, Tuple

import numpy as np

CHRLEN = 80
_PREC_RANGE = (15, 307)  # PRECISION(1.0_RFREAL), RANGE(1.0_RFREAL) for double
_NV = {"Tetrahedra": 4, "Hexahedra": 8, "Prisms": 6, "Pyramids": 5}
_CELL_KEYS = ("Tetrahedra", "Hexahedra", "Prisms", "Pyramids")


@dataclass
class GridPatch:
    tri2v: np.ndarray                      # (nBTris, 3), 1-based
    quad2v: np.ndarray                     # (nBQuads, 4), 1-based
    bvc: Optional[np.ndarray] = None       # (nBCellsVirt,) virtual cells (v2 boundaries)


@dataclass
class Grid:
    xyz: np.ndarray                        # (nVert, 3)
    tet2v: np.ndarray                      # (nTets, 4), 1-based
    hex2v: np.ndarray                      # (nHexs, 8)
    pri2v: np.ndarray                      # (nPris, 6)
    pyr2v: np.ndarray                      # (nPyrs, 5)
    patches: List[GridPatch] = field(default_factory=list)
    time: float = 0.0

    def conn(self, key: str) -> np.ndarray:
        return {"Tetrahedra": self.tet2v, "Hexahedra": self.hex2v, "Prisms": self.pri2v,
                "Pyramids": self.pyr2v}[key]


@dataclass
class Flow:
    cv: np.ndarray                         # (nCells, nCv): cv(iLoc, icg) transposed
    time: float = 0.0
    res_init: float = 0.0


# ---- Fortran edit descriptors ----------------------------------------------

def _e23_16(x: float) -> str:
    """Fortran E23.16: 0.d1..d16 with a two-digit exponent after E, or a
    three-digit one without the E when it is beyond +-99."""
    x = float(x)
    if not np.isfinite(x):
        raise ValueError("non-finite value in a Fortran E field")
    neg = x < 0.0 or (x == 0.0 and np.copysign(1.0, x) < 0.0)
    if x == 0.0:
        digits, e = "0" * 16, 0
    else:
        s = "%.15e" % abs(x)
        digits = s[0] + s[2:17]
        e = int(s[18:]) + 1
    exp = ("E%+03d" % e) if abs(e) <= 99 else ("%+04d" % e)
    return ("-" if neg else " ") + "0." + digits + exp


_EXP_NO_E = re.compile(r"^([+-]?[0-9.]+)([+-][0-9]+)$")


def _read_e(field_: str) -> float:
    t = field_.strip().upper().replace("D", "E")
    if "E" not in t:
        m = _EXP_NO_E.match(t)
        if m:
            t = m.group(1) + "E" + m.group(2)
    return float(t)


def _write_reals(lines: list, a, per_line: int = 5):
    a = np.asarray(a, np.float64).ravel()
    for i in range(0, a.shape[0], per_line):
        lines.append("".join(_e23_16(v) for v in a[i:i + per_line]))


def _write_ints(lines: list, a, per_line: int = 10, width: int = 16):
    a = np.asarray(a, np.int64).ravel()
    for i in range(0, a.shape[0], per_line):
        lines.append("".join("%*d" % (width, v) for v in a[i:i + per_line]))


class _Lines:
    def __init__(self, text: str):
        self.lines = text.splitlines()
        self.i = 0

    def line(self) -> str:
        if self.i >= len(self.lines):
            raise ValueError("unexpected end of file")
        s = self.lines[self.i]
        self.i += 1
        return s

    def section(self) -> str:
        s = self.line().rstrip()
        if not s.startswith("# "):
            raise ValueError(f"invalid section marker: {s!r}")
        return s[2:]

    def fields(self, n: int, width: int, per_line: int):
        out = []
        while len(out) < n:
            s = self.line()
            k = min(per_line, n - len(out))
            for j in range(k):
                out.append(s[j * width:(j + 1) * width])
        return out

    def reals(self, n: int, per_line: int = 5) -> np.ndarray:
        return np.array([_read_e(f) for f in self.fields(n, 23, per_line)], np.float64)

    def ints(self, n: int, per_line: int = 10, width: int = 16) -> np.ndarray:
        return np.array([int(f) for f in self.fields(n, width, per_line)], np.int64)


# ---- grid files --------------------------------------------------------------

def write_grid_ascii(path: str, g: Grid) -> None:
    L: list = ["# ROCFLU grid file", "# Precision and range", "%8d%8d" % _PREC_RANGE,
               "# Physical time", _e23_16(g.time), "# Dimensions"]
    dims = [g.xyz.shape[0]] + [g.conn(k).shape[0] for k in _CELL_KEYS]
    _write_ints(L, dims, per_line=5)
    L.append("# Coordinates")
    for i in range(3):
        _write_reals(L, g.xyz[:, i])
    for k in _CELL_KEYS:
        c = g.conn(k)
        if c.shape[0] > 0:
            L.append("# " + k)
            for i in range(_NV[k]):
                _write_ints(L, c[:, i])
    L.append("# Boundaries (v2)")
    _write_ints(L, [len(g.patches)], per_line=1)
    for p in g.patches:
        nv = 0 if p.bvc is None else p.bvc.shape[0]
        _write_ints(L, [p.tri2v.shape[0], p.quad2v.shape[0], nv], per_line=3)
        for j in range(3):
            if p.tri2v.shape[0] > 0:
                _write_ints(L, p.tri2v[:, j])
        for j in range(4):
            if p.quad2v.shape[0] > 0:
                _write_ints(L, p.quad2v[:, j])
        if nv > 0:
            _write_ints(L, p.bvc)
    L.append("# End")
    with open(path, "w") as f:
        f.write("\n".join(L) + "\n")


def read_grid_ascii(path: str) -> Grid:
    with open(path) as f:
        r = _Lines(f.read())
    if r.section() != "ROCFLU grid file":
        raise ValueError("not a ROCFLU grid file")
    time, dims = 0.0, None
    xyz = None
    conn = {k: np.zeros((0, _NV[k]), np.int32) for k in _CELL_KEYS}
    patches: List[GridPatch] = []
    while True:
        sec = r.section()
        if sec == "Precision and range":
            r.ints(2, per_line=2, width=8)
        elif sec == "Physical time":
            time = float(r.reals(1, per_line=1)[0])
        elif sec == "Dimensions":
            dims = r.ints(5, per_line=5)
        elif sec == "Coordinates":
            xyz = np.stack([r.reals(int(dims[0])) for _ in range(3)], axis=1)
        elif sec in _NV:
            n = int(dims[1 + _CELL_KEYS.index(sec)])
            conn[sec] = np.stack([r.ints(n) for _ in range(_NV[sec])], axis=1).astype(np.int32)
        elif sec in ("Boundaries", "Boundaries (v2)"):
            v2 = sec.endswith("(v2)")
            npat = int(r.ints(1, per_line=1)[0])
            for _ in range(npat):
                hd = r.ints(3 if v2 else 2, per_line=3 if v2 else 2)
                nt, nq = int(hd[0]), int(hd[1])
                nvc = int(hd[2]) if v2 else 0
                tri = (np.stack([r.ints(nt) for _ in range(3)], axis=1) if nt > 0
                       else np.zeros((0, 3), np.int64))
                quad = (np.stack([r.ints(nq) for _ in range(4)], axis=1) if nq > 0
                        else np.zeros((0, 4), np.int64))
                bvc = r.ints(nvc) if nvc > 0 else None
                patches.append(GridPatch(tri.astype(np.int32), quad.astype(np.int32),
                                         None if bvc is None else bvc.astype(np.int32)))
        elif sec == "End":
            break
        else:
            raise ValueError(f"unknown grid section {sec!r}")
    if xyz is None or dims is None:
        raise ValueError("grid file without coordinates")
    return Grid(xyz, conn["Tetrahedra"], conn["Hexahedra"], conn["Prisms"], conn["Pyramids"],
                patches, time)


class _RecordWriter:
    def __init__(self, f, endian: str):
        self.f, self.e = f, endian

    def rec(self, payload: bytes):
        n = struct.pack(self.e + "i", len(payload))
        self.f.write(n + payload + n)

    def text(self, s: str):
        self.rec(s.ljust(CHRLEN).encode("ascii"))

    def ints(self, a, fmt: str = "i"):
        self.rec(np.asarray(a, self.e + fmt).tobytes())

    def reals(self, a):
        self.rec(np.asarray(a, self.e + "f8").tobytes())


class _RecordReader:
    def __init__(self, data: bytes, endian: str):
        self.d, self.p, self.e = data, 0, endian

    def rec(self) -> bytes:
        if self.p + 4 > len(self.d):
            raise ValueError("unexpected end of file")
        (n,) = struct.unpack_from(self.e + "i", self.d, self.p)
        if n < 0 or self.p + 8 + n > len(self.d):
            raise ValueError("corrupt record marker")
        b = self.d[self.p + 4:self.p + 4 + n]
        (n2,) = struct.unpack_from(self.e + "i", self.d, self.p + 4 + n)
        if n2 != n:
            raise ValueError("record markers disagree")
        self.p += 8 + n
        return b

    def text(self) -> str:
        return self.rec().decode("ascii").rstrip()

    def ints(self) -> np.ndarray:
        return np.frombuffer(self.rec(), self.e + "i4").astype(np.int64)

    def reals(self) -> np.ndarray:
        return np.frombuffer(self.rec(), self.e + "f8").astype(np.float64)


def write_grid_binary(path: str, g: Grid, endian: str = "<") -> None:
    with open(path, "wb") as f:
        w = _RecordWriter(f, endian)
        w.text("# ROCFLU grid file")
        w.text("# Precision and range")
        w.ints(_PREC_RANGE)
        w.text("# Physical time")
        w.reals([g.time])
        w.text("# Dimensions")
        w.ints([g.xyz.shape[0]] + [g.conn(k).shape[0] for k in _CELL_KEYS])
        w.text("# Coordinates")
        for i in range(3):
            w.reals(g.xyz[:, i])
        for k in _CELL_KEYS:
            c = g.conn(k)
            if c.shape[0] > 0:
                w.text("# " + k)
                for i in range(_NV[k]):
                    w.ints(c[:, i])
        w.text("# Boundaries (v2)")
        w.ints([len(g.patches)])
        for p in g.patches:
            nv = 0 if p.bvc is None else p.bvc.shape[0]
            w.ints([p.tri2v.shape[0], p.quad2v.shape[0], nv])
            if p.tri2v.shape[0] > 0:
                for j in range(3):
                    w.ints(p.tri2v[:, j])
            if p.quad2v.shape[0] > 0:
                for j in range(4):
                    w.ints(p.quad2v[:, j])
            if nv > 0:
                w.ints(p.bvc)
        w.text("# End")


def read_grid_binary(path: str, endian: str = "<") -> Grid:
    with open(path, "rb") as f:
        r = _RecordReader(f.read(), endian)
    if r.text() != "# ROCFLU grid file":
        raise ValueError("not a ROCFLU grid file")
    time, dims, xyz = 0.0, None, None
    conn = {k: np.zeros((0, _NV[k]), np.int32) for k in _CELL_KEYS}
    patches: List[GridPatch] = []
    while True:
        sec = r.text()
        if not sec.startswith("# "):
            raise ValueError(f"invalid section marker: {sec!r}")
        sec = sec[2:]
        if sec == "Precision and range":
            r.ints()
        elif sec == "Physical time":
            time = float(r.reals()[0])
        elif sec == "Dimensions":
            dims = r.ints()
        elif sec == "Coordinates":
            xyz = np.stack([r.reals() for _ in range(3)], axis=1)
        elif sec in _NV:
            conn[sec] = np.stack([r.ints() for _ in range(_NV[sec])], axis=1).astype(np.int32)
        elif sec in ("Boundaries", "Boundaries (v2)"):
            v2 = sec.endswith("(v2)")
            npat = int(r.ints()[0])
            for _ in range(npat):
                hd = r.ints()
                nt, nq = int(hd[0]), int(hd[1])
                nvc = int(hd[2]) if v2 else 0
                tri = np.stack([r.ints() for _ in range(3)], axis=1) if nt > 0 else np.zeros((0, 3))
                quad = np.stack([r.ints() for _ in range(4)], axis=1) if nq > 0 else np.zeros((0, 4))
                bvc = r.ints() if nvc > 0 else None
                patches.append(GridPatch(tri.astype(np.int32), quad.astype(np.int32),
                                         None if bvc is None else bvc.astype(np.int32)))
        elif sec == "End":
            break
        else:
            raise ValueError(f"unknown grid section {sec!r}")
    if xyz is None or dims is None:
        raise ValueError("grid file without coordinates")
    return Grid(xyz, conn["Tetrahedra"], conn["Hexahedra"], conn["Prisms"], conn["Pyramids"],
                patches, time)


# ---- flow files (v2) -----------------------------------------------------------

def write_flow_ascii(path: str, fl: Flow) -> None:
    n, ncv = fl.cv.shape
    L = ["# ROCFLU flow file (v2)", "# Precision and range", "%8d%8d" % _PREC_RANGE,
         "# Initial residual", _e23_16(fl.res_init), "# Physical time", _e23_16(fl.time),
         "# Dimensions"]
    _write_ints(L, [n, ncv], per_line=2)
    for iloc in range(ncv):
        L.append("# %2d" % (iloc + 1))
        _write_reals(L, fl.cv[:, iloc])
    L.append("# End")
    with open(path, "w") as f:
        f.write("\n".join(L) + "\n")


def read_flow_ascii(path: str) -> Flow:
    with open(path) as f:
        r = _Lines(f.read())
    if r.section() != "ROCFLU flow file (v2)":
        raise ValueError("not a ROCFLU v2 flow file")
    time = res = 0.0
    dims = None
    cv = None
    seen = set()
    while True:
        sec = r.section()
        if sec == "Precision and range":
            r.ints(2, per_line=2, width=8)
        elif sec == "Initial residual":
            res = float(r.reals(1, per_line=1)[0])
        elif sec == "Physical time":
            time = float(r.reals(1, per_line=1)[0])
        elif sec == "Dimensions":
            dims = r.ints(2, per_line=2)
            cv = np.zeros((int(dims[0]), int(dims[1])), np.float64)
        elif sec == "End":
            break
        else:
            iloc = int(sec[:2])
            if dims is None or iloc < 1 or iloc > dims[1]:
                raise ValueError(f"invalid cv location {sec!r}")
            cv[:, iloc - 1] = r.reals(int(dims[0]))
            seen.add(iloc)
    if cv is None or len(seen) != cv.shape[1]:
        raise ValueError("flow file does not hold every cv location")
    return Flow(cv, time, res)


def write_flow_binary(path: str, fl: Flow, endian: str = "<") -> None:
    n, ncv = fl.cv.shape
    with open(path, "wb") as f:
        w = _RecordWriter(f, endian)
        w.text("# ROCFLU flow file (v2)")
        w.text("# Precision and range")
        w.ints(_PREC_RANGE)
        w.text("# Initial residual")
        w.reals([fl.res_init])
        w.text("# Physical time")
        w.reals([fl.time])
        w.text("# Dimensions")
        w.ints([n, ncv])
        for iloc in range(ncv):
            w.text("# %2d" % (iloc + 1))
            w.reals(fl.cv[:, iloc])
        w.text("# End")


def read_flow_binary(path: str, endian: str = "<") -> Flow:
    with open(path, "rb") as f:
        r = _RecordReader(f.read(), endian)
    if r.text() != "# ROCFLU flow file (v2)":
        raise ValueError("not a ROCFLU v2 flow file")
    time = res = 0.0
    cv, dims, seen = None, None, set()
    while True:
        sec = r.text()
        if not sec.startswith("# "):
            raise ValueError(f"invalid section marker: {sec!r}")
        sec = sec[2:]
        if sec == "Precision and range":
            r.ints()
        elif sec == "Initial residual":
            res = float(r.reals()[0])
        elif sec == "Physical time":
            time = float(r.reals()[0])
        elif sec == "Dimensions":
            dims = r.ints()
            cv = np.zeros((int(dims[0]), int(dims[1])), np.float64)
        elif sec == "End":
            break
        else:
            iloc = int(sec[:2])
            if dims is None or iloc < 1 or iloc > dims[1]:
                raise ValueError(f"invalid cv location {sec!r}")
            cv[:, iloc - 1] = r.reals()
            seen.add(iloc)
    if cv is None or len(seen) != cv.shape[1]:
        raise ValueError("flow file does not hold every cv location")
    return Flow(cv, time, res)


# ---- bridges to the engine -------------------------------------------------------

def grid_of_mesh(m) -> Grid:
    """The grid file content of a mesh built by rocflupicl_gb300.mesh (cells in
    its global order, each patch's boundary faces as triangles and quads)."""
    pats = []
    for p in m.patches:
        tri = p.bf2v[:, 3] == 0
        pats.append(GridPatch(p.bf2v[tri][:, :3].astype(np.int32),
                              p.bf2v[~tri].astype(np.int32)))
    return Grid(m.xyz.copy(), m.conn[0], m.conn[1], m.conn[2], m.conn[3], pats)


def mesh_of_grid(g: Grid, threads: int = 0, stencils: str = "host"):
    """Region arrays of a grid: face list, geometry, stencils and moments by the
    same builder as the synthetic meshes."""
    from . import mesh as M
    return M.from_grid(g.xyz, g.tet2v, g.hex2v, g.pri2v, g.pyr2v,
                       [(p.tri2v, p.quad2v) for p in g.patches], threads=threads,
                       stencils=stencils)
