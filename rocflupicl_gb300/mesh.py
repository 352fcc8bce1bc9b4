"""Python view of the host mesh builder (include/rfmesh.h).

A `BoxMesh` holds the region arrays in the layout the Fortran host passes to
the engine: Fortran column-major arrays with 1-based cell indices, e.g.
``f2c`` has shape ``(nFaces, 2)`` in NumPy (C order) which is the memory image
of the Fortran array ``f2c(2,nFaces)``.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import _build

HEX, TET, MIXED, GRID = 0, 1, 2, 3
XLO, XHI, YLO, YHI, ZLO, ZHI = range(6)
_NSIZES = 11

_lib = None


def _load():
    global _lib
    if _lib is None:
        path = _build.build_mesh()
        lib = C.CDLL(str(path))
        vp = C.c_void_p
        lib.rfmesh_create_box.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int,
                                          C.POINTER(C.c_double), C.POINTER(C.c_double),
                                          C.c_double, C.c_ulonglong, C.c_int, C.POINTER(vp)]
        lib.rfmesh_create_box_ex.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int,
                                             C.POINTER(C.c_double), C.POINTER(C.c_double),
                                             C.c_double, C.c_ulonglong, C.c_int, C.c_int,
                                             C.POINTER(vp)]
        for name in ("cell_verts", "cell_nverts", "v2c_offsets", "v2c"):
            f = getattr(lib, "rfmesh_" + name)
            f.argtypes = [vp]
            f.restype = C.POINTER(C.c_int)
        lib.rfmesh_cofg_view.argtypes = [vp]
        lib.rfmesh_cofg_view.restype = C.POINTER(C.c_double)
        lib.rfmesh_set_stencils.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                            C.POINTER(C.c_double)]
        ip_ = C.POINTER(C.c_int)
        lib.rfmesh_build_stencils.argtypes = [C.c_int, C.c_int, ip_, ip_, ip_, ip_,
                                              C.POINTER(C.c_double), C.c_int, ip_, ip_,
                                              C.POINTER(C.c_double)]
        ipp = C.POINTER(C.POINTER(C.c_int))
        lib.rfmesh_create_grid.argtypes = [C.c_int, C.POINTER(C.c_double),
                                           C.c_int, C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_int),
                                           C.c_int, C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_int),
                                           C.c_int, C.POINTER(C.c_int), ipp, C.POINTER(C.c_int),
                                           ipp, C.c_int, C.c_int, C.POINTER(vp)]
        lib.rfmesh_cell_conn.argtypes = [vp, C.c_int]
        lib.rfmesh_cell_conn.restype = C.POINTER(C.c_int)
        lib.rfmesh_bf2v.argtypes = [vp, C.c_int]
        lib.rfmesh_bf2v.restype = C.POINTER(C.c_int)
        lib.rfmesh_destroy.argtypes = [vp]
        lib.rfmesh_sizes.argtypes = [vp, C.POINTER(C.c_longlong)]
        lib.rfmesh_patch_nbfaces.argtypes = [vp, C.c_int]
        for name in ("xyz", "vol", "cofg", "fn", "fc", "xyzmoms"):
            f = getattr(lib, "rfmesh_" + name)
            f.argtypes = [vp]
            f.restype = C.POINTER(C.c_double)
        for name in ("f2c", "c2cs_offsets", "c2cs_members", "cell_type"):
            f = getattr(lib, "rfmesh_" + name)
            f.argtypes = [vp]
            f.restype = C.POINTER(C.c_int)
        lib.rfmesh_bf2c.argtypes = [vp, C.c_int]
        lib.rfmesh_bf2c.restype = C.POINTER(C.c_int)
        for name in ("bfn", "bfc"):
            f = getattr(lib, "rfmesh_" + name)
            f.argtypes = [vp, C.c_int]
            f.restype = C.POINTER(C.c_double)
        _lib = lib
    return _lib


def _copy(ptr, n, dtype, shape):
    if n == 0:
        return np.zeros(shape, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True).reshape(shape)


@dataclass
class Patch:
    """One boundary patch: faces bf2c (1-based), fn (nB,4), fc (nB,3), and the
    face vertices bf2v (nB,4), 1-based, 0 for the 4th vertex of a triangle."""
    bf2c: np.ndarray
    fn: np.ndarray
    fc: np.ndarray
    bf2v: Optional[np.ndarray] = None
    # partitioned regions: positions of these faces in the whole mesh's patch
    global_faces: Optional[np.ndarray] = None
    # partitioned regions: the patch's faces on virtual cells (the reference's
    # FACE_KIND_VB faces, pPatch%nBFaces+1..nBFacesTot), bf2c (1-based local),
    # fn, fc; only the positivity check of RECONST 2 reads them
    vb_bf2c: Optional[np.ndarray] = None
    vb_fn: Optional[np.ndarray] = None
    vb_fc: Optional[np.ndarray] = None

    @property
    def n(self) -> int:
        return int(self.bf2c.shape[0])

    @property
    def n_vb(self) -> int:
        return 0 if self.vb_bf2c is None else int(self.vb_bf2c.shape[0])

    def all_faces(self):
        """(bf2c, fn, fc) of the actual faces followed by the virtual ones."""
        if not self.n_vb:
            return self.bf2c, self.fn, self.fc
        return (np.concatenate([self.bf2c, self.vb_bf2c]), np.concatenate([self.fn, self.vb_fn]),
                np.concatenate([self.fc, self.vb_fc]))


@dataclass
class Border:
    """One border of a partitioned region (t_border, modfloflu/ModBorder.F90:87-99):
    the neighbour's global region id (1-based), the 1-based index of the
    matching border in the neighbour, the actual cells sent (1-based local)
    and the virtual cells received (1-based local).  Send cell k here pairs
    with receive cell k of the matching border."""
    iRegionGlobal: int
    iBorder: int
    icgSend: np.ndarray
    icgRecv: np.ndarray


@dataclass
class BoxMesh:
    kind: int
    dims: tuple
    nCells: int                 # actual cells
    nFaces: int
    xyz: np.ndarray
    vol: np.ndarray
    cofg: np.ndarray            # (nCells,3)
    f2c: np.ndarray             # (nFaces,2) 1-based
    fn: np.ndarray              # (nFaces,4)
    fc: np.ndarray              # (nFaces,3)
    c2cs_off: np.ndarray        # (nCells+1,) 0-based offsets
    c2cs_mem: np.ndarray        # (nMembs,) 1-based
    xyzmoms: np.ndarray         # (nCells,10)
    cell_type: np.ndarray
    patches: List[Patch] = field(default_factory=list)
    n_of_type: tuple = (0, 0, 0, 0)
    # cell-to-vertex lists per type (tet, hex, prism, pyramid), 1-based, (n, nv)
    conn: List[np.ndarray] = field(default_factory=list)
    # partitioned regions: actual + virtual cells (0: no virtual cells; the
    # per-cell arrays vol, cofg, c2cs_off, xyzmoms, cell_type then have
    # nCellsTot rows), the global region id and the borders
    nCellsTot: int = 0
    iRegionGlobal: int = 1
    borders: List[Border] = field(default_factory=list)
    # whole-mesh (0-based) ids of a partitioned region's cells, actual then virtual
    global_cells: Optional[np.ndarray] = None
    # partitioned regions: the interior faces beyond the flux faces, between
    # two virtual cells (FACE_KIND_VV) and between a virtual cell and a cell
    # outside the region (FACE_KIND_VX, outside side 0), f2c (n,2) 1-based
    # local, fn, fc; only the positivity check of RECONST 2 reads them
    vf2c: Optional[np.ndarray] = None
    vfn: Optional[np.ndarray] = None
    vfc: Optional[np.ndarray] = None

    @property
    def nTot(self) -> int:
        return self.nCellsTot if self.nCellsTot > 0 else self.nCells

    @property
    def nBFaces(self) -> int:
        return sum(p.n for p in self.patches)

    @property
    def nMembs(self) -> int:
        return int(self.c2cs_mem.shape[0])

    @property
    def nFacesAll(self) -> int:
        """Interior faces of every kind: the flux faces, then VV and VX faces."""
        return self.nFaces + (0 if self.vf2c is None else int(self.vf2c.shape[0]))

    def all_faces(self):
        """(f2c, fn, fc) of all interior faces, flux faces first."""
        if self.nFacesAll == self.nFaces:
            return self.f2c, self.fn, self.fc
        return (np.concatenate([self.f2c, self.vf2c]), np.concatenate([self.fn, self.vfn]),
                np.concatenate([self.fc, self.vfc]))


RFMESH_DEFER_STENCILS = 1
RFMESH_CELLS_ONLY = 2


def box(kind: int, nx: int, ny: int, nz: int, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0),
        jitter: float = 0.0, seed: int = 0, threads: int = 0, stencils: str = "host") -> BoxMesh:
    """Build a box mesh (HEX / Kuhn TET / MIXED) and return its region arrays.
    stencils="device" builds the c2c stencils and WLSQ moments on the GPU
    (rfgpu_mesh_stencils: the host builder's per-cell routine, identical
    output) and the rest on the host; stencils="all-device" builds everything
    but the vertices and cells on the GPU (rfgpu_mesh_build: face list,
    geometry, vertex-to-cell lists, stencils, moments; identical output)."""
    if stencils not in ("host", "device", "all-device"):
        raise ValueError(stencils)
    lib = _load()
    h = C.c_void_p()
    lo_a = (C.c_double * 3)(*lo)
    hi_a = (C.c_double * 3)(*hi)
    if stencils == "all-device":
        rc = lib.rfmesh_create_box_ex(kind, nx, ny, nz, lo_a, hi_a, float(jitter), int(seed),
                                      int(threads), RFMESH_CELLS_ONLY, C.byref(h))
        if rc != 0:
            raise RuntimeError(f"rfmesh_create_box failed with code {rc}")
        try:
            return _from_device(lib, h, kind, (nx, ny, nz), lo, hi)
        finally:
            lib.rfmesh_destroy(h)
    flags = RFMESH_DEFER_STENCILS if stencils == "device" else 0
    rc = lib.rfmesh_create_box_ex(kind, nx, ny, nz, lo_a, hi_a, float(jitter), int(seed),
                                  int(threads), flags, C.byref(h))
    if rc != 0:
        raise RuntimeError(f"rfmesh_create_box failed with code {rc}")
    try:
        return _extract(lib, h, kind, (nx, ny, nz), stencils)
    finally:
        lib.rfmesh_destroy(h)


_NV = (4, 8, 6, 5)


def _from_device(lib, h, kind, dims, lo, hi) -> BoxMesh:
    """Region arrays of a cells-only rfmesh handle, built by rfgpu_mesh_build."""
    from . import engine
    s = (C.c_longlong * _NSIZES)()
    lib.rfmesh_sizes(h, s)
    nV, nC = s[0], s[1]
    xyz = _copy(lib.rfmesh_xyz(h), 3 * nV, np.float64, (nV, 3))
    cv8 = _copy(lib.rfmesh_cell_verts(h), 8 * nC, np.int32, (nC, 8))
    nv = _copy(lib.rfmesh_cell_nverts(h), nC, np.int32, (nC,))
    ct = _copy(lib.rfmesh_cell_type(h), nC, np.int32, (nC,))
    r = engine.mesh_build(nV, xyz, cv8, nv, ct, lo, hi)
    m = BoxMesh(kind=kind, dims=dims, nCells=nC, nFaces=r["f2c"].shape[0], xyz=xyz, vol=r["vol"],
                cofg=r["cofg"], f2c=r["f2c"], fn=r["fn"], fc=r["fc"], c2cs_off=r["c2cs_off"],
                c2cs_mem=r["c2cs_mem"], xyzmoms=r["xyzmoms"], cell_type=ct,
                n_of_type=(s[5], s[6], s[7], s[8]))
    for pa in r["patches"]:
        m.patches.append(Patch(bf2c=pa["bf2c"], fn=pa["fn"], fc=pa["fc"], bf2v=pa["bf2v"] + 1))
    m.conn = [_copy(lib.rfmesh_cell_conn(h, t), _NV[t] * int(s[5 + t]), np.int32,
                    (int(s[5 + t]), _NV[t])) + 1 for t in range(4)]
    return m


def _extract(lib, h, kind, dims, stencils) -> BoxMesh:
    """Region arrays of a built rfmesh handle (stencils built on the GPU first
    when they were deferred)."""
    if stencils == "device":
        from . import engine
        s = (C.c_longlong * _NSIZES)()
        lib.rfmesh_sizes(h, s)
        nV, nC = s[0], s[1]
        view = lambda p, n: np.ctypeslib.as_array(p, shape=(n,))
        vo = view(lib.rfmesh_v2c_offsets(h), nV + 1)
        off, mem, mom = engine.mesh_stencils(
            nC, nV, view(lib.rfmesh_cell_verts(h), 8 * nC), view(lib.rfmesh_cell_nverts(h), nC),
            vo, view(lib.rfmesh_v2c(h), int(vo[-1])), view(lib.rfmesh_cofg_view(h), 3 * nC))
        rc = lib.rfmesh_set_stencils(h, off.ctypes.data_as(C.POINTER(C.c_int)),
                                     mem.ctypes.data_as(C.POINTER(C.c_int)),
                                     mom.ctypes.data_as(C.POINTER(C.c_double)))
        if rc != 0:
            raise RuntimeError(f"rfmesh_set_stencils failed with code {rc}")
    s = (C.c_longlong * _NSIZES)()
    lib.rfmesh_sizes(h, s)
    nV, nC, nF, nP, nM = s[0], s[1], s[2], s[3], s[4]
    m = BoxMesh(
        kind=kind, dims=dims, nCells=nC, nFaces=nF,
        xyz=_copy(lib.rfmesh_xyz(h), 3 * nV, np.float64, (nV, 3)),
        vol=_copy(lib.rfmesh_vol(h), nC, np.float64, (nC,)),
        cofg=_copy(lib.rfmesh_cofg(h), 3 * nC, np.float64, (nC, 3)),
        f2c=_copy(lib.rfmesh_f2c(h), 2 * nF, np.int32, (nF, 2)),
        fn=_copy(lib.rfmesh_fn(h), 4 * nF, np.float64, (nF, 4)),
        fc=_copy(lib.rfmesh_fc(h), 3 * nF, np.float64, (nF, 3)),
        c2cs_off=_copy(lib.rfmesh_c2cs_offsets(h), nC + 1, np.int32, (nC + 1,)),
        c2cs_mem=_copy(lib.rfmesh_c2cs_members(h), nM, np.int32, (nM,)),
        xyzmoms=_copy(lib.rfmesh_xyzmoms(h), 10 * nC, np.float64, (nC, 10)),
        cell_type=_copy(lib.rfmesh_cell_type(h), nC, np.int32, (nC,)),
        n_of_type=(s[5], s[6], s[7], s[8]),
    )
    for ip in range(nP):
        nb = lib.rfmesh_patch_nbfaces(h, ip)
        m.patches.append(Patch(
            bf2c=_copy(lib.rfmesh_bf2c(h, ip), nb, np.int32, (nb,)),
            fn=_copy(lib.rfmesh_bfn(h, ip), 4 * nb, np.float64, (nb, 4)),
            fc=_copy(lib.rfmesh_bfc(h, ip), 3 * nb, np.float64, (nb, 3)),
            bf2v=_copy(lib.rfmesh_bf2v(h, ip), 4 * nb, np.int32, (nb, 4)) + 1))
    m.conn = [_copy(lib.rfmesh_cell_conn(h, t), _NV[t] * int(s[5 + t]), np.int32,
                    (int(s[5 + t]), _NV[t])) + 1 for t in range(4)]
    return m


def build_stencils(cell_verts, cell_nverts, v2c_off, v2c, cofg, threads: int = 0):
    """rfmesh_build_stencils: c2c stencils and WLSQ moments of every cell of
    the given connectivity (0-based cell vertices padded to 8 with -1, vertex
    counts, vertex-to-cell CSR in ascending cell order, centroids (n,3)) with
    the host builder.  Returns (offsets (n+1, 0-based), members (1-based),
    moments (n, 10))."""
    lib = _load()
    cv = np.ascontiguousarray(cell_verts, np.int32).reshape(-1)
    nv = np.ascontiguousarray(cell_nverts, np.int32)
    vo = np.ascontiguousarray(v2c_off, np.int32)
    vc = np.ascontiguousarray(v2c, np.int32)
    cg = np.ascontiguousarray(cofg, np.float64)
    n = nv.shape[0]
    off = np.empty(n + 1, np.int32)
    mem = np.empty(40 * n, np.int32)
    mom = np.empty((n, 10), np.float64)
    ip = C.POINTER(C.c_int)
    rc = lib.rfmesh_build_stencils(n, vo.shape[0] - 1, cv.ctypes.data_as(ip), nv.ctypes.data_as(ip),
                                   vo.ctypes.data_as(ip), vc.ctypes.data_as(ip),
                                   cg.ctypes.data_as(C.POINTER(C.c_double)), int(threads),
                                   off.ctypes.data_as(ip), mem.ctypes.data_as(ip),
                                   mom.ctypes.data_as(C.POINTER(C.c_double)))
    if rc != 0:
        raise RuntimeError(f"rfmesh_build_stencils failed with code {rc}")
    return off, mem[:off[-1]].copy(), mom


def cell_vertices(m: BoxMesh):
    """Cell vertex lists of a mesh in its cell numbering (tets, hexes, prisms,
    pyramids): (nCells, 8) 0-based padded with -1, and the counts."""
    n = sum(int(c.shape[0]) for c in m.conn)
    cv8 = np.full((n, 8), -1, np.int32)
    nv = np.zeros(n, np.int32)
    k = 0
    for t, c in enumerate(m.conn):
        nt = int(c.shape[0])
        cv8[k:k + nt, :_NV[t]] = c - 1
        nv[k:k + nt] = _NV[t]
        k += nt
    return cv8, nv


def from_grid(xyz, tet2v=None, hex2v=None, pri2v=None, pyr2v=None, patches=(),
              threads: int = 0, stencils: str = "host") -> BoxMesh:
    """Region arrays of a grid in the reference's layout (rfmesh_create_grid):
    xyz (nVert,3); tet2v (n,4), hex2v (n,8), pri2v (n,6), pyr2v (n,5), 1-based;
    patches = [(tri2v (n,3), quad2v (n,4)), ...], 1-based."""
    if stencils not in ("host", "device"):
        raise ValueError(stencils)
    lib = _load()
    ip_t = C.POINTER(C.c_int)
    keep = []

    def arr(a, cols, dt=np.int32):
        a = np.zeros((0, cols), dt) if a is None else np.ascontiguousarray(a, dt).reshape(-1, cols)
        keep.append(a)
        return a

    xyz_a = arr(xyz, 3, np.float64)
    conn = [arr(tet2v, 4), arr(hex2v, 8), arr(pri2v, 6), arr(pyr2v, 5)]
    nP = len(patches)
    tris = [arr(t, 3) for t, _ in patches]
    quads = [arr(q, 4) for _, q in patches]
    nT = (C.c_int * max(1, nP))(*[t.shape[0] for t in tris])
    nQ = (C.c_int * max(1, nP))(*[q.shape[0] for q in quads])
    pT = (ip_t * max(1, nP))(*[t.ctypes.data_as(ip_t) for t in tris])
    pQ = (ip_t * max(1, nP))(*[q.ctypes.data_as(ip_t) for q in quads])
    h = C.c_void_p()
    flags = RFMESH_DEFER_STENCILS if stencils == "device" else 0
    rc = lib.rfmesh_create_grid(
        xyz_a.shape[0], xyz_a.ctypes.data_as(C.POINTER(C.c_double)),
        *[v for c in conn for v in (c.shape[0], c.ctypes.data_as(ip_t))],
        nP, nT, pT, nQ, pQ, int(threads), flags, C.byref(h))
    if rc != 0:
        raise RuntimeError(f"rfmesh_create_grid failed with code {rc}")
    try:
        return _extract(lib, h, GRID, (0, 0, 0), stencils)
    finally:
        lib.rfmesh_destroy(h)
