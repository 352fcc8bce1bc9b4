"""Partitioned regions with virtual cells, as the engine's multi-region path
consumes them.

In RocfluMP a partitioned case comes from the preprocessor (rflupart): each
region holds its actual cells, then virtual cells copied from its neighbours,
the faces between actual cells and between actual and virtual cells, its
share of the boundary patches, stencils built over its own cells, and one
border per neighbour listing the cells it sends and receives
(utilities/part/RFLU_ModPartitionRegion.F90:135-420, the second-order rule of
utilities/part/RFLU_ModPartitionRegionUtils.F90:269-648).  This module builds
the same structure from a whole mesh so partitioned cases can be run and
checked here:

  * ownership: the cells sorted by one centroid coordinate and cut into
    equal slabs;
  * virtual cells (second order): the stencil members and face neighbours of
    the region's actual cells that it does not own, then two more layers of
    the stencil members of the virtual cells added last, each layer in
    ascending global id after the actual cells (the reference's ``vc`` list
    is kept sorted the same way);
  * faces: every interior face with an actual cell (the flux faces, AA and
    AV), in the whole mesh's face order; then, for the virtual cells' own
    face lists, the faces between two virtual cells (VV) and between a
    virtual cell and a cell outside the region (VX, the outside side 0),
    each in the whole mesh's order, as the reference's face list orders
    face kinds (modflu/RFLU_ModFaceList.F90:1317-1360); boundary faces of
    the actual cells patch by patch, and after them each patch's faces on
    virtual cells (VB);
  * stencils and WLSQ moments rebuilt over the region's own cells, as the
    reference's solver builds them for nCellsTot cells;
  * borders: one per neighbour region in ascending region id; send cell k of
    a border pairs with receive cell k of the neighbour's matching border.
"""
from __future__ import annotations

from dataclasses import replace
from typing import List

import numpy as np

from . import mesh as M


def _csr_rows(off: np.ndarray, data: np.ndarray, rows: np.ndarray) -> np.ndarray:
    """Concatenated CSR rows `rows` of (off, data)."""
    if rows.size == 0:
        return np.zeros(0, data.dtype)
    lens = off[rows + 1] - off[rows]
    starts = np.repeat(off[rows] - np.cumsum(lens) + lens, lens)
    return data[starts + np.arange(int(lens.sum()))]


def owners(m: M.BoxMesh, n_regions: int, axis: int = 0) -> np.ndarray:
    """Region (0-based) of every cell: equal slabs of the cells sorted by one
    centroid coordinate (ties by cell id)."""
    n = m.nCells
    order = np.argsort(m.cofg[:, axis], kind="stable")
    own = np.empty(n, np.int32)
    own[order] = (np.arange(n, dtype=np.int64) * n_regions // n).astype(np.int32)
    return own


def partition(m: M.BoxMesh, n_regions: int, axis: int = 0, layers: int = 2,
              threads: int = 0) -> List[M.BoxMesh]:
    """Split a whole (unpartitioned) mesh into n_regions regions with virtual
    cells and borders.  Returns one mesh per region (iRegionGlobal = 1..n)."""
    if m.nCellsTot not in (0, m.nCells):
        raise ValueError("the mesh is already a partitioned region")
    nC = m.nCells
    own = owners(m, n_regions, axis)
    mem0 = m.c2cs_mem.astype(np.int64) - 1
    off = m.c2cs_off.astype(np.int64)
    f2c0 = m.f2c.astype(np.int64) - 1
    cv8, nv = M.cell_vertices(m)
    # face neighbours per cell (CSR)
    a, b = f2c0[:, 0], f2c0[:, 1]
    src = np.concatenate([a, b])
    dst = np.concatenate([b, a])
    o = np.argsort(src, kind="stable")
    fn_off = np.zeros(nC + 1, np.int64)
    np.add.at(fn_off, src + 1, 1)
    fn_off = np.cumsum(fn_off)
    fn_dat = dst[o]

    regions = []
    for r in range(n_regions):
        act = np.flatnonzero(own == r)
        taken = np.zeros(nC, bool)
        taken[act] = True
        vlist = []
        new = np.unique(np.concatenate([_csr_rows(off, mem0, act), _csr_rows(fn_off, fn_dat, act)]))
        new = new[~taken[new]]
        taken[new] = True
        vlist.append(new)
        for _ in range(layers):
            nxt = np.unique(_csr_rows(off, mem0, new))
            nxt = nxt[~taken[nxt]]
            taken[nxt] = True
            vlist.append(nxt)
            new = nxt
        virt = np.sort(np.concatenate(vlist))
        regions.append((act, virt))

    out = []
    for r, (act, virt) in enumerate(regions):
        loc = np.concatenate([act, virt])
        nT = loc.shape[0]
        g2l = np.full(nC, -1, np.int64)
        g2l[loc] = np.arange(nT)
        inA = np.zeros(nC, bool)
        inA[act] = True
        fsel = np.flatnonzero(inA[a] | inA[b])
        if np.any(g2l[f2c0[fsel]] < 0):
            raise RuntimeError("a face of an actual cell leads outside the region")
        inV = np.zeros(nC, bool)
        inV[virt] = True
        vv = np.flatnonzero(inV[a] & inV[b])
        vx = np.flatnonzero((inV[a] & (g2l[b] < 0)) | (inV[b] & (g2l[a] < 0)))
        vsel = np.concatenate([vv, vx])
        vf2c = np.where(g2l[f2c0[vsel]] >= 0, g2l[f2c0[vsel]] + 1, 0).astype(np.int32)
        patches = []
        for p in m.patches:
            sel = np.flatnonzero(inA[p.bf2c - 1])
            vbs = np.flatnonzero(inV[p.bf2c - 1])
            patches.append(M.Patch(bf2c=(g2l[p.bf2c[sel] - 1] + 1).astype(np.int32),
                                   fn=p.fn[sel].copy(), fc=p.fc[sel].copy(),
                                   bf2v=None if p.bf2v is None else p.bf2v[sel].copy(),
                                   global_faces=sel,
                                   vb_bf2c=(g2l[p.bf2c[vbs] - 1] + 1).astype(np.int32),
                                   vb_fn=p.fn[vbs].copy(), vb_fc=p.fc[vbs].copy()))
        # stencils over the region's own cells: vertex-to-cell lists of the
        # region's cells in ascending local id
        lcv = cv8[loc]
        lnv = nv[loc]
        vs = lcv.reshape(-1)
        cs = np.repeat(np.arange(nT), 8)
        keep = vs >= 0
        vs, cs = vs[keep], cs[keep]
        oo = np.lexsort((cs, vs))
        nV = int(m.xyz.shape[0])
        voff = np.zeros(nV + 1, np.int64)
        np.add.at(voff, vs + 1, 1)
        voff = np.cumsum(voff).astype(np.int32)
        cofg = m.cofg[loc].copy()
        soff, smem, moms = M.build_stencils(lcv, lnv, voff, cs[oo].astype(np.int32), cofg,
                                            threads)
        out.append(M.BoxMesh(
            kind=m.kind, dims=m.dims, nCells=int(act.shape[0]), nFaces=int(fsel.shape[0]),
            xyz=m.xyz, vol=m.vol[loc].copy(), cofg=cofg,
            f2c=(g2l[f2c0[fsel]] + 1).astype(np.int32), fn=m.fn[fsel].copy(),
            fc=m.fc[fsel].copy(), c2cs_off=soff, c2cs_mem=smem, xyzmoms=moms,
            cell_type=m.cell_type[loc].copy(), patches=patches, n_of_type=m.n_of_type, conn=[],
            nCellsTot=int(nT), iRegionGlobal=r + 1, borders=[], global_cells=loc,
            vf2c=vf2c, vfn=m.fn[vsel].copy(), vfc=m.fc[vsel].copy()))

    # borders
    recv = {}
    for r, (act, virt) in enumerate(regions):
        nA = act.shape[0]
        vo = own[virt]
        for s in np.unique(vo):
            idx = np.flatnonzero(vo == s)
            recv[(r, int(s))] = (virt[idx], (nA + idx + 1).astype(np.int32))
    nbrs = [sorted({s for (q, s) in recv if q == r} | {q for (q, s) in recv if s == r})
            for r in range(n_regions)]
    for r in range(n_regions):
        g2l = np.full(nC, -1, np.int64)
        g2l[out[r].global_cells] = np.arange(out[r].nTot)
        for s in nbrs[r]:
            sent = recv.get((s, r), (np.zeros(0, np.int64), None))[0]
            icg_recv = recv.get((r, s), (None, np.zeros(0, np.int32)))[1]
            out[r].borders.append(M.Border(
                iRegionGlobal=s + 1, iBorder=nbrs[s].index(r) + 1,
                icgSend=(g2l[sent] + 1).astype(np.int32), icgRecv=icg_recv))
    return out


def partition_case(case, n_regions: int, axis: int = 0, layers: int = 2, threads: int = 0):
    """The regions of `case` (its mesh partitioned as above), each a Case with
    the region's state rows cv, dv (actual then virtual cells) and the same
    boundary conditions and numerics."""
    parts = partition(case.mesh, n_regions, axis, layers, threads)
    out = []
    for p in parts:
        bcs = []
        for bc, pa, whole in zip(case.bcs, p.patches, case.mesh.patches):
            # per-face patch values follow their faces
            v, po = bc.vals, bc.pout
            if v is not None and np.ndim(v) == 2 and np.shape(v)[0] == whole.n:
                v = np.asarray(v)[pa.global_faces]
            if po is not None and np.size(po) == whole.n and whole.n > 1:
                po = np.asarray(po)[pa.global_faces]
            bcs.append(replace(bc, vals=v, pout=po))
        out.append(replace(case, name=f"{case.name}.r{p.iRegionGlobal}", mesh=p, bcs=bcs,
                           cv=case.cv[p.global_cells].copy(), dv=case.dv[p.global_cells].copy()))
    return out


def gather(cases, field: str = "cv") -> np.ndarray:
    """Whole-mesh array of a per-region field from the regions' actual cells."""
    n = sum(c.mesh.nCells for c in cases)
    width = getattr(cases[0], field).shape[1]
    out = np.empty((n, width))
    for c in cases:
        out[c.mesh.global_cells[:c.mesh.nCells]] = getattr(c, field)[:c.mesh.nCells]
    return out
