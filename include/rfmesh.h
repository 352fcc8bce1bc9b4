/*
 * rfmesh.h - host-side mesh builder that produces the region arrays the
 * residual engine (rfgpu.h) registers.
 *
 * In RocfluMP these arrays come from the Fortran initialisation chain
 * (rocflu/RFLU_InitFlowSolver.F90:604-1071): face list, geometry,
 * vertex-to-cell lists, cell-to-cell stencils and WLSQ moments.  This library
 * restates that chain for synthetic box meshes so the engine and the CPU oracle
 * can be fed identical, reference-shaped inputs without the Fortran host:
 *
 *   - cell numbering by type: tets, hexes, prisms, pyramids
 *       (modflu/RFLU_ModCellMapping.F90:330-432)
 *   - face vectors / centroids (libfloflu/FaceVector.F90:79-136,
 *       libfloflu/FaceCentroid.F90:77-122), volumes and centroids by the
 *       divergence theorem (modflu/RFLU_ModGeometry.F90:307-672), approximate
 *       centroids = vertex averages (RFLU_ModGeometry.F90:1277-1460)
 *   - c2c stencils: vertex neighbours ranked by shared-vertex fraction with the
 *       reference's quicksort, truncated to 10x the minimum size and re-sorted
 *       (modflu/RFLU_ModStencilsCells.F90:750-1416,2816-2909,
 *        modflu/RFLU_ModStencilsUtils.F90:696-979,1093-1137,
 *        modfloflu/ModSortSearch.F90:898-990), layer growth decided by the
 *       singular-value ratio test of libflu/RFLU_InvertMatrixSVD.F90:150-190
 *   - WLSQ moments (modflu/RFLU_ModWeights.F90:1770-1894)
 *
 * Face order is this library's own (first encounter while sweeping cells in
 * global order); the engine and the oracle consume it as given, exactly as the
 * engine consumes whatever face list the Fortran host passes.
 *
 * All arrays are returned in Fortran layout (column-major, first index fastest)
 * with 1-based cell indices, i.e. exactly what the Fortran host would pass
 * through ISO_C_BINDING.  Pointers stay valid until rfmesh_destroy.
 */
#ifndef RFMESH_H
#define RFMESH_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct rfmesh_s *rfmesh_t;

enum {
  RFMESH_HEX = 0,   /* nx*ny*nz hexahedra */
  RFMESH_TET = 1,   /* every hex split into 6 Kuhn (Freudenthal) tets */
  RFMESH_MIXED = 2, /* hexes; x>mid -> 2 prisms; z>mid -> 6 tets (prism
                       precedence); pyramid/tet transition cubes where a tet
                       cube meets a quad face, so the mesh is conforming */
  RFMESH_GRID = 3   /* any grid of the reference's cell types (rfmesh_create_grid) */
};

/* patch order of box meshes */
enum { RFMESH_XLO = 0, RFMESH_XHI, RFMESH_YLO, RFMESH_YHI, RFMESH_ZLO, RFMESH_ZHI,
       RFMESH_NPATCH };

/* size slots of rfmesh_sizes */
enum {
  RFMESH_NVERT = 0, RFMESH_NCELLS, RFMESH_NFACES, RFMESH_NPATCHES, RFMESH_NMEMBS,
  RFMESH_NTETS, RFMESH_NHEXS, RFMESH_NPRIS, RFMESH_NPYRS, RFMESH_NBFACES,
  RFMESH_MAXMEMBS, RFMESH_NSIZES
};

/* Return codes */
enum { RFMESH_OK = 0, RFMESH_ERR_ARG = 1, RFMESH_ERR_GEOM = 2, RFMESH_ERR_NOMEM = 3 };

/* flags of rfmesh_create_box_ex */
enum {
  RFMESH_DEFER_STENCILS = 1, /* build everything but the c2c stencils and moments; supply
                                them with rfmesh_set_stencils (e.g. from the GPU builder
                                rfgpu_mesh_stencils, which runs the same per-cell routine) */
  RFMESH_CELLS_ONLY = 2      /* generate the vertices and cells only (rfmesh_xyz,
                                rfmesh_cell_verts, rfmesh_cell_nverts, rfmesh_cell_type,
                                rfmesh_cell_conn); the face list, geometry, vertex-to-cell
                                lists and stencils come from the device builder
                                rfgpu_mesh_build, which reproduces this library's */
};

/* Build a box mesh over [lo,hi] with nx*ny*nz base hexes.  Interior vertices
 * are displaced by U(-jitter,+jitter)*h per coordinate from a 64-bit Mersenne
 * twister seeded with `seed`.  nThreads <= 0 uses all host threads. */
int rfmesh_create_box(int kind, int nx, int ny, int nz, const double lo[3],
                      const double hi[3], double jitter, unsigned long long seed,
                      int nThreads, rfmesh_t *out);
int rfmesh_create_box_ex(int kind, int nx, int ny, int nz, const double lo[3],
                         const double hi[3], double jitter, unsigned long long seed,
                         int nThreads, int flags, rfmesh_t *out);
/* Build from a grid in the reference's layout (what a .grda / .grd file
 * holds, modflu/RFLU_ModReadWriteGrid.F90): xyz(3,nVert); tet2v(4,nTets),
 * hex2v(8,nHexs), pri2v(6,nPris), pyr2v(5,nPyrs), 1-based, vertex orders of
 * modflu/RFLU_ModGrid.F90:92-102; per patch its boundary triangles
 * bTri2v[ip](3,nBTris[ip]) and quads bQuad2v[ip](4,nBQuads[ip]), 1-based.
 * Cells are numbered tets, hexes, prisms, pyramids in file order; each
 * boundary face is matched to its patch by vertex set, and a patch's faces
 * keep the file's order (triangles, then quads).  Every index is validated
 * (RFMESH_ERR_ARG); a boundary face in no patch, or a patch face that bounds
 * no cell, gives RFMESH_ERR_GEOM. */
int rfmesh_create_grid(int nVert, const double *xyz, int nTets, const int *tet2v, int nHexs,
                       const int *hex2v, int nPris, const int *pri2v, int nPyrs,
                       const int *pyr2v, int nPatches, const int *nBTris,
                       const int *const *bTri2v, const int *nBQuads,
                       const int *const *bQuad2v, int nThreads, int flags, rfmesh_t *out);
/* cell-to-vertex lists of one type (0 tet, 1 hex, 2 prism, 3 pyramid),
 * 0-based, (nv,nOfType) */
const int *rfmesh_cell_conn(rfmesh_t m, int type);
/* boundary face vertices of a patch, 0-based, (4,nBFaces), -1 for the 4th
 * vertex of a triangle; oriented outward */
const int *rfmesh_bf2v(rfmesh_t m, int iPatch);
int rfmesh_destroy(rfmesh_t m);
int rfmesh_sizes(rfmesh_t m, long long sizes[RFMESH_NSIZES]);
int rfmesh_patch_nbfaces(rfmesh_t m, int iPatch);

/* Fortran-layout views */
const double *rfmesh_xyz(rfmesh_t m);      /* (3,nVert) */
const double *rfmesh_vol(rfmesh_t m);      /* (nCells) */
const double *rfmesh_cofg(rfmesh_t m);     /* (3,nCells) */
const int *rfmesh_f2c(rfmesh_t m);         /* (2,nFaces), 1-based */
const double *rfmesh_fn(rfmesh_t m);       /* (4,nFaces): unit normal + area */
const double *rfmesh_fc(rfmesh_t m);       /* (3,nFaces) */
const int *rfmesh_c2cs_offsets(rfmesh_t m);/* (nCells+1), 0-based CSR offsets */
const int *rfmesh_c2cs_members(rfmesh_t m);/* (nMembs), 1-based cell ids */
const double *rfmesh_xyzmoms(rfmesh_t m);  /* (10,nCells) XYZ_MOM_11..44 */
const int *rfmesh_cell_type(rfmesh_t m);   /* (nCells) 0 tet 1 hex 2 pri 3 pyr */
const int *rfmesh_bf2c(rfmesh_t m, int iPatch);   /* (nBFaces), 1-based */
const double *rfmesh_bfn(rfmesh_t m, int iPatch); /* (4,nBFaces) */
const double *rfmesh_bfc(rfmesh_t m, int iPatch); /* (3,nBFaces) */

/* Connectivity the stencil builders take (0-based): cell vertices padded to
 * 8 with -1 (8,nCells), vertex counts (nCells), vertex-to-cell lists in
 * ascending cell order (offsets (nVert+1), cells (offsets[nVert])), and the
 * centroids (3,nCells) (the same array as rfmesh_cofg). */
const int *rfmesh_cell_verts(rfmesh_t m);
const int *rfmesh_cell_nverts(rfmesh_t m);
const int *rfmesh_v2c_offsets(rfmesh_t m);
const int *rfmesh_v2c(rfmesh_t m);
const double *rfmesh_cofg_view(rfmesh_t m);

/* Install c2c stencils (0-based CSR offsets (nCells+1), 1-based members, at
 * most 40 per cell) and moments (10,nCells) built elsewhere. */
int rfmesh_set_stencils(rfmesh_t m, const int *offsets, const int *members, const double *moms);

/* The host stencil builder on connectivity given as arrays (the inputs of
 * rfgpu_mesh_stencils, same outputs): e.g. the cells of one partitioned
 * region, actual and virtual, whose stencils the reference builds from the
 * region's own cells (RFLU_BuildC2CStencilWrapper over nCellsTot).
 * c2csMembers needs room for 40 per cell.  RFMESH_ERR_ARG for a bad index,
 * RFMESH_ERR_GEOM when a cell has more than 256 vertex-neighbour entries. */
int rfmesh_build_stencils(int nCells, int nVerts, const int *cellVerts, const int *cellNVerts,
                          const int *v2cOffsets, const int *v2c, const double *cofg, int nThreads,
                          int *c2csOffsets, int *c2csMembers, double *xyzMoms);

#ifdef __cplusplus
}
#endif
#endif
