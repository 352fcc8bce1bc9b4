// rfmesh_geom.h - cell face tables and face geometry shared by the host mesh
// builder (rfmesh.cpp) and the device builder (rfgpu_mesh_build), so both
// enumerate the same faces in the same vertex order and compute the same face
// vectors and centroids bit for bit (FP64, no contraction on either side).
#pragma once

#include "rfmesh_stencil.h"  // RFM_HD

namespace rfm {

enum { T_TET = 0, T_HEX = 1, T_PRI = 2, T_PYR = 3 };

// Local faces of the four cell types, cyclic vertex order, -1 padded for
// triangles (vertex orders of modflu/RFLU_ModGrid.F90:92-102; face numbering
// of the reference's face-list build, RFLU_ModFaceList.F90:784-1609).
#define RFM_FACE_TABLE                                                                     \
  {{{0, 2, 1, -1}, {0, 1, 3, -1}, {1, 2, 3, -1}, {0, 3, 2, -1}, {-1, -1, -1, -1},          \
    {-1, -1, -1, -1}},                                                                     \
   {{0, 3, 2, 1}, {4, 5, 6, 7}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}},   \
   {{0, 2, 1, -1}, {3, 4, 5, -1}, {0, 1, 4, 3}, {1, 2, 5, 4}, {2, 0, 3, 5},                 \
    {-1, -1, -1, -1}},                                                                     \
   {{0, 3, 2, 1}, {0, 1, 4, -1}, {1, 2, 4, -1}, {2, 3, 4, -1}, {3, 0, 4, -1},              \
    {-1, -1, -1, -1}}}

RFM_HD inline int cell_nv(int t) { return t == T_TET ? 4 : t == T_HEX ? 8 : t == T_PRI ? 6 : 5; }
RFM_HD inline int cell_nf(int t) { return t == T_TET ? 4 : t == T_HEX ? 6 : 5; }
RFM_HD inline int face_local(int t, int f, int a) {
  const signed char tab[4][6][4] = RFM_FACE_TABLE;
  return tab[t][f][a];
}

// FaceVectorTria / FaceVectorQuad (libfloflu/FaceVector.F90:79-136) and
// FaceCentroidTria / FaceCentroidQuad (libfloflu/FaceCentroid.F90:77-122) of
// face vertices fv (fv[3] < 0: triangle), xyz(3,nVert).
RFM_HD inline void face_vec_cen(const double *xyz, const int *fv, double S[3], double C[3]) {
  if (fv[3] < 0) {
    const double *p1 = xyz + 3 * (size_t)fv[0], *p2 = xyz + 3 * (size_t)fv[1],
                 *p3 = xyz + 3 * (size_t)fv[2];
    double dxa = p1[0] - p2[0], dya = p1[1] - p2[1], dza = p1[2] - p2[2];
    double dxb = p1[0] - p3[0], dyb = p1[1] - p3[1], dzb = p1[2] - p3[2];
    S[0] = 0.5 * (dya * dzb - dyb * dza);
    S[1] = -0.5 * (dxa * dzb - dxb * dza);
    S[2] = 0.5 * (dxa * dyb - dxb * dya);
    const double thrd = 1.0 / 3.0;
    C[0] = thrd * (p1[0] + p2[0] + p3[0]);
    C[1] = thrd * (p1[1] + p2[1] + p3[1]);
    C[2] = thrd * (p1[2] + p2[2] + p3[2]);
  } else {
    const double *p1 = xyz + 3 * (size_t)fv[0], *p2 = xyz + 3 * (size_t)fv[1],
                 *p3 = xyz + 3 * (size_t)fv[2], *p4 = xyz + 3 * (size_t)fv[3];
    double dxa = p3[0] - p1[0], dya = p3[1] - p1[1], dza = p3[2] - p1[2];
    double dxb = p2[0] - p4[0], dyb = p2[1] - p4[1], dzb = p2[2] - p4[2];
    S[0] = 0.5 * (dza * dyb - dya * dzb);
    S[1] = 0.5 * (dxa * dzb - dza * dxb);
    S[2] = 0.5 * (dya * dxb - dxa * dyb);
    C[0] = 0.25 * (p1[0] + p2[0] + p3[0] + p4[0]);
    C[1] = 0.25 * (p1[1] + p2[1] + p3[1] + p4[1]);
    C[2] = 0.25 * (p1[2] + p2[2] + p3[2] + p4[2]);
  }
}

// A cell's contribution of one face to the divergence-theorem sums of
// RFLU_BuildGeometry (RFLU_ModGeometry.F90:307-672): volume term
// (C - cofgApp).S and centroid term (C.S) C, added on the face's first cell
// and subtracted on its second.
RFM_HD inline void face_contrib(const double S[3], const double C[3], const double *ca, double sgn,
                                double *vol, double *cg) {
  double term = (C[0] - ca[0]) * S[0] + (C[1] - ca[1]) * S[1] + (C[2] - ca[2]) * S[2];
  if (sgn > 0) *vol = *vol + term; else *vol = *vol - term;
  term = C[0] * S[0] + C[1] * S[1] + C[2] * S[2];
  for (int d = 0; d < 3; ++d) {
    if (sgn > 0) cg[d] = cg[d] + term * C[d];
    else cg[d] = cg[d] - term * C[d];
  }
}

}  // namespace rfm
