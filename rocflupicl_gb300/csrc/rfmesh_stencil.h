// rfmesh_stencil.h - per-cell c2c stencil and WLSQ moments, shared by the
// host mesh builder (rfmesh.cpp, OpenMP over cells) and the device builder
// (rfgpu_mesh_stencils, one thread per cell), so both produce the same
// members in the same order and the same moments bit for bit (FP64, no
// contraction on either side, IEEE division and square root).
//
//   candidates  vertex neighbours of the cell (RFLU_ModStencilsCells.F90:
//               750-1416): cells sharing a vertex, ranked by the fraction of
//               shared vertices with Wirth's quicksort (ModSortSearch.F90:
//               898-990, unstable tie-breaking kept), the top 10x-minimum
//               kept and re-sorted by cell id (:2816-2909)
//   layers      grown by RFLU_AddCellLayer (RFLU_ModStencilsUtils.F90:
//               696-979) while the singular-value ratio test of
//               RFLU_InvertMatrixSVD.F90:150-190 finds the scaled offset
//               matrix rank deficient (4x4 Jacobi eigen solve of A^T A in
//               place of LAPACK dgesdd; only the rank decision is used)
//   moments     xyzMoms of RFLU_ModWeights.F90:1770-1894
#pragma once

#include <math.h>

#ifdef __CUDACC__
#define RFM_HD __host__ __device__
#else
#define RFM_HD
#endif

namespace rfm {

constexpr int kStencilMin = 4;   // RFLU_ComputeStencilSize(3,1,1) = 2*3*4/6
constexpr int kStencilMax = 40;  // 10x the minimum
constexpr int kLayersMax = 6;
constexpr int kMaxCand = 256;    // vertex-neighbour entries (with repeats) per cell

// Cell connectivity as the builders hold it: cv[8*c + a] = vertex a of cell c
// (0-based, nv[c] of them), v2c[v2cOff[v] .. v2cOff[v+1]) = cells of vertex v
// in ascending order, cofg[3*c + d] = centroid.
struct CellView {
  const double *cofg;
  const int *cv;
  const int *nv;
  const int *v2cOff;
  const int *v2c;
};

// Wirth's non-recursive quicksort of a[0..n) carrying b, restated from
// modfloflu/ModSortSearch.F90:898-990 with its 1-based index math shifted.
RFM_HD inline void quicksort_real_int(double *a, int *b, int n) {
  if (n <= 0) return;
  int stackl[50], stackr[50];
  int s = 1;
  stackl[0] = 1;
  stackr[0] = n;
  int l, r;
  do {
    l = stackl[s - 1];
    r = stackr[s - 1];
    s = s - 1;
    do {
      int i = l, j = r;
      int k = (l + r) / 2;
      double x = a[k - 1];
      for (;;) {
        while (a[i - 1] < x) i = i + 1;
        while (x < a[j - 1]) j = j - 1;
        if (i <= j) {
          double w = a[i - 1];
          a[i - 1] = a[j - 1];
          a[j - 1] = w;
          int v = b[i - 1];
          b[i - 1] = b[j - 1];
          b[j - 1] = v;
          i = i + 1;
          j = j - 1;
          if (i > j) break;
        } else {
          break;
        }
      }
      if (j - l >= r - i) {
        if (l < j) {
          s = s + 1;
          stackl[s - 1] = l;
          stackr[s - 1] = j;
        }
        l = i;
      } else {
        if (i < r) {
          s = s + 1;
          stackl[s - 1] = i;
          stackr[s - 1] = r;
        }
        r = j;
      }
    } while (l < r);
  } while (s != 0);
}

// ascending insertion sort of distinct-or-repeated ints
RFM_HD inline void sort_int(int *a, int n) {
  for (int i = 1; i < n; ++i) {
    const int x = a[i];
    int j = i - 1;
    while (j >= 0 && a[j] > x) {
      a[j + 1] = a[j];
      --j;
    }
    a[j + 1] = x;
  }
}

// first position in sorted a[0..n) whose value is not below x
RFM_HD inline int lower_bound_int(const int *a, int n, int x) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (a[mid] < x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

RFM_HD inline bool contains_int(const int *a, int n, int x) {
  const int p = lower_bound_int(a, n, x);
  return p < n && a[p] == x;
}

// Number of (near-)zero singular values by the ratio test of
// RFLU_InvertMatrixSVD.F90:150-190 for the column-scaled rows x 4 matrix A:
// singular values (descending) from the eigenvalues of A^T A by cyclic Jacobi.
RFM_HD inline int svd_scount(const double *A, int rows) {
  double g[4][4];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      double acc = 0.0;
      for (int r = 0; r < rows; ++r) acc += A[r * 4 + i] * A[r * 4 + j];
      g[i][j] = acc;
    }
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < 4; ++p)
      for (int q = p + 1; q < 4; ++q) off += g[p][q] * g[p][q];
    if (off < 1e-300) break;
    for (int p = 0; p < 4; ++p)
      for (int q = p + 1; q < 4; ++q) {
        if (g[p][q] == 0.0) continue;
        double theta = (g[q][q] - g[p][p]) / (2.0 * g[p][q]);
        double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
        for (int k = 0; k < 4; ++k) {
          double gkp = g[k][p], gkq = g[k][q];
          g[k][p] = c * gkp - sn * gkq;
          g[k][q] = sn * gkp + c * gkq;
        }
        for (int k = 0; k < 4; ++k) {
          double gpk = g[p][k], gqk = g[q][k];
          g[p][k] = c * gpk - sn * gqk;
          g[q][k] = sn * gpk + c * gqk;
        }
      }
  }
  double s[4];
  for (int i = 0; i < 4; ++i) s[i] = sqrt(g[i][i] > 0.0 ? g[i][i] : 0.0);
  for (int i = 1; i < 4; ++i) {  // descending
    const double x = s[i];
    int j = i - 1;
    while (j >= 0 && s[j] < x) {
      s[j + 1] = s[j];
      --j;
    }
    s[j + 1] = x;
  }
  const double eps = 2.220446049250313080847e-16;  // DBL_EPSILON
  int sCount = 0;
  if (!(s[0] > 100.0 * eps)) sCount = 1;
  for (int i = 1; i < 4; ++i) {
    if (s[i] > 0.01 * s[i - 1]) continue;
    sCount += 4 - i;
    break;
  }
  return sCount;
}

// Scratch of one cell's build.
struct Scratch {
  int tmp[kMaxCand];
  double frac[kMaxCand];
  int help[kStencilMax];
  int sorted[kStencilMax];
  double A[4 * kStencilMax];
};

// Stencil members of cell icg into c2cs[0..degr) (0-based ids) and its ten
// moments into mo; returns degr, or -1 when the cell has more than kMaxCand
// vertex-neighbour entries.
RFM_HD inline int cell_stencil(const CellView &m, int icg, int *c2cs, double *mo, Scratch &w) {
  const int nVert = m.nv[icg];
  const int *v = m.cv + 8 * (long long)icg;
  const double iNVert = 1.0 / (double)nVert;
  int nt = 0;
  for (int a = 0; a < nVert; ++a)
    for (int e = m.v2cOff[v[a]]; e < m.v2cOff[v[a] + 1]; ++e) {
      if (nt >= kMaxCand) return -1;
      w.tmp[nt++] = m.v2c[e];
    }
  sort_int(w.tmp, nt);
  int nu = 0;  // unique, without the cell itself
  for (int q = 0; q < nt; ++q)
    if ((nu == 0 || w.tmp[nu - 1] != w.tmp[q]) && w.tmp[q] != icg) w.tmp[nu++] = w.tmp[q];
  int vs[8];
  for (int a = 0; a < nVert; ++a) vs[a] = v[a];
  sort_int(vs, nVert);
  const int nC2 = nu;
  for (int q = 0; q < nC2; ++q) {
    const int c2 = w.tmp[q];
    const int n2 = m.nv[c2];
    int vs2[8];
    const int *v2 = m.cv + 8 * (long long)c2;
    for (int a = 0; a < n2; ++a) vs2[a] = v2[a];
    sort_int(vs2, n2);
    int common = 0, ia = 0, ib = 0;
    while (ia < nVert && ib < n2) {
      if (vs[ia] == vs2[ib]) {
        ++common;
        ++ia;
        ++ib;
      } else if (vs[ia] < vs2[ib]) {
        ++ia;
      } else {
        ++ib;
      }
    }
    w.frac[q] = (double)common * iNVert;
  }
  quicksort_real_int(w.frac, w.tmp, nC2);
  int degr = 0;
  const int qLo = nC2 - kStencilMax + 1 > 1 ? nC2 - kStencilMax + 1 : 1;
  for (int q = nC2; q >= qLo; --q) c2cs[degr++] = w.tmp[q - 1];
  sort_int(c2cs, degr);
  int layBeg = 0, layEnd = degr;  // previous layer [beg, end)
  const double *c0 = m.cofg + 3 * (long long)icg;
  for (int iLayer = 2; iLayer <= kLayersMax; ++iLayer) {
    int sCount = 0;
    if (degr >= kStencilMin) {
      for (int s = 0; s < degr; ++s) {
        const double *c1 = m.cofg + 3 * (long long)c2cs[s];
        double dx = c1[0] - c0[0], dy = c1[1] - c0[1], dz = c1[2] - c0[2];
        double term = 1.0 / sqrt(dx * dx + dy * dy + dz * dz);
        w.A[4 * s + 0] = term;
        w.A[4 * s + 1] = term * dx;
        w.A[4 * s + 2] = term * dy;
        w.A[4 * s + 3] = term * dz;
      }
      for (int col = 0; col < 4; ++col) {
        double cm = -1.7976931348623157e308;
        for (int s = 0; s < degr; ++s) {
          const double x = fabs(w.A[4 * s + col]);
          cm = cm < x ? x : cm;
        }
        for (int s = 0; s < degr; ++s) w.A[4 * s + col] = w.A[4 * s + col] / cm;
      }
      sCount = svd_scount(w.A, degr);
    }
    if (sCount != 0 || degr < kStencilMin) {
      // RFLU_AddCellLayer: cells sharing a vertex with the previous layer, not
      // yet members, ascending, until kStencilMax are collected
      for (int s = 0; s < degr; ++s) w.sorted[s] = c2cs[s];
      sort_int(w.sorted, degr);
      int nh = 0;
      bool full = false;
      for (int s = layBeg; s < layEnd && !full; ++s) {
        const int c1 = c2cs[s];
        const int *v1 = m.cv + 8 * (long long)c1;
        for (int a = 0; a < m.nv[c1] && !full; ++a)
          for (int e = m.v2cOff[v1[a]]; e < m.v2cOff[v1[a] + 1]; ++e) {
            const int c2 = m.v2c[e];
            if (c2 == icg) continue;
            if (contains_int(w.sorted, degr, c2)) continue;
            if (contains_int(w.help, nh, c2)) continue;
            if (nh < kStencilMax) {
              int p = nh;  // insert after equal keys (none: c2 is new)
              while (p > 0 && w.help[p - 1] > c2) {
                w.help[p] = w.help[p - 1];
                --p;
              }
              w.help[p] = c2;
              ++nh;
            } else {
              full = true;
              break;
            }
          }
      }
      const int newBeg = degr;
      for (int s = 0; s < nh; ++s)
        if (degr < kStencilMax) c2cs[degr++] = w.help[s];
      layBeg = newBeg;
      layEnd = degr;
    } else {
      break;
    }
  }
  // moments
  for (int k = 0; k < 10; ++k) mo[k] = 0.0;
  double s6[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int s = 0; s < degr; ++s) {
    const double *c1 = m.cofg + 3 * (long long)c2cs[s];
    double dx = c1[0] - c0[0], dy = c1[1] - c0[1], dz = c1[2] - c0[2];
    double wt = 1.0 / sqrt(dx * dx + dy * dy + dz * dz);
    dx = wt * dx;
    dy = wt * dy;
    dz = wt * dz;
    s6[0] = s6[0] + dx * dx;
    s6[1] = s6[1] + dx * dy;
    s6[2] = s6[2] + dy * dy;
    s6[3] = s6[3] + dx * dz;
    s6[4] = s6[4] + dy * dz;
    s6[5] = s6[5] + dz * dz;
    s6[6] = s6[6] + wt * dx;
    s6[7] = s6[7] + wt * dy;
    s6[8] = s6[8] + wt * dz;
    s6[9] = s6[9] + wt * wt;
  }
  double r11 = sqrt(s6[0]);
  double ir11 = 1.0 / r11;
  double r12 = ir11 * s6[1];
  double r22 = sqrt(s6[2] - r12 * r12);
  double ir22 = 1.0 / r22;
  double r13 = ir11 * s6[3];
  double r23 = ir22 * (s6[4] - r12 * r13);
  double r33 = sqrt(s6[5] - (r13 * r13 + r23 * r23));
  double ir33 = 1.0 / r33;
  double r14 = ir11 * s6[6];
  double r24 = ir22 * (s6[7] - r12 * r14);
  double r34 = ir33 * (s6[8] - (r13 * r14 + r23 * r24));
  double r44 = sqrt(s6[9] - (r14 * r14 + r24 * r24 + r34 * r34));
  mo[0] = r11;
  mo[1] = r12;
  mo[2] = r22;
  mo[3] = r13;
  mo[4] = r23;
  mo[5] = r33;
  mo[6] = r14;
  mo[7] = r24;
  mo[8] = r34;
  mo[9] = r44;
  return degr;
}

}  // namespace rfm
