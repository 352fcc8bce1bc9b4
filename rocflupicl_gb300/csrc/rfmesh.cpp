// rfmesh.cpp - host mesh builder for the residual engine (see include/rfmesh.h).
//
// Compiled with -ffp-contract=off so the geometry is bit-identical on every
// host (x86_64 here, aarch64 on the GPU nodes) and matches the unfused
// Fortran arithmetic it restates.
#include "rfmesh.h"
#include "rfmesh_geom.h"
#include "rfmesh_stencil.h"

#include <algorithm>
#include <array>
#include <map>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <new>
#include <random>
#include <stdexcept>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using rfm::T_TET;
using rfm::T_HEX;
using rfm::T_PRI;
using rfm::T_PYR;
const int kNV[4] = {4, 8, 6, 5};
const int kNF[4] = {4, 6, 5, 5};
// local faces, cyclic vertex order, -1 padded (tri faces); the table the
// device builder uses too
const int kFaces[4][6][4] = RFM_FACE_TABLE;

struct Patch {
  std::vector<int> bf2c;    // 0-based internally
  std::vector<int> bf2v;    // 4 per face
  std::vector<double> fn, fc;
  std::vector<int> bf2c1;   // 1-based export
};

}  // namespace

struct rfmesh_s {
  int kind = 0;
  double lo[3], hi[3];
  std::vector<double> xyz;
  // cells grouped by type; global numbering tets, hexes, prisms, pyramids
  std::vector<int> c2v[4];
  long long nOfType[4] = {0, 0, 0, 0};
  long long nCells = 0;
  std::vector<int> ctype, cloc;  // per global cell: type, local index
  std::vector<double> cofgApp, cofg, vol;
  std::vector<int> f2c;          // 2 per interior face, 0-based
  std::vector<int> f2v;          // 4 per interior face
  std::vector<double> fn, fc;
  std::vector<int> f2c1;         // 1-based export
  std::vector<Patch> patch = std::vector<Patch>(RFMESH_NPATCH);
  // grid meshes: boundary faces of patch ip, sorted-vertex keys in the grid
  // file's order (triangles, then quads), and the key -> (patch, position) map
  bool fromGrid = false;
  std::vector<std::vector<std::array<int, 4>>> gridPatchKeys;
  std::vector<int> v2cOff, v2c;
  std::vector<int> csOff, csMem, csMem1;
  std::vector<double> moms;
  int maxMembs = 0;
  std::vector<int> cv8, nv8;  // connectivity padded to 8 vertices, vertex counts
  bool skipStencils = false;  // stencils and moments come from rfmesh_set_stencils

  int nv(long long icg) const { return kNV[ctype[icg]]; }
  const int *verts(long long icg) const {
    int t = ctype[icg];
    return &c2v[t][(size_t)cloc[icg] * kNV[t]];
  }
};

namespace {

using rfm::face_vec_cen;  // FaceVector / FaceCentroid, shared with the device builder

inline uint64_t vid(int i, int j, int k, int nx, int ny) {
  return (uint64_t)i + (uint64_t)(nx + 1) * ((uint64_t)j + (uint64_t)(ny + 1) * (uint64_t)k);
}

// ---------------------------------------------------------------------------
// generators

struct Gen {
  int nx, ny, nz;
  std::vector<int> cells[4];  // vertex lists per type, in creation order
};

void add_cell(Gen &g, int t, const int *v) {
  for (int i = 0; i < kNV[t]; ++i) g.cells[t].push_back(v[i]);
}

void generate(rfmesh_s *m, int nx, int ny, int nz, double jitter, unsigned long long seed) {
  long long nvBase = (long long)(nx + 1) * (ny + 1) * (nz + 1);
  double h[3] = {(m->hi[0] - m->lo[0]) / nx, (m->hi[1] - m->lo[1]) / ny,
                 (m->hi[2] - m->lo[2]) / nz};
  m->xyz.resize(3 * (size_t)nvBase);
  std::mt19937_64 rng(seed);
  const double two53 = 1.0 / 9007199254740992.0;
  for (int k = 0; k <= nz; ++k)
    for (int j = 0; j <= ny; ++j)
      for (int i = 0; i <= nx; ++i) {
        uint64_t v = vid(i, j, k, nx, ny);
        double p[3] = {m->lo[0] + h[0] * i, m->lo[1] + h[1] * j, m->lo[2] + h[2] * k};
        if (i == nx) p[0] = m->hi[0];
        if (j == ny) p[1] = m->hi[1];
        if (k == nz) p[2] = m->hi[2];
        bool interior = i > 0 && i < nx && j > 0 && j < ny && k > 0 && k < nz;
        if (jitter > 0.0 && interior) {
          for (int d = 0; d < 3; ++d) {
            double u = (double)(rng() >> 11) * two53;  // [0,1)
            p[d] += (2.0 * u - 1.0) * jitter * h[d];
          }
        }
        m->xyz[3 * v + 0] = p[0];
        m->xyz[3 * v + 1] = p[1];
        m->xyz[3 * v + 2] = p[2];
      }
  Gen g;
  int midx = nx / 2, midz = nz / 2;
  static const int kuhn[6][4] = {{0, 1, 2, 6}, {0, 1, 5, 6}, {0, 3, 2, 6},
                                 {0, 3, 7, 6}, {0, 4, 5, 6}, {0, 4, 7, 6}};
  // hex faces (cyclic) and their Freudenthal diagonal split into two triangles
  static const int quadFace[6][4] = {{0, 3, 2, 1}, {4, 5, 6, 7}, {0, 1, 5, 4},
                                     {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}};
  static const int kuhnTri[6][2][3] = {{{0, 1, 2}, {0, 2, 3}}, {{4, 5, 6}, {4, 6, 7}},
                                       {{0, 1, 5}, {0, 5, 4}}, {{1, 2, 6}, {1, 6, 5}},
                                       {{3, 2, 6}, {3, 6, 7}}, {{0, 4, 7}, {0, 7, 3}}};
  auto region = [&](int i, int k) -> int {  // 0 hex, 1 prism, 2 tet (mixed mesh)
    if (m->kind == RFMESH_HEX) return 0;
    if (m->kind == RFMESH_TET) return 2;
    if (i >= midx) return 1;
    if (k >= midz) return 2;
    return 0;
  };
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        int cv[8] = {(int)vid(i, j, k, nx, ny),         (int)vid(i + 1, j, k, nx, ny),
                     (int)vid(i + 1, j + 1, k, nx, ny), (int)vid(i, j + 1, k, nx, ny),
                     (int)vid(i, j, k + 1, nx, ny),     (int)vid(i + 1, j, k + 1, nx, ny),
                     (int)vid(i + 1, j + 1, k + 1, nx, ny), (int)vid(i, j + 1, k + 1, nx, ny)};
        int reg = region(i, k);
        if (reg == 0) {
          add_cell(g, T_HEX, cv);
        } else if (reg == 1) {
          int p0[6] = {cv[0], cv[1], cv[2], cv[4], cv[5], cv[6]};
          int p1[6] = {cv[0], cv[2], cv[3], cv[4], cv[6], cv[7]};
          add_cell(g, T_PRI, p0);
          add_cell(g, T_PRI, p1);
        } else {
          // quad neighbours across the -z face (hex below) and +x face (prism)
          bool quad[6] = {false, false, false, false, false, false};
          if (m->kind == RFMESH_MIXED) {
            if (k - 1 >= 0 && region(i, k - 1) != 2) quad[0] = true;
            if (i + 1 < nx && region(i + 1, k) != 2) quad[3] = true;
          }
          bool transition = false;
          for (int f = 0; f < 6; ++f) transition |= quad[f];
          if (!transition) {
            for (int t = 0; t < 6; ++t) {
              int tv[4] = {cv[kuhn[t][0]], cv[kuhn[t][1]], cv[kuhn[t][2]], cv[kuhn[t][3]]};
              add_cell(g, T_TET, tv);
            }
          } else {
            // centroid vertex, then a pyramid on each quad face and two tets on
            // every other face (split along its Freudenthal diagonal)
            int c = (int)(m->xyz.size() / 3);
            double pc[3] = {0, 0, 0};
            for (int a = 0; a < 8; ++a)
              for (int d = 0; d < 3; ++d) pc[d] += m->xyz[3 * (size_t)cv[a] + d];
            for (int d = 0; d < 3; ++d) m->xyz.push_back(0.125 * pc[d]);
            for (int f = 0; f < 6; ++f) {
              if (quad[f]) {
                int pv[5] = {cv[quadFace[f][0]], cv[quadFace[f][1]], cv[quadFace[f][2]],
                             cv[quadFace[f][3]], c};
                add_cell(g, T_PYR, pv);
              } else {
                for (int s = 0; s < 2; ++s) {
                  int tv[4] = {cv[kuhnTri[f][s][0]], cv[kuhnTri[f][s][1]],
                               cv[kuhnTri[f][s][2]], c};
                  add_cell(g, T_TET, tv);
                }
              }
            }
          }
        }
      }
  for (int t = 0; t < 4; ++t) {
    m->nOfType[t] = (long long)(g.cells[t].size() / kNV[t]);
    m->c2v[t].swap(g.cells[t]);
  }
}

// ---------------------------------------------------------------------------

void set_stencils(rfmesh_s *m, const std::vector<int> &cnt, const std::vector<int> &memb);

// Global cell numbering (tets, hexes, prisms, pyramids) and the connectivity
// padded to 8 vertices that the stencil and device builders take.
void cells(rfmesh_s *m) {
  m->nCells = m->nOfType[0] + m->nOfType[1] + m->nOfType[2] + m->nOfType[3];
  const long long nC = m->nCells;
  m->ctype.resize(nC);
  m->cloc.resize(nC);
  {
    long long icg = 0;
    for (int t = 0; t < 4; ++t)
      for (long long l = 0; l < m->nOfType[t]; ++l, ++icg) {
        m->ctype[icg] = t;
        m->cloc[icg] = (int)l;
      }
  }
  m->cv8.assign(8 * (size_t)nC, -1);
  m->nv8.resize(nC);
  for (long long c = 0; c < nC; ++c) {
    m->nv8[c] = m->nv(c);
    const int *v = m->verts(c);
    for (int a = 0; a < m->nv(c); ++a) m->cv8[8 * (size_t)c + a] = v[a];
  }
}

void build(rfmesh_s *m, int nThreads) {
  (void)nThreads;
  cells(m);
  const long long nC = m->nCells;
  const long long nV = (long long)(m->xyz.size() / 3);
  // approximate centroids: vertex averages (RFLU_ModGeometry.F90:1277-1460)
  m->cofgApp.assign(3 * (size_t)nC, 0.0);
  for (long long icg = 0; icg < nC; ++icg) {
    int n = m->nv(icg);
    const int *v = m->verts(icg);
    double term = 1.0 / (double)n;
    for (int d = 0; d < 3; ++d) {
      double s = 0.0;
      for (int a = 0; a < n; ++a) s = s + m->xyz[3 * (size_t)v[a] + d];
      m->cofgApp[3 * icg + d] = term * s;
    }
  }
  // face list: first encounter sweeping cells in global order; faces keyed by
  // their sorted vertex set, chained on the smallest vertex id
  std::vector<int> fvAll;    // 4 per face
  std::vector<int> fc1, fc2;
  std::vector<int64_t> head(nV, -1), next;
  std::vector<int> keyAll;   // sorted key, 4 per face
  fvAll.reserve(4 * (size_t)nC * 3);
  for (long long icg = 0; icg < nC; ++icg) {
    int t = m->ctype[icg];
    const int *v = m->verts(icg);
    for (int f = 0; f < kNF[t]; ++f) {
      int fv[4];
      for (int a = 0; a < 4; ++a) fv[a] = kFaces[t][f][a] < 0 ? -1 : v[kFaces[t][f][a]];
      int key[4] = {fv[0], fv[1], fv[2], fv[3]};
      int nk = key[3] < 0 ? 3 : 4;
      std::sort(key, key + nk);
      if (nk == 3) key[3] = -1;
      int64_t hit = -1;
      for (int64_t e = head[key[0]]; e >= 0; e = next[e]) {
        const int *k2 = &keyAll[4 * e];
        if (k2[1] == key[1] && k2[2] == key[2] && k2[3] == key[3]) {
          hit = e;
          break;
        }
      }
      if (hit >= 0) {
        fc2[hit] = (int)icg;
      } else {
        int64_t e = (int64_t)fc1.size();
        fc1.push_back((int)icg);
        fc2.push_back(-1);
        for (int a = 0; a < 4; ++a) {
          fvAll.push_back(fv[a]);
          keyAll.push_back(key[a]);
        }
        next.push_back(head[key[0]]);
        head[key[0]] = e;
      }
    }
  }
  std::vector<int64_t>().swap(head);
  std::vector<int64_t>().swap(next);
  std::vector<int>().swap(keyAll);
  const int64_t nAll = (int64_t)fc1.size();
  // grid meshes: boundary face key -> (patch, position in the patch's file list)
  std::map<std::array<int, 4>, std::pair<int, int>> gridKey;
  std::vector<std::vector<std::pair<int, int64_t>>> gridSlot;  // per patch: (position, face)
  if (m->fromGrid) {
    gridSlot.resize(m->patch.size());
    for (size_t ip = 0; ip < m->gridPatchKeys.size(); ++ip)
      for (size_t q = 0; q < m->gridPatchKeys[ip].size(); ++q)
        gridKey[m->gridPatchKeys[ip][q]] = {(int)ip, (int)q};
  }
  // orient every face outward from its first cell, then split interior/boundary
  const double tolx = 1e-9 * (m->hi[0] - m->lo[0]), toly = 1e-9 * (m->hi[1] - m->lo[1]),
               tolz = 1e-9 * (m->hi[2] - m->lo[2]);
  for (int64_t e = 0; e < nAll; ++e) {
    int *fv = &fvAll[4 * e];
    double S[3], C[3];
    face_vec_cen(m->xyz.data(), fv, S, C);
    const double *ca = &m->cofgApp[3 * (size_t)fc1[e]];
    double dot = (C[0] - ca[0]) * S[0] + (C[1] - ca[1]) * S[1] + (C[2] - ca[2]) * S[2];
    if (dot < 0.0) {
      if (fv[3] < 0)
        std::swap(fv[1], fv[2]);
      else
        std::swap(fv[1], fv[3]);
    }
    if (fc2[e] >= 0) {
      m->f2c.push_back(fc1[e]);
      m->f2c.push_back(fc2[e]);
      for (int a = 0; a < 4; ++a) m->f2v.push_back(fv[a]);
    } else if (m->fromGrid) {
      std::array<int, 4> key{fv[0], fv[1], fv[2], fv[3]};
      const int nk = key[3] < 0 ? 3 : 4;
      std::sort(key.begin(), key.begin() + nk);
      auto it = gridKey.find(key);
      if (it == gridKey.end()) throw std::runtime_error("boundary face in no patch");
      gridSlot[it->second.first].push_back({it->second.second, e});
    } else {
      int ip = -1;
      if (std::fabs(C[0] - m->lo[0]) < tolx) ip = RFMESH_XLO;
      else if (std::fabs(C[0] - m->hi[0]) < tolx) ip = RFMESH_XHI;
      else if (std::fabs(C[1] - m->lo[1]) < toly) ip = RFMESH_YLO;
      else if (std::fabs(C[1] - m->hi[1]) < toly) ip = RFMESH_YHI;
      else if (std::fabs(C[2] - m->lo[2]) < tolz) ip = RFMESH_ZLO;
      else if (std::fabs(C[2] - m->hi[2]) < tolz) ip = RFMESH_ZHI;
      if (ip < 0) throw std::runtime_error("boundary face off the box surface");
      m->patch[ip].bf2c.push_back(fc1[e]);
      for (int a = 0; a < 4; ++a) m->patch[ip].bf2v.push_back(fv[a]);
    }
  }
  if (m->fromGrid) {  // patch faces in the grid file's order
    for (size_t ip = 0; ip < gridSlot.size(); ++ip) {
      std::sort(gridSlot[ip].begin(), gridSlot[ip].end());
      if (gridSlot[ip].size() != m->gridPatchKeys[ip].size())
        throw std::runtime_error("patch face that bounds no cell");
      for (auto &sf : gridSlot[ip]) {
        m->patch[ip].bf2c.push_back(fc1[sf.second]);
        for (int a = 0; a < 4; ++a) m->patch[ip].bf2v.push_back(fvAll[4 * sf.second + a]);
      }
    }
  }
  const int64_t nF = (int64_t)(m->f2c.size() / 2);
  // geometry (RFLU_ModGeometry.F90:307-672)
  m->vol.assign(nC, 0.0);
  m->cofg.assign(3 * (size_t)nC, 0.0);
  m->fn.resize(4 * (size_t)nF);
  m->fc.resize(3 * (size_t)nF);
  auto contrib = [&](int c, const double S[3], const double C[3], double sgn) {
    rfm::face_contrib(S, C, &m->cofgApp[3 * (size_t)c], sgn, &m->vol[c], &m->cofg[3 * (size_t)c]);
  };
  for (int64_t f = 0; f < nF; ++f) {
    double S[3], C[3];
    face_vec_cen(m->xyz.data(), &m->f2v[4 * f], S, C);
    double fVecM = std::sqrt(S[0] * S[0] + S[1] * S[1] + S[2] * S[2]);
    double term = 1.0 / fVecM;
    m->fn[4 * f + 0] = S[0] * term;
    m->fn[4 * f + 1] = S[1] * term;
    m->fn[4 * f + 2] = S[2] * term;
    m->fn[4 * f + 3] = fVecM;
    m->fc[3 * f + 0] = C[0];
    m->fc[3 * f + 1] = C[1];
    m->fc[3 * f + 2] = C[2];
    contrib(m->f2c[2 * f], S, C, 1.0);
    contrib(m->f2c[2 * f + 1], S, C, -1.0);
  }
  for (int ip = 0; ip < (int)m->patch.size(); ++ip) {
    Patch &p = m->patch[ip];
    size_t nb = p.bf2c.size();
    p.fn.resize(4 * nb);
    p.fc.resize(3 * nb);
    for (size_t f = 0; f < nb; ++f) {
      double S[3], C[3];
      face_vec_cen(m->xyz.data(), &p.bf2v[4 * f], S, C);
      double fVecM = std::sqrt(S[0] * S[0] + S[1] * S[1] + S[2] * S[2]);
      double term = 1.0 / fVecM;
      p.fn[4 * f + 0] = S[0] * term;
      p.fn[4 * f + 1] = S[1] * term;
      p.fn[4 * f + 2] = S[2] * term;
      p.fn[4 * f + 3] = fVecM;
      p.fc[3 * f + 0] = C[0];
      p.fc[3 * f + 1] = C[1];
      p.fc[3 * f + 2] = C[2];
      contrib(p.bf2c[f], S, C, 1.0);
    }
  }
  const double THRD = 1.0 / 3.0;
  for (long long c = 0; c < nC; ++c) {
    m->vol[c] = THRD * m->vol[c];
    if (!(m->vol[c] > 0.0)) throw std::runtime_error("non-positive cell volume");
    double term = 1.0 / (4.0 * m->vol[c]);
    for (int d = 0; d < 3; ++d) m->cofg[3 * c + d] = term * m->cofg[3 * c + d];
  }
  // vertex-to-cell lists, ascending cell id
  m->v2cOff.assign(nV + 1, 0);
  for (long long c = 0; c < nC; ++c) {
    const int *v = m->verts(c);
    for (int a = 0; a < m->nv(c); ++a) m->v2cOff[v[a] + 1]++;
  }
  for (long long v = 0; v < nV; ++v) m->v2cOff[v + 1] += m->v2cOff[v];
  m->v2c.resize(m->v2cOff[nV]);
  {
    std::vector<int> fill(m->v2cOff.begin(), m->v2cOff.end() - 1);
    for (long long c = 0; c < nC; ++c) {
      const int *v = m->verts(c);
      for (int a = 0; a < m->nv(c); ++a) m->v2c[fill[v[a]]++] = (int)c;
    }
  }
  // 1-based exports
  m->f2c1.resize(m->f2c.size());
  for (size_t i = 0; i < m->f2c.size(); ++i) m->f2c1[i] = m->f2c[i] + 1;
  for (int ip = 0; ip < (int)m->patch.size(); ++ip) {
    Patch &p = m->patch[ip];
    p.bf2c1.resize(p.bf2c.size());
    for (size_t i = 0; i < p.bf2c.size(); ++i) p.bf2c1[i] = p.bf2c[i] + 1;
  }
  // c2c stencils (RFLU_ModStencilsCells.F90:750-1416) and moments
  // (RFLU_ModWeights.F90:1770-1894): the per-cell routine shared with the
  // device builder (rfmesh_stencil.h)
  if (m->skipStencils) return;
  const rfm::CellView view{m->cofg.data(), m->cv8.data(), m->nv8.data(), m->v2cOff.data(),
                           m->v2c.data()};
  std::vector<int> cnt(nC, 0);
  std::vector<int> memb((size_t)nC * rfm::kStencilMax);
  m->moms.assign(10 * (size_t)nC, 0.0);
  int overflow = 0;
#pragma omp parallel reduction(| : overflow)
  {
    rfm::Scratch w;
#pragma omp for schedule(dynamic, 1024)
    for (long long icg = 0; icg < nC; ++icg) {
      const int degr = rfm::cell_stencil(view, (int)icg, &memb[(size_t)icg * rfm::kStencilMax],
                                         &m->moms[10 * (size_t)icg], w);
      if (degr < 0) overflow = 1;
      cnt[icg] = degr < 0 ? 0 : degr;
    }
  }
  if (overflow) throw std::runtime_error("vertex-neighbour list longer than the stencil builder holds");
  set_stencils(m, cnt, memb);
}

// CSR stencils (1-based members) and the maximum size from per-cell lists of
// kStencilMax slots.
void set_stencils(rfmesh_s *m, const std::vector<int> &cnt, const std::vector<int> &memb) {
  const long long nC = m->nCells;
  m->csOff.assign(nC + 1, 0);
  for (long long c = 0; c < nC; ++c) {
    m->csOff[c + 1] = m->csOff[c] + cnt[c];
    m->maxMembs = std::max(m->maxMembs, cnt[c]);
  }
  m->csMem1.resize(m->csOff[nC]);
  for (long long c = 0; c < nC; ++c)
    for (int s = 0; s < cnt[c]; ++s)
      m->csMem1[m->csOff[c] + s] = memb[(size_t)c * rfm::kStencilMax + s] + 1;
}

}  // namespace

extern "C" {

int rfmesh_create_box(int kind, int nx, int ny, int nz, const double lo[3], const double hi[3],
                      double jitter, unsigned long long seed, int nThreads, rfmesh_t *out) {
  return rfmesh_create_box_ex(kind, nx, ny, nz, lo, hi, jitter, seed, nThreads, 0, out);
}

int rfmesh_create_box_ex(int kind, int nx, int ny, int nz, const double lo[3], const double hi[3],
                         double jitter, unsigned long long seed, int nThreads, int flags,
                         rfmesh_t *out) {
  if (!out || !lo || !hi || nx < 1 || ny < 1 || nz < 1 || kind < 0 || kind > 2 || jitter < 0 ||
      jitter >= 0.25)
    return RFMESH_ERR_ARG;
  *out = nullptr;
  rfmesh_s *m = new (std::nothrow) rfmesh_s();
  if (!m) return RFMESH_ERR_NOMEM;
  m->kind = kind;
  m->skipStencils = (flags & RFMESH_DEFER_STENCILS) != 0;
  for (int d = 0; d < 3; ++d) {
    m->lo[d] = lo[d];
    m->hi[d] = hi[d];
  }
#ifdef _OPENMP
  int saved = omp_get_max_threads();
  if (nThreads > 0) omp_set_num_threads(nThreads);
#endif
  int rc = RFMESH_OK;
  try {
    generate(m, nx, ny, nz, jitter, seed);
    if (flags & RFMESH_CELLS_ONLY)
      cells(m);
    else
      build(m, nThreads);
  } catch (const std::bad_alloc &) {
    rc = RFMESH_ERR_NOMEM;
  } catch (...) {
    rc = RFMESH_ERR_GEOM;
  }
#ifdef _OPENMP
  omp_set_num_threads(saved);
#endif
  if (rc != RFMESH_OK) {
    delete m;
    return rc;
  }
  *out = m;
  return RFMESH_OK;
}

int rfmesh_create_grid(int nVert, const double *xyz, int nTets, const int *tet2v, int nHexs,
                       const int *hex2v, int nPris, const int *pri2v, int nPyrs,
                       const int *pyr2v, int nPatches, const int *nBTris,
                       const int *const *bTri2v, const int *nBQuads,
                       const int *const *bQuad2v, int nThreads, int flags, rfmesh_t *out) {
  if (!out || nVert <= 0 || !xyz || nTets < 0 || nHexs < 0 || nPris < 0 || nPyrs < 0 ||
      nPatches < 0 || (nPatches > 0 && (!nBTris || !nBQuads || !bTri2v || !bQuad2v)))
    return RFMESH_ERR_ARG;
  const int nCt[4] = {nTets, nHexs, nPris, nPyrs};
  const int *c2v[4] = {tet2v, hex2v, pri2v, pyr2v};
  for (int t = 0; t < 4; ++t) {
    if (nCt[t] > 0 && !c2v[t]) return RFMESH_ERR_ARG;
    for (long long i = 0; i < (long long)nCt[t] * kNV[t]; ++i)
      if (c2v[t][i] < 1 || c2v[t][i] > nVert) return RFMESH_ERR_ARG;
  }
  if ((long long)nTets + nHexs + nPris + nPyrs <= 0) return RFMESH_ERR_ARG;
  for (int ip = 0; ip < nPatches; ++ip) {
    if (nBTris[ip] < 0 || nBQuads[ip] < 0 || (nBTris[ip] > 0 && !bTri2v[ip]) ||
        (nBQuads[ip] > 0 && !bQuad2v[ip]))
      return RFMESH_ERR_ARG;
    for (long long i = 0; i < 3LL * nBTris[ip]; ++i)
      if (bTri2v[ip][i] < 1 || bTri2v[ip][i] > nVert) return RFMESH_ERR_ARG;
    for (long long i = 0; i < 4LL * nBQuads[ip]; ++i)
      if (bQuad2v[ip][i] < 1 || bQuad2v[ip][i] > nVert) return RFMESH_ERR_ARG;
  }
  *out = nullptr;
  rfmesh_s *m = new (std::nothrow) rfmesh_s();
  if (!m) return RFMESH_ERR_NOMEM;
  int rc = RFMESH_OK;
#ifdef _OPENMP
  int saved = omp_get_max_threads();
  if (nThreads > 0) omp_set_num_threads(nThreads);
#endif
  try {
    m->kind = RFMESH_GRID;
    m->fromGrid = true;
    m->skipStencils = (flags & RFMESH_DEFER_STENCILS) != 0;
    m->xyz.assign(xyz, xyz + 3 * (size_t)nVert);
    for (int d = 0; d < 3; ++d) {
      m->lo[d] = m->hi[d] = xyz[d];
      for (int v = 0; v < nVert; ++v) {
        m->lo[d] = std::min(m->lo[d], xyz[3 * (size_t)v + d]);
        m->hi[d] = std::max(m->hi[d], xyz[3 * (size_t)v + d]);
      }
    }
    for (int t = 0; t < 4; ++t) {
      m->nOfType[t] = nCt[t];
      m->c2v[t].resize((size_t)nCt[t] * kNV[t]);
      for (size_t i = 0; i < m->c2v[t].size(); ++i) m->c2v[t][i] = c2v[t][i] - 1;
    }
    m->patch.assign(nPatches, Patch());
    m->gridPatchKeys.resize(nPatches);
    for (int ip = 0; ip < nPatches; ++ip) {
      for (int q = 0; q < nBTris[ip]; ++q) {
        std::array<int, 4> k{bTri2v[ip][3 * q] - 1, bTri2v[ip][3 * q + 1] - 1,
                             bTri2v[ip][3 * q + 2] - 1, -1};
        std::sort(k.begin(), k.begin() + 3);
        m->gridPatchKeys[ip].push_back(k);
      }
      for (int q = 0; q < nBQuads[ip]; ++q) {
        std::array<int, 4> k{bQuad2v[ip][4 * q] - 1, bQuad2v[ip][4 * q + 1] - 1,
                             bQuad2v[ip][4 * q + 2] - 1, bQuad2v[ip][4 * q + 3] - 1};
        std::sort(k.begin(), k.end());
        m->gridPatchKeys[ip].push_back(k);
      }
    }
    build(m, nThreads);
  } catch (const std::bad_alloc &) {
    rc = RFMESH_ERR_NOMEM;
  } catch (...) {
    rc = RFMESH_ERR_GEOM;
  }
#ifdef _OPENMP
  omp_set_num_threads(saved);
#endif
  if (rc != RFMESH_OK) {
    delete m;
    return rc;
  }
  *out = m;
  return RFMESH_OK;
}

const int *rfmesh_bf2v(rfmesh_t m, int ip) {
  return (m && ip >= 0 && ip < (int)m->patch.size()) ? m->patch[ip].bf2v.data() : nullptr;
}

const int *rfmesh_cell_conn(rfmesh_t m, int type) {
  return (m && type >= 0 && type < 4) ? m->c2v[type].data() : nullptr;
}

int rfmesh_destroy(rfmesh_t m) {
  delete m;
  return RFMESH_OK;
}

int rfmesh_sizes(rfmesh_t m, long long s[RFMESH_NSIZES]) {
  if (!m || !s) return RFMESH_ERR_ARG;
  s[RFMESH_NVERT] = (long long)(m->xyz.size() / 3);
  s[RFMESH_NCELLS] = m->nCells;
  s[RFMESH_NFACES] = (long long)(m->f2c.size() / 2);
  s[RFMESH_NPATCHES] = (long long)m->patch.size();
  s[RFMESH_NMEMBS] = (long long)m->csMem1.size();
  for (int t = 0; t < 4; ++t) s[RFMESH_NTETS + t] = m->nOfType[t];
  long long nb = 0;
  for (int ip = 0; ip < (int)m->patch.size(); ++ip) nb += (long long)m->patch[ip].bf2c.size();
  s[RFMESH_NBFACES] = nb;
  s[RFMESH_MAXMEMBS] = m->maxMembs;
  return RFMESH_OK;
}

int rfmesh_patch_nbfaces(rfmesh_t m, int ip) {
  if (!m || ip < 0 || ip >= (int)m->patch.size()) return -1;
  return (int)m->patch[ip].bf2c.size();
}

const double *rfmesh_xyz(rfmesh_t m) { return m ? m->xyz.data() : nullptr; }
const double *rfmesh_vol(rfmesh_t m) { return m ? m->vol.data() : nullptr; }
const double *rfmesh_cofg(rfmesh_t m) { return m ? m->cofg.data() : nullptr; }
const int *rfmesh_f2c(rfmesh_t m) { return m ? m->f2c1.data() : nullptr; }
const double *rfmesh_fn(rfmesh_t m) { return m ? m->fn.data() : nullptr; }
const double *rfmesh_fc(rfmesh_t m) { return m ? m->fc.data() : nullptr; }
const int *rfmesh_c2cs_offsets(rfmesh_t m) { return m ? m->csOff.data() : nullptr; }
const int *rfmesh_c2cs_members(rfmesh_t m) { return m ? m->csMem1.data() : nullptr; }
const double *rfmesh_xyzmoms(rfmesh_t m) { return m ? m->moms.data() : nullptr; }
const int *rfmesh_cell_type(rfmesh_t m) { return m ? m->ctype.data() : nullptr; }
const int *rfmesh_cell_verts(rfmesh_t m) { return m ? m->cv8.data() : nullptr; }
const int *rfmesh_cell_nverts(rfmesh_t m) { return m ? m->nv8.data() : nullptr; }
const int *rfmesh_v2c_offsets(rfmesh_t m) { return m ? m->v2cOff.data() : nullptr; }
const int *rfmesh_v2c(rfmesh_t m) { return m ? m->v2c.data() : nullptr; }
const double *rfmesh_cofg_view(rfmesh_t m) { return m ? m->cofg.data() : nullptr; }

int rfmesh_set_stencils(rfmesh_t m, const int *offsets, const int *members, const double *moms) {
  if (!m || !offsets || !members || !moms) return RFMESH_ERR_ARG;
  const long long nC = m->nCells;
  if (offsets[0] != 0) return RFMESH_ERR_ARG;
  for (long long c = 0; c < nC; ++c) {
    const int k = offsets[c + 1] - offsets[c];
    if (k < 0 || k > rfm::kStencilMax) return RFMESH_ERR_ARG;
  }
  try {
    std::vector<int> cnt(nC), memb((size_t)nC * rfm::kStencilMax, 0);
    for (long long c = 0; c < nC; ++c) {
      cnt[c] = offsets[c + 1] - offsets[c];
      for (int s = 0; s < cnt[c]; ++s) {
        const int x = members[offsets[c] + s];
        if (x < 1 || x > nC) return RFMESH_ERR_ARG;
        memb[(size_t)c * rfm::kStencilMax + s] = x - 1;
      }
    }
    m->maxMembs = 0;
    set_stencils(m, cnt, memb);
    m->moms.assign(moms, moms + 10 * (size_t)nC);
  } catch (const std::bad_alloc &) {
    return RFMESH_ERR_NOMEM;
  }
  m->skipStencils = false;
  return RFMESH_OK;
}

int rfmesh_build_stencils(int nCells, int nVerts, const int *cellVerts, const int *cellNVerts,
                          const int *v2cOffsets, const int *v2c, const double *cofg, int nThreads,
                          int *c2csOffsets, int *c2csMembers, double *xyzMoms) {
  if (nCells <= 0 || nVerts <= 0 || !cellVerts || !cellNVerts || !v2cOffsets || !v2c || !cofg ||
      !c2csOffsets || !c2csMembers || !xyzMoms)
    return RFMESH_ERR_ARG;
  for (long long c = 0; c < nCells; ++c) {
    if (cellNVerts[c] < 4 || cellNVerts[c] > 8) return RFMESH_ERR_ARG;
    for (int a = 0; a < cellNVerts[c]; ++a)
      if (cellVerts[8 * c + a] < 0 || cellVerts[8 * c + a] >= nVerts) return RFMESH_ERR_ARG;
  }
  if (v2cOffsets[0] != 0) return RFMESH_ERR_ARG;
  for (long long v = 0; v < nVerts; ++v)
    if (v2cOffsets[v + 1] < v2cOffsets[v]) return RFMESH_ERR_ARG;
  for (long long e = 0; e < v2cOffsets[nVerts]; ++e)
    if (v2c[e] < 0 || v2c[e] >= nCells) return RFMESH_ERR_ARG;
  const rfm::CellView view{cofg, cellVerts, cellNVerts, v2cOffsets, v2c};
  std::vector<int> cnt(nCells, 0), memb((size_t)nCells * rfm::kStencilMax);
  int overflow = 0;
  int saved = omp_get_max_threads();
  if (nThreads > 0) omp_set_num_threads(nThreads);
#pragma omp parallel reduction(| : overflow)
  {
    rfm::Scratch w;
#pragma omp for schedule(dynamic, 1024)
    for (long long icg = 0; icg < nCells; ++icg) {
      const int degr = rfm::cell_stencil(view, (int)icg, &memb[(size_t)icg * rfm::kStencilMax],
                                         &xyzMoms[10 * (size_t)icg], w);
      if (degr < 0) overflow = 1;
      cnt[icg] = degr < 0 ? 0 : degr;
    }
  }
  omp_set_num_threads(saved);
  if (overflow) return RFMESH_ERR_GEOM;
  c2csOffsets[0] = 0;
  for (long long c = 0; c < nCells; ++c) {
    c2csOffsets[c + 1] = c2csOffsets[c] + cnt[c];
    for (int k = 0; k < cnt[c]; ++k)
      c2csMembers[c2csOffsets[c] + k] = memb[(size_t)c * rfm::kStencilMax + k] + 1;
  }
  return RFMESH_OK;
}

const int *rfmesh_bf2c(rfmesh_t m, int ip) {
  return (m && ip >= 0 && ip < (int)m->patch.size()) ? m->patch[ip].bf2c1.data() : nullptr;
}
const double *rfmesh_bfn(rfmesh_t m, int ip) {
  return (m && ip >= 0 && ip < (int)m->patch.size()) ? m->patch[ip].fn.data() : nullptr;
}
const double *rfmesh_bfc(rfmesh_t m, int ip) {
  return (m && ip >= 0 && ip < (int)m->patch.size()) ? m->patch[ip].fc.data() : nullptr;
}

}  // extern "C"
