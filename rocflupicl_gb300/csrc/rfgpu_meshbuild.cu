// rfgpu_meshbuild.cu - device-side mesh preprocessing (include/rfgpu.h,
// rfgpu_mesh_build): the face list, face and cell geometry, vertex-to-cell
// lists, c2c stencils and WLSQ moments of a mesh given by its vertices and
// cells, the same arrays the host builder of rfmesh.cpp makes, bit for bit.
//
// The host builder numbers faces by first encounter while sweeping the cells
// in order (cell c, local face f), orients each face outward from the cell
// that met it first, splits interior faces from boundary faces (box meshes:
// the patch is the box plane the face centroid lies on) and sums the
// divergence-theorem terms face by face (interior faces ascending, then the
// patches in order).  Here:
//   1. every (cell, local face) slot gets its sorted vertex key; a stable
//      two-pass radix sort by key keeps equal keys in slot order, so the
//      first slot of each run is the face's first encounter;
//   2. faces are ranked by that first slot (the host's face order), oriented
//      and classified (interior / patch) one thread per face;
//   3. a stable sort by class gives interior faces, then each patch's faces,
//      each in face order: the host's arrays;
//   4. face geometry one thread per face, cell volumes and centroids one
//      thread per cell, adding its faces in the host's order;
//   5. vertex-to-cell lists by a stable sort of (vertex, cell) pairs, then the
//      stencil kernel of rfmesh_stencil.h.
// Compiled without FMA contraction, as the host builder (-ffp-contract=off).
// References: RFLU_BuildFaceList (modflu/RFLU_ModFaceList.F90:784-1609),
// RFLU_BuildGeometry (modflu/RFLU_ModGeometry.F90:307-672, approximate
// centroids :1277-1460), FaceVector / FaceCentroid (libfloflu/FaceVector.F90:
// 79-136, FaceCentroid.F90:77-122), RFLU_BuildVertCellsList and the c2c
// stencils (modflu/RFLU_ModStencilsCells.F90:750-1416).
#include "rfgpu.h"
#include "rfgpu_internal.h"
#include "rfmesh_geom.h"

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <new>
#include <stdexcept>
#include <vector>

namespace {

constexpr int kSlots = 6;  // local faces per cell (at most)
enum { MB_NONMANIFOLD = 1, MB_OFFBOX = 2, MB_VOLUME = 4 };

// 1: approximate centroids, vertex averages (RFLU_ModGeometry.F90:1277-1460)
__global__ void k_cofg_app(const double *__restrict__ xyz, const int *__restrict__ cv8,
                           const int *__restrict__ nv8, int nC, double *__restrict__ ca) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nC) return;
  const int n = nv8[c];
  const double term = 1.0 / (double)n;
  for (int d = 0; d < 3; ++d) {
    double s = 0.0;
    for (int a = 0; a < n; ++a) s = s + xyz[3 * (size_t)cv8[8 * (size_t)c + a] + d];
    ca[3 * (size_t)c + d] = term * s;
  }
}

__device__ __forceinline__ void slot_face(const int *cv8, int c, int t, int f, int fv[4]) {
  for (int a = 0; a < 4; ++a) {
    const int l = rfm::face_local(t, f, a);
    fv[a] = l < 0 ? -1 : cv8[8 * (size_t)c + l];
  }
}

// sorted-vertex key of slot s = 6c + f as two 64-bit halves; unused slots
// get the largest key and sort last
__global__ void k_slot_keys(const int *__restrict__ cv8, const int *__restrict__ ctype, int nC,
                            unsigned long long *__restrict__ hi, unsigned long long *__restrict__ lo,
                            int *__restrict__ idx) {
  const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= (long long)nC * kSlots) return;
  const int c = (int)(s / kSlots), f = (int)(s % kSlots), t = ctype[c];
  idx[s] = (int)s;
  if (f >= rfm::cell_nf(t)) {
    hi[s] = lo[s] = ~0ull;
    return;
  }
  int k[4];
  slot_face(cv8, c, t, f, k);
  const int nk = k[3] < 0 ? 3 : 4;
  for (int i = 1; i < nk; ++i) {  // insertion sort of 3 or 4 ids
    const int x = k[i];
    int j = i - 1;
    while (j >= 0 && k[j] > x) {
      k[j + 1] = k[j];
      --j;
    }
    k[j + 1] = x;
  }
  if (nk == 3) k[3] = -1;
  hi[s] = ((unsigned long long)(unsigned)k[0] << 32) | (unsigned)k[1];
  lo[s] = ((unsigned long long)(unsigned)k[2] << 32) | (unsigned)(k[3] + 1);
}

__global__ void k_gather_u64(const unsigned long long *__restrict__ src, const int *__restrict__ idx,
                             long long n, unsigned long long *__restrict__ dst) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[idx[i]];
}

// 1 at the first slot of each run of equal keys among the valid slots
__global__ void k_heads(const unsigned long long *__restrict__ hi,
                        const unsigned long long *__restrict__ lo, const int *__restrict__ slot,
                        long long nValid, int *__restrict__ head, int *__restrict__ err) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nValid) return;
  const int s = slot[i];
  const unsigned long long h = hi[s], l = lo[s];
  const bool first = i == 0 || hi[slot[i - 1]] != h || lo[slot[i - 1]] != l;
  head[i] = first ? 1 : 0;
  if (first && i + 2 < nValid && hi[slot[i + 2]] == h && lo[slot[i + 2]] == l)
    atomicOr(err, MB_NONMANIFOLD);  // three cells on one face
}

// faces (runs): first slot (the first encounter) and second slot or -1
__global__ void k_runs(const unsigned long long *__restrict__ hi,
                       const unsigned long long *__restrict__ lo, const int *__restrict__ slot,
                       const int *__restrict__ head, const int *__restrict__ pos, long long nValid,
                       unsigned *__restrict__ first, int *__restrict__ second,
                       int *__restrict__ runId) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nValid || !head[i]) return;
  const int g = pos[i];
  const int s = slot[i];
  first[g] = (unsigned)s;
  runId[g] = g;
  int s2 = -1;
  if (i + 1 < nValid && hi[slot[i + 1]] == hi[s] && lo[slot[i + 1]] == lo[s]) s2 = slot[i + 1];
  second[g] = s2;
}

// face e (in first-encounter order): oriented vertices, class (0 interior,
// 1 + patch of a box boundary face)
__global__ void k_orient(const double *__restrict__ xyz, const int *__restrict__ cv8,
                         const int *__restrict__ ctype, const double *__restrict__ ca,
                         const unsigned *__restrict__ first, const int *__restrict__ second,
                         const int *__restrict__ order, int nAll, const double *lohi,
                         int *__restrict__ fv4, int *__restrict__ cls, int *__restrict__ c1,
                         int *__restrict__ c2, int *__restrict__ err) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nAll) return;
  const int g = order[e];
  const int s = (int)first[g];
  const int c = s / kSlots, f = s % kSlots;
  int fv[4];
  slot_face(cv8, c, ctype[c], f, fv);
  double S[3], C[3];
  rfm::face_vec_cen(xyz, fv, S, C);
  const double *cc = ca + 3 * (size_t)c;
  const double dot = (C[0] - cc[0]) * S[0] + (C[1] - cc[1]) * S[1] + (C[2] - cc[2]) * S[2];
  if (dot < 0.0) {
    if (fv[3] < 0) {
      const int x = fv[1];
      fv[1] = fv[2];
      fv[2] = x;
    } else {
      const int x = fv[1];
      fv[1] = fv[3];
      fv[3] = x;
    }
  }
  for (int a = 0; a < 4; ++a) fv4[4 * (size_t)e + a] = fv[a];
  const int s2 = second[g];
  c1[e] = c;
  c2[e] = s2 >= 0 ? s2 / kSlots : -1;
  int k = 0;
  if (s2 < 0) {  // box patch by the face centroid's plane (rfmesh.cpp's test)
    const double *lo = lohi, *hi = lohi + 3;
    const double tolx = 1e-9 * (hi[0] - lo[0]), toly = 1e-9 * (hi[1] - lo[1]),
                 tolz = 1e-9 * (hi[2] - lo[2]);
    int ip = -1;
    if (fabs(C[0] - lo[0]) < tolx) ip = 0;
    else if (fabs(C[0] - hi[0]) < tolx) ip = 1;
    else if (fabs(C[1] - lo[1]) < toly) ip = 2;
    else if (fabs(C[1] - hi[1]) < toly) ip = 3;
    else if (fabs(C[2] - lo[2]) < tolz) ip = 4;
    else if (fabs(C[2] - hi[2]) < tolz) ip = 5;
    if (ip < 0) {
      atomicOr(err, MB_OFFBOX);
      ip = 0;
    }
    k = 1 + ip;
  }
  cls[e] = k;
}

// 4: face geometry at its final position p (interior faces first, then the
// patches in order); slot -> (p, side) for the cell pass
__global__ void k_face_geom(const double *__restrict__ xyz, const int *__restrict__ fv4,
                            const int *__restrict__ sortedE, const unsigned *__restrict__ first,
                            const int *__restrict__ second, const int *__restrict__ order,
                            int nAll, double *__restrict__ Sa, double *__restrict__ Ca,
                            double *__restrict__ fnA, int *__restrict__ slotFace) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nAll) return;
  const int e = sortedE[p];
  int fv[4];
  for (int a = 0; a < 4; ++a) fv[a] = fv4[4 * (size_t)e + a];
  double S[3], C[3];
  rfm::face_vec_cen(xyz, fv, S, C);
  const double fVecM = sqrt(S[0] * S[0] + S[1] * S[1] + S[2] * S[2]);
  const double term = 1.0 / fVecM;
  fnA[4 * (size_t)p + 0] = S[0] * term;
  fnA[4 * (size_t)p + 1] = S[1] * term;
  fnA[4 * (size_t)p + 2] = S[2] * term;
  fnA[4 * (size_t)p + 3] = fVecM;
  for (int d = 0; d < 3; ++d) {
    Sa[3 * (size_t)p + d] = S[d];
    Ca[3 * (size_t)p + d] = C[d];
  }
  const int g = order[e];
  slotFace[first[g]] = 2 * p;
  if (second[g] >= 0) slotFace[second[g]] = 2 * p + 1;
}

// cell volumes and centroids: the cell's faces in the host's order (final
// position ascending), + on the first cell, - on the second
__global__ void k_cell_geom(const int *__restrict__ ctype, const double *__restrict__ ca,
                            const int *__restrict__ slotFace, const double *__restrict__ Sa,
                            const double *__restrict__ Ca, int nC, double *__restrict__ vol,
                            double *__restrict__ cofg, int *__restrict__ err) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nC) return;
  const int nf = rfm::cell_nf(ctype[c]);
  int code[kSlots];
  for (int f = 0; f < nf; ++f) {
    code[f] = slotFace[kSlots * (size_t)c + f];
    if (code[f] < 0) {  // a slot left out of every face (a face on three cells)
      atomicOr(err, MB_NONMANIFOLD);
      return;
    }
  }
  for (int i = 1; i < nf; ++i) {  // ascending position
    const int x = code[i];
    int j = i - 1;
    while (j >= 0 && code[j] > x) {
      code[j + 1] = code[j];
      --j;
    }
    code[j + 1] = x;
  }
  double v = 0.0, cg[3] = {0.0, 0.0, 0.0};
  for (int i = 0; i < nf; ++i) {
    const int p = code[i] >> 1;
    double S[3], C[3];
    for (int d = 0; d < 3; ++d) {
      S[d] = Sa[3 * (size_t)p + d];
      C[d] = Ca[3 * (size_t)p + d];
    }
    rfm::face_contrib(S, C, ca + 3 * (size_t)c, (code[i] & 1) ? -1.0 : 1.0, &v, cg);
  }
  const double THRD = 1.0 / 3.0;
  v = THRD * v;
  if (!(v > 0.0)) atomicOr(err, MB_VOLUME);
  const double term = 1.0 / (4.0 * v);
  vol[c] = v;
  for (int d = 0; d < 3; ++d) cofg[3 * (size_t)c + d] = term * cg[d];
}

__global__ void k_v2c_pairs(const int *__restrict__ cv8, const int *__restrict__ nv8, int nC,
                            int *__restrict__ vkey, int *__restrict__ cval,
                            int *__restrict__ count) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 8LL * nC) return;
  const int c = (int)(i / 8), a = (int)(i % 8);
  if (a < nv8[c]) {
    const int v = cv8[8 * (size_t)c + a];
    vkey[i] = v;
    atomicAdd(count + v, 1);
  } else {
    vkey[i] = 0x7fffffff;  // sorts last
  }
  cval[i] = c;
}

// 3: which class run each position belongs to
__global__ void k_class_bounds(const int *__restrict__ clsSorted, int nAll, int *__restrict__ start) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nAll) return;
  const int k = clsSorted[p];
  if (p == 0 || clsSorted[p - 1] != k)
    for (int q = (p == 0 ? 0 : clsSorted[p - 1] + 1); q <= k; ++q) start[q] = p;
  if (p == nAll - 1)
    for (int q = k + 1; q <= 7; ++q) start[q] = nAll;
}

inline unsigned grid_of(long long n, int b = 256) { return (unsigned)((n + b - 1) / b); }

}  // namespace

struct rfgpu_mesh_s {
  long long nFaces = 0, nMembs = 0;
  long long nB[6] = {0, 0, 0, 0, 0, 0};
  std::vector<int> f2c1;             // (2,nFaces), 1-based
  std::vector<double> fn, fc;        // (4,nFaces), (3,nFaces)
  std::vector<double> vol, cofg;     // (nCells), (3,nCells)
  std::vector<int> csOff, csMem1;    // stencils, 1-based members
  std::vector<double> moms;          // (10,nCells)
  std::vector<int> v2cOff, v2c;      // 0-based
  std::vector<int> bf2c1[6], bf2v[6];  // per patch: 1-based cells, 0-based vertices (4, -1 pad)
  std::vector<double> bfn[6], bfc[6];
};

extern "C" {

int rfgpu_mesh_build(int nCells, int nVerts, const double *xyz, const int *cellVerts,
                     const int *cellNVerts, const int *cellType, const double lo[3],
                     const double hi[3], rfgpu_mesh_t *out) {
  if (!out) return RFGPU_ERR_ARG;
  *out = nullptr;
  if (nCells <= 0 || nVerts <= 0 || !xyz || !cellVerts || !cellNVerts || !cellType || !lo || !hi ||
      (long long)nCells * kSlots > 0x7fffffffLL)
    return RFGPU_ERR_ARG;
  long long nValid = 0;
  for (long long c = 0; c < nCells; ++c) {  // every index a kernel follows, checked first
    const int t = cellType[c];
    if (t < 0 || t > 3 || cellNVerts[c] != rfm::cell_nv(t)) return RFGPU_ERR_ARG;
    for (int a = 0; a < 8; ++a) {
      const int v = cellVerts[8 * c + a];
      if (a < cellNVerts[c] ? (v < 0 || v >= nVerts) : v != -1) return RFGPU_ERR_ARG;
    }
    nValid += rfm::cell_nf(t);
  }
  const size_t N = (size_t)nCells, NS = N * kSlots;
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return RFGPU_ERR_CUDA;
  std::vector<void *> bufs;
  bool ok = true;
  auto dalloc = [&](size_t bytes) -> void * {
    void *p = nullptr;
    if (cudaMallocAsync(&p, bytes ? bytes : 1, s) != cudaSuccess) {
      ok = false;
      return nullptr;
    }
    bufs.push_back(p);
    return p;
  };
  rfgpu_mesh_s *m = new (std::nothrow) rfgpu_mesh_s();
  int rc = m ? RFGPU_OK : RFGPU_ERR_NOMEM;
  try {
    double *dxyz = (double *)dalloc(3 * (size_t)nVerts * 8), *dlohi = (double *)dalloc(48);
    int *dcv = (int *)dalloc(8 * N * 4), *dnv = (int *)dalloc(N * 4), *dty = (int *)dalloc(N * 4);
    int *derr = (int *)dalloc(4);
    double *dca = (double *)dalloc(3 * N * 8);
    unsigned long long *khi = (unsigned long long *)dalloc(NS * 8),
                       *klo = (unsigned long long *)dalloc(NS * 8),
                       *k1 = (unsigned long long *)dalloc(NS * 8),
                       *k2 = (unsigned long long *)dalloc(NS * 8);
    int *idx0 = (int *)dalloc(NS * 4), *idx1 = (int *)dalloc(NS * 4), *idx2 = (int *)dalloc(NS * 4);
    int *head = (int *)dalloc(NS * 4), *pos = (int *)dalloc(NS * 4);
    if (!ok) throw std::bad_alloc();
    double lohi[6] = {lo[0], lo[1], lo[2], hi[0], hi[1], hi[2]};
    cudaMemcpyAsync(dxyz, xyz, 3 * (size_t)nVerts * 8, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(dlohi, lohi, 48, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(dcv, cellVerts, 8 * N * 4, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(dnv, cellNVerts, N * 4, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(dty, cellType, N * 4, cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(derr, 0, 4, s);
    k_cofg_app<<<grid_of(N), 256, 0, s>>>(dxyz, dcv, dnv, nCells, dca);
    k_slot_keys<<<grid_of(NS), 256, 0, s>>>(dcv, dty, nCells, khi, klo, idx0);
    // 1. stable LSD sort by (hi, lo): by lo, then by hi carried in lo order
    size_t tb = 0, tb2 = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tb, klo, k1, idx0, idx1, (long long)NS, 0, 64, s);
    cub::DeviceScan::ExclusiveSum(nullptr, tb2, head, pos, (long long)NS, s);
    void *tmp = dalloc(std::max(tb, tb2));
    if (!ok) throw std::bad_alloc();
    cub::DeviceRadixSort::SortPairs(tmp, tb, klo, k1, idx0, idx1, (long long)NS, 0, 64, s);
    k_gather_u64<<<grid_of(NS), 256, 0, s>>>(khi, idx1, (long long)NS, k1);
    cub::DeviceRadixSort::SortPairs(tmp, tb, k1, k2, idx1, idx2, (long long)NS, 0, 64, s);
    // idx2: slots in key order, equal keys in slot order; the valid ones first
    k_heads<<<grid_of(nValid), 256, 0, s>>>(khi, klo, idx2, nValid, head, derr);
    cub::DeviceScan::ExclusiveSum(tmp, tb2, head, pos, nValid, s);
    int nAll = 0, lastHead = 0, lastPos = 0;
    cudaMemcpyAsync(&lastHead, head + nValid - 1, 4, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&lastPos, pos + nValid - 1, 4, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) throw std::runtime_error("cuda");
    nAll = lastPos + lastHead;
    unsigned *first = (unsigned *)dalloc((size_t)nAll * 4), *firstS = (unsigned *)dalloc((size_t)nAll * 4);
    int *second = (int *)dalloc((size_t)nAll * 4), *runId = (int *)dalloc((size_t)nAll * 4),
        *order = (int *)dalloc((size_t)nAll * 4);
    if (!ok) throw std::bad_alloc();
    k_runs<<<grid_of(nValid), 256, 0, s>>>(khi, klo, idx2, head, pos, nValid, first, second, runId);
    // 2. faces in first-encounter order: runs sorted by their first slot
    size_t tb3 = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tb3, first, firstS, runId, order, nAll, 0, 32, s);
    void *tmp3 = dalloc(tb3);
    int *fv4 = (int *)dalloc(4 * (size_t)nAll * 4), *cls = (int *)dalloc((size_t)nAll * 4),
        *c1 = (int *)dalloc((size_t)nAll * 4), *c2 = (int *)dalloc((size_t)nAll * 4),
        *eIdx = (int *)dalloc((size_t)nAll * 4), *clsS = (int *)dalloc((size_t)nAll * 4),
        *sortedE = (int *)dalloc((size_t)nAll * 4), *start = (int *)dalloc(8 * 4);
    if (!ok) throw std::bad_alloc();
    cub::DeviceRadixSort::SortPairs(tmp3, tb3, first, firstS, runId, order, nAll, 0, 32, s);
    k_orient<<<grid_of(nAll), 256, 0, s>>>(dxyz, dcv, dty, dca, first, second, order, nAll, dlohi,
                                          fv4, cls, c1, c2, derr);
    // 3. interior faces, then each patch, each in face order
    std::vector<int> iota(nAll);
    for (int e = 0; e < nAll; ++e) iota[e] = e;
    cudaMemcpyAsync(eIdx, iota.data(), (size_t)nAll * 4, cudaMemcpyHostToDevice, s);
    size_t tb4 = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tb4, cls, clsS, eIdx, sortedE, nAll, 0, 3, s);
    void *tmp4 = dalloc(tb4);
    if (!ok) throw std::bad_alloc();
    cub::DeviceRadixSort::SortPairs(tmp4, tb4, cls, clsS, eIdx, sortedE, nAll, 0, 3, s);
    k_class_bounds<<<grid_of(nAll), 256, 0, s>>>(clsS, nAll, start);
    // 4. geometry
    double *Sa = (double *)dalloc(3 * (size_t)nAll * 8), *Ca = (double *)dalloc(3 * (size_t)nAll * 8),
           *fnA = (double *)dalloc(4 * (size_t)nAll * 8), *dvol = (double *)dalloc(N * 8),
           *dcofg = (double *)dalloc(3 * N * 8);
    int *slotFace = (int *)dalloc(NS * 4);
    if (!ok) throw std::bad_alloc();
    cudaMemsetAsync(slotFace, 0xff, NS * 4, s);  // -1: no face
    k_face_geom<<<grid_of(nAll), 256, 0, s>>>(dxyz, fv4, sortedE, first, second, order, nAll, Sa,
                                             Ca, fnA, slotFace);
    k_cell_geom<<<grid_of(N), 256, 0, s>>>(dty, dca, slotFace, Sa, Ca, nCells, dvol, dcofg, derr);
    // 5. vertex-to-cell lists, ascending cell per vertex
    int *vkey = (int *)dalloc(8 * N * 4), *cval = (int *)dalloc(8 * N * 4),
        *vkeyS = (int *)dalloc(8 * N * 4), *cvalS = (int *)dalloc(8 * N * 4),
        *vcnt = (int *)dalloc(((size_t)nVerts + 1) * 4), *voff = (int *)dalloc(((size_t)nVerts + 1) * 4);
    if (!ok) throw std::bad_alloc();
    cudaMemsetAsync(vcnt, 0, ((size_t)nVerts + 1) * 4, s);
    k_v2c_pairs<<<grid_of(8 * N), 256, 0, s>>>(dcv, dnv, nCells, vkey, cval, vcnt);
    size_t tb5 = 0, tb6 = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tb5, vkey, vkeyS, cval, cvalS, (long long)(8 * N), 0, 32, s);
    cub::DeviceScan::ExclusiveSum(nullptr, tb6, vcnt, voff, nVerts + 1, s);
    void *tmp5 = dalloc(std::max(tb5, tb6));
    if (!ok) throw std::bad_alloc();
    cub::DeviceRadixSort::SortPairs(tmp5, tb5, vkey, vkeyS, cval, cvalS, (long long)(8 * N), 0, 32, s);
    cub::DeviceScan::ExclusiveSum(tmp5, tb6, vcnt, voff, nVerts + 1, s);
    // stencils and moments (the kernel of rfgpu_mesh_stencils)
    const size_t K = rfm::kStencilMax;
    int *dcnt = (int *)dalloc(N * 4), *dmemb = (int *)dalloc(K * N * 4), *dov = (int *)dalloc(4);
    double *dmoms = (double *)dalloc(10 * N * 8);
    if (!ok) throw std::bad_alloc();
    cudaMemsetAsync(dov, 0, 4, s);
    rfgpu::launch_mesh_stencils(dcofg, dcv, dnv, voff, cvalS, nCells, dcnt, dmemb, dmoms, dov, s);
    // results to the host
    int hstart[8] = {0}, herr = 0, overflow = 0;
    std::vector<int> fvh(4 * (size_t)nAll), c1h(nAll), c2h(nAll), sE(nAll), cnt(N), memb(K * N);
    std::vector<double> fnh(4 * (size_t)nAll), Ch(3 * (size_t)nAll);
    m->vol.resize(N);
    m->cofg.resize(3 * N);
    m->moms.resize(10 * N);
    m->v2cOff.resize((size_t)nVerts + 1);
    cudaMemcpyAsync(hstart, start, 32, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&herr, derr, 4, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&overflow, dov, 4, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(fvh.data(), fv4, 16 * (size_t)nAll, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(c1h.data(), c1, 4 * (size_t)nAll, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(c2h.data(), c2, 4 * (size_t)nAll, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(sE.data(), sortedE, 4 * (size_t)nAll, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(fnh.data(), fnA, 32 * (size_t)nAll, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(Ch.data(), Ca, 24 * (size_t)nAll, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(m->vol.data(), dvol, N * 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(m->cofg.data(), dcofg, 3 * N * 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(m->moms.data(), dmoms, 10 * N * 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(cnt.data(), dcnt, N * 4, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(memb.data(), dmemb, K * N * 4, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(m->v2cOff.data(), voff, ((size_t)nVerts + 1) * 4, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess || cudaGetLastError() != cudaSuccess)
      throw std::runtime_error("cuda");
    m->v2c.resize((size_t)m->v2cOff[nVerts]);
    cudaMemcpyAsync(m->v2c.data(), cvalS, 4 * m->v2c.size(), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) throw std::runtime_error("cuda");
    if (herr & (MB_NONMANIFOLD | MB_OFFBOX)) {
      rc = RFGPU_ERR_ARG;
    } else if (herr & MB_VOLUME) {
      rc = RFGPU_ERR_ARG;
    } else if (overflow) {
      rc = RFGPU_ERR_UNSUPPORTED;
    } else {
      const int nF = hstart[1];
      m->nFaces = nF;
      m->f2c1.resize(2 * (size_t)nF);
      m->fn.resize(4 * (size_t)nF);
      m->fc.resize(3 * (size_t)nF);
      for (int p = 0; p < nF; ++p) {
        const int e = sE[p];
        m->f2c1[2 * (size_t)p] = c1h[e] + 1;
        m->f2c1[2 * (size_t)p + 1] = c2h[e] + 1;
        for (int k = 0; k < 4; ++k) m->fn[4 * (size_t)p + k] = fnh[4 * (size_t)p + k];
        for (int k = 0; k < 3; ++k) m->fc[3 * (size_t)p + k] = Ch[3 * (size_t)p + k];
      }
      for (int ip = 0; ip < 6; ++ip) {
        const int b0 = hstart[1 + ip], b1 = hstart[2 + ip];
        m->nB[ip] = b1 - b0;
        for (int p = b0; p < b1; ++p) {
          const int e = sE[p];
          m->bf2c1[ip].push_back(c1h[e] + 1);
          for (int k = 0; k < 4; ++k) m->bf2v[ip].push_back(fvh[4 * (size_t)e + k]);
          for (int k = 0; k < 4; ++k) m->bfn[ip].push_back(fnh[4 * (size_t)p + k]);
          for (int k = 0; k < 3; ++k) m->bfc[ip].push_back(Ch[3 * (size_t)p + k]);
        }
      }
      m->csOff.assign(N + 1, 0);
      for (size_t c = 0; c < N; ++c) m->csOff[c + 1] = m->csOff[c] + cnt[c];
      m->csMem1.resize((size_t)m->csOff[N]);
      for (size_t c = 0; c < N; ++c)
        for (int k = 0; k < cnt[c]; ++k) m->csMem1[m->csOff[c] + k] = memb[K * c + k] + 1;
      m->nMembs = m->csOff[N];
    }
  } catch (const std::bad_alloc &) {
    rc = RFGPU_ERR_NOMEM;
  } catch (...) {
    rc = RFGPU_ERR_CUDA;
  }
  for (void *p : bufs) cudaFreeAsync(p, s);
  cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  if (rc != RFGPU_OK) {
    delete m;
    return rc;
  }
  *out = m;
  return RFGPU_OK;
}

int rfgpu_mesh_sizes(rfgpu_mesh_t m, long long sizes[8]) {
  if (!m || !sizes) return RFGPU_ERR_ARG;
  sizes[0] = m->nFaces;
  sizes[1] = m->nMembs;
  for (int ip = 0; ip < 6; ++ip) sizes[2 + ip] = m->nB[ip];
  return RFGPU_OK;
}

int rfgpu_mesh_faces(rfgpu_mesh_t m, int *f2c, double *fn, double *fc) {
  if (!m) return RFGPU_ERR_ARG;
  if (f2c) std::copy(m->f2c1.begin(), m->f2c1.end(), f2c);
  if (fn) std::copy(m->fn.begin(), m->fn.end(), fn);
  if (fc) std::copy(m->fc.begin(), m->fc.end(), fc);
  return RFGPU_OK;
}

int rfgpu_mesh_cells(rfgpu_mesh_t m, double *vol, double *cofg, int *c2csOffsets,
                     int *c2csMembers, double *xyzMoms, int *v2cOffsets, int *v2c) {
  if (!m) return RFGPU_ERR_ARG;
  if (vol) std::copy(m->vol.begin(), m->vol.end(), vol);
  if (cofg) std::copy(m->cofg.begin(), m->cofg.end(), cofg);
  if (c2csOffsets) std::copy(m->csOff.begin(), m->csOff.end(), c2csOffsets);
  if (c2csMembers) std::copy(m->csMem1.begin(), m->csMem1.end(), c2csMembers);
  if (xyzMoms) std::copy(m->moms.begin(), m->moms.end(), xyzMoms);
  if (v2cOffsets) std::copy(m->v2cOff.begin(), m->v2cOff.end(), v2cOffsets);
  if (v2c) std::copy(m->v2c.begin(), m->v2c.end(), v2c);
  return RFGPU_OK;
}

int rfgpu_mesh_patch(rfgpu_mesh_t m, int ip, int *bf2c, double *fn, double *fc, int *bf2v) {
  if (!m || ip < 0 || ip >= 6) return RFGPU_ERR_ARG;
  if (bf2c) std::copy(m->bf2c1[ip].begin(), m->bf2c1[ip].end(), bf2c);
  if (fn) std::copy(m->bfn[ip].begin(), m->bfn[ip].end(), fn);
  if (fc) std::copy(m->bfc[ip].begin(), m->bfc[ip].end(), fc);
  if (bf2v) std::copy(m->bf2v[ip].begin(), m->bf2v[ip].end(), bf2v);
  return RFGPU_OK;
}

int rfgpu_mesh_destroy(rfgpu_mesh_t m) {
  if (!m) return RFGPU_ERR_ARG;
  delete m;
  return RFGPU_OK;
}

}  // extern "C"
