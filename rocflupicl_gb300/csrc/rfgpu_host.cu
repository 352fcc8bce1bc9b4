// rfgpu_host.cu - C ABI of the residual engine (include/rfgpu.h): region
// registration (Fortran image -> 0-based SoA + SELL-32 lists on the device),
// stage / step / residual / time-step drivers, CUDA-graph replay and batches.
#include "rfgpu.h"
#include "rfgpu_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <vector>

using namespace rfgpu;

namespace {

struct DevAlloc {
  std::vector<void *> ptrs;
  long long bytes = 0;
  template <typename T>
  T *alloc(size_t n) {
    if (n == 0) n = 1;
    void *p = nullptr;
    if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) throw std::bad_alloc();
    ptrs.push_back(p);
    bytes += (long long)(n * sizeof(T));
    return (T *)p;
  }
  template <typename T>
  T *upload(const std::vector<T> &v, cudaStream_t s) {
    T *d = alloc<T>(v.size());
    if (!v.empty() &&
        cudaMemcpyAsync(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s) != cudaSuccess)
      throw std::bad_alloc();
    return d;
  }
  void free_all() {
    for (void *p : ptrs) cudaFree(p);
    ptrs.clear();
  }
};

struct Sell {
  std::vector<long long> off;  // per slice
  std::vector<int> cnt;        // per cell
  long long total = 0;
  void build(const std::vector<int> &counts) {
    int N = (int)counts.size();
    int nSl = (N + kSlice - 1) / kSlice;
    off.assign(nSl + 1, 0);
    cnt = counts;
    for (int s = 0; s < nSl; ++s) {
      int w = 0;
      for (int l = 0; l < kSlice && s * kSlice + l < N; ++l) w = std::max(w, counts[s * kSlice + l]);
      off[s + 1] = off[s] + (long long)w * kSlice;
    }
    total = off[nSl];
  }
  long long at(int c, int k) const { return off[c / kSlice] + (long long)k * kSlice + c % kSlice; }
};

// Per-kernel CUDA-event profiler: a pair of events recorded on the launching
// stream around every launch while enabled; resolved into per-class totals
// when read.
struct ProfState {
  bool on = false;
  std::vector<cudaEvent_t> pool;
  size_t used = 0;
  std::vector<std::pair<int, std::pair<size_t, size_t>>> spans;  // kind, (start ev, stop ev)
  size_t open[KP_COUNT] = {0};
  Prof hook{};
  cudaEvent_t get() {
    if (used == pool.size()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      pool.push_back(e);
    }
    return pool[used++];
  }
  static void mark(void *ctx, int kind, int phase, cudaStream_t s) {
    ProfState *p = (ProfState *)ctx;
    size_t idx = p->used;
    cudaEvent_t e = p->get();
    cudaEventRecord(e, s);
    if (phase == 0)
      p->open[kind] = idx;
    else
      p->spans.push_back({kind, {p->open[kind], idx}});
  }
  const Prof *hookp() {
    if (!on) return nullptr;
    hook.mark = &ProfState::mark;
    hook.ctx = this;
    return &hook;
  }
  void reset() {
    used = 0;
    spans.clear();
  }
  void destroy() {
    for (auto e : pool) cudaEventDestroy(e);
    pool.clear();
    reset();
  }
};

// Tile lists of the tuned launch shapes, made once per item stride and kept
// for the handle's lifetime (a few bytes per 64 items).
struct TileCache {
  std::map<int, std::pair<Tile *, int>> cells, faces;
};

}  // namespace

// One border of a partitioned region: its send and receive cells in the
// device numbering (host copies for matching borders into a coupled batch,
// device copies for the border calls).
struct BorderH {
  int iRegionGlobal = 0, iBorder = 0;
  std::vector<int> send, recv;
  int *dSend = nullptr, *dRecv = nullptr;
};

struct rfgpu_region_s {
  int prec = 0;
  int device = 0;                           // the GPU the region was created on
  int nCells = 0, nFaces = 0, nBFaces = 0;  // nCells: actual + virtual (nCellsTot)
  int nAct = 0;                             // actual cells
  int iRegionGlobal = 0;
  double gvCp = 0.0, gvMol = 0.0;
  std::vector<BorderH> borders;
  double *bbuf = nullptr;                   // border buffer, 5 x the largest border
  cudaEvent_t evA = nullptr, evB = nullptr; // ordering of border copies between streams
  // mixed-path transfers: copies on xstream, conversions on stream, chunk by
  // chunk, so a chunk's copy overlaps its neighbour's conversion
  cudaStream_t xstream = nullptr;
  cudaEvent_t xev[9] = {};
  // rfgpu_step_host (mixed path): cell tiles grouped by transfer phase, made on
  // first use; phOff[0] gradient phases over phGrad, phOff[1] update phases over phUpd,
  // phOff[2] the last stage's interior-face phases over phFace, phOff[3] its
  // gradient phases over phGradL, phOff[4] its boundary-face phases over phBface
  Tile *phGrad = nullptr, *phUpd = nullptr, *phFace = nullptr, *phGradL = nullptr,
       *phBface = nullptr;
  int phOff[5][9] = {};
  int phN = 0;
  // mixed-path transfers: the device cells of each chunk in ascending device
  // order (xList[xOff[k] .. xOff[k+1])), so the conversions touch the device
  // state coalesced
  int *xList = nullptr;
  int xOff[9] = {};
  // rfgpu_step_host: the upload's conversions run on their own stream, beside
  // the first stage's gradient phases on the region's stream
  cudaStream_t cstream = nullptr;
  cudaEvent_t cev[9] = {};
  int rkScheme = 2, nSteps = 3, spaceOrder = 2, reconst = 11;
  cudaStream_t stream = nullptr;
  DevAlloc mem;
  RegionDev<double> rd64{};
  RegionDev<float> rd32{};
  void *regsDev = nullptr;  // RegionDev<R>[1]
  Tile *cellTiles = nullptr, *faceTiles = nullptr, *bfaceTiles = nullptr;
  Work work{};
  double *stage = nullptr;   // staging for AoS transfers, 5*N doubles
  double *stage2 = nullptr;  // second staging buffer (dv), 3*N doubles, mixed path
  long long launches = 0;
  // graph cache
  cudaGraphExec_t graph = nullptr;
  double gkey[4] = {0, 0, 0, 0};
  long long perStep = 0;
  ProfState prof;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  const int *cellNew = nullptr, *cellOld = nullptr;  // device numbering (null: host's)
  TileCache tiles;
};

struct rfgpu_batch_s {
  int prec = 0;
  std::vector<rfgpu_region_t> regs;
  cudaStream_t stream = nullptr;
  DevAlloc mem;
  void *regsDev = nullptr;
  Work work{};
  int spaceOrder = 1, reconst = 0, nSteps = 3;
  long long launches = 0;
  cudaGraphExec_t graph = nullptr;
  double gkey[4] = {0, 0, 0, 0};
  long long perStep = 0;
  ProfState prof;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  TileCache tiles;
  std::vector<int> nCells, nFaces;  // per member region, for its tile lists
};

namespace {

int cuda_rc(cudaError_t e) { return e == cudaSuccess ? RFGPU_OK : RFGPU_ERR_CUDA; }

// Limit of a persistent stage launch's grid-barrier wait, in SM clock cycles
// (about a second at GB300's clocks).
constexpr long long kBarrierSpin = 2000000000ll;

// Synchronise a stream and report a persistent stage launch whose bounded
// barrier wait ran out (the error word is read and cleared).
int sync_and_check(cudaStream_t s, GridBar *bar) {
  if (cudaStreamSynchronize(s) != cudaSuccess) return RFGPU_ERR_CUDA;
  if (!bar) return RFGPU_OK;
  unsigned err = 0;
  if (cudaMemcpyAsync(&err, &bar->err, sizeof(unsigned), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return RFGPU_ERR_CUDA;
  if (!err) return RFGPU_OK;
  if (cudaMemsetAsync(&bar->err, 0, sizeof(unsigned), s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return RFGPU_ERR_CUDA;
  return RFGPU_ERR_TIMEOUT;
}

void rk_coeffs(int scheme, Phys &ph) {
  for (int i = 0; i < 5; ++i) ph.ark[i] = ph.grk[i] = 0.0;
  if (scheme == RFGPU_RK_SCHEME_4_CLASSICAL) {
    ph.ark[0] = 0.5; ph.ark[1] = 0.5; ph.ark[2] = 1.0; ph.ark[3] = 1.0 / 6.0;
    ph.grk[0] = 1.0; ph.grk[1] = 2.0; ph.grk[2] = 2.0; ph.grk[3] = 1.0;
    ph.nSteps = 4;
  } else if (scheme == RFGPU_RK_SCHEME_3_WRAY) {  // libflu/RFLU_DerivedInputValues.F90:374-389
    ph.ark[0] = 8.0 / 15.0; ph.ark[1] = 5.0 / 12.0; ph.ark[2] = 0.75;
    ph.grk[0] = 0.0; ph.grk[1] = 17.0 / 25.0; ph.grk[2] = 5.0 / 9.0;
    ph.nSteps = 3;
  } else {
    ph.ark[0] = 1.0; ph.grk[0] = 1.0;
    ph.nSteps = 1;
  }
}

std::vector<Tile> make_tiles(int region, int n, int block) {
  std::vector<Tile> t;
  for (int i = 0; i < n; i += block) t.push_back(Tile{region, i});
  return t;
}

int check_desc(const rfgpu_region_desc_t *d) {
  if (!d || d->nCells <= 0 || d->nFaces < 0 || d->nPatches < 0 || !d->cv || !d->vol ||
      !d->cofg || (d->nFaces > 0 && (!d->f2c || !d->fn || !d->fc)) || d->f2cLd < 2 ||
      !d->c2csOffsets || !d->c2csMembers || !d->xyzMoms || (d->nPatches > 0 && !d->patches))
    return RFGPU_ERR_ARG;
  if (d->gasModel != RFGPU_GAS_MODEL_TCPERF || d->flowModel != RFGPU_FLOW_EULER)
    return RFGPU_ERR_UNSUPPORTED;
  if (d->spaceDiscr != RFGPU_DISCR_UPW_ROE && d->spaceDiscr != RFGPU_DISCR_UPW_HLLC &&
      d->spaceDiscr != RFGPU_DISCR_UPW_AUSMPLUS && d->spaceDiscr != RFGPU_DISCR_UPW_AUSMPLUSUP)
    return RFGPU_ERR_UNSUPPORTED;
  if (d->spaceOrder != 1 && d->spaceOrder != 2) return RFGPU_ERR_UNSUPPORTED;
  if (d->reconst != RFGPU_RECONST_NONE && d->reconst != RFGPU_RECONST_LIM_VENKAT &&
      d->reconst != RFGPU_RECONST_WENO_XYZ)
    return RFGPU_ERR_UNSUPPORTED;
  if (d->rkScheme < 1 || d->rkScheme > 3) return RFGPU_ERR_UNSUPPORTED;
  if (d->precision != RFGPU_PREC_FP64 && d->precision != RFGPU_PREC_MIXED &&
      d->precision != RFGPU_PREC_SPLIT)
    return RFGPU_ERR_UNSUPPORTED;
  if (d->cellOrder != RFGPU_ORDER_LOCALITY && d->cellOrder != RFGPU_ORDER_HOST)
    return RFGPU_ERR_UNSUPPORTED;
  for (int ip = 0; ip < d->nPatches; ++ip) {
    const rfgpu_patch_t &p = d->patches[ip];
    if (p.nBFaces < 0 || (p.nBFaces > 0 && (!p.bf2c || !p.fn || !p.fc))) return RFGPU_ERR_ARG;
    if (p.nBFacesTot != 0 && (p.nBFacesTot < p.nBFaces || !p.bf2c || !p.fc)) return RFGPU_ERR_ARG;
    if (p.bcType != RFGPU_BC_SLIPWALL && p.bcType != RFGPU_BC_OUTFLOW &&
        p.bcType != RFGPU_BC_FARFIELD && p.bcType != RFGPU_BC_INJECTION &&
        p.bcType != RFGPU_BC_INFLOW_TOTANG && p.bcType != RFGPU_BC_INFLOW_VELTEMP)
      return RFGPU_ERR_UNSUPPORTED;
    if (p.spaceOrder != 1 && p.spaceOrder != 2) return RFGPU_ERR_UNSUPPORTED;
    if (p.nData < 0) return RFGPU_ERR_ARG;
    const int nData = p.nData > 0 ? p.nData : 1;
    if (p.bcType == RFGPU_BC_OUTFLOW) {
      if (p.bcOptType < 0 || p.bcOptType > 2) return RFGPU_ERR_UNSUPPORTED;
      if (p.bcOptType != RFGPU_BCOPT_SUPERSONIC && !p.vals) return RFGPU_ERR_ARG;
    }
    if (p.bcType == RFGPU_BC_FARFIELD) {
      if (p.bcOptType != 0) return RFGPU_ERR_UNSUPPORTED;  // lift correction (airfoil-specific)
      if (!p.vals || nData < 5) return RFGPU_ERR_ARG;
    }
    if (p.bcType == RFGPU_BC_INJECTION && (!p.vals || nData < 2)) return RFGPU_ERR_ARG;
    if (p.bcType == RFGPU_BC_INFLOW_TOTANG || p.bcType == RFGPU_BC_INFLOW_VELTEMP) {
      if (p.bcOptType < 0 || p.bcOptType > 2) return RFGPU_ERR_UNSUPPORTED;
      if (p.bcOptFixed < 0 || p.bcOptFixed > 1) return RFGPU_ERR_UNSUPPORTED;
      if (!p.vals || nData < 5) return RFGPU_ERR_ARG;
    }
  }
  if (d->nCellsTot != 0 && d->nCellsTot < d->nCells) return RFGPU_ERR_ARG;
  const long long N = d->nCellsTot > 0 ? d->nCellsTot : d->nCells;
  if (d->nBorders < 0 || (d->nBorders > 0 && !d->borders)) return RFGPU_ERR_ARG;
  for (int ib = 0; ib < d->nBorders; ++ib) {
    const rfgpu_border_t &b = d->borders[ib];
    if (b.nCellsSend < 0 || b.nCellsRecv < 0 || (b.nCellsSend > 0 && !b.icgSend) ||
        (b.nCellsRecv > 0 && !b.icgRecv) || b.iBorder < 1)
      return RFGPU_ERR_ARG;
    for (int k = 0; k < b.nCellsSend; ++k)  // actual cells
      if (b.icgSend[k] < 1 || b.icgSend[k] > d->nCells) return RFGPU_ERR_ARG;
    for (int k = 0; k < b.nCellsRecv; ++k)  // virtual cells
      if (b.icgRecv[k] <= d->nCells || b.icgRecv[k] > N) return RFGPU_ERR_ARG;
  }
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (int f = 0; f < d->nFaces; ++f)
    for (int k = 0; k < 2; ++k) {
      int c = d->f2c[(long long)f * d->f2cLd + k];
      if (c < 1 || c > N) bad = 1;
    }
  if (bad) return RFGPU_ERR_ARG;
  // faces past the flux faces (VV, VX): at least one side a virtual cell; the
  // other a cell of the region or outside it (any value outside 1..N)
  if (d->nFacesAll != 0 && d->nFacesAll < d->nFaces) return RFGPU_ERR_ARG;
  for (int f = d->nFaces; f < d->nFacesAll; ++f) {
    const int a = d->f2c[(long long)f * d->f2cLd], b = d->f2c[(long long)f * d->f2cLd + 1];
    const bool va = a > d->nCells && a <= N, vb = b > d->nCells && b <= N;
    const bool ina = a >= 1 && a <= N, inb = b >= 1 && b <= N;
    if (!(va || vb) || (ina && !va && !vb) || (inb && !va && !vb)) return RFGPU_ERR_ARG;
  }
  if (d->c2csOffsets[0] != 0) return RFGPU_ERR_ARG;
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (long long c = 0; c < N; ++c)
    if (d->c2csOffsets[c + 1] < d->c2csOffsets[c]) bad = 1;
  if (bad) return RFGPU_ERR_ARG;
  const long long nMem = d->c2csOffsets[N];
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (long long e = 0; e < nMem; ++e)
    if (d->c2csMembers[e] < 1 || d->c2csMembers[e] > N) bad = 1;
  if (bad) return RFGPU_ERR_ARG;
  // stencils are at most 10x the minimum size (RFLU_ModStencilsCells.F90:2865-2873)
  // in the reference; the engine stages up to 400 members per cell on chip
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (long long c = 0; c < N; ++c)
    if (d->c2csOffsets[c + 1] - d->c2csOffsets[c] > 400) bad = 1;
  if (bad) return RFGPU_ERR_UNSUPPORTED;
  for (int ip = 0; ip < d->nPatches; ++ip) {
    const rfgpu_patch_t &p = d->patches[ip];
    for (int b = 0; b < p.nBFaces; ++b)
      if (p.bf2c[b] < 1 || p.bf2c[b] > N) return RFGPU_ERR_ARG;
    for (int b = p.nBFaces; b < p.nBFacesTot; ++b)  // faces on virtual cells
      if (p.bf2c[b] <= d->nCells || p.bf2c[b] > N) return RFGPU_ERR_ARG;
  }
  return RFGPU_OK;
}

template <typename R>
std::vector<R> cast(const std::vector<double> &v) {
  std::vector<R> out(v.size());
  const long long n = (long long)v.size();
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < n; ++i) out[i] = (R)v[i];
  return out;
}

template <typename R>
RegionDev<R> &rd(rfgpu_region_s *h);
template <>
RegionDev<double> &rd<double>(rfgpu_region_s *h) { return h->rd64; }
template <>
RegionDev<float> &rd<float>(rfgpu_region_s *h) { return h->rd32; }

// Free-stream state of a farfield face (RFLU_SetRindStateFarfieldPerf,
// modflu/RFLU_ModRindStates.F90:249-421, the part that depends only on the
// patch values): ri = p/(R T), pi = p, qi = M sqrt(g R T) and its components
// along the angles of attack and sideslip, in this order of operations.
void farfield_state(const Phys &ph, const double *v, double dat[16]) {
  const double machInf = v[0], alphaInf = v[1], betaInf = v[2], pInf = v[3], tInf = v[4];
  const double rGas = ph.gvR, gGas = ph.gvG;
  const double ri = pInf / (rGas * tInf);
  const double qi = machInf * std::sqrt(gGas * rGas * tInf);
  dat[0] = ri;
  dat[1] = pInf;
  dat[2] = qi;
  dat[3] = qi * std::cos(alphaInf) * std::cos(betaInf);
  dat[4] = qi * std::sin(alphaInf) * std::cos(betaInf);
  dat[5] = qi * std::sin(betaInf);
  dat[6] = machInf;
  dat[7] = 0.0;
}

// Total-pressure / total-temperature inflow (libfloflu/BcondInflowPerf.F90:
// 93-272), the parts that depend only on the patch values: a02 = g R ttot,
// the flow-angle cosines and sines, and the prescribed state of the
// supersonic branch (Mach from the patch; also the MIXED type's state when the
// interior normal velocity is supersonic), MixtPerf_P_GMaPo, _T_GMaTo, _D_PRT,
// _C_GRT, _Eo_DGPUVW in their order of operations.  The reference leaves ksg
// unset on the supersonic branch; it is 0 here.
void inflow_totang_state(const Phys &ph, const double *v, int opt, int fixed, double dat[16]) {
  const double ptot = v[0], ttot = v[1], betah = v[2], betav = v[3];
  const double mach = opt != RFGPU_BCOPT_SUBSONIC ? v[4] : 0.0;
  const double rgas = ph.gvR, g = ph.gvG;
  dat[0] = ptot;
  dat[1] = ttot;
  dat[2] = g * rgas * ttot;  // MixtPerf_C2_GRT
  dat[3] = std::cos(betah);
  dat[4] = std::sin(betah);
  dat[5] = std::cos(betav);
  dat[6] = std::sin(betav);
  dat[7] = fixed;
  const double pr = ptot / (std::pow(1.0 + 0.5 * (g - 1.0) * mach * mach, g / (g - 1.0)));
  const double tr = ttot / (1.0 + 0.5 * (g - 1.0) * mach * mach);
  const double rr = pr / (rgas * tr);
  const double ar = std::sqrt(g * rgas * tr);
  const double ur = mach * ar * std::cos(betah) * std::cos(betav);
  const double vr = mach * ar * std::sin(betah);
  const double wr = mach * ar * std::cos(betah) * std::sin(betav);
  dat[8] = rr;
  dat[9] = rr * ur;
  dat[10] = rr * vr;
  dat[11] = rr * wr;
  dat[12] = rr * (pr / (rr * (g - 1.0)) + 0.5 * (ur * ur + vr * vr + wr * wr) + 0.0);
  dat[13] = pr;
}

// Device numbering of cells and interior faces.  Empty maps: the host's.
struct Order {
  std::vector<int> cOld, cNew;  // device cell -> host cell, host cell -> device cell
  std::vector<int> fOld, fNew;  // the same for interior faces
  int oc(int c) const { return cOld.empty() ? c : cOld[c]; }
  int nc(int c) const { return cNew.empty() ? c : cNew[c]; }
  int of(int f) const { return fOld.empty() ? f : fOld[f]; }
  int nf(int f) const { return fNew.empty() ? f : fNew[f]; }
};

// Interleave the low 21 bits of v with two zero bits between each.
unsigned long long spread3(unsigned long long v) {
  v &= 0x1fffffull;
  v = (v | v << 32) & 0x1f00000000ffffull;
  v = (v | v << 16) & 0x1f0000ff0000ffull;
  v = (v | v << 8) & 0x100f00f00f00f00full;
  v = (v | v << 4) & 0x10c30c30c30c30c3ull;
  v = (v | v << 2) & 0x1249249249249249ull;
  return v;
}

// Locality numbering.  Cells: ascending 63-bit Morton key of the centroid
// (one scale for all three axes, so the curve follows physical distance),
// ties by host index, by a stable LSD radix sort (6 passes of 11 bits).
// Interior faces: grouped by their lower device cell, ascending, then by the
// higher one (a counting sort on the lower cell, short runs sorted in place).
Order locality_order(const rfgpu_region_desc_t *d) {
  Order o;
  const int N = d->nCellsTot > 0 ? d->nCellsTot : d->nCells, F = d->nFaces;
  const int nAct = d->nCells;
  double lo[3], hi[3];
  for (int k = 0; k < 3; ++k) lo[k] = hi[k] = d->cofg[k];
  for (int c = 0; c < N; ++c)
    for (int k = 0; k < 3; ++k) {
      const double x = d->cofg[3 * (size_t)c + k];
      lo[k] = x < lo[k] ? x : lo[k];
      hi[k] = x > hi[k] ? x : hi[k];
    }
  double ext = 0.0;
  for (int k = 0; k < 3; ++k) ext = hi[k] - lo[k] > ext ? hi[k] - lo[k] : ext;
  const double scale = ext > 0.0 ? 2097151.0 / ext : 0.0;
  std::vector<unsigned long long> key(N), key2(N);
  std::vector<int> idx(N), idx2(N);
#pragma omp parallel for schedule(static)
  for (int c = 0; c < N; ++c) {
    unsigned long long m = 0;
    for (int k = 0; k < 3; ++k) {
      double q = (d->cofg[3 * (size_t)c + k] - lo[k]) * scale;
      q = q < 0.0 ? 0.0 : (q > 2097151.0 ? 2097151.0 : q);
      m |= spread3((unsigned long long)q) << k;
    }
    // virtual cells after the actual ones (bit 63 is above the 63-bit key)
    if (c >= nAct) m |= 1ull << 63;
    key[c] = m;
    idx[c] = c;
  }
  std::vector<int> count(2048);
  for (int pass = 0; pass < 6; ++pass) {
    const int sh = 11 * pass;
    std::fill(count.begin(), count.end(), 0);
    for (int i = 0; i < N; ++i) count[(key[i] >> sh) & 2047]++;
    int run = 0;
    for (int b = 0; b < 2048; ++b) {
      const int t = count[b];
      count[b] = run;
      run += t;
    }
    for (int i = 0; i < N; ++i) {
      const int dst = count[(key[i] >> sh) & 2047]++;
      key2[dst] = key[i];
      idx2[dst] = idx[i];
    }
    key.swap(key2);
    idx.swap(idx2);
  }
  o.cOld = idx;
  o.cNew.assign(N, 0);
  for (int i = 0; i < N; ++i) o.cNew[o.cOld[i]] = i;
  // faces
  std::vector<int> lowOf(F), highOf(F), start(N + 1, 0);
  for (int f = 0; f < F; ++f) {
    const int a = o.cNew[d->f2c[(long long)f * d->f2cLd] - 1];
    const int b = o.cNew[d->f2c[(long long)f * d->f2cLd + 1] - 1];
    lowOf[f] = a < b ? a : b;
    highOf[f] = a < b ? b : a;
    start[lowOf[f] + 1]++;
  }
  for (int c = 0; c < N; ++c) start[c + 1] += start[c];
  o.fOld.assign(F, 0);
  {
    std::vector<int> fill(start.begin(), start.end() - 1);
    for (int f = 0; f < F; ++f) o.fOld[fill[lowOf[f]]++] = f;
  }
  for (int c = 0; c < N; ++c) {
    // insertion sort of the run by the higher cell, ties by host index
    for (int i = start[c] + 1; i < start[c + 1]; ++i) {
      const int f = o.fOld[i];
      int j = i - 1;
      while (j >= start[c] && (highOf[o.fOld[j]] > highOf[f] ||
                               (highOf[o.fOld[j]] == highOf[f] && o.fOld[j] > f))) {
        o.fOld[j + 1] = o.fOld[j];
        --j;
      }
      o.fOld[j + 1] = f;
    }
  }
  o.fNew.assign(F, 0);
  for (int i = 0; i < F; ++i) o.fNew[o.fOld[i]] = i;
  return o;
}

// Fill device arrays of precision R, in the device numbering o.
template <typename R>
void build_region(rfgpu_region_s *h, const rfgpu_region_desc_t *d, const Phys &ph, const Order &o) {
  cudaStream_t s = h->stream;
  DevAlloc &M = h->mem;
  const int N = d->nCellsTot > 0 ? d->nCellsTot : d->nCells, F = d->nFaces;
  RegionDev<R> g{};
  g.nCells = N;
  g.nAct = d->nCells;
  g.nFaces = F;
  g.ph = ph;
  // ---- cells
  std::vector<double> cofg(3 * (size_t)N), vol(N), epsq(N), moms(6 * (size_t)N);
#pragma omp parallel for schedule(static)
  for (int c = 0; c < N; ++c) {
    const size_t oc = (size_t)o.oc(c);
    for (int k = 0; k < 3; ++k) cofg[(size_t)k * N + c] = d->cofg[3 * oc + k];
    vol[c] = d->vol[oc];
    // eps^2 = (K*vol^(1/3))^3, K = 1 (modflu/RFLU_ModLimiters.F90:386,459-462)
    double ds = std::pow(d->vol[oc], 1.0 / 3.0);
    epsq[c] = ds * ds * ds;
    for (int k = 0; k < 6; ++k) moms[(size_t)k * N + c] = d->xyzMoms[10 * oc + k];
  }
  g.vol = M.upload(vol, s);
  {
    std::vector<float> iv(N);
#pragma omp parallel for schedule(static)
    for (int c = 0; c < N; ++c) iv[c] = (float)(1.0 / vol[c]);
    g.ivolF = M.upload(iv, s);
  }
  g.epsq = M.upload(cast<R>(epsq), s);
  // Mixed path: the WLSQ weight of a member is A d / |d|^2, A the symmetric
  // matrix of the cell's factor terms (RFLU_ModDifferentiationCells.F90:
  // 1029-1042, 1064-1076 expanded): cwt = Axx, Axy, Axz, Ayy, Ayz, Azz
  if (sizeof(R) == 4) {
    std::vector<double> cw(6 * (size_t)N);
#pragma omp parallel for schedule(static)
    for (int c = 0; c < N; ++c) {
      const double *mo = d->xyzMoms + 10 * (size_t)o.oc(c);
      double c11 = 1.0 / mo[0], c22 = 1.0 / mo[2], c33 = 1.0 / mo[5];
      double c12 = -c11 * mo[1];
      double c13 = -(c11 * mo[3] + c12 * c22 * mo[4]);
      double c23 = -c22 * mo[4];
      const double q1 = c11 * c11, q2 = c22 * c22, q3 = c33 * c33;
      cw[c] = q1 + c12 * c12 * q2 + c13 * c13 * q3;
      cw[(size_t)N + c] = c12 * q2 + c13 * c23 * q3;
      cw[2 * (size_t)N + c] = c13 * q3;
      cw[3 * (size_t)N + c] = q2 + c23 * c23 * q3;
      cw[4 * (size_t)N + c] = c23 * q3;
      cw[5 * (size_t)N + c] = q3;
    }
    g.cwt = M.upload(cast<R>(cw), s);
  }
  // ---- stencil SELL
  {
    std::vector<int> cnt(N);
#pragma omp parallel for schedule(static)
    for (int c = 0; c < N; ++c) cnt[c] = d->c2csOffsets[o.oc(c) + 1] - d->c2csOffsets[o.oc(c)];
    Sell sl;
    sl.build(cnt);
    std::vector<int> idx(sl.total, 0);
#pragma omp parallel for schedule(static)
    for (int c = 0; c < N; ++c) {
      const int *mem = d->c2csMembers + d->c2csOffsets[o.oc(c)];
      for (int k = 0; k < cnt[c]; ++k) idx[sl.at(c, k)] = o.nc(mem[k] - 1);  // stored order
    }
    g.stOff = M.upload(sl.off, s);
    g.stCnt = M.upload(sl.cnt, s);
    g.stIdx = M.upload(idx, s);
    g.stTotal = sl.total;
    if (sizeof(R) == 8) {
      // weights on the device with the reference arithmetic (FP64 unit)
      double *dcofg = M.alloc<double>(cofg.size());
      double *dmoms = M.alloc<double>(moms.size());
      cudaMemcpyAsync(dcofg, cofg.data(), cofg.size() * 8, cudaMemcpyHostToDevice, s);
      cudaMemcpyAsync(dmoms, moms.data(), moms.size() * 8, cudaMemcpyHostToDevice, s);
      double *w64 = M.alloc<double>(3 * (size_t)sl.total);
      launch_weights64(g.stOff, g.stCnt, g.stIdx, N, dcofg, dmoms, w64, s, sl.total);
      g.stW = (const R *)w64;
    }
  }
  // ---- faces
  std::vector<int> f2c(2 * (size_t)F);
  std::vector<double> fnA(4 * (size_t)F), fdl(3 * (size_t)F), fdr(3 * (size_t)F);
#pragma omp parallel for schedule(static)
  for (int f = 0; f < F; ++f) {
    const long long of = o.of(f);
    int c1 = o.nc(d->f2c[of * d->f2cLd] - 1), c2 = o.nc(d->f2c[of * d->f2cLd + 1] - 1);
    f2c[f] = c1;
    f2c[(size_t)F + f] = c2;
    for (int k = 0; k < 4; ++k) fnA[4 * (size_t)f + k] = d->fn[4 * of + k];
    for (int k = 0; k < 3; ++k) {
      double xc = d->fc[3 * of + k];
      fdl[(size_t)k * F + f] = xc - cofg[(size_t)k * N + c1];
      fdr[(size_t)k * F + f] = xc - cofg[(size_t)k * N + c2];
    }
  }
  g.f2c = M.upload(f2c, s);
  g.fnA = M.upload(cast<R>(fnA), s);
  g.fdl = M.upload(cast<R>(fdl), s);
  g.fdr = M.upload(cast<R>(fdr), s);
  g.flux = M.alloc<R>(8 * (size_t)F);
  // ---- boundary faces, patches in order
  std::vector<int> bf2c, bkind;
  std::vector<double> bfnA, bfdA, bpout, bdat;
  for (int ip = 0; ip < d->nPatches; ++ip) {
    const rfgpu_patch_t &p = d->patches[ip];
    const int type = p.bcType == RFGPU_BC_SLIPWALL         ? BK_SLIP
                     : p.bcType == RFGPU_BC_OUTFLOW        ? BK_OUTFLOW
                     : p.bcType == RFGPU_BC_FARFIELD       ? BK_FARFIELD
                     : p.bcType == RFGPU_BC_INFLOW_TOTANG  ? BK_INFLOW_TA
                     : p.bcType == RFGPU_BC_INFLOW_VELTEMP ? BK_INFLOW_VT
                                                           : BK_INJECTION;
    const int nData = p.nData > 0 ? p.nData : 1;
    for (int b = 0; b < p.nBFaces; ++b) {
      int c = o.nc(p.bf2c[b] - 1);
      bf2c.push_back(c);
      const bool withOpt = type == BK_OUTFLOW || type == BK_INFLOW_TA || type == BK_INFLOW_VT;
      bkind.push_back(bk_pack(type, p.spaceOrder, withOpt ? p.bcOptType : 0));
      double pout = 0.0;
      const double *v = p.vals ? p.vals + (size_t)nData * (p.distrib ? b : 0) : nullptr;
      if (type == BK_OUTFLOW && p.bcOptType != RFGPU_BCOPT_SUPERSONIC) pout = v[0];
      bpout.push_back(pout);
      double dat[kBData] = {0};
      if (type == BK_FARFIELD) farfield_state(ph, v, dat);
      if (type == BK_INJECTION) {
        dat[0] = v[0];  // MFRATE
        dat[1] = v[1];  // TEMP
      }
      if (type == BK_INFLOW_TA) inflow_totang_state(ph, v, p.bcOptType, p.bcOptFixed, dat);
      if (type == BK_INFLOW_VT)
        for (int k = 0; k < 5; ++k) dat[k] = v[k];  // U, V, W, T, P
      bdat.insert(bdat.end(), dat, dat + kBData);
      for (int k = 0; k < 4; ++k) bfnA.push_back(p.fn[4 * (size_t)b + k]);
      for (int k = 0; k < 3; ++k) bfdA.push_back(p.fc[3 * (size_t)b + k] - cofg[(size_t)k * N + c]);
    }
  }
  const int B = (int)bf2c.size();
  g.nBFaces = B;
  std::vector<double> bfd(3 * (size_t)B);
  for (int b = 0; b < B; ++b)
    for (int k = 0; k < 3; ++k) bfd[(size_t)k * B + b] = bfdA[3 * (size_t)b + k];
  g.bf2c = M.upload(bf2c, s);
  g.bkind = M.upload(bkind, s);
  g.bpout = M.upload(bpout, s);
  g.bdat = M.upload(cast<R>(bdat), s);
  g.bfnA = M.upload(cast<R>(bfnA), s);
  g.bfd = M.upload(cast<R>(bfd), s);
  g.bflux = M.alloc<R>(8 * (size_t)B);
  // ---- cell -> face lists in the reference accumulation order
  {
    std::vector<int> cnt(N, 0);
    for (int f = 0; f < F; ++f) {
      cnt[f2c[f]]++;
      cnt[f2c[(size_t)F + f]]++;
    }
    for (int b = 0; b < B; ++b) cnt[bf2c[b]]++;
    Sell sl;
    sl.build(cnt);
    std::vector<int> code(sl.total, 0), nb(sl.total, -1);
    std::vector<double> cd(3 * (size_t)sl.total, 0.0);
    std::vector<int> fill(N, 0);
    for (int fh = 0; fh < F; ++fh) {  // host face order: the reference's accumulation order
      const int f = o.nf(fh);
      for (int side = 0; side < 2; ++side) {
        int c = f2c[(size_t)side * F + f];
        long long e = sl.at(c, fill[c]++);
        code[e] = 2 * f + side;
        nb[e] = f2c[(size_t)(1 - side) * F + f];
        const std::vector<double> &fd = side == 0 ? fdl : fdr;
        for (int k = 0; k < 3; ++k) cd[(size_t)k * sl.total + e] = -fd[(size_t)k * F + f];
      }
    }
    for (int b = 0; b < B; ++b) {
      int c = bf2c[b];
      long long e = sl.at(c, fill[c]++);
      code[e] = -(b + 1);
    }
    g.cfOff = M.upload(sl.off, s);
    g.cfCnt = M.upload(sl.cnt, s);
    g.cfCode = M.upload(code, s);
    g.cfNb = M.upload(nb, s);
    g.cfD = M.upload(cast<R>(cd), s);
    g.cfTotal = sl.total;
  }
  // ---- RECONST 2 in a partitioned region: each virtual cell's offsets fc - xc
  // to all of its faces (flux faces, VV and VX faces, the patches' faces on
  // virtual cells) for RFLU_LimitGradCellsSimple, which walks every face of
  // every cell; CSR over the virtual cells, SoA offsets
  if (d->reconst == RFGPU_RECONST_WENO_XYZ && d->spaceOrder > 1 && N > d->nCells) {
    const int nA = d->nCells, nV = N - nA;
    const int nFA = d->nFacesAll > d->nFaces ? d->nFacesAll : d->nFaces;
    std::vector<long long> off(nV + 1, 0);
    auto dev = [&](int oneBased) { return oneBased >= 1 && oneBased <= N ? o.nc(oneBased - 1) : -1; };
    auto each = [&](auto fn) {
      for (int f = 0; f < nFA; ++f)
        for (int k = 0; k < 2; ++k) {
          const int c = dev(d->f2c[(long long)f * d->f2cLd + k]);
          if (c >= nA) fn(c - nA, d->fc + 3 * (size_t)f);
        }
      for (int ip = 0; ip < d->nPatches; ++ip) {
        const rfgpu_patch_t &p = d->patches[ip];
        const int nb = p.nBFacesTot > p.nBFaces ? p.nBFacesTot : p.nBFaces;
        for (int b = 0; b < nb; ++b) {
          const int c = dev(p.bf2c[b]);
          if (c >= nA) fn(c - nA, p.fc + 3 * (size_t)b);
        }
      }
    };
    each([&](int v, const double *) { off[v + 1]++; });
    for (int v = 0; v < nV; ++v) off[v + 1] += off[v];
    const long long P = off[nV];
    std::vector<double> pd(3 * (size_t)P);
    std::vector<long long> fill(off.begin(), off.end() - 1);
    each([&](int v, const double *fcx) {
      const long long e = fill[v]++;
      const int c = nA + v;
      for (int k = 0; k < 3; ++k) pd[(size_t)k * P + e] = fcx[k] - cofg[(size_t)k * N + c];
    });
    g.vposOff = M.upload(off, s);
    g.vposD = M.upload(cast<R>(pd), s);
    g.vposTotal = P;
  }
  // ---- state (FP64 SoA on the FP64 path; float-float pairs on the mixed path)
  if (sizeof(R) == 8) {
    g.cv = M.alloc<double>(5 * (size_t)N);
    g.dv = M.alloc<double>(3 * (size_t)N);
    g.cvOld = ph.rkScheme == RFGPU_RK_SCHEME_4_CLASSICAL ? M.alloc<double>(5 * (size_t)N) : nullptr;
    g.rhsSum = M.alloc<double>(5 * (size_t)N);
    cudaMemsetAsync(g.rhsSum, 0, 5 * (size_t)N * sizeof(double), s);
  } else if (h->prec == RFGPU_PREC_SPLIT) {
    // FP64 state, history and 1/V; dv only as the download's image
    g.cv = M.alloc<double>(5 * (size_t)N);
    g.cvOld = ph.rkScheme == RFGPU_RK_SCHEME_4_CLASSICAL ? M.alloc<double>(5 * (size_t)N) : nullptr;
    g.rhsSum = M.alloc<double>(5 * (size_t)N);
    cudaMemsetAsync(g.rhsSum, 0, 5 * (size_t)N * sizeof(double), s);
    std::vector<double> iv(N);
#pragma omp parallel for schedule(static)
    for (int c = 0; c < N; ++c) iv[c] = 1.0 / vol[c];
    g.ivol = M.upload(iv, s);
  } else {
    g.rhsSumF = M.alloc<float>(5 * (size_t)N);
    cudaMemsetAsync(g.rhsSumF, 0, 5 * (size_t)N * sizeof(float), s);
    g.cvF = M.alloc<float>(10 * (size_t)N);
    if (ph.rkScheme == RFGPU_RK_SCHEME_4_CLASSICAL) g.cvOldF = M.alloc<float>(10 * (size_t)N);
  }
  g.rhs = M.alloc<double>(5 * (size_t)N);
  {
    std::vector<double> recx(8 * (size_t)N, 0.0);  // centroid slots; state filled by k_prim
#pragma omp parallel for schedule(static)
    for (int c = 0; c < N; ++c)
      for (int k = 0; k < 3; ++k) recx[8 * (size_t)c + 5 + k] = cofg[(size_t)k * N + c];
    g.rec = M.upload(cast<R>(recx), s);
  }
  g.grad = M.alloc<R>(16 * (size_t)N);
  g.gradRaw = (d->reconst == RFGPU_RECONST_WENO_XYZ && d->spaceOrder > 1)
                  ? M.alloc<R>((sizeof(R) == 8 ? 32 : 16) * (size_t)N)
                  : nullptr;
  cudaMemsetAsync(g.grad, 0, 16 * (size_t)N * sizeof(R), s);
  g.dtBits = M.alloc<unsigned long long>(1);
  unsigned long long inf = 0x7FF0000000000000ull;
  cudaMemcpyAsync(g.dtBits, &inf, 8, cudaMemcpyHostToDevice, s);
  g.scal = M.alloc<double>(8);
  cudaMemsetAsync(g.scal, 0, 8 * sizeof(double), s);
  g.status = M.alloc<unsigned>(1);
  cudaMemsetAsync(g.status, 0, sizeof(unsigned), s);
  if (!o.cOld.empty()) {
    g.cellNew = M.upload(o.cNew, s);
    g.cellOld = M.upload(o.cOld, s);
  }
  // ---- borders (device numbering)
  size_t maxB = 0;
  h->borders.resize(d->nBorders);
  for (int ib = 0; ib < d->nBorders; ++ib) {
    const rfgpu_border_t &b = d->borders[ib];
    BorderH &bh = h->borders[ib];
    bh.iRegionGlobal = b.iRegionGlobal;
    bh.iBorder = b.iBorder;
    for (int k = 0; k < b.nCellsSend; ++k) bh.send.push_back(o.nc(b.icgSend[k] - 1));
    for (int k = 0; k < b.nCellsRecv; ++k) bh.recv.push_back(o.nc(b.icgRecv[k] - 1));
    bh.dSend = M.upload(bh.send, s);
    bh.dRecv = M.upload(bh.recv, s);
    maxB = std::max(maxB, std::max(bh.send.size(), bh.recv.size()));
  }
  if (d->nBorders > 0) h->bbuf = M.alloc<double>(5 * maxB);
  h->cellNew = g.cellNew;
  h->cellOld = g.cellOld;
  h->nBFaces = B;
  rd<R>(h) = g;
  RegionDev<R> *dregs = M.alloc<RegionDev<R>>(1);
  cudaMemcpyAsync(dregs, &rd<R>(h), sizeof(RegionDev<R>), cudaMemcpyHostToDevice, s);
  h->regsDev = dregs;
  cudaStreamSynchronize(s);  // host vectors above go out of scope
}

template <typename R>
const RegionDev<R> *regs_of(rfgpu_region_s *h) {
  return (const RegionDev<R> *)h->regsDev;
}

constexpr int kXChunks = 8;  // transfer chunks of the mixed path

// Tiles [t0, t1) of chunk k, and its host cells [c0, c1).  With the full 8
// chunks the first and last are smaller (weights 1,2,3,3,3,3,2,1): the first
// download copy starts sooner and the work left after the last upload copy is
// shorter (measured on 12.6 M cells: rfgpu_step_host 14.19 -> 14.11 ms, upload
// + step + download 16.19 -> 16.08 ms against even chunks); regions under 36
// tiles get even chunks.
void chunk_range(const rfgpu_region_s *h, int k, int nk, int &t0, int &t1, size_t &c0,
                 size_t &c1) {
  const int nT = h->work.nCellTiles;
  static const int cum[kXChunks + 1] = {0, 1, 3, 6, 9, 12, 15, 17, 18};
  if (nk == kXChunks && nT >= 2 * cum[kXChunks]) {
    t0 = (int)((long long)nT * cum[k] / cum[kXChunks]);
    t1 = (int)((long long)nT * cum[k + 1] / cum[kXChunks]);
  } else {
    t0 = (int)((long long)nT * k / nk);
    t1 = (int)((long long)nT * (k + 1) / nk);
  }
  c0 = (size_t)t0 * h->work.block;
  c1 = std::min((size_t)t1 * h->work.block, (size_t)h->nCells);
}

int n_chunks(const rfgpu_region_s *h) { return std::min(kXChunks, std::max(1, h->work.nCellTiles)); }

// The second stream, the events and the per-chunk device cell lists of the
// chunked transfers, made on first use.
int transfer_setup(rfgpu_region_s *h) {
  if (h->xstream) return RFGPU_OK;
  const int N = h->nCells;
  const int nk = n_chunks(h);
  std::vector<int> old(N), chunk(N), list(N);
  if (h->cellOld) {
    if (cudaMemcpyAsync(old.data(), h->cellOld, (size_t)N * 4, cudaMemcpyDeviceToHost,
                        h->stream) != cudaSuccess ||
        cudaStreamSynchronize(h->stream) != cudaSuccess)
      return RFGPU_ERR_CUDA;
  } else {
    for (int d = 0; d < N; ++d) old[d] = d;
  }
  std::vector<int> cnt(nk + 1, 0);
  for (int k = 0; k < nk; ++k) {
    int t0, t1;
    size_t c0, c1;
    chunk_range(h, k, nk, t0, t1, c0, c1);
    for (size_t i = c0; i < c1; ++i) chunk[i] = k;
  }
  for (int d = 0; d < N; ++d) cnt[chunk[old[d]] + 1]++;
  for (int k = 0; k < nk; ++k) cnt[k + 1] += cnt[k];
  for (int k = 0; k <= nk; ++k) h->xOff[k] = cnt[k];
  for (int d = 0; d < N; ++d) list[cnt[chunk[old[d]]]++] = d;
  try {
    h->xList = h->mem.upload(list, h->stream);
  } catch (const std::bad_alloc &) {
    return RFGPU_ERR_NOMEM;
  }
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) return RFGPU_ERR_CUDA;
  // conversions run on a stream of the highest priority, so their blocks go
  // before the stage kernels they run beside
  int loPrio = 0, hiPrio = 0;
  cudaDeviceGetStreamPriorityRange(&loPrio, &hiPrio);
  if (cudaStreamCreateWithFlags(&h->xstream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithPriority(&h->cstream, cudaStreamNonBlocking, hiPrio) != cudaSuccess)
    return RFGPU_ERR_CUDA;
  for (cudaEvent_t &e : h->xev)
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return RFGPU_ERR_CUDA;
  for (cudaEvent_t &e : h->cev)
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return RFGPU_ERR_CUDA;
  return RFGPU_OK;
}

// Conversions of chunk k between the staged Fortran images and the device state.
void upload_chunk(rfgpu_region_s *h, int k, const double *cvS, const double *dvS,
                  cudaStream_t s) {
  launch_upload_list<float>(regs_of<float>(h), h->xList + h->xOff[k], h->xOff[k + 1] - h->xOff[k],
                            cvS, dvS, h->prec == RFGPU_PREC_SPLIT, s);
  h->launches++;
}
void download_chunk(rfgpu_region_s *h, int k, double *cvS, double *dvS,
                    cudaStream_t st = nullptr) {
  launch_download_list<float>(regs_of<float>(h), h->xList + h->xOff[k],
                              h->xOff[k + 1] - h->xOff[k], cvS, dvS,
                              h->prec == RFGPU_PREC_SPLIT, st ? st : h->stream);
  h->launches++;
}

int upload_state(rfgpu_region_s *h, const double *cv, const double *dv) {
  cudaStream_t s = h->stream;
  const int N = h->nCells;
  if (h->prec) {  // mixed: DMA copies into the staging buffers, fused conversion, chunk by chunk
    int rc = transfer_setup(h);
    if (rc != RFGPU_OK) return rc;
    cudaStream_t x = h->xstream;
    // the copies start after the work already queued on the region's stream
    if (cudaEventRecord(h->xev[kXChunks], s) != cudaSuccess ||
        cudaStreamWaitEvent(x, h->xev[kXChunks], 0) != cudaSuccess)
      return RFGPU_ERR_CUDA;
    const int nk = n_chunks(h);
    for (int k = 0; k < nk; ++k) {
      int t0, t1;
      size_t c0, c1;
      chunk_range(h, k, nk, t0, t1, c0, c1);
      if (t1 <= t0) continue;
      if (cudaMemcpyAsync(h->stage + 5 * c0, cv + 5 * c0, 5 * (c1 - c0) * 8,
                          cudaMemcpyHostToDevice, x) != cudaSuccess)
        return RFGPU_ERR_CUDA;
      if (dv && cudaMemcpyAsync(h->stage2 + 3 * c0, dv + 3 * c0, 3 * (c1 - c0) * 8,
                                cudaMemcpyHostToDevice, x) != cudaSuccess)
        return RFGPU_ERR_CUDA;
      if (cudaEventRecord(h->xev[k], x) != cudaSuccess ||
          cudaStreamWaitEvent(s, h->xev[k], 0) != cudaSuccess)
        return RFGPU_ERR_CUDA;
      upload_chunk(h, k, h->stage, dv ? h->stage2 : nullptr, s);
    }
    return cuda_rc(cudaGetLastError());
  }
  // FP64 path: staged copies into the SoA state, then records (and dv) from it
  if (cudaMemcpyAsync(h->stage, cv, 5 * (size_t)N * 8, cudaMemcpyHostToDevice, s) != cudaSuccess)
    return RFGPU_ERR_CUDA;
  launch_aos_to_soa(h->stage, h->rd64.cv, N, 5, h->cellNew, s);
  if (dv) {
    if (cudaMemcpyAsync(h->stage, dv, 3 * (size_t)N * 8, cudaMemcpyHostToDevice, s) != cudaSuccess)
      return RFGPU_ERR_CUDA;
    launch_aos_to_soa(h->stage, h->rd64.dv, N, 3, h->cellNew, s);
  }
  launch_prim<double>(regs_of<double>(h), h->work, dv ? 0 : 1, s);
  h->launches += dv ? 3 : 2;
  return cuda_rc(cudaGetLastError());
}

// Groups the cell tiles by transfer phase for rfgpu_step_host, once per region.
// Gradient phase j holds the tiles whose every gathered record (own, stencil
// members, face neighbours) travels in chunks 0..j, so it runs as soon as chunk
// j is converted; update phase k holds the tiles whose first own cell travels
// in chunk k, so chunk k can go back to the host once update phases 0..k ran.
int phase_setup(rfgpu_region_s *h) {
  if (h->phN) return RFGPU_OK;
  const Work &w = h->work;
  const int nT = w.nCellTiles;
  const int nk = n_chunks(h);
  ChunkMap m{};
  m.nk = nk;
  m.block = w.block;
  for (int k = 0; k < nk; ++k) {
    int t0, t1;
    size_t c0, c1;
    chunk_range(h, k, nk, t0, t1, c0, c1);
    m.tEnd[k] = t1;
  }
  cudaStream_t s = h->stream;
  int *d = h->mem.alloc<int>(2 * (size_t)std::max(1, nT));
  std::vector<int> last(nT), first(nT);
  std::vector<Tile> tiles(nT);
  if (nT > 0) {
    if (cudaMemsetAsync(d, 0, (size_t)nT * 4, s) != cudaSuccess ||
        cudaMemsetAsync(d + nT, 0x7f, (size_t)nT * 4, s) != cudaSuccess)
      return RFGPU_ERR_CUDA;
    launch_tile_phases<float>(regs_of<float>(h), w, m, d, d + nT, s);
    h->launches++;
    if (cudaMemcpyAsync(last.data(), d, (size_t)nT * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(first.data(), d + nT, (size_t)nT * 4, cudaMemcpyDeviceToHost, s) !=
            cudaSuccess ||
        cudaMemcpyAsync(tiles.data(), w.cellTiles, (size_t)nT * sizeof(Tile),
                        cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return RFGPU_ERR_CUDA;
  }
  std::vector<Tile> grad, upd;
  grad.reserve(nT);
  upd.reserve(nT);
  auto clampk = [&](int v) { return std::min(nk - 1, std::max(0, v)); };
  for (int j = 0; j < nk; ++j) {
    h->phOff[0][j] = (int)grad.size();
    h->phOff[1][j] = (int)upd.size();
    for (int t = 0; t < nT; ++t) {
      if (clampk(last[t]) == j) grad.push_back(tiles[t]);
      if (clampk(first[t]) == j) upd.push_back(tiles[t]);
    }
  }
  h->phOff[0][nk] = h->phOff[1][nk] = nT;
  h->phGrad = h->mem.upload(grad, s);
  h->phUpd = h->mem.upload(upd, s);
  // The face tables on the host once (the region's own 128-face and
  // 128-boundary-face tiles, whatever face shape a tuning chose).
  const int F = h->nFaces, nFT = (F + w.block - 1) / w.block;
  const int B = h->nBFaces, nBT = (B + w.block - 1) / w.block;
  std::vector<int> f2c(2 * (size_t)F), bf2c(B);
  std::vector<Tile> ftiles(nFT), btiles(nBT);
  if ((nFT > 0 &&
       (cudaMemcpyAsync(f2c.data(), h->rd32.f2c, 2 * (size_t)F * 4, cudaMemcpyDeviceToHost, s) !=
            cudaSuccess ||
        cudaMemcpyAsync(ftiles.data(), h->faceTiles, (size_t)nFT * sizeof(Tile),
                        cudaMemcpyDeviceToHost, s) != cudaSuccess)) ||
      (nBT > 0 &&
       (cudaMemcpyAsync(bf2c.data(), h->rd32.bf2c, (size_t)B * 4, cudaMemcpyDeviceToHost, s) !=
            cudaSuccess ||
        cudaMemcpyAsync(btiles.data(), h->bfaceTiles, (size_t)nBT * sizeof(Tile),
                        cudaMemcpyDeviceToHost, s) != cudaSuccess)) ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return RFGPU_ERR_CUDA;
  // tile lists by phase: list[j] holds the tiles whose phase is j
  auto by_phase = [&](const std::vector<Tile> &all, const std::vector<int> &ph, int slot,
                      Tile *&dev) {
    std::vector<Tile> out;
    out.reserve(all.size());
    for (int j = 0; j < nk; ++j) {
      h->phOff[slot][j] = (int)out.size();
      for (size_t t = 0; t < all.size(); ++t)
        if (ph[t] == j) out.push_back(all[t]);
    }
    h->phOff[slot][nk] = (int)out.size();
    dev = out.empty() ? nullptr : h->mem.upload(out, s);
  };
  const int bs = w.block;
  std::vector<int> u(nT);  // update phase of each cell tile
  for (int t = 0; t < nT; ++t) u[t] = clampk(first[t]);
  // interior faces of the last stage: a 128-face tile runs in the phase of
  // the earliest update tile any of its faces feeds, so update phase k finds
  // every face of its cells done (face phases 0..k run before it)
  std::vector<int> phi(nFT, nk - 1);
  for (int t = 0; t < nFT; ++t)
    for (int f = ftiles[t].first; f < std::min(F, ftiles[t].first + bs); ++f)
      for (int q = 0; q < 2; ++q) phi[t] = std::min(phi[t], u[f2c[(size_t)q * F + f] / bs]);
  by_phase(ftiles, phi, 2, h->phFace);
  if (nT > 0 && h->nSteps >= 2 && h->reconst != RFGPU_RECONST_WENO_XYZ) {
    // the last stage's gradient and boundary faces by phase too (stages after
    // the first, without the WENO pass that needs every gradient): a boundary
    // tile runs in the earliest update phase of its cells; a gradient tile no
    // later than every face and boundary tile that reads its cells'
    // gradients and than every update that rewrites a record it reads
    std::vector<int> gam(nT, nk - 1), beta(nBT, nk - 1);
    int *du = h->mem.upload(u, s);
    int *dg = h->mem.upload(gam, s);
    launch_member_phase<float>(regs_of<float>(h), w, du, dg, s);
    h->launches++;
    if (cudaMemcpyAsync(gam.data(), dg, (size_t)nT * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return RFGPU_ERR_CUDA;
    for (int t = 0; t < nFT; ++t)
      for (int f = ftiles[t].first; f < std::min(F, ftiles[t].first + bs); ++f)
        for (int q = 0; q < 2; ++q) {
          int &g = gam[f2c[(size_t)q * F + f] / bs];
          g = std::min(g, phi[t]);
        }
    for (int t = 0; t < nBT; ++t) {
      const int b0 = btiles[t].first, b1 = std::min(B, b0 + bs);
      for (int b = b0; b < b1; ++b) beta[t] = std::min(beta[t], u[bf2c[b] / bs]);
      for (int b = b0; b < b1; ++b) gam[bf2c[b] / bs] = std::min(gam[bf2c[b] / bs], beta[t]);
    }
    by_phase(tiles, gam, 3, h->phGradL);
    by_phase(btiles, beta, 4, h->phBface);
  }
  if (cudaStreamSynchronize(s) != cudaSuccess) return RFGPU_ERR_CUDA;
  h->phN = nk;
  return RFGPU_OK;
}

// One time step of a host-resident state (mixed path), its transfers
// overlapped with the step: chunk k of cv goes up on the copy stream while a
// conversion stream converts chunk k-1 and the region's stream runs the
// stage-1 gradient phases whose records have all arrived; the last stage runs
// phase by phase (its faces and update always, its gradient and boundary
// faces too when it is not the first stage and has no WENO pass), each phase
// followed by its chunk's conversion on the conversion stream and the copy
// back.  The arithmetic per cell is that of rfgpu_upload + rfgpu_step +
// rfgpu_download.  Second order only (the stage-1 gradient pass carries the
// time step).
int step_host_mixed(rfgpu_region_s *h, double *cv, double *dv, const DtArgs &da) {
  int rc = transfer_setup(h);
  if (rc != RFGPU_OK) return rc;
  rc = phase_setup(h);
  if (rc != RFGPU_OK) return rc;
  cudaStream_t s = h->stream, x = h->xstream;
  const RegionDev<float> *regs = regs_of<float>(h);
  const Work &w = h->work;
  const int nk = h->phN;
  const int nS = h->nSteps;
  const Prof *prof = h->prof.hookp();
  cudaStream_t cs = h->cstream;
  if (cudaEventRecord(h->xev[kXChunks], s) != cudaSuccess ||
      cudaStreamWaitEvent(x, h->xev[kXChunks], 0) != cudaSuccess ||
      cudaStreamWaitEvent(cs, h->xev[kXChunks], 0) != cudaSuccess)
    return RFGPU_ERR_CUDA;
  // upload: copies on x, conversions on cs, the stage-1 gradient phases on s
  // behind the conversions they need (cs runs in order, so the last wait
  // covers every earlier chunk)
  for (int k = 0; k < nk; ++k) {
    int t0, t1;
    size_t c0, c1;
    chunk_range(h, k, nk, t0, t1, c0, c1);
    if (cudaMemcpyAsync(h->stage + 5 * c0, cv + 5 * c0, 5 * (c1 - c0) * 8,
                        cudaMemcpyHostToDevice, x) != cudaSuccess ||
        cudaEventRecord(h->xev[k], x) != cudaSuccess ||
        cudaStreamWaitEvent(cs, h->xev[k], 0) != cudaSuccess)
      return RFGPU_ERR_CUDA;
    upload_chunk(h, k, h->stage, nullptr, cs);
    if (cudaEventRecord(h->cev[k], cs) != cudaSuccess ||
        cudaStreamWaitEvent(s, h->cev[k], 0) != cudaSuccess)
      return RFGPU_ERR_CUDA;
    const int n = h->phOff[0][k + 1] - h->phOff[0][k];
    if (n > 0) {
      launch_grad_tiles<float>(regs, w, h->phGrad + h->phOff[0][k], n, 1, s);
      h->launches++;
    }
  }
  for (int is = 1; is <= nS; ++is) {
    StepArgs sa{is, 1, 0.0, 0, 1, is == 1 ? 1 : 0, da};
    // the last stage runs its interior faces and its update phase by phase,
    // and with phGradL its gradient and boundary faces as well
    const bool allPhased = is == nS && h->phGradL;
    const int parts = (is == 1 ? 0 : SP_GRADIENT) | SP_FLUX |
                      (is == nS ? (h->phFace ? SP_NOFACE : 0) : SP_UPDATE);
    if (!allPhased)
      launch_stage<float>(regs, w, sa, s, &h->launches, h->spaceOrder, h->reconst, prof, parts);
    if (is < nS) continue;
    // last stage phase by phase: the gradients, faces and boundary faces the
    // phase's update tiles need, the update, then each chunk converted and
    // copied back behind it
    for (int k = 0; k < nk; ++k) {
      if (allPhased) {
        const int ng = h->phOff[3][k + 1] - h->phOff[3][k];
        if (ng > 0) {
          launch_grad_tiles<float>(regs, w, h->phGradL + h->phOff[3][k], ng, 0, s);
          h->launches++;
        }
      }
      const int nf = h->phFace ? h->phOff[2][k + 1] - h->phOff[2][k] : 0;
      if (nf > 0) {
        launch_face_tiles<float>(regs, w, h->phFace + h->phOff[2][k], nf, s);
        h->launches++;
      }
      const int nb = h->phBface && allPhased ? h->phOff[4][k + 1] - h->phOff[4][k] : 0;
      if (nb > 0) {
        launch_bface_tiles<float>(regs, w, h->phBface + h->phOff[4][k], nb, s);
        h->launches++;
      }
      const int n = h->phOff[1][k + 1] - h->phOff[1][k];
      if (n > 0) {
        launch_update_tiles<float>(regs, w, h->phUpd + h->phOff[1][k], n, sa, s);
        h->launches++;
      }
      int t0, t1;
      size_t c0, c1;
      chunk_range(h, k, nk, t0, t1, c0, c1);
      // the chunk's conversion (FP64 state and EOS, FP64-pipe bound) on the
      // high-priority conversion stream beside the next phase's FP32 kernels;
      // its copy back behind it
      if (cudaEventRecord(h->cev[k], s) != cudaSuccess ||
          cudaStreamWaitEvent(cs, h->cev[k], 0) != cudaSuccess)
        return RFGPU_ERR_CUDA;
      download_chunk(h, k, h->stage, dv ? h->stage2 : nullptr, cs);
      if (cudaEventRecord(h->xev[k], cs) != cudaSuccess ||
          cudaStreamWaitEvent(x, h->xev[k], 0) != cudaSuccess)
        return RFGPU_ERR_CUDA;
      if (cudaMemcpyAsync(cv + 5 * c0, h->stage + 5 * c0, 5 * (c1 - c0) * 8,
                          cudaMemcpyDeviceToHost, x) != cudaSuccess)
        return RFGPU_ERR_CUDA;
      if (dv && cudaMemcpyAsync(dv + 3 * c0, h->stage2 + 3 * c0, 3 * (c1 - c0) * 8,
                                cudaMemcpyDeviceToHost, x) != cudaSuccess)
        return RFGPU_ERR_CUDA;
    }
  }
  if (cudaGetLastError() != cudaSuccess) return RFGPU_ERR_CUDA;
  return cuda_rc(cudaStreamSynchronize(x));
}

void stage_launch(rfgpu_region_s *h, const StepArgs &a) {
  if (h->prec)
    launch_stage<float>(regs_of<float>(h), h->work, a, h->stream, &h->launches, h->spaceOrder,
                        h->reconst, h->prof.hookp());
  else
    launch_stage<double>(regs_of<double>(h), h->work, a, h->stream, &h->launches, h->spaceOrder,
                         h->reconst, h->prof.hookp());
}

void dt_launch(rfgpu_region_s *h, const DtArgs &a) {
  if (h->prec)
    launch_dt<float>(regs_of<float>(h), h->work, a, h->stream, &h->launches, h->prof.hookp());
  else
    launch_dt<double>(regs_of<double>(h), h->work, a, h->stream, &h->launches, h->prof.hookp());
}

// The launch shapes of rfgpu_tuning_t applied to a Work: tile lists of the
// requested strides over the regions whose cell / face counts are given (in
// batch order), made on first use.
int apply_tuning(Work &w, TileCache &tc, DevAlloc &M, cudaStream_t s, const rfgpu_tuning_t &t,
                 const std::vector<int> &nCells, const std::vector<int> &nFaces) {
  auto okBlock = [](int b) { return b == 0 || b == 64 || b == 128 || b == 256; };
  if (t.gridCap < 0 || !okBlock(t.gradBlock) || !okBlock(t.faceBlock) || !okBlock(t.cellBlock) ||
      t.facesPerThread < 0 || t.facesPerThread > 2 || t.persistentStage < 0 ||
      t.persistentStage > 1)
    return RFGPU_ERR_ARG;
  auto dflt = [](int b) { return b == 0 || b == 128; };
  if (t.persistentStage && !(dflt(t.gradBlock) && dflt(t.faceBlock) && dflt(t.cellBlock) &&
                             t.facesPerThread <= 1))
    return RFGPU_ERR_ARG;  // the persistent kernel walks the default 128-item tiles
  if (t.persistentStage && !w.bar) return RFGPU_ERR_ARG;
  auto list = [&](std::map<int, std::pair<Tile *, int>> &cache, const std::vector<int> &counts,
                  int stride) -> std::pair<Tile *, int> {
    auto it = cache.find(stride);
    if (it != cache.end()) return it->second;
    std::vector<Tile> v;
    for (size_t r = 0; r < counts.size(); ++r) {
      auto a = make_tiles((int)r, counts[r], stride);
      v.insert(v.end(), a.begin(), a.end());
    }
    Tile *d = M.upload(v, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) throw std::bad_alloc();
    return cache[stride] = {d, (int)v.size()};
  };
  try {
    const int gb = t.gradBlock ? t.gradBlock : 128, cb = t.cellBlock ? t.cellBlock : 128;
    const int fb = t.faceBlock ? t.faceBlock : 128, fpt = t.facesPerThread ? t.facesPerThread : 1;
    w.grid = t.gridCap;
    if (gb == 128) {
      w.gradTiles = nullptr;
      w.nGradTiles = 0;
    } else {
      auto p = list(tc.cells, nCells, gb);
      w.gradTiles = p.first;
      w.nGradTiles = p.second;
    }
    w.gradBlock = gb;
    if (cb == 128) {
      w.updTiles = nullptr;
      w.nUpdTiles = 0;
    } else {
      auto p = list(tc.cells, nCells, cb);
      w.updTiles = p.first;
      w.nUpdTiles = p.second;
    }
    w.cellBlock = cb;
    auto p = list(tc.faces, nFaces, fb * fpt);
    w.faceTiles = p.first;
    w.nFaceTiles = p.second;
    w.faceBlock = fb;
    w.facesPerThread = fpt;
    w.coop = t.persistentStage;
  } catch (const std::bad_alloc &) {
    return RFGPU_ERR_NOMEM;
  }
  return RFGPU_OK;
}

void step_launch(rfgpu_region_s *h, double cfl, double dtImposed, double dtMinLimit,
                 double endTime) {
  DtArgs da{cfl, dtImposed, dtMinLimit, endTime, 1, 0.0};
  if (h->prec)
    launch_step<float>(regs_of<float>(h), h->work, da, h->nSteps, h->stream, &h->launches,
                       h->spaceOrder, h->reconst, h->prof.hookp());
  else
    launch_step<double>(regs_of<double>(h), h->work, da, h->nSteps, h->stream, &h->launches,
                        h->spaceOrder, h->reconst, h->prof.hookp());
}

}  // namespace

extern "C" {

int rfgpu_region_create(const rfgpu_region_desc_t *d, rfgpu_region_t *out) {
  if (!out) return RFGPU_ERR_ARG;
  *out = nullptr;
  int rc = check_desc(d);
  if (rc != RFGPU_OK) return rc;
  rfgpu_region_s *h = new (std::nothrow) rfgpu_region_s();
  if (!h) return RFGPU_ERR_NOMEM;
  h->prec = d->precision;
  if (cudaGetDevice(&h->device) != cudaSuccess) {
    delete h;
    return RFGPU_ERR_CUDA;
  }
  h->nCells = d->nCellsTot > 0 ? d->nCellsTot : d->nCells;
  h->nAct = d->nCells;
  h->iRegionGlobal = d->iRegionGlobal;
  h->gvCp = d->gvCp;
  h->gvMol = d->gvMol;
  h->nFaces = d->nFaces;
  h->rkScheme = d->rkScheme;
  h->spaceOrder = d->spaceOrder;
  h->reconst = d->spaceOrder > 1 ? d->reconst : 0;
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete h;
    return RFGPU_ERR_CUDA;
  }
  Phys ph{};
  ph.refCp = d->refCp;
  ph.refGamma = d->refGamma;
  ph.gcRef = d->refCp - d->refCp / d->refGamma;   // MixtPerf_R_CpG
  ph.gvCp = d->gvCp;
  ph.gvMol = d->gvMol;
  ph.gvR = 8314.3 / d->gvMol;                     // MixtPerf_R_M
  ph.gvG = d->gvCp / (d->gvCp - ph.gvR);          // MixtPerf_G_CpR
  ph.gvRinv = 1.0 / ph.gvR;
  ph.epsentr = d->epsentr;
  ph.dissFact = d->dissFact;
  rk_coeffs(d->rkScheme, ph);
  ph.rkScheme = d->rkScheme;
  ph.spaceDiscr = d->spaceDiscr;
  ph.spaceOrder = d->spaceOrder;
  ph.reconst = h->reconst;
  ph.venkatGuard = d->venkatGuard;
  ph.refCpF = (float)ph.refCp;
  ph.refGammaF = (float)ph.refGamma;
  ph.gcRefF = (float)ph.gcRef;
  ph.gvGF = (float)ph.gvG;
  ph.epsentrF = (float)ph.epsentr;
  ph.dissFactF = (float)ph.dissFact;
  ph.ausmSigma = d->ausmSigma;
  ph.ausmKp = d->ausmKp;
  ph.ausmKu = d->ausmKu;
  ph.ausmMInf = d->ausmMInf;
  ph.ausmSigmaF = (float)ph.ausmSigma;
  ph.ausmKpF = (float)ph.ausmKp;
  ph.ausmKuF = (float)ph.ausmKu;
  for (int i = 0; i < 5; ++i) ph.grkF[i] = (float)ph.grk[i];
  h->nSteps = ph.nSteps;
  try {
    const Order order = d->cellOrder == RFGPU_ORDER_LOCALITY ? locality_order(d) : Order{};
    if (h->prec)
      build_region<float>(h, d, ph, order);
    else
      build_region<double>(h, d, ph, order);
    const int block = 128;
    auto ct = make_tiles(0, h->nCells, block);
    auto ft = make_tiles(0, h->nFaces, block);
    auto bt = make_tiles(0, h->nBFaces, block);
    h->cellTiles = h->mem.upload(ct, h->stream);
    h->faceTiles = h->mem.upload(ft, h->stream);
    h->bfaceTiles = h->mem.upload(bt, h->stream);
    h->work = Work{h->cellTiles, h->faceTiles, h->bfaceTiles, (int)ct.size(), (int)ft.size(),
                   (int)bt.size(), 0, block, 1};
    h->tiles.faces[block] = {h->faceTiles, (int)ft.size()};
    h->work.split = h->prec == RFGPU_PREC_SPLIT;
    h->work.bar = h->mem.alloc<GridBar>(1);
    h->work.barSpin = kBarrierSpin;
    cudaMemsetAsync(h->work.bar, 0, sizeof(GridBar), h->stream);
    h->stage = h->mem.alloc<double>(5 * (size_t)h->nCells);
    if (h->prec) h->stage2 = h->mem.alloc<double>(3 * (size_t)h->nCells);
    cudaStreamSynchronize(h->stream);
  } catch (const std::bad_alloc &) {
    h->mem.free_all();
    cudaStreamDestroy(h->stream);
    delete h;
    return RFGPU_ERR_NOMEM;
  }
  rc = upload_state(h, d->cv, d->dv);
  if (rc == RFGPU_OK) rc = cuda_rc(cudaStreamSynchronize(h->stream));
  if (rc != RFGPU_OK) {
    cudaStreamSynchronize(h->stream);
    if (h->xstream) {
      cudaStreamSynchronize(h->xstream);
      cudaStreamSynchronize(h->cstream);
      for (cudaEvent_t e : h->xev)
        if (e) cudaEventDestroy(e);
      for (cudaEvent_t e : h->cev)
        if (e) cudaEventDestroy(e);
      cudaStreamDestroy(h->xstream);
      if (h->cstream) cudaStreamDestroy(h->cstream);
    }
    h->mem.free_all();
    cudaStreamDestroy(h->stream);
    delete h;
    return rc;
  }
  *out = h;
  return RFGPU_OK;
}

int rfgpu_region_destroy(rfgpu_region_t h) {
  if (!h) return RFGPU_ERR_ARG;
  cudaStreamSynchronize(h->stream);
  if (h->graph) cudaGraphExecDestroy(h->graph);
  if (h->evA) cudaEventDestroy(h->evA);
  if (h->evB) cudaEventDestroy(h->evB);
  if (h->xstream) {
    cudaStreamSynchronize(h->xstream);
    cudaStreamSynchronize(h->cstream);
    for (cudaEvent_t e : h->xev)
      if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : h->cev)
      if (e) cudaEventDestroy(e);
    cudaStreamDestroy(h->xstream);
    if (h->cstream) cudaStreamDestroy(h->cstream);
  }
  if (h->t0) cudaEventDestroy(h->t0);
  if (h->t1) cudaEventDestroy(h->t1);
  h->prof.destroy();
  h->mem.free_all();
  cudaStreamDestroy(h->stream);
  delete h;
  return RFGPU_OK;
}

int rfgpu_stage(rfgpu_region_t h, int istage, double dtMin) {
  if (!h || istage < 1 || istage > h->nSteps) return RFGPU_ERR_ARG;
  StepArgs a{istage, 0, dtMin, 0, 1, 0, DtArgs{}};
  stage_launch(h, a);
  return cuda_rc(cudaGetLastError());
}

int rfgpu_dt(rfgpu_region_t h, double cfl, double dtImposed, double dtMinLimit,
             double currentTime, double *dtMin) {
  if (!h || !dtMin) return RFGPU_ERR_ARG;
  DtArgs a{cfl, dtImposed, dtMinLimit, 0.0, 0, currentTime};
  dt_launch(h, a);
  double *scal = h->prec ? h->rd32.scal : h->rd64.scal;
  if (cudaMemcpyAsync(dtMin, scal, 8, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess)
    return RFGPU_ERR_CUDA;
  return cuda_rc(cudaStreamSynchronize(h->stream));
}

int rfgpu_step(rfgpu_region_t h, double cfl, double dtImposed, double dtMinLimit, double endTime) {
  if (!h) return RFGPU_ERR_ARG;
  if (!h->borders.empty()) return RFGPU_ERR_UNSUPPORTED;  // needs its neighbours between stages
  step_launch(h, cfl, dtImposed, dtMinLimit, endTime);
  return cuda_rc(cudaGetLastError());
}

int rfgpu_steps_graph(rfgpu_region_t h, int nSteps, double cfl, double dtImposed,
                      double dtMinLimit, double endTime) {
  if (!h || nSteps < 0) return RFGPU_ERR_ARG;
  if (!h->borders.empty()) return RFGPU_ERR_UNSUPPORTED;
  double key[4] = {cfl, dtImposed, dtMinLimit, endTime};
  if (!h->graph || std::memcmp(key, h->gkey, sizeof(key)) != 0) {
    if (h->graph) {
      cudaGraphExecDestroy(h->graph);
      h->graph = nullptr;
    }
    cudaGraph_t g;
    if (cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
      return RFGPU_ERR_CUDA;
    long long before = h->launches;
    bool profOn = h->prof.on;
    h->prof.on = false;
    step_launch(h, cfl, dtImposed, dtMinLimit, endTime);
    h->prof.on = profOn;
    h->perStep = h->launches - before;  // counted at replay
    h->launches = before;
    if (cudaStreamEndCapture(h->stream, &g) != cudaSuccess) return RFGPU_ERR_CUDA;
    cudaError_t e = cudaGraphInstantiate(&h->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return RFGPU_ERR_CUDA;
    std::memcpy(h->gkey, key, sizeof(key));
  }
  for (int i = 0; i < nSteps; ++i)
    if (cudaGraphLaunch(h->graph, h->stream) != cudaSuccess) return RFGPU_ERR_CUDA;
  h->launches += h->perStep * nSteps;
  return RFGPU_OK;
}

int rfgpu_residual(rfgpu_region_t h, double *rhs) {
  if (!h) return RFGPU_ERR_ARG;
  StepArgs a{1, 0, 0.0, 1, 0, 0, DtArgs{}};
  stage_launch(h, a);
  if (!rhs) return cuda_rc(cudaGetLastError());
  const int N = h->nCells;
  double *drhs = h->prec ? h->rd32.rhs : h->rd64.rhs;
  launch_soa_to_aos(drhs, h->stage, N, 5, h->cellNew, h->stream);
  h->launches++;
  if (cudaMemcpyAsync(rhs, h->stage, 5 * (size_t)N * 8, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess)
    return RFGPU_ERR_CUDA;
  return cuda_rc(cudaStreamSynchronize(h->stream));
}

int rfgpu_download(rfgpu_region_t h, double *cv, double *dv) {
  if (!h) return RFGPU_ERR_ARG;
  const int N = h->nCells;
  if (h->prec) {  // mixed: fused conversion into the staging buffers and DMA copies, chunk by chunk
    if (!cv && !dv) return RFGPU_OK;
    int rc = transfer_setup(h);
    if (rc != RFGPU_OK) return rc;
    cudaStream_t x = h->xstream;
    const int nk = n_chunks(h);
    for (int k = 0; k < nk; ++k) {
      int t0, t1;
      size_t c0, c1;
      chunk_range(h, k, nk, t0, t1, c0, c1);
      if (t1 <= t0) continue;
      download_chunk(h, k, cv ? h->stage : nullptr, dv ? h->stage2 : nullptr);
      if (cudaEventRecord(h->xev[k], h->stream) != cudaSuccess ||
          cudaStreamWaitEvent(x, h->xev[k], 0) != cudaSuccess)
        return RFGPU_ERR_CUDA;
      if (cv && cudaMemcpyAsync(cv + 5 * c0, h->stage + 5 * c0, 5 * (c1 - c0) * 8,
                                cudaMemcpyDeviceToHost, x) != cudaSuccess)
        return RFGPU_ERR_CUDA;
      if (dv && cudaMemcpyAsync(dv + 3 * c0, h->stage2 + 3 * c0, 3 * (c1 - c0) * 8,
                                cudaMemcpyDeviceToHost, x) != cudaSuccess)
        return RFGPU_ERR_CUDA;
    }
    if (cudaGetLastError() != cudaSuccess) return RFGPU_ERR_CUDA;
    return cuda_rc(cudaStreamSynchronize(x));
  }
  if (cv) {
    launch_soa_to_aos(h->rd64.cv, h->stage, N, 5, h->cellNew, h->stream);
    h->launches++;
    if (cudaMemcpyAsync(cv, h->stage, 5 * (size_t)N * 8, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess)
      return RFGPU_ERR_CUDA;
  }
  if (dv) {
    // stage is reused: wait for the cv copy first
    if (cv && cudaStreamSynchronize(h->stream) != cudaSuccess) return RFGPU_ERR_CUDA;
    launch_soa_to_aos(h->rd64.dv, h->stage, N, 3, h->cellNew, h->stream);
    h->launches++;
    if (cudaMemcpyAsync(dv, h->stage, 3 * (size_t)N * 8, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess)
      return RFGPU_ERR_CUDA;
  }
  return cuda_rc(cudaStreamSynchronize(h->stream));
}

int rfgpu_upload(rfgpu_region_t h, const double *cv, const double *dv) {
  if (!h || !cv) return RFGPU_ERR_ARG;
  int rc = upload_state(h, cv, dv);
  if (rc != RFGPU_OK) return rc;
  return cuda_rc(cudaStreamSynchronize(h->stream));
}

int rfgpu_step_host(rfgpu_region_t h, double *cv, double *dv, double cfl, double dtImposed,
                    double dtMinLimit, double endTime) {
  if (!h || !cv) return RFGPU_ERR_ARG;
  if (!h->borders.empty()) return RFGPU_ERR_UNSUPPORTED;  // needs its neighbours between stages
  DtArgs da{cfl, dtImposed, dtMinLimit, endTime, 1, 0.0};
  if (h->prec && h->spaceOrder > 1 && h->work.nCellTiles > 0) {
    try {
      return step_host_mixed(h, cv, dv, da);
    } catch (const std::bad_alloc &) {
      return RFGPU_ERR_NOMEM;
    }
  }
  // FP64 path and first order: the three calls in sequence
  int rc = upload_state(h, cv, nullptr);
  if (rc != RFGPU_OK) return rc;
  step_launch(h, cfl, dtImposed, dtMinLimit, endTime);
  if (cudaGetLastError() != cudaSuccess) return RFGPU_ERR_CUDA;
  return rfgpu_download(h, cv, dv);
}

int rfgpu_download_grad(rfgpu_region_t h, double *grad) {
  if (!h || !grad) return RFGPU_ERR_ARG;
  const int N = h->nCells;
  double *tmp = nullptr;
  if (cudaMalloc(&tmp, 15 * (size_t)N * 8) != cudaSuccess) return RFGPU_ERR_NOMEM;
  if (h->prec)
    launch_grad_export_f32(h->rd32.grad, tmp, N, h->cellNew, h->stream);
  else
    launch_grad_export(h->rd64.grad, tmp, N, h->cellNew, h->stream);
  h->launches++;
  cudaError_t e = cudaMemcpyAsync(grad, tmp, 15 * (size_t)N * 8, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(tmp);
  return cuda_rc(e);
}

int rfgpu_time(rfgpu_region_t h, double *currentTime, double *dtMin) {
  if (!h) return RFGPU_ERR_ARG;
  double sc[4];
  double *scal = h->prec ? h->rd32.scal : h->rd64.scal;
  if (cudaMemcpyAsync(sc, scal, sizeof(sc), cudaMemcpyDeviceToHost, h->stream) != cudaSuccess)
    return RFGPU_ERR_CUDA;
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) return RFGPU_ERR_CUDA;
  if (currentTime) *currentTime = sc[1];
  if (dtMin) *dtMin = sc[2];
  return RFGPU_OK;
}

int rfgpu_set_time(rfgpu_region_t h, double currentTime) {
  if (!h) return RFGPU_ERR_ARG;
  double *scal = h->prec ? h->rd32.scal : h->rd64.scal;
  if (cudaMemcpyAsync(scal + 1, &currentTime, 8, cudaMemcpyHostToDevice, h->stream) != cudaSuccess)
    return RFGPU_ERR_CUDA;
  return cuda_rc(cudaStreamSynchronize(h->stream));
}

int rfgpu_status(rfgpu_region_t h, int *flags) {
  if (!h || !flags) return RFGPU_ERR_ARG;
  const int brc = sync_and_check(h->stream, h->work.bar);
  if (brc != RFGPU_OK) return brc;
  unsigned *st = h->prec ? h->rd32.status : h->rd64.status;
  unsigned v = 0;
  if (cudaMemcpyAsync(&v, st, 4, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess) return RFGPU_ERR_CUDA;
  if (cudaMemsetAsync(st, 0, 4, h->stream) != cudaSuccess) return RFGPU_ERR_CUDA;
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) return RFGPU_ERR_CUDA;
  *flags = (int)v;
  return (v & (RFGPU_ST_NAN | RFGPU_ST_NEGPOS)) ? RFGPU_ERR_STATE : RFGPU_OK;
}

int rfgpu_sync(rfgpu_region_t h) {
  if (!h) return RFGPU_ERR_ARG;
  return sync_and_check(h->stream, h->work.bar);
}

void *rfgpu_stream(rfgpu_region_t h) { return h ? (void *)h->stream : nullptr; }
long long rfgpu_device_bytes(rfgpu_region_t h) { return h ? h->mem.bytes : -1; }
long long rfgpu_launch_count(rfgpu_region_t h) { return h ? h->launches : -1; }

int rfgpu_set_tuning(rfgpu_region_t h, const rfgpu_tuning_t *t) {
  if (!h || !t) return RFGPU_ERR_ARG;
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) return RFGPU_ERR_CUDA;
  const int rc = apply_tuning(h->work, h->tiles, h->mem, h->stream, *t, {h->nCells}, {h->nFaces});
  if (rc != RFGPU_OK) return rc;
  if (h->graph) {
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
  }
  return RFGPU_OK;
}

// ---- borders --------------------------------------------------------------------

int rfgpu_border_copy(rfgpu_region_t src, int iBorder, rfgpu_region_t dst) {
  if (!src || !dst || src == dst || src->prec != dst->prec || iBorder < 1 ||
      iBorder > (int)src->borders.size())
    return RFGPU_ERR_ARG;
  const BorderH &b = src->borders[iBorder - 1];
  if (b.iRegionGlobal != dst->iRegionGlobal || b.iBorder > (int)dst->borders.size())
    return RFGPU_ERR_ARG;
  const BorderH &b2 = dst->borders[b.iBorder - 1];
  if (b2.iRegionGlobal != src->iRegionGlobal || b2.recv.size() != b.send.size())
    return RFGPU_ERR_ARG;
  if (src->gvCp != dst->gvCp || src->gvMol != dst->gvMol) return RFGPU_ERR_UNSUPPORTED;
  if (!src->evA && cudaEventCreateWithFlags(&src->evA, cudaEventDisableTiming) != cudaSuccess)
    return RFGPU_ERR_CUDA;
  if (!dst->evB && cudaEventCreateWithFlags(&dst->evB, cudaEventDisableTiming) != cudaSuccess)
    return RFGPU_ERR_CUDA;
  // dst waits for src's queued work (the state it reads), src's later work
  // waits for the copy (the state it will overwrite)
  if (cudaEventRecord(src->evA, src->stream) != cudaSuccess ||
      cudaStreamWaitEvent(dst->stream, src->evA, 0) != cudaSuccess)
    return RFGPU_ERR_CUDA;
  if (src->prec)
    launch_halo_pair<float>(regs_of<float>(src), regs_of<float>(dst), b.dSend, b2.dRecv,
                            (int)b.send.size(), dst->stream);
  else
    launch_halo_pair<double>(regs_of<double>(src), regs_of<double>(dst), b.dSend, b2.dRecv,
                             (int)b.send.size(), dst->stream);
  if (!b.send.empty()) dst->launches++;
  if (cudaGetLastError() != cudaSuccess || cudaEventRecord(dst->evB, dst->stream) != cudaSuccess ||
      cudaStreamWaitEvent(src->stream, dst->evB, 0) != cudaSuccess)
    return RFGPU_ERR_CUDA;
  return RFGPU_OK;
}

int rfgpu_border_pack(rfgpu_region_t h, int iBorder, double *sendBuff) {
  if (!h || !sendBuff || iBorder < 1 || iBorder > (int)h->borders.size()) return RFGPU_ERR_ARG;
  const BorderH &b = h->borders[iBorder - 1];
  const int n = (int)b.send.size();
  if (n == 0) return RFGPU_OK;
  if (h->prec)
    launch_border_pack<float>(regs_of<float>(h), b.dSend, n, h->bbuf, h->stream);
  else
    launch_border_pack<double>(regs_of<double>(h), b.dSend, n, h->bbuf, h->stream);
  h->launches++;
  if (cudaGetLastError() != cudaSuccess ||
      cudaMemcpyAsync(sendBuff, h->bbuf, 5 * (size_t)n * 8, cudaMemcpyDefault, h->stream) !=
          cudaSuccess)
    return RFGPU_ERR_CUDA;
  return cuda_rc(cudaStreamSynchronize(h->stream));
}

int rfgpu_border_unpack(rfgpu_region_t h, int iBorder, const double *recvBuff) {
  if (!h || !recvBuff || iBorder < 1 || iBorder > (int)h->borders.size()) return RFGPU_ERR_ARG;
  const BorderH &b = h->borders[iBorder - 1];
  const int n = (int)b.recv.size();
  if (n == 0) return RFGPU_OK;
  if (cudaMemcpyAsync(h->bbuf, recvBuff, 5 * (size_t)n * 8, cudaMemcpyDefault, h->stream) !=
      cudaSuccess)
    return RFGPU_ERR_CUDA;
  if (h->prec)
    launch_border_unpack<float>(regs_of<float>(h), b.dRecv, n, h->bbuf, h->stream);
  else
    launch_border_unpack<double>(regs_of<double>(h), b.dRecv, n, h->bbuf, h->stream);
  h->launches++;
  if (cudaGetLastError() != cudaSuccess) return RFGPU_ERR_CUDA;
  return cuda_rc(cudaStreamSynchronize(h->stream));
}

// ---- batches ------------------------------------------------------------------

int rfgpu_batch_create(rfgpu_region_t *regions, int n, rfgpu_batch_t *out) {
  return rfgpu_batch_create_ex(regions, n, 0, out);
}

int rfgpu_batch_create_ex(rfgpu_region_t *regions, int n, int flags, rfgpu_batch_t *out) {
  if (!regions || n <= 0 || !out || (flags & ~RFGPU_BATCH_COUPLED)) return RFGPU_ERR_ARG;
  *out = nullptr;
  int prec = regions[0] ? regions[0]->prec : -1;
  for (int i = 0; i < n; ++i)
    if (!regions[i] || regions[i]->prec != prec) return RFGPU_ERR_ARG;
  const bool coupled = (flags & RFGPU_BATCH_COUPLED) != 0;
  // halo links: every border's send cells go to the receive cells of the
  // neighbour's matching border (RFLU_MPI_CopyWrapper's pairing)
  std::vector<HaloLink> links;
  if (coupled) {
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < i; ++j)
        if (regions[i]->iRegionGlobal == regions[j]->iRegionGlobal || regions[i] == regions[j])
          return RFGPU_ERR_ARG;
    for (int i = 0; i < n; ++i) {
      const rfgpu_region_s *a = regions[i];
      if (a->gvCp != regions[0]->gvCp || a->gvMol != regions[0]->gvMol)
        return RFGPU_ERR_UNSUPPORTED;
      for (const BorderH &b : a->borders) {
        int j = -1;
        for (int k = 0; k < n; ++k)
          if (regions[k]->iRegionGlobal == b.iRegionGlobal) j = k;
        if (j < 0 || b.iBorder > (int)regions[j]->borders.size()) return RFGPU_ERR_ARG;
        const BorderH &b2 = regions[j]->borders[b.iBorder - 1];
        if (b2.iRegionGlobal != a->iRegionGlobal || b2.recv.size() != b.send.size())
          return RFGPU_ERR_ARG;
        for (size_t k = 0; k < b.send.size(); ++k)
          links.push_back(HaloLink{i, b.send[k], j, b2.recv[k]});
      }
    }
  } else {
    for (int i = 0; i < n; ++i)
      if (!regions[i]->borders.empty()) return RFGPU_ERR_UNSUPPORTED;
  }
  rfgpu_batch_s *b = new (std::nothrow) rfgpu_batch_s();
  if (!b) return RFGPU_ERR_NOMEM;
  b->prec = prec;
  b->regs.assign(regions, regions + n);
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete b;
    return RFGPU_ERR_CUDA;
  }
  const int block = 128;
  std::vector<Tile> ct, ft, bt;
  for (int i = 0; i < n; ++i) {
    rfgpu_region_s *h = regions[i];
    cudaStreamSynchronize(h->stream);
    auto a = make_tiles(i, h->nCells, block), f = make_tiles(i, h->nFaces, block),
         c = make_tiles(i, h->nBFaces, block);
    ct.insert(ct.end(), a.begin(), a.end());
    ft.insert(ft.end(), f.begin(), f.end());
    bt.insert(bt.end(), c.begin(), c.end());
    b->nCells.push_back(h->nCells);
    b->nFaces.push_back(h->nFaces);
    b->spaceOrder = std::max(b->spaceOrder, h->spaceOrder);
    // launch the WENO-XYZ pass when any region needs it (it skips the others)
    if (b->reconst != RFGPU_RECONST_WENO_XYZ)
      b->reconst = h->reconst == RFGPU_RECONST_WENO_XYZ ? h->reconst : std::max(b->reconst, h->reconst);
    if (i == 0) b->nSteps = h->nSteps;
    if (h->nSteps != b->nSteps) {
      cudaStreamDestroy(b->stream);
      delete b;
      return RFGPU_ERR_UNSUPPORTED;
    }
  }
  try {
    Tile *dct = b->mem.upload(ct, b->stream), *dft = b->mem.upload(ft, b->stream),
         *dbt = b->mem.upload(bt, b->stream);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    b->work = Work{dct, dft, dbt, (int)ct.size(), (int)ft.size(), (int)bt.size(), sms * 8, block, n};
    b->tiles.faces[block] = {dft, (int)ft.size()};
    b->work.split = prec == RFGPU_PREC_SPLIT;
    b->work.bar = b->mem.alloc<GridBar>(1);
    b->work.barSpin = kBarrierSpin;
    cudaMemsetAsync(b->work.bar, 0, sizeof(GridBar), b->stream);
    if (coupled) {
      b->work.coupled = 1;
      b->work.halo = links.empty() ? nullptr : b->mem.upload(links, b->stream);
      b->work.nHalo = (int)links.size();
    }
    if (prec) {
      std::vector<RegionDev<float>> v;
      for (int i = 0; i < n; ++i) v.push_back(regions[i]->rd32);
      b->regsDev = b->mem.upload(v, b->stream);
    } else {
      std::vector<RegionDev<double>> v;
      for (int i = 0; i < n; ++i) v.push_back(regions[i]->rd64);
      b->regsDev = b->mem.upload(v, b->stream);
    }
    cudaStreamSynchronize(b->stream);
  } catch (const std::bad_alloc &) {
    b->mem.free_all();
    cudaStreamDestroy(b->stream);
    delete b;
    return RFGPU_ERR_NOMEM;
  }
  *out = b;
  return RFGPU_OK;
}

int rfgpu_batch_destroy(rfgpu_batch_t b) {
  if (!b) return RFGPU_ERR_ARG;
  cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  if (b->t0) cudaEventDestroy(b->t0);
  if (b->t1) cudaEventDestroy(b->t1);
  b->prof.destroy();
  b->mem.free_all();
  cudaStreamDestroy(b->stream);
  delete b;
  return RFGPU_OK;
}

static void batch_step_launch(rfgpu_batch_t b, double cfl, double dtImposed, double dtMinLimit,
                              double endTime) {
  DtArgs da{cfl, dtImposed, dtMinLimit, endTime, 1, 0.0};
  if (b->prec)
    launch_step<float>((const RegionDev<float> *)b->regsDev, b->work, da, b->nSteps, b->stream,
                       &b->launches, b->spaceOrder, b->reconst, b->prof.hookp());
  else
    launch_step<double>((const RegionDev<double> *)b->regsDev, b->work, da, b->nSteps, b->stream,
                        &b->launches, b->spaceOrder, b->reconst, b->prof.hookp());
}

int rfgpu_batch_step(rfgpu_batch_t b, double cfl, double dtImposed, double dtMinLimit,
                     double endTime) {
  if (!b) return RFGPU_ERR_ARG;
  batch_step_launch(b, cfl, dtImposed, dtMinLimit, endTime);
  return cuda_rc(cudaGetLastError());
}

int rfgpu_batch_steps_graph(rfgpu_batch_t b, int nSteps, double cfl, double dtImposed,
                            double dtMinLimit, double endTime) {
  if (!b || nSteps < 0) return RFGPU_ERR_ARG;
  double key[4] = {cfl, dtImposed, dtMinLimit, endTime};
  if (!b->graph || std::memcmp(key, b->gkey, sizeof(key)) != 0) {
    if (b->graph) {
      cudaGraphExecDestroy(b->graph);
      b->graph = nullptr;
    }
    cudaGraph_t g;
    if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
      return RFGPU_ERR_CUDA;
    long long before = b->launches;
    bool profOn = b->prof.on;
    b->prof.on = false;
    batch_step_launch(b, cfl, dtImposed, dtMinLimit, endTime);
    b->prof.on = profOn;
    b->perStep = b->launches - before;  // counted at replay
    b->launches = before;
    if (cudaStreamEndCapture(b->stream, &g) != cudaSuccess) return RFGPU_ERR_CUDA;
    cudaError_t e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return RFGPU_ERR_CUDA;
    std::memcpy(b->gkey, key, sizeof(key));
  }
  for (int i = 0; i < nSteps; ++i)
    if (cudaGraphLaunch(b->graph, b->stream) != cudaSuccess) return RFGPU_ERR_CUDA;
  b->launches += b->perStep * nSteps;
  return RFGPU_OK;
}

int rfgpu_batch_set_tuning(rfgpu_batch_t b, const rfgpu_tuning_t *t) {
  if (!b || !t) return RFGPU_ERR_ARG;
  if (cudaStreamSynchronize(b->stream) != cudaSuccess) return RFGPU_ERR_CUDA;
  const int rc = apply_tuning(b->work, b->tiles, b->mem, b->stream, *t, b->nCells, b->nFaces);
  if (rc != RFGPU_OK) return rc;
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  return RFGPU_OK;
}

int rfgpu_batch_sync(rfgpu_batch_t b) {
  if (!b) return RFGPU_ERR_ARG;
  return sync_and_check(b->stream, b->work.bar);
}

int rfgpu_batch_test_barrier(rfgpu_batch_t b, int extra, long long spinCycles) {
  if (!b || extra < 0 || spinCycles < 0) return RFGPU_ERR_ARG;
  if (cudaStreamSynchronize(b->stream) != cudaSuccess) return RFGPU_ERR_CUDA;
  b->work.barExtra = extra;
  b->work.barSpin = spinCycles > 0 ? spinCycles : kBarrierSpin;
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  return RFGPU_OK;
}

void *rfgpu_batch_stream(rfgpu_batch_t b) { return b ? (void *)b->stream : nullptr; }

static int prof_read(ProfState &p, cudaStream_t s, double *ms, long long *count, int n) {
  if (cudaStreamSynchronize(s) != cudaSuccess) return RFGPU_ERR_CUDA;
  for (int k = 0; k < n; ++k) {
    ms[k] = 0.0;
    if (count) count[k] = 0;
  }
  for (auto &sp : p.spans) {
    float t = 0.f;
    if (cudaEventElapsedTime(&t, p.pool[sp.second.first], p.pool[sp.second.second]) != cudaSuccess)
      return RFGPU_ERR_CUDA;
    if (sp.first < n) {
      ms[sp.first] += t;
      if (count) count[sp.first] += 1;
    }
  }
  p.reset();
  return RFGPU_OK;
}

int rfgpu_profile(rfgpu_region_t h, int enable) {
  if (!h) return RFGPU_ERR_ARG;
  cudaStreamSynchronize(h->stream);
  h->prof.on = enable != 0;
  h->prof.reset();
  return RFGPU_OK;
}

int rfgpu_profile_read(rfgpu_region_t h, double *ms, long long *count, int n) {
  if (!h || !ms || n < 0) return RFGPU_ERR_ARG;
  return prof_read(h->prof, h->stream, ms, count, n);
}

int rfgpu_batch_profile(rfgpu_batch_t b, int enable) {
  if (!b) return RFGPU_ERR_ARG;
  cudaStreamSynchronize(b->stream);
  b->prof.on = enable != 0;
  b->prof.reset();
  return RFGPU_OK;
}

int rfgpu_batch_profile_read(rfgpu_batch_t b, double *ms, long long *count, int n) {
  if (!b || !ms || n < 0) return RFGPU_ERR_ARG;
  return prof_read(b->prof, b->stream, ms, count, n);
}

long long rfgpu_batch_launch_count(rfgpu_batch_t b) { return b ? b->launches : -1; }

static int timer_start(cudaEvent_t &t0, cudaEvent_t &t1, cudaStream_t s) {
  if (!t0 && cudaEventCreate(&t0) != cudaSuccess) return RFGPU_ERR_CUDA;
  if (!t1 && cudaEventCreate(&t1) != cudaSuccess) return RFGPU_ERR_CUDA;
  return cuda_rc(cudaEventRecord(t0, s));
}

static int timer_stop(cudaEvent_t t0, cudaEvent_t t1, cudaStream_t s, double *ms) {
  if (!t0 || !t1 || !ms) return RFGPU_ERR_ARG;
  if (cudaEventRecord(t1, s) != cudaSuccess) return RFGPU_ERR_CUDA;
  if (cudaEventSynchronize(t1) != cudaSuccess) return RFGPU_ERR_CUDA;
  float f = 0.f;
  if (cudaEventElapsedTime(&f, t0, t1) != cudaSuccess) return RFGPU_ERR_CUDA;
  *ms = f;
  return RFGPU_OK;
}

int rfgpu_timer_start(rfgpu_region_t h) { return h ? timer_start(h->t0, h->t1, h->stream) : RFGPU_ERR_ARG; }
int rfgpu_timer_stop(rfgpu_region_t h, double *ms) {
  return h ? timer_stop(h->t0, h->t1, h->stream, ms) : RFGPU_ERR_ARG;
}
int rfgpu_batch_timer_start(rfgpu_batch_t b) { return b ? timer_start(b->t0, b->t1, b->stream) : RFGPU_ERR_ARG; }
int rfgpu_batch_timer_stop(rfgpu_batch_t b, double *ms) {
  return b ? timer_stop(b->t0, b->t1, b->stream, ms) : RFGPU_ERR_ARG;
}

int rfgpu_set_device(int device) { return cuda_rc(cudaSetDevice(device)); }

int rfgpu_mem_info(long long *freeBytes, long long *totalBytes) {
  size_t f = 0, t = 0;
  if (cudaMemGetInfo(&f, &t) != cudaSuccess) return RFGPU_ERR_CUDA;
  if (freeBytes) *freeBytes = (long long)f;
  if (totalBytes) *totalBytes = (long long)t;
  return RFGPU_OK;
}

int rfgpu_sm_count(int *sms) {
  if (!sms) return RFGPU_ERR_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return RFGPU_ERR_CUDA;
  return cuda_rc(cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, dev));
}

void *rfgpu_host_alloc(long long bytes) {
  void *p = nullptr;
  if (bytes <= 0 || cudaHostAlloc(&p, (size_t)bytes, cudaHostAllocDefault) != cudaSuccess) return nullptr;
  return p;
}

int rfgpu_host_free(void *p) { return p ? cuda_rc(cudaFreeHost(p)) : RFGPU_ERR_ARG; }

// ---- residual without device allocation -----------------------------------------
// Fixed scratch for rfgpu_residual_noalloc: RFGPU_NOALLOC_SCRATCH_BYTES of
// device memory, reserved in every GPU that loads the library until the
// process exits.  It holds the face fluxes (8 working-precision values per
// interior face) followed by the residual (5 doubles per cell).  Host code must
// not use the symbol itself as a device address: the address comes from
// cudaGetSymbolAddress, taken once per device with that device current.

}  // extern "C"

static __device__ __align__(256) unsigned char g_noallocScratch[RFGPU_NOALLOC_SCRATCH_BYTES];

namespace {
std::mutex g_noallocMutex;
void *g_noallocPtr[256] = {nullptr};
// Makes a device current for a scope and restores the caller's on exit.
struct DeviceScope {
  int prev = -1;
  bool ok = false;
  explicit DeviceScope(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) return;
    ok = prev == dev || cudaSetDevice(dev) == cudaSuccess;
    if (prev == dev) prev = -1;
  }
  ~DeviceScope() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};
}  // namespace

extern "C" {

int rfgpu_residual_noalloc(rfgpu_region_t h, double *rhs) {
  if (!h || !rhs) return RFGPU_ERR_ARG;
  const long long N = h->nCells, F = h->nFaces;
  const long long fluxBytes = F * 8 * (h->prec ? 4 : 8);
  const long long fluxAligned = (fluxBytes + 255) / 256 * 256;
  if (fluxAligned + N * 5 * 8 > (long long)RFGPU_NOALLOC_SCRATCH_BYTES) return RFGPU_ERR_NOALLOC_LIMIT;
  // everything runs with the region's device current: the scratch address
  // is that device's (looked up once per device) and the launches go to the
  // region's stream; the caller's current device is restored on return
  const int dev = h->device;
  if (dev < 0 || dev >= 256) return RFGPU_ERR_CUDA;
  DeviceScope scope(dev);
  if (!scope.ok) return RFGPU_ERR_CUDA;
  void *base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noallocMutex);
    if (!g_noallocPtr[dev]) {
      void *p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noallocScratch) != cudaSuccess || !p) return RFGPU_ERR_CUDA;
      g_noallocPtr[dev] = p;
    }
    base = g_noallocPtr[dev];
  }
  double *drhs = (double *)((unsigned char *)base + fluxAligned);
  // every face flux and every residual entry is written before it is read, so
  // nothing left from an earlier call needs clearing
  if (h->prec)
    launch_residual_scratch<float>(regs_of<float>(h), h->rd32, h->work, h->spaceOrder,
                                   (float *)base, drhs, h->stream);
  else
    launch_residual_scratch<double>(regs_of<double>(h), h->rd64, h->work, h->spaceOrder,
                                    (double *)base, drhs, h->stream);
  if (cudaGetLastError() != cudaSuccess) return RFGPU_ERR_CUDA;
  if (cudaMemcpyAsync(rhs, drhs, (size_t)N * 5 * 8, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess)
    return RFGPU_ERR_CUDA;
  return cuda_rc(cudaStreamSynchronize(h->stream));
}

int rfgpu_mesh_stencils(int nCells, int nVerts, const int *cellVerts, const int *cellNVerts,
                        const int *v2cOffsets, const int *v2c, const double *cofg,
                        int *c2csOffsets, int *c2csMembers, double *xyzMoms) {
  if (nCells <= 0 || nVerts <= 0 || !cellVerts || !cellNVerts || !v2cOffsets || !v2c || !cofg ||
      !c2csOffsets || !c2csMembers || !xyzMoms)
    return RFGPU_ERR_ARG;
  // every index the kernel follows is checked here first
  for (long long c = 0; c < nCells; ++c) {
    const int n = cellNVerts[c];
    if (n < 1 || n > 8) return RFGPU_ERR_ARG;
    for (int a = 0; a < n; ++a)
      if (cellVerts[8 * c + a] < 0 || cellVerts[8 * c + a] >= nVerts) return RFGPU_ERR_ARG;
  }
  if (v2cOffsets[0] != 0) return RFGPU_ERR_ARG;
  for (long long v = 0; v < nVerts; ++v)
    if (v2cOffsets[v + 1] < v2cOffsets[v]) return RFGPU_ERR_ARG;
  const long long nV2c = v2cOffsets[nVerts];
  for (long long e = 0; e < nV2c; ++e)
    if (v2c[e] < 0 || v2c[e] >= nCells) return RFGPU_ERR_ARG;
  const size_t N = (size_t)nCells, K = 40;
  // stream-ordered allocations: no device-wide synchronisation, so a serving
  // loop can build stencils for a new request while its batch runs
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return RFGPU_ERR_CUDA;
  std::vector<void *> bufs;
  auto dalloc = [&](size_t bytes) -> void * {
    void *p = nullptr;
    if (cudaMallocAsync(&p, bytes ? bytes : 1, s) != cudaSuccess) return nullptr;
    bufs.push_back(p);
    return p;
  };
  int rc = RFGPU_OK;
  double *dcofg = (double *)dalloc(3 * N * 8), *dmoms = (double *)dalloc(10 * N * 8);
  int *dcv = (int *)dalloc(8 * N * 4), *dnv = (int *)dalloc(N * 4);
  int *doff = (int *)dalloc(((size_t)nVerts + 1) * 4), *dv2c = (int *)dalloc((size_t)nV2c * 4);
  int *dcnt = (int *)dalloc(N * 4), *dmemb = (int *)dalloc(K * N * 4), *dov = (int *)dalloc(4);
  if (bufs.size() != 9) {
    rc = RFGPU_ERR_NOMEM;
  } else {
    try {
      std::vector<int> cnt(N), memb(K * N);
      int overflow = 0;
      cudaMemcpyAsync(dcofg, cofg, 3 * N * 8, cudaMemcpyHostToDevice, s);
      cudaMemcpyAsync(dcv, cellVerts, 8 * N * 4, cudaMemcpyHostToDevice, s);
      cudaMemcpyAsync(dnv, cellNVerts, N * 4, cudaMemcpyHostToDevice, s);
      cudaMemcpyAsync(doff, v2cOffsets, ((size_t)nVerts + 1) * 4, cudaMemcpyHostToDevice, s);
      if (nV2c > 0) cudaMemcpyAsync(dv2c, v2c, (size_t)nV2c * 4, cudaMemcpyHostToDevice, s);
      cudaMemsetAsync(dov, 0, 4, s);
      launch_mesh_stencils(dcofg, dcv, dnv, doff, dv2c, nCells, dcnt, dmemb, dmoms, dov, s);
      cudaMemcpyAsync(cnt.data(), dcnt, N * 4, cudaMemcpyDeviceToHost, s);
      cudaMemcpyAsync(memb.data(), dmemb, K * N * 4, cudaMemcpyDeviceToHost, s);
      cudaMemcpyAsync(xyzMoms, dmoms, 10 * N * 8, cudaMemcpyDeviceToHost, s);
      cudaMemcpyAsync(&overflow, dov, 4, cudaMemcpyDeviceToHost, s);
      if (cudaStreamSynchronize(s) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
        rc = RFGPU_ERR_CUDA;
      } else if (overflow) {
        rc = RFGPU_ERR_UNSUPPORTED;
      } else {
        c2csOffsets[0] = 0;
        for (size_t c = 0; c < N; ++c) {
          const int n = cnt[c];
          for (int k = 0; k < n; ++k) c2csMembers[c2csOffsets[c] + k] = memb[K * c + k] + 1;
          c2csOffsets[c + 1] = c2csOffsets[c] + n;
        }
      }
    } catch (const std::bad_alloc &) {
      rc = RFGPU_ERR_NOMEM;
    }
  }
  for (void *p : bufs) cudaFreeAsync(p, s);
  cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  return rc;
}

}  // extern "C"
