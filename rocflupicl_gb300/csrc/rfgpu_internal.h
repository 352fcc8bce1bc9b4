// rfgpu_internal.h - device-side data layout shared by the engine's
// translation units (host API, FP64 kernels, mixed-precision kernels).
//
// Layout in HBM (per region, N = nCells, F = nFaces, B = nBFaces).  Data a
// thread streams through is SoA (coalesced); data gathered through an index
// is AoS, one record per cell or face, so a gather touches one 32-byte sector
// (mixed path) instead of one per component:
//   cell state   cv[5][N], rhsSum[5][N], dv[3][N] (p,T,a)        FP64 SoA
//   cell record  rec[N][8] = rho,u,v,w,p,x,y,z                   R    AoS
//   gradients    grad[N][16] = d(rho,u,v,w,p)/d(x,y,z)           R    AoS
//   stencil      SELL-32: member k of cell c at stOff[c/32] + 32*k + c%32;
//                stIdx (0-based); stW[3][stTotal] precomputed WLSQ weights
//                (FP64 path); cwt[6][N] WLSQ factor terms (mixed path,
//                weights rebuilt on the fly from rec x,y,z)
//   cell->face   SELL-32 list in the reference accumulation order (interior
//                faces ascending, then boundary faces by patch); code >= 0:
//                2*face + side, code < 0: -(bface+1); cfNb = other cell,
//                cfD[3] = cofg - fc (limiter vector)
//   faces        f2c[2][F], fnA[F][4] (normal, area), fdl/fdr[3][F] = fc - cofg(c1/c2)
//   boundary     bf2c[B], bfnA[B][4], bfd[3][B], bkind[B], bpout[B], bdat[B][16]
//   scratch      flux[F][8], bflux[B][8] (R, 5 used)
// Cells and faces are in the device numbering (the host's, or a locality
// order chosen at registration, cellNew/cellOld); the face indices stored in
// the cell->face lists keep each cell's host summation order.
// R is double on the FP64 path and float on the mixed path.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace rfgpu {

constexpr int kSlice = 32;

// boundary kind bits
enum { BK_SLIP = 0, BK_OUTFLOW = 1, BK_FARFIELD = 2, BK_INJECTION = 3, BK_INFLOW_TA = 4,
       BK_INFLOW_VT = 5 };
constexpr int kBData = 16;  // per boundary face data slots (bdat)
__host__ __device__ inline int bk_pack(int type, int order, int opt) {
  return type | (order << 4) | (opt << 8);
}

struct Phys {
  double refCp, refGamma, gcRef;    // flux kernels: cp, g, R = cp - cp/g
  double gvR, gvG, gvCp, gvMol;     // EOS / conversions: R = 8314.3/M, g = cp/(cp-R)
  double epsentr, dissFact;
  double ark[5], grk[5];
  int nSteps, rkScheme, spaceDiscr, spaceOrder, reconst, venkatGuard;
  // FP32 copies for the mixed-path kernels (no per-thread FP64 conversions)
  float refCpF, refGammaF, gcRefF, gvGF, epsentrF, dissFactF, grkF[5];
  // AUSM+up parameters (sigma, kp, ku; mInf is read by the reference but its
  // flux function 2 overwrites the factor that uses it)
  double ausmSigma, ausmKp, ausmKu, ausmMInf;
  float ausmSigmaF, ausmKpF, ausmKuF;
  double gvRinv;  // 1 / gvR (mixed-path download EOS)
};

template <typename R>
struct RegionDev {
  // nCells: all cells of the region, actual then virtual (the extent and
  // stride of every per-cell array); nAct: the actual cells, the ones the
  // update, the checks and the time step cover
  int nCells, nFaces, nBFaces, nAct;
  // state.  FP64 path: SoA cv, dv, rhsSum.  The mixed path advances its state
  // as float-float pairs, cvF[2][5][N] (hi rows, then lo rows; the pair's sum
  // carries about 48 significand bits) with the RK increment history in FP32
  // (rhsSumF); its cv and dv exist only as host images, converted in one pass
  // on upload / download.  The split path (R = float, cvF null) keeps cv,
  // cvOld and rhsSum in FP64 SoA like the FP64 path, and no dv on the device.
  double *cv, *cvOld, *rhsSum, *dv, *rhs;
  float *rhsSumF;
  float *cvF, *cvOldF;
  // gathered per-cell records (AoS): rec[8*c..] = rho,u,v,w,p,x,y,z;
  // grad[16*c + 3*v + d] (15 used)
  R *rec, *grad;
  // geometry
  const double *vol;
  const float *ivolF;  // 1/vol in FP32 (mixed-path update)
  const double *ivol;  // 1/vol in FP64 (split-path update)
  const R *epsq;
  const R *cwt;   // [6][N] Axx,Axy,Axz,Ayy,Ayz,Azz: weight = A d/|d|^2 (mixed path)
  // RECONST 2, what the WENO-XYZ pass reads (null otherwise): mixed path the
  // unweighted gradients [N][16]; FP64 path each component's weight
  // s = 1/(g^2 + 1e-15) and s*g, [N][32] (s in 0..14, s*g in 16..30)
  R *gradRaw;
  // stencil (SELL-32)
  const long long *stOff;
  const int *stCnt, *stIdx;
  const R *stW;   // [3][stTotal] precomputed weights (FP64 path)
  long long stTotal;
  // cell -> face (SELL-32)
  const long long *cfOff;
  const int *cfCnt, *cfCode, *cfNb;
  const R *cfD;
  long long cfTotal;
  // RECONST 2 in a partitioned region: per virtual cell (index c - nAct) the
  // offsets fc - xc to all its faces, CSR vposOff[nCells - nAct + 1],
  // vposD[3][vposTotal]; null otherwise
  const long long *vposOff;
  const R *vposD;
  long long vposTotal;
  // faces
  const int *f2c;      // [2][F]
  const R *fnA;        // [F][4] nx,ny,nz,area
  const R *fdl, *fdr;  // [3][F]
  R *flux;             // [F][8] (5 used)
  // boundary faces
  const int *bf2c;
  const R *bfnA;       // [B][4]
  const R *bfd;        // [3][B]
  const int *bkind;
  const double *bpout;
  // per boundary face data [B][kBData], evaluated once on the host:
  //   farfield   ri, pi, qi, ui, vi, wi, machInf
  //   injection  mInj, tInj
  //   inflow TOTANG   ptot, ttot, a02 = g R ttot, cos/sin betah, cos/sin betav,
  //                   fixed, then the prescribed state of the supersonic / mixed
  //                   branch rr, rur, rvr, rwr, rer, pr (slots 8..13)
  //   inflow VELTEMP  ur, vr, wr, tr, pr
  const R *bdat;
  R *bflux;            // [B][8]
  // time step
  unsigned long long *dtBits;
  double *scal;   // [0] dtMin, [1] current time, [2] dtMin of the previous step,
                  // [3..7] ark(1..5)*dtMin of the current step
  unsigned *status;
  // device numbering (null when it is the host's): cellNew[hostCell],
  // cellOld[deviceCell]
  const int *cellNew, *cellOld;
  Phys ph;
};

// A tile of work: blockDim.x consecutive items of one region.
struct Tile {
  int region;
  int first;
};

// One received virtual cell of a coupled batch: the state of cell srcCell of
// region srcRegion goes to cell dstCell of region dstRegion (device numbering).
struct HaloLink {
  int srcRegion, srcCell, dstRegion, dstCell;
};

// Grid-wide barrier of the persistent stage launch: arrivals and generation
// (cleared before every launch) and a sticky error word (bit 0: a bounded
// wait ran out), read and cleared by the host's sync calls.
struct GridBar {
  unsigned count, gen, err, pad;
};

struct Work {
  const Tile *cellTiles, *faceTiles, *bfaceTiles;
  int nCellTiles, nFaceTiles, nBFaceTiles;
  int grid;     // blocks per launch (persistent when smaller than the tile count)
  int block;    // items per tile == threads per block
  int nRegions;
  // coupled batches: one time step for all regions, and the halo exchange
  // after every stage's update
  int coupled;
  const HaloLink *halo;
  int nHalo;
  // tuned launch shapes (zero: 128 threads, one item per thread, the cell
  // tiles above): the gradient pass over gradTiles of gradBlock cells, the
  // interior-face pass over faceTiles of faceBlock * facesPerThread faces
  // (faceBlock threads, facesPerThread faces each), the gather/update pass
  // over updTiles of cellBlock cells
  const Tile *gradTiles, *updTiles;
  int nGradTiles, nUpdTiles;
  int gradBlock, faceBlock, facesPerThread, cellBlock;
  // 1: the regions run the split precision mode (R = float, FP64 state)
  int split;
  // 1: a full stage is one cooperative launch (every pass, separated by
  // grid-wide barriers) instead of one launch per pass
  int coop;
  GridBar *bar;
  // barrier arrivals expected beyond the grid (0; a test sets it so the wait
  // runs out) and the wait's limit in SM clock cycles
  int barExtra;
  long long barSpin;
};

struct DtArgs {
  double cfl, dtImposed, dtMinLimit, endTime;
  int useDeviceTime;  // 1: current time from scal[1] and advance it
  double timeHost;
};

// step parameters (host-side values; dt may alternatively come from the device)
struct StepArgs {
  int istage;
  int useDeviceDt;   // 1: dtMin from scal[0]
  double dtHost;
  int writeRhs;      // 1: store the residual into rhs
  int update;        // 0: residual only (no RK update)
  int fuseDt;        // 1: the gradient pass also reduces the time step (stage 1)
  DtArgs dt;         // time-step parameters when fuseDt
};

// Parts of a stage, for a caller that launches some passes itself over subsets
// of the cell tiles: the gradient pass; the time-step finalisation (when the
// gradient pass reduces it) and the face passes; the update (and halo).
enum { SP_GRADIENT = 1, SP_FLUX = 2, SP_UPDATE = 4, SP_ALL = 7, SP_NOFACE = 8 };

// Host-state step (rfgpu_step_host): the host images move in chunks of cell
// tiles, chunk k covering host cells [tEnd[k-1], tEnd[k]) * block.
struct ChunkMap {
  int nk, block;
  int tEnd[8];
};

// Kernel classes for the per-kernel event profiler.
enum { KP_GRADIENT = 0, KP_LIMITER, KP_FACE_FLUX, KP_BFACE_FLUX, KP_GATHER_UPDATE, KP_DT_FACE,
       KP_DT_BFACE, KP_DT_CELL, KP_DT_FINAL, KP_HALO, KP_STAGE, KP_COUNT };
// KP_GRADIENT times the fused gradient + limiter kernel; KP_LIMITER the
// WENO-XYZ weighting and positivity pass of RECONST 2; KP_DT_FACE and
// KP_DT_BFACE are no longer launched separately (kept for the ABI's class
// numbering); KP_STAGE times a whole stage run as one persistent launch.

// Optional hook called around every kernel launch (phase 0 before, 1 after),
// used to record CUDA events on the launching stream.
struct Prof {
  void (*mark)(void *ctx, int kind, int phase, cudaStream_t s);
  void *ctx;
};

// Launchers, instantiated for R = double (FP64 unit, no FMA contraction) and
// R = float (mixed unit).  `regs` is a device array of RegionDev<R>.
template <typename R>
void launch_prim(const RegionDev<R> *regs, const Work &w, int computeDv, cudaStream_t s);
// Mixed path: fused conversion between the Fortran images cv(5,N), dv(3,N)
// (host numbering, in device staging buffers) and the device state of one
// region (regs[0]), for the device cells list[0..n) (ascending); either image
// may be null where the call allows it.
template <typename R>
void launch_upload_list(const RegionDev<R> *regs, const int *list, int n, const double *cvH,
                        const double *dvH, int split, cudaStream_t s);
template <typename R>
void launch_download_list(const RegionDev<R> *regs, const int *list, int n, double *cvH,
                          double *dvH, int split, cudaStream_t s);
// Halo exchange: the links of a coupled batch (regs indexed by region), or
// one border between two handles (send cells of src -> receive cells of dst,
// device numbering).  Copies the conserved state and rebuilds the received
// cells' dependent variables and records.
template <typename R>
void launch_halo(const RegionDev<R> *regs, const HaloLink *links, int n, cudaStream_t s);
template <typename R>
void launch_halo_pair(const RegionDev<R> *src, const RegionDev<R> *dst, const int *srcCells,
                      const int *dstCells, int n, cudaStream_t s);
// Border buffers in the Fortran layout buf(5,n): pack cv(:,cells) / unpack
// into cv(:,cells) with the dependent variables and records of those cells.
template <typename R>
void launch_border_pack(const RegionDev<R> *g, const int *cells, int n, double *buf,
                        cudaStream_t s);
template <typename R>
void launch_border_unpack(const RegionDev<R> *g, const int *cells, int n, const double *buf,
                          cudaStream_t s);
// Residual with the face fluxes and the result in caller-supplied scratch
// (used by rfgpu_residual_noalloc): rhs in the Fortran layout rhs(5,nCells), host numbering.
template <typename R>
void launch_residual_scratch(const RegionDev<R> *regs, const RegionDev<R> &g, const Work &w,
                             int spaceOrder, R *flux, double *rhs, cudaStream_t s);
template <typename R>
void launch_stage(const RegionDev<R> *regs, const Work &w, const StepArgs &a, cudaStream_t s,
                  long long *launches, int spaceOrder, int reconst, const Prof *prof,
                  int parts = SP_ALL);
// Phases of the host-state step, per cell tile (index into w.cellTiles): the
// last transfer chunk its gradient pass reads from (own record, stencil
// members, face neighbours) and the first chunk among its own cells.
// tileLast must hold zeros and tileFirst values >= m.nk on entry.
template <typename R>
void launch_tile_phases(const RegionDev<R> *regs, const Work &w, const ChunkMap &m,
                        int *tileLast, int *tileFirst, cudaStream_t s);
// The gradient pass (with the stage-1 time-step reduction when fuseDt) and the
// update of one stage over a list of cell tiles.
template <typename R>
void launch_grad_tiles(const RegionDev<R> *regs, const Work &w, const Tile *tiles, int nTiles,
                       int fuseDt, cudaStream_t s);
template <typename R>
void launch_update_tiles(const RegionDev<R> *regs, const Work &w, const Tile *tiles, int nTiles,
                         const StepArgs &a, cudaStream_t s);
// The interior-face pass over a list of 128-face tiles; the boundary-face
// pass over a list of boundary-face tiles.
template <typename R>
void launch_face_tiles(const RegionDev<R> *regs, const Work &w, const Tile *tiles, int nTiles,
                       cudaStream_t s);
template <typename R>
void launch_bface_tiles(const RegionDev<R> *regs, const Work &w, const Tile *tiles, int nTiles,
                        cudaStream_t s);
// Per cell tile, the minimum of tilePhase over the tiles of its cells, their
// stencil members and face neighbours (atomicMin into out).
template <typename R>
void launch_member_phase(const RegionDev<R> *regs, const Work &w, const int *tilePhase, int *out,
                         cudaStream_t s);
template <typename R>
void launch_dt(const RegionDev<R> *regs, const Work &w, const DtArgs &a, cudaStream_t s,
               long long *launches, const Prof *prof);
// One time step: stage 1 with the time-step reduction fused into its gradient
// pass (finalized before the stage's update), then the remaining stages.
template <typename R>
void launch_step(const RegionDev<R> *regs, const Work &w, const DtArgs &da, int nStages,
                 cudaStream_t s, long long *launches, int spaceOrder, int reconst,
                 const Prof *prof);

// Setup kernels of the FP64 unit.  WLSQ weights of every stencil member,
// w64[3][stTotal], with the arithmetic of RFLU_ComputeGradCellsFast_3D
// (modflu/RFLU_ModDifferentiationCells.F90:1029-1080); cofg is [3][N] SoA,
// moms [6][N] (r11,r12,r22,r13,r23,r33).
void launch_weights64(const long long *stOff, const int *stCnt, const int *stIdx, int nCells,
                      const double *cofg, const double *moms, double *w64, cudaStream_t s,
                      long long stTotal);
void launch_to_f32(const double *src, float *dst, long long n, cudaStream_t s);
// c2c stencils (memb[40*c + s], cnt[c]) and moments (moms[10*c + k]) of every
// cell from the connectivity views of rfmesh.h; overflow counts cells whose
// vertex-neighbour list exceeds the builder's capacity.
void launch_mesh_stencils(const double *cofg, const int *cv, const int *nv, const int *v2cOff,
                          const int *v2c, int nCells, int *cnt, int *memb, double *moms,
                          int *overflow, cudaStream_t s);
// Fortran image a(ncomp,N) in host numbering <-> SoA [ncomp][N] in device
// numbering; cellNew maps a host cell to its device cell (null: identity)
void launch_aos_to_soa(const double *aos, double *soa, int N, int ncomp, const int *cellNew,
                       cudaStream_t s);
void launch_soa_to_aos(const double *soa, double *aos, int N, int ncomp, const int *cellNew,
                       cudaStream_t s);
// grad[N][16] -> grad(3,5,N) Fortran image in FP64, host numbering
void launch_grad_export(const double *g16, double *out, int N, const int *cellNew,
                        cudaStream_t s);
void launch_grad_export_f32(const float *g16, double *out, int N, const int *cellNew,
                            cudaStream_t s);

}  // namespace rfgpu
