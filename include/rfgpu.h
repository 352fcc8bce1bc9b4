/*
 * rfgpu.h - C ABI of the GB300 residual engine for RocfluMP.
 *
 * The engine replaces the per-region body of the Runge-Kutta stage loop and
 * the time-step computation of the Fortran solver.  Each entry point names
 * the reference routine(s) it stands in for.  Arrays are passed exactly as the
 * Fortran host holds them (column-major, 1-based cell indices, C_LOC of
 * contiguous arrays); the engine converts them once to 0-based
 * structure-of-arrays device copies and keeps the state resident on the GPU.
 *
 * Error convention: every entry returns an int, RFGPU_OK (0) on success.  The
 * Fortran shim maps non-zero codes onto ModError codes and calls ErrorStop
 * (modfloflu/ModError.F90:486).  Device-detected invalid states (NaN,
 * non-positive density or pressure) are latched in a device status word and
 * reported by rfgpu_status, replacing the host checks of AfterUpdateMP
 * (libfloflu/AfterUpdateMP.F90:134-136).
 *
 * Threading: a handle is used by one host thread at a time.  Calls are
 * stream-ordered and asynchronous; rfgpu_dt, rfgpu_download, rfgpu_status,
 * rfgpu_residual (with a host output) and rfgpu_sync synchronise.
 */
#ifndef RFGPU_H
#define RFGPU_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct rfgpu_region_s *rfgpu_region_t;
typedef struct rfgpu_batch_s *rfgpu_batch_t;

enum {
  RFGPU_OK = 0,
  RFGPU_ERR_ARG = 1,          /* bad pointer / size / index */
  RFGPU_ERR_UNSUPPORTED = 2,  /* option outside the supported envelope */
  RFGPU_ERR_CUDA = 3,         /* CUDA runtime error */
  RFGPU_ERR_NOMEM = 4,        /* device allocation failed */
  RFGPU_ERR_STATE = 5,        /* invalid flow state detected on the device */
  RFGPU_ERR_TIMEOUT = 6,      /* a bounded device wait expired */
  RFGPU_ERR_NOALLOC_LIMIT = 7 /* problem larger than rfgpu_residual_noalloc's fixed scratch */
};

/* status bits returned by rfgpu_status */
enum {
  RFGPU_ST_NAN = 1,     /* RFLU_CheckValidity would stop (NaN rho,u,v,w,p,T) */
  RFGPU_ST_NEGPOS = 2,  /* RFLU_CheckPositivity would stop (rho<=0 or p<=0) */
  RFGPU_ST_PFLOOR = 4,  /* CheckPositivity energy floor applied */
  RFGPU_ST_PCLAMP = 8   /* EnforceBounds clamped a tiny negative pressure */
};

/* values of the keys below (modfloflu/ModParameters.F90) */
enum {
  RFGPU_DISCR_UPW_ROE = 1, RFGPU_DISCR_UPW_HLLC = 3, RFGPU_DISCR_UPW_AUSMPLUS = 4,
  RFGPU_DISCR_UPW_AUSMPLUSUP = 5,
  RFGPU_RECONST_NONE = 0, RFGPU_RECONST_WENO_XYZ = 2, RFGPU_RECONST_LIM_VENKAT = 11,
  RFGPU_RK_SCHEME_4_CLASSICAL = 1, RFGPU_RK_SCHEME_3_WRAY = 2, RFGPU_RK_SCHEME_1_EULER = 3,
  RFGPU_BC_INFLOW_TOTANG = 10, RFGPU_BC_INFLOW_VELTEMP = 11,
  RFGPU_BC_OUTFLOW = 20, RFGPU_BC_SLIPWALL = 60, RFGPU_BC_FARFIELD = 80,
  RFGPU_BC_INJECTION = 90,
  RFGPU_BCOPT_SUPERSONIC = 0, RFGPU_BCOPT_SUBSONIC = 1, RFGPU_BCOPT_MIXED = 2,
  RFGPU_GAS_MODEL_TCPERF = 1, RFGPU_FLOW_EULER = 0,
  RFGPU_PREC_FP64 = 0,   /* everything FP64; bit-identical to the reference order */
  RFGPU_PREC_MIXED = 1,  /* FP32 prim/gradients/limiter/flux with compensated
                            residual sums; float-float (~48-bit) conserved
                            state and RK update; FP32 EOS for the next stage
                            (the energy's low part kept); FP64 cv/dv on
                            download */
  RFGPU_PREC_SPLIT = 2,  /* FP32 prim/gradients/limiter/reconstruction/flux;
                            FP64 residual accumulation, FP64 conserved state
                            and RK update, FP64 EOS of the new state (rounded
                            to FP32 for the next stage's gathers) */
  /* Device numbering.  LOCALITY: cells renumbered along a Morton curve of
   * their centroids and interior faces grouped by their lower-numbered cell,
   * so a block's stencil and face gathers stay within a compact patch of the
   * mesh.  Every per-cell summation keeps the host's order (stencil members
   * as stored, interior faces by ascending host index, then boundary faces),
   * so results do not depend on this choice; arrays crossing the ABI are
   * always in the host's numbering.  HOST: keep the host's numbering. */
  RFGPU_ORDER_LOCALITY = 0, RFGPU_ORDER_HOST = 1
};

/* One boundary patch (modfloflu/ModBndPatch.F90:112-162). */
typedef struct {
  int bcType;            /* RFGPU_BC_SLIPWALL or RFGPU_BC_OUTFLOW */
  int spaceOrder;        /* .bc ORDER: 1 or 2 */
  int bcOptType;         /* outflow, inflow TYPE: BCOPT_*; farfield: the CORR switch (0 only) */
  int nBFaces;
  const int *bf2c;       /* bf2c(nBFaces), 1-based */
  const double *fn;      /* fn(4,nBFaces): unit normal, area */
  const double *fc;      /* fc(3,nBFaces) */
  const double *vals;    /* pPatch%mixt%vals from its first used column: vals(nData,nBFaces)
                            if distrib, else vals(nData,1); outflow: PRESS; farfield: MACH,
                            ATTACK, SLIP, PRESS, TEMP (angles in radians); injection:
                            MFRATE, TEMP; inflow TOTANG: PTOT, TTOT, BETAH, BETAV, MACH;
                            inflow VELTEMP: U, V, W, T, P (modfloflu/ModParameters.F90:
                            452-493) */
  int distrib;
  int nData;             /* leading dimension of vals; 0 is read as 1 */
  int bcOptFixed;        /* inflow TOTANG FIXED switch (BCOPT_FIXED_NO 0 / YES 1) */
  int nBFacesTot;        /* pPatch%nBFacesTot: in a partitioned region the patch's
                            faces on actual cells (1..nBFaces) are followed in bf2c,
                            fn and fc by its faces on virtual cells (FACE_KIND_VB);
                            only RECONST 2's positivity check of the virtual cells
                            reads those.  0 is read as nBFaces */
} rfgpu_patch_t;

/* One border of a partitioned region: the cells it sends to one neighbour
 * region and the virtual cells it receives from it (t_border,
 * modfloflu/ModBorder.F90:87-99).  Send cell k of this border pairs with
 * receive cell k of the neighbour's matching border. */
typedef struct {
  int iRegionGlobal;     /* border%iRegionGlobal: the neighbour region */
  int iBorder;           /* border%iBorder: 1-based index of the matching border in the neighbour */
  int nCellsSend;        /* border%nCellsSend */
  const int *icgSend;    /* border%icgSend(nCellsSend): actual cells of this region, 1-based */
  int nCellsRecv;        /* border%nCellsRecv */
  const int *icgRecv;    /* border%icgRecv(nCellsRecv): virtual cells of this region, 1-based */
} rfgpu_border_t;

/* Everything RFLU_InitFlowSolver has built for one region, plus the numerics
 * keys.  Mirrors t_region / t_grid / t_mixt_input fields
 * (modfloflu/ModDataStruct.F90:100-167, ModGrid.F90:84-317,
 * ModMixture.F90:76-195). */
typedef struct {
  int nCells;            /* actual cells (grid%nCells); see nCellsTot for virtual cells */
  int nFaces;            /* interior faces (nFaces); f2c may have a larger leading dim */
  int f2cLd;             /* leading dimension of f2c (>= 2) */
  const int *f2c;        /* f2c(f2cLd,nFaces), 1-based */
  const double *fn;      /* fn(4,nFaces) */
  const double *fc;      /* fc(3,nFaces) */
  const double *cofg;    /* cofg(3,nCells) */
  const double *vol;     /* vol(nCells) */
  const int *c2csOffsets;/* (nCells+1) 0-based offsets into c2csMembers */
  const int *c2csMembers;/* flattened c2cs(icg)%cellMembs, 1-based */
  const double *xyzMoms; /* xyzMoms(10,nCells) (XYZ_MOM_11..44) */
  int nPatches;
  const rfgpu_patch_t *patches;
  const double *cv;      /* cv(5,nCells) conserved state */
  const double *dv;      /* dv(3,nCells) p, T, a; NULL: computed from cv */
  /* numerics */
  int gasModel, flowModel;
  int spaceDiscr, spaceOrder, reconst, rkScheme;
  double refCp, refGamma;  /* global%refCp, global%refGamma (flux kernels) */
  double gvCp, gvMol;      /* gv(GV_MIXT_CP), gv(GV_MIXT_MOL) (EOS, conversions) */
  double epsentr, dissFact;
  int precision;           /* RFGPU_PREC_* */
  int venkatGuard;         /* 0: limiter term exactly as the reference;
                              1: guard added with the sign of the denominator */
  int cellOrder;           /* RFGPU_ORDER_*: device numbering of cells and faces */
  double ausmSigma, ausmKp, ausmKu, ausmMInf; /* AUSM+up (DISCR 5) SIGMA, KP, KU, MINF
                              (libfloflu/ReadNumericsSection.F90:239-276) */
  /* Partitioned regions.  nCellsTot (grid%nCellsTot) counts the actual cells
   * 1..nCells followed by the virtual cells nCells+1..nCellsTot; 0 means
   * nCells (no virtual cells).  With virtual cells, cofg, vol, c2csOffsets,
   * xyzMoms, cv and dv cover nCellsTot cells, stencil members and f2c may
   * name virtual cells (nFaces holds the actual-actual and actual-virtual
   * faces), and every per-cell array crossing this ABI (cv, dv, rhs, grad)
   * has nCellsTot columns.  As in the reference, gradients and limiter cover
   * all nCellsTot cells (CellGradientsMP), residuals of virtual cells are
   * zero (ZeroDummyCellsMP) and the update, EOS, checks and time step cover
   * the actual cells; virtual cells change only through the border calls
   * below or a coupled batch. */
  int nCellsTot;
  int iRegionGlobal;       /* pRegion%iRegionGlobal: matches borders between regions */
  int nBorders;            /* grid%nBorders */
  const rfgpu_border_t *borders;
  /* Interior faces of every kind in f2c, fn and fc (0 is read as nFaces):
   * the flux faces 1..nFaces (FACE_KIND_AA and AV), then the faces between
   * two virtual cells (FACE_KIND_VV) and between a virtual cell and a cell
   * outside the region (FACE_KIND_VX, modflu/RFLU_ModFaceList.F90:1317-1360),
   * an f2c entry outside 1..nCellsTot marking the outside side.  Only
   * RECONST 2's positivity check of the virtual cells reads faces past nFaces
   * (RFLU_LimitGradCellsSimple walks every face of every cell). */
  int nFacesAll;
} rfgpu_region_desc_t;

/* Register a region: copies and reorders the arrays to device-resident SoA.
 * Replaces nothing in the reference (one-time setup after
 * rocflu/RFLU_InitFlowSolver.F90:1071); refuses options outside the
 * supported envelope with RFGPU_ERR_UNSUPPORTED. */
int rfgpu_region_create(const rfgpu_region_desc_t *desc, rfgpu_region_t *out);
int rfgpu_region_destroy(rfgpu_region_t h);

/* One RK stage for the region (libfloflu/RungeKuttaMP.F90:219-260 and
 * :280-370): RKInitMP, CellGradientsMP, ConvectiveFluxesMP, ZeroResidualsMP,
 * SourceTermsMP, ZeroDummyCellsMP, RKUpdateMP, RFLU_SetVarsContWrapper,
 * AfterUpdateMP.  istage in 1..nrkSteps; dtMin = global%dtMin. */
int rfgpu_stage(rfgpu_region_t h, int istage, double dtMin);

/* RFLU_TimeStepInviscid + RFLU_MinimumTimeStep
 * (rocflu/RFLU_TimeStepping.F90:458,473): returns global%dtMin.  Synchronous. */
int rfgpu_dt(rfgpu_region_t h, double cfl, double dtImposed, double dtMinLimit,
             double currentTime, double *dtMin);

/* One full time step on the device without host round trips: dt as above
 * using the device-resident current time, clipped so time does not pass
 * endTime (rocflu/RFLU_TimeStepping.F90:490-493; endTime <= 0 disables the
 * clip), then nrkSteps stages, then time += dtMin.  A region with borders
 * needs its neighbours between stages: it is stepped through a coupled batch
 * (rfgpu_batch_create_ex) or rfgpu_stage plus the border calls, and gets
 * RFGPU_ERR_UNSUPPORTED here and from rfgpu_steps_graph. */
int rfgpu_step(rfgpu_region_t h, double cfl, double dtImposed, double dtMinLimit,
               double endTime);

/* Capture rfgpu_step in a CUDA graph and replay it nSteps times. */
int rfgpu_steps_graph(rfgpu_region_t h, int nSteps, double cfl, double dtImposed,
                      double dtMinLimit, double endTime);

/* Residual only: CellGradientsMP + ConvectiveFluxesMP (libfloflu/RungeKuttaMP.F90:223-233)
 * on the resident state, which it does not modify.  rhs (5,nCellsTot) host
 * output (zero for virtual cells) or NULL (result stays on the device). */
int rfgpu_residual(rfgpu_region_t h, double *rhs);

/* Host copies: cv(5,nCellsTot), dv(3,nCellsTot); either may be NULL. */
int rfgpu_download(rfgpu_region_t h, double *cv, double *dv);
/* Restart / host edits: cv(5,nCellsTot); dv NULL recomputes dv from cv. */
int rfgpu_upload(rfgpu_region_t h, const double *cv, const double *dv);

/* One time step of a state the host keeps: the body of the time-step loop of
 * rocflu/RFLU_TimeStepping.F90:458-520 (dt, the nrkSteps stages of
 * libfloflu/RungeKuttaMP.F90, time += dtMin) for a caller whose cv lives in its
 * own arrays.  cv(5,nCells) is read and overwritten with the new state; dv
 * (3,nCells) is output only, or NULL.  Results equal rfgpu_upload(cv, NULL) +
 * rfgpu_step + rfgpu_download(cv, dv) bit for bit; on the mixed path at second
 * order the copies overlap the step (the first stage's gradient pass starts on
 * the cells whose neighbourhoods have arrived, the last stage runs in phases
 * and hands cells back as they finish).  Synchronous; pinned host memory lets the copies
 * run at full rate.  Regions with borders: RFGPU_ERR_UNSUPPORTED. */
int rfgpu_step_host(rfgpu_region_t h, double *cv, double *dv, double cfl, double dtImposed,
                    double dtMinLimit, double endTime);

/* Limited gradients of the last residual/stage: grad(3,5,nCellsTot). */
int rfgpu_download_grad(rfgpu_region_t h, double *grad);

/* Time state: current time and last dtMin. */
int rfgpu_time(rfgpu_region_t h, double *currentTime, double *dtMin);
int rfgpu_set_time(rfgpu_region_t h, double currentTime);

/* Latched status bits since the last call (clears them).  Synchronous. */
int rfgpu_status(rfgpu_region_t h, int *flags);
int rfgpu_sync(rfgpu_region_t h);
/* The cudaStream_t the handle launches on. */
void *rfgpu_stream(rfgpu_region_t h);
/* Device bytes held by the handle. */
long long rfgpu_device_bytes(rfgpu_region_t h);
/* Kernel launches issued by the handle since creation. */
long long rfgpu_launch_count(rfgpu_region_t h);
/* Launch shapes of the stage passes, chosen by the autotuner
 * (rocflupicl_gb300/autotune.py) by timing real steps.  Block sizes, faces per
 * thread and the grid leave every result bit for bit unchanged; the persistent
 * stage does on the FP64 path, and on the reduced-precision paths changes
 * results by FP32 rounding at most (the compiler may contract a product into
 * an FMA differently inside the one large kernel).  A zero field keeps the
 * default.  No counterpart in the reference (its loops run serially on the
 * host). */
typedef struct {
  int gridCap;         /* blocks per launch of every tiled pass; a grid smaller than
                          the tile count walks the tiles persistently; 0 = one
                          block per tile */
  int gradBlock;       /* threads (= cells) per block of the gradient + limiter
                          pass: 64, 128 (default) or 256 */
  int faceBlock;       /* threads per block of the interior-face flux pass: 64,
                          128 (default) or 256 */
  int facesPerThread;  /* interior faces per thread of that pass: 1 (default) or 2 */
  int cellBlock;       /* threads (= cells) per block of the residual gather and
                          update pass: 64, 128 (default) or 256 */
  int persistentStage; /* 1: each RK stage is one cooperative launch that runs all
                          its passes over every tile, separated by grid-wide
                          barriers (the block sizes above must then be the
                          defaults); 0: one launch per pass.  A barrier wait is
                          bounded (about a second); one that runs out ends the
                          launch and the next rfgpu_sync / rfgpu_batch_sync /
                          rfgpu_status returns RFGPU_ERR_TIMEOUT */
} rfgpu_tuning_t;
/* RFGPU_ERR_ARG for a shape outside the values above.  Drops a captured
 * graph (the next rfgpu_steps_graph captures again). */
int rfgpu_set_tuning(rfgpu_region_t h, const rfgpu_tuning_t *t);

/* Per-kernel profiler (the engine's counterpart of the reference's ROCPROF
 * FPROFILER_BEGINS/ENDS markers): while enabled, CUDA events are recorded on
 * the handle's stream around every kernel; rfgpu_profile_read synchronises and
 * returns, per kernel class, the summed milliseconds and launch counts, then
 * resets.  Classes: 0 gradient, 1 limiter, 2 face flux, 3 boundary-face flux,
 * 4 gather+update, 5 dt faces, 6 dt boundary faces, 7 dt cells, 8 dt finalize,
 * 9 halo exchange, 10 a whole stage run as one persistent launch.  Graph
 * replays are not profiled. */
#define RFGPU_NPROF 11
int rfgpu_profile(rfgpu_region_t h, int enable);
int rfgpu_profile_read(rfgpu_region_t h, double *ms, long long *count, int n);

/* Stream timers: CUDA events recorded on the handle's stream; stop
 * synchronises on the stop event and returns the elapsed milliseconds. */
int rfgpu_timer_start(rfgpu_region_t h);
int rfgpu_timer_stop(rfgpu_region_t h, double *ms);

/* Device selection for the calling host thread (one process per GPU), and
 * page-locked host buffers for the host<->device copies of a drop-in caller. */
int rfgpu_set_device(int device);
/* Free and total device memory of the current GPU (admission control). */
int rfgpu_mem_info(long long *freeBytes, long long *totalBytes);
/* Streaming multiprocessors of the current GPU (cudaDevAttrMultiProcessorCount):
 * the unit the autotuner sizes persistent grids in. */
int rfgpu_sm_count(int *sms);
void *rfgpu_host_alloc(long long bytes);
int rfgpu_host_free(void *p);

/* Halo exchange between partitioned regions (iBorder is 1-based).
 *
 * rfgpu_border_copy: RFLU_MPI_CopyWrapper for one border of src
 * (modflu/RFLU_ModMPI.F90:564-666, RFLU_MPI_CopyCellData :332-390) followed by
 * RFLU_SetVarsContWrapper of the received virtual cells
 * (libfloflu/RungeKuttaMP.F90:381-396): cv of the border's send cells in src
 * goes to the receive cells of the matching border in dst (the border's
 * iRegionGlobal / iBorder), whose dv and cell records are recomputed.  Both
 * handles must live on the same device; the copy is ordered after the work
 * already queued on both handles' streams, and later work on either waits
 * for it.
 *
 * rfgpu_border_pack / rfgpu_border_unpack: the buffer sides of
 * RFLU_MPI_ISendWrapper / RFLU_MPI_RecvWrapper (RFLU_ModMPI.F90:2469-2555,
 * 2856-2940) for a neighbour in another process: sendBuff(5,nCellsSend) =
 * cv(:,icgSend) and cv(:,icgRecv) = recvBuff(5,nCellsRecv) plus the virtual
 * cells' dv.  The buffers may be host or device memory (a CUDA-aware MPI can
 * take device buffers directly).  Synchronous.  The engine's stage applies
 * the update and AfterUpdateMP in one pass, so a pack after rfgpu_stage sees
 * the state after AfterUpdateMP; the reference's ISendWrapper packs before
 * it, which differs only where AfterUpdateMP changed a border cell
 * (RFGPU_ST_PFLOOR / RFGPU_ST_PCLAMP). */
int rfgpu_border_copy(rfgpu_region_t src, int iBorder, rfgpu_region_t dst);
int rfgpu_border_pack(rfgpu_region_t h, int iBorder, double *sendBuff);
int rfgpu_border_unpack(rfgpu_region_t h, int iBorder, const double *recvBuff);

/* Batches: many regions advanced together, one launch per pass over all
 * regions (a persistent grid walking a tile work list).  Regions of a plain
 * batch are independent solves (each its own time step) and may not have
 * borders.  RFGPU_BATCH_COUPLED makes the batch the regions of one
 * partitioned case on this device (global%nRegionsLocal): one time step, the
 * minimum over the batch (rocflu/RFLU_MinimumTimeStep.F90:131-208, the
 * MPI_Allreduce over local regions), and after every stage's update the halo
 * exchange of every border (RFLU_MPI_CopyWrapper + RFLU_SetVarsContWrapper of
 * the virtual cells) in one launch.  Every border's neighbour must be in the
 * batch (RFGPU_ERR_ARG otherwise) and the regions must share the gas
 * constants (RFGPU_ERR_UNSUPPORTED). */
enum { RFGPU_BATCH_COUPLED = 1 };
int rfgpu_batch_create(rfgpu_region_t *regions, int nRegions, rfgpu_batch_t *out);
int rfgpu_batch_create_ex(rfgpu_region_t *regions, int nRegions, int flags, rfgpu_batch_t *out);
int rfgpu_batch_destroy(rfgpu_batch_t b);
int rfgpu_batch_step(rfgpu_batch_t b, double cfl, double dtImposed, double dtMinLimit,
                     double endTime);
int rfgpu_batch_steps_graph(rfgpu_batch_t b, int nSteps, double cfl, double dtImposed,
                            double dtMinLimit, double endTime);
int rfgpu_batch_sync(rfgpu_batch_t b);
/* Launch shapes of the batch's passes (rfgpu_tuning_t, as for a region). */
int rfgpu_batch_set_tuning(rfgpu_batch_t b, const rfgpu_tuning_t *t);
/* Failure-detection hook for tests (no counterpart in the reference): with
 * extra > 0 the batch's persistent stage launches wait at their grid-wide
 * barriers for `extra` blocks that never arrive, with a wait limit of
 * spinCycles SM clock cycles (0 keeps the default), so the bounded wait runs
 * out and rfgpu_batch_sync returns RFGPU_ERR_TIMEOUT; extra = 0 restores
 * normal operation.  The state of a stage that timed out is not valid. */
int rfgpu_batch_test_barrier(rfgpu_batch_t b, int extra, long long spinCycles);
void *rfgpu_batch_stream(rfgpu_batch_t b);
int rfgpu_batch_profile(rfgpu_batch_t b, int enable);
int rfgpu_batch_profile_read(rfgpu_batch_t b, double *ms, long long *count, int n);
long long rfgpu_batch_launch_count(rfgpu_batch_t b);
int rfgpu_batch_timer_start(rfgpu_batch_t b);
int rfgpu_batch_timer_stop(rfgpu_batch_t b, double *ms);

/* Residual that allocates nothing (no counterpart in the reference; an
 * addition of this library).  For callers that may not allocate device
 * memory: a Fortran or C host whose device memory is budgeted once at start-up
 * (a server admitting work by its HBM footprint, a solver sized to fill the
 * GPU), or code running where the CUDA runtime must not be asked for memory,
 * such as a host callback.  Same result as rfgpu_residual(h, rhs): the
 * CellGradientsMP + ConvectiveFluxesMP residual of the resident state into the
 * caller's host array rhs(5,nCells).  The face fluxes and the residual are
 * staged in one static device array of RFGPU_NOALLOC_SCRATCH_BYTES (32 MiB)
 * that every GPU loading the library reserves until the process exits; a
 * region needs 8*sizeof(working precision) bytes per interior face (rounded
 * up to 256) plus 40 bytes per cell, and larger regions get
 * RFGPU_ERR_NOALLOC_LIMIT before anything runs.  The call runs on the device
 * the region was created on (made current for the call, the caller's current
 * device restored after); the first call on a device looks up the array's
 * device address there (cudaGetSymbolAddress); make that first call before
 * any stream capture.  The mixed path's result equals rfgpu_residual's bit
 * for bit, like the FP64 path's.  All calls
 * share the one array, which keeps the last call's contents: calls whose work
 * overlaps on the GPU (other threads, other handles' streams) race on it and
 * must be serialised by the caller.  Synchronous, like rfgpu_residual. */
#define RFGPU_NOALLOC_SCRATCH_BYTES (32u << 20)
int rfgpu_residual_noalloc(rfgpu_region_t h, double *rhs);

/* Device-side mesh preprocessing: the c2c stencils and WLSQ moments of every
 * cell (RFLU_BuildC2CStencilWrapper, RFLU_ModStencilsCells.F90:750-1416, and
 * the moments of RFLU_ModWeights.F90:1770-1894), one GPU thread per cell,
 * with the same per-cell routine as the host builder of rfmesh.h, so members
 * and moments are identical to it bit for bit.  Inputs (0-based): cell
 * vertices padded to 8 with -1 (8,nCells), vertex counts (nCells),
 * vertex-to-cell lists in ascending cell order (offsets (nVerts+1), cells),
 * centroids cofg(3,nCells).  Outputs: c2csOffsets (nCells+1, 0-based),
 * c2csMembers (1-based, room for 40 per cell), xyzMoms (10,nCells).  Every
 * index is validated on the host first (RFGPU_ERR_ARG); a cell with more
 * than 256 vertex-neighbour entries gives RFGPU_ERR_UNSUPPORTED.
 * Synchronous; allocates and frees its own device buffers. */
int rfgpu_mesh_stencils(int nCells, int nVerts, const int *cellVerts, const int *cellNVerts,
                        const int *v2cOffsets, const int *v2c, const double *cofg,
                        int *c2csOffsets, int *c2csMembers, double *xyzMoms);

/* Device-side mesh preprocessing of a whole box mesh: the face list, face
 * and cell geometry, vertex-to-cell lists, c2c stencils and WLSQ moments
 * (RFLU_BuildFaceList, modflu/RFLU_ModFaceList.F90:784-1609; RFLU_BuildGeometry,
 * modflu/RFLU_ModGeometry.F90:307-672; the stencils and moments as
 * rfgpu_mesh_stencils), the arrays rfmesh.h's host builder makes for the same
 * cells, bit for bit: faces numbered by first encounter sweeping the cells,
 * oriented outward from their first cell, interior faces then the six box
 * patches (XLO, XHI, YLO, YHI, ZLO, ZHI) by the plane their centroid lies on.
 * Inputs: xyz(3,nVerts); cell vertices (8,nCells) 0-based padded with -1, the
 * vertex counts and the cell types (0 tet, 1 hex, 2 prism, 3 pyramid, vertex
 * counts 4/8/6/5), cells numbered by type as rfmesh.h numbers them; the box
 * bounds.  Every index is validated on the host (RFGPU_ERR_ARG); a face on
 * three cells, a boundary face off the box or a non-positive volume gives
 * RFGPU_ERR_ARG, a cell with more than 256 vertex-neighbour entries
 * RFGPU_ERR_UNSUPPORTED.  Synchronous; the results are held by the handle.
 * sizes: nFaces, nMembs, then the boundary faces of the six patches.
 * Outputs in the layouts of rfmesh.h: f2c(2,nFaces) 1-based, fn(4,nFaces),
 * fc(3,nFaces), vol(nCells), cofg(3,nCells), stencil offsets (nCells+1,
 * 0-based) and members (1-based), xyzMoms(10,nCells), vertex-to-cell offsets
 * (nVerts+1) and cells (0-based); per patch bf2c (1-based), fn(4,n), fc(3,n)
 * and the face vertices (4,n) 0-based, -1 for a triangle's fourth.  Any output
 * pointer may be NULL. */
typedef struct rfgpu_mesh_s *rfgpu_mesh_t;
int rfgpu_mesh_build(int nCells, int nVerts, const double *xyz, const int *cellVerts,
                     const int *cellNVerts, const int *cellType, const double lo[3],
                     const double hi[3], rfgpu_mesh_t *out);
int rfgpu_mesh_sizes(rfgpu_mesh_t m, long long sizes[8]);
int rfgpu_mesh_faces(rfgpu_mesh_t m, int *f2c, double *fn, double *fc);
int rfgpu_mesh_cells(rfgpu_mesh_t m, double *vol, double *cofg, int *c2csOffsets,
                     int *c2csMembers, double *xyzMoms, int *v2cOffsets, int *v2c);
int rfgpu_mesh_patch(rfgpu_mesh_t m, int iPatch, int *bf2c, double *fn, double *fc, int *bf2v);
int rfgpu_mesh_destroy(rfgpu_mesh_t m);

#ifdef __cplusplus
}
#endif
#endif
