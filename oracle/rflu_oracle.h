/*
 * rflu_oracle.h - CPU FP64 restatement of RocfluMP's residual / Runge-Kutta
 * stage path.  TEST INFRASTRUCTURE ONLY: the parity tests, the smoke check and
 * the CPU-baseline leg of the benchmark call it as the checker; the engine
 * never links or calls it.
 *
 * Parity status: the reference is Fortran 90 + MPI and cannot be compiled in
 * this environment (no Fortran compiler, no MPI), and its own tests hold no
 * golden vectors for this path, so this restatement is "parity unpinned" with
 * respect to reference outputs.  It is pinned instead to the reference-defined
 * known answers: WLSQ exactness on the linear `gtlin` field, flux consistency,
 * free-stream preservation, discrete conservation and the Sod shock tube
 * against an exact Riemann solution (tests/test_oracle_kats.py).
 *
 * Arrays use the Fortran memory image the reference works on: cv(5,nCells),
 * dv(3,nCells), grad(3,5,nCells), f2c(2,nFaces) with 1-based cell ids, etc.
 */
#ifndef RFLU_ORACLE_H
#define RFLU_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_PATCHES 16

typedef struct {
  int bcType;      /* BC_INFLOW_TOTANG=10, BC_INFLOW_VELTEMP=11, BC_OUTFLOW=20,
                      BC_SLIPWALL=60, BC_FARFIELD=80, BC_INJECTION=90
                      (modfloflu/ModParameters.F90:398-434) */
  int spaceOrder;  /* 1 or 2 */
  int bcOptType;   /* outflow: BCOPT_SUPERSONIC=0, SUBSONIC=1, MIXED=2 */
  int nBFaces;
  const int *bf2c;      /* (nBFaces) 1-based */
  const double *fn;     /* (4,nBFaces) */
  const double *fc;     /* (3,nBFaces) */
  const double *vals;   /* vals(nData,nBFaces) if distrib else vals(nData,1): outflow PRESS;
                           farfield MACH, ATTACK, SLIP, PRESS, TEMP; injection MFRATE, TEMP */
  int distrib;
  int nData;            /* leading dimension of vals (0 read as 1) */
  int bcOptFixed;       /* inflow TOTANG FIXED switch */
  /* pPatch%nBFacesTot: the patch's faces on actual cells (1..nBFaces), then
   * on virtual cells (FACE_KIND_VB); bf2c/fn/fc hold nBFacesTot rows.  0 is
   * read as nBFaces.  Only RFLU_LimitGradCellsSimple walks the VB faces. */
  int nBFacesTot;
} orc_patch_t;

typedef struct {
  int nCells, nFaces, nPatches;
  const int *f2c;       /* (2,nFaces) 1-based */
  const double *fn;     /* (4,nFaces) */
  const double *fc;     /* (3,nFaces) */
  const double *cofg;   /* (3,nCells) */
  const double *vol;    /* (nCells) */
  const int *csOff;     /* (nCells+1) 0-based */
  const int *csMem;     /* (nMembs) 1-based */
  const double *xyzMoms;/* (10,nCells) */
  orc_patch_t patches[ORC_MAX_PATCHES];
  /* numerics (libflu/RFLU_InitInputValues.F90 keys) */
  int spaceDiscr;   /* DISCR_UPW_ROE=1, HLLC=3, AUSMPLUS=4, AUSMPLUSUP=5 */
  int spaceOrder;   /* 1 or 2 */
  int reconst;      /* RECONST_NONE=0, RECONST_WENO_XYZ=2, RECONST_LIM_VENKAT=11 */
  int rkScheme;     /* RK_SCHEME_4_CLASSICAL=1, RK_SCHEME_3_WRAY=2, RK_SCHEME_1_EULER=3 */
  double refCp, refGamma;  /* global%refCp, refGamma: used by the flux kernels */
  double gvCp, gvMol;      /* gv(GV_MIXT_CP), gv(GV_MIXT_MOL): used by EOS/conversions */
  double epsentr, dissFact;
  /* 0: the reference limiter term numer/(denom+1e-12) verbatim; 1: the
   * labelled extension numer/(denom+copysign(1e-12,denom)), which keeps the
   * guard from cancelling a negative denominator (see venkat_term) */
  int venkatGuard;
  /* AUSM+up (DISCR_UPW_AUSMPLUSUP=5) parameters sigma, kp, ku, mInf
   * (libfloflu/ReadNumericsSection.F90:239-276; defaults 1, 0.25, 0.75, 0.1) */
  double ausmSigma, ausmKp, ausmKu, ausmMInf;
  /* grid%nCellsTot: actual cells 1..nCells then virtual cells (0: nCells).
   * Conversions, gradients and limiter cover all nCellsTot cells
   * (CellGradientsMP, RFLU_ModLimiters.F90:393-412, RFLU_ModConvertCv.F90:845),
   * residuals of virtual cells are zeroed (ZeroDummyCellsMP), the update, EOS,
   * checks and time step cover 1..nCells; every per-cell array is sized
   * nCellsTot. */
  int nCellsTot;
  /* Interior faces of every kind (0: nFaces): the flux faces 1..nFaces
   * (FACE_KIND_AA, AV), then FACE_KIND_VV and FACE_KIND_VX faces, which only
   * the virtual cells' face lists hold (tet2f / hex2f / ... of
   * RFLU_LimitGradCellsSimple); f2c/fn/fc hold nFacesAll rows, a VX face's
   * outside side is 0. */
  int nFacesAll;
} orc_region_t;

/* status bits, shared with the engine */
#define ORC_ST_NAN     1  /* RFLU_CheckValidity would stop */
#define ORC_ST_NEGPOS  2  /* RFLU_CheckPositivity would stop */
#define ORC_ST_PFLOOR  4  /* CheckPositivity energy floor applied */
#define ORC_ST_PCLAMP  8  /* EnforceBounds clamped a tiny negative pressure */

/* One RK stage exactly as libfloflu/RungeKuttaMP.F90:219-370 runs it for one
 * region: RKInit, CellGradients, ConvectiveFluxes, SourceTerms round trip,
 * RKUpdate, SetDependentVars(1,nCells), AfterUpdate.  cvOld, rhsSum and grad
 * are caller-owned work arrays ((5,nCells), (5,nCells), (3,5,nCells)); rhs
 * receives the residual.  Returns status bits. */
int orc_rk_stage(const orc_region_t *r, int istage, double dtMin, double *cv, double *dv,
                 double *cvOld, double *rhs, double *rhsSum, double *grad);

/* Residual only: CellGradientsMP + ConvectiveFluxesMP on a private copy of cv
 * (so repeated calls see the same state).  grad may be NULL. */
void orc_residual(const orc_region_t *r, const double *cv, const double *dv, double *rhs,
                  double *grad);

/* Same stage, OpenMP over cells: face fluxes in parallel, then a per-cell
 * gather that adds each cell's face fluxes in the reference's order (interior
 * faces ascending, then patches), so the result is bit-identical to
 * orc_rk_stage.  Used as the multi-core CPU baseline. */
int orc_rk_stage_omp(const orc_region_t *r, int istage, double dtMin, double *cv, double *dv,
                     double *cvOld, double *rhs, double *rhsSum, double *grad, int nThreads);

/* The OpenMP stage's and time step's cell -> face lists, built once per
 * region (orc_rk_stage_omp builds and frees them on every call). */
typedef struct orc_omp_plan_s *orc_omp_plan_t;
orc_omp_plan_t orc_omp_plan_create(const orc_region_t *r);
void orc_omp_plan_destroy(orc_omp_plan_t plan);
int orc_rk_stage_omp_plan(const orc_region_t *r, orc_omp_plan_t plan, int istage, double dtMin,
                          double *cv, double *dv, double *cvOld, double *rhs, double *rhsSum,
                          double *grad, int nThreads);
/* orc_dt with OpenMP over faces and cells; bit-identical to orc_dt. */
double orc_dt_omp(const orc_region_t *r, orc_omp_plan_t plan, const double *cv, const double *dv,
                  double cfl, double dtImposed, double dtMinLimit, double currentTime,
                  int nThreads);

/* RFLU_TimeStepInviscid + RFLU_MinimumTimeStep for one region. */
double orc_dt(const orc_region_t *r, const double *cv, const double *dv, double cfl,
              double dtImposed, double dtMinLimit, double currentTime);

/* RFLU_SetDependentVars (TCPERF) over all cells: dv from cv. */
void orc_set_dv(const orc_region_t *r, const double *cv, double *dv);
/* The same over cells first..last-1 (0-based), e.g. the virtual cells after a
 * halo exchange (RFLU_SetVarsContWrapper(nCells+1,nCellsTot)). */
void orc_set_dv_range(const orc_region_t *r, const double *cv, double *dv, long first, long last);

/* Flux functions on one face for known-answer tests.  left/right = (r,u,v,w,p);
 * n = (nx,ny,nz,nm); returns flux(5). */
void orc_face_flux(const orc_region_t *r, const double *left, const double *right,
                   const double *n, double *flux);

#ifdef __cplusplus
}
#endif
#endif
