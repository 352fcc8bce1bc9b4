// rflu_oracle.cpp - CPU FP64 restatement of RocfluMP's residual / RK stage
// path.  TEST INFRASTRUCTURE ONLY (see rflu_oracle.h): the engine never links
// or calls this file; tests, the smoke check and the benchmark's CPU-baseline
// leg use it as the checker.
//
// Every expression keeps the Fortran evaluation order of the routine it
// restates (left-to-right for operators of equal precedence, no contraction:
// built with -ffp-contract=off).  ksg (PICL sub-grid energy) and the particle
// volume fraction are identically zero: the `#else` (no-PICL) semantics of
// modflu/RFLU_ModConvertCv.F90:589, equal to a PICL build with no particles.
#include "rflu_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// modfloflu/ModParameters.F90
const int BC_INFLOW_TOTANG = 10, BC_INFLOW_VELTEMP = 11, BC_OUTFLOW = 20, BC_SLIPWALL = 60,
          BC_FARFIELD = 80, BC_INJECTION = 90;
const int BCOPT_FIXED_NO = 0;
const int BCOPT_SUPERSONIC = 0, BCOPT_SUBSONIC = 1, BCOPT_MIXED = 2;
const int DISCR_UPW_ROE = 1, DISCR_UPW_HLLC = 3, DISCR_UPW_AUSMPLUS = 4, DISCR_UPW_AUSMPLUSUP = 5;
const int RECONST_LIM_VENKAT = 11;
const int RECONST_WENO_XYZ = 2;  // modfloflu/ModParameters.F90:680
const int RK_SCHEME_4_CLASSICAL = 1, RK_SCHEME_3_WRAY = 2, RK_SCHEME_1_EULER = 3;
const double KSG = 0.0;

// ---- libfloflu/MixtPerf_*.F90 ---------------------------------------------
inline double R_M(double M) { return 8314.3 / M; }                       // MixtPerf_R.F90
inline double R_CpG(double Cp, double G) { return Cp - Cp / G; }         // MixtPerf_R.F90
inline double G_CpR(double Cp, double R) { return Cp / (Cp - R); }       // MixtPerf_G.F90
inline double Eo_DGPUVW(double D, double G, double P, double U, double V, double W, double K) {
  return P / (D * (G - 1.0)) + 0.5 * (U * U + V * V + W * W) + K;        // MixtPerf_E.F90
}
inline double P_DEoGVm2(double D, double Eo, double G, double Vm2, double K) {
  return (G - 1.0) * D * (Eo - 0.5 * Vm2 - K);                            // MixtPerf_P.F90:78
}
inline double T_DPR(double D, double P, double R) { return P / (D * R); }  // MixtPerf_T.F90
inline double C_GRT(double G, double R, double T) { return std::sqrt(G * R * T); }
inline double C_DGP(double D, double G, double P) { return std::sqrt(G * P / D); }
inline double C_GHoVm2(double G, double Ho, double Vm2) { return std::sqrt((G - 1.0) * (Ho - 0.5 * Vm2)); }
inline double Ho_CpTUVW(double Cp, double T, double U, double V, double W, double K) {
  return Cp * T + 0.5 * (U * U + V * V + W * W) + K;                       // MixtPerf_H.F90
}
inline double fmin_f(double a, double b) { return b < a ? b : a; }
inline double fmax_f(double a, double b) { return b > a ? b : a; }

// modflu/RFLU_ModEntropyFixes.F90:95-106
inline double EntropyFixHartenHyman(double l, double d) {
  if (l > d) return l;
  return (l * l + d * d) / (2.0 * d);
}

// ---- flux functions on reconstructed states ---------------------------------

// RFLU_AUSM_FluxFunction, modflu/RFLU_ModAUSMFlux.F90:282-367
void ausm_flux_function(double nx, double ny, double nz, double nm, double fs, double rl,
                        double ul, double vl, double wl, double pl, double Hl, double al,
                        double rr, double ur, double vr, double wr, double pr, double Hr,
                        double ar, double flx[5]) {
  double ql = ul * nx + vl * ny + wl * nz - fs;
  double qr = ur * nx + vr * ny + wr * nz - fs;
  double af = 0.5 * (al + ar);
  double ml = ql / af, mla = std::fabs(ml);
  double mr = qr / af, mra = std::fabs(mr);
  double mlp, wtl, mrm, wtr;
  if (mla <= 1.0) {
    mlp = 0.25 * (ml + 1.0) * (ml + 1.0) + 0.125 * (ml * ml - 1.0) * (ml * ml - 1.0);
    wtl = 0.25 * (ml + 1.0) * (ml + 1.0) * (2.0 - ml) + 0.1875 * ml * (ml * ml - 1.0) * (ml * ml - 1.0);
  } else {
    mlp = 0.5 * (ml + mla);
    wtl = 0.5 * (1.0 + ml / mla);
  }
  if (mra <= 1.0) {
    mrm = -(0.25 * (mr - 1.0) * (mr - 1.0)) - 0.125 * (mr * mr - 1.0) * (mr * mr - 1.0);
    wtr = 0.25 * (mr - 1.0) * (mr - 1.0) * (2.0 + mr) - 0.1875 * mr * (mr * mr - 1.0) * (mr * mr - 1.0);
  } else {
    mrm = 0.5 * (mr - mra);
    wtr = 0.5 * (1.0 - mr / mra);
  }
  double mf = mlp + mrm, mfa = std::fabs(mf);
  double mfp = 0.5 * (mf + mfa), mfm = 0.5 * (mf - mfa);
  double pf = wtl * pl + wtr * pr;
  flx[0] = (af * (mfp * rl + mfm * rr)) * nm;
  flx[1] = (af * (mfp * rl * ul + mfm * rr * ur) + pf * nx) * nm;
  flx[2] = (af * (mfp * rl * vl + mfm * rr * vr) + pf * ny) * nm;
  flx[3] = (af * (mfp * rl * wl + mfm * rr * wr) + pf * nz) * nm;
  flx[4] = (af * (mfp * rl * Hl + mfm * rr * Hr) + pf * fs) * nm;
}

// AUSM+ from reconstructed primitive states, RFLU_ModAUSMFlux.F90:2787-2846
void ausm_states(const orc_region_t *r, const double L[5], const double R[5], const double n[4],
                 double fs, double flx[5]) {
  double cp = r->refCp, g = r->refGamma, gc = R_CpG(cp, g);
  double tl = T_DPR(L[0], L[4], gc);
  double al = C_GRT(g, gc, tl);
  double Hl = Ho_CpTUVW(cp, tl, L[1], L[2], L[3], KSG);
  double tr = T_DPR(R[0], R[4], gc);
  double ar = C_GRT(g, gc, tr);
  double Hr = Ho_CpTUVW(cp, tr, R[1], R[2], R[3], KSG);
  ausm_flux_function(n[0], n[1], n[2], n[3], fs, L[0], L[1], L[2], L[3], L[4], Hl, al, R[0], R[1],
                     R[2], R[3], R[4], Hr, ar, flx);
}

// Roe, RFLU_ModRoeFlux.F90:2725-2855
void roe_states(const orc_region_t *r, const double L[5], const double R[5], const double n[4],
                double fs, double flx[5]) {
  double cp = r->refCp, g = r->refGamma, gc = R_CpG(cp, g);
  double nx = n[0], ny = n[1], nz = n[2], nm = n[3];
  double rl = L[0], ul = L[1], vl = L[2], wl = L[3], pl = L[4];
  double rr = R[0], ur = R[1], vr = R[2], wr = R[3], pr = R[4];
  double tl = T_DPR(rl, pl, gc);
  double Hl = Ho_CpTUVW(cp, tl, ul, vl, wl, KSG);
  double ql = ul * nx + vl * ny + wl * nz - fs;
  double tr = T_DPR(rr, pr, gc);
  double Hr = Ho_CpTUVW(cp, tr, ur, vr, wr, KSG);
  double qr = ur * nx + vr * ny + wr * nz - fs;
  double rh = std::sqrt(rl * rr);
  double wt = rl / (rl + rh);
  double uh = wt * ul + (1.0 - wt) * ur;
  double vh = wt * vl + (1.0 - wt) * vr;
  double wh = wt * wl + (1.0 - wt) * wr;
  double Hh = wt * Hl + (1.0 - wt) * Hr;
  double qh = uh * nx + vh * ny + wh * nz - fs;
  double sh = 0.5 * (uh * uh + vh * vh + wh * wh);
  double ah = C_GHoVm2(g, Hh, 2.0 * sh);
  double l1 = std::fabs(qh - ah), l2 = std::fabs(qh), l5 = std::fabs(qh + ah);
  double efc = r->epsentr * l5;
  l1 = EntropyFixHartenHyman(l1, efc);
  l2 = EntropyFixHartenHyman(l2, efc);
  l5 = EntropyFixHartenHyman(l5, efc);
  double dr = rr - rl, du = ur - ul, de = vr - vl, dw = wr - wl, dp = pr - pl;
  double dq = du * nx + de * ny + dw * nz;
  double dv1 = (dp - rh * ah * dq) / (2.0 * ah * ah);
  double dv5 = (dp + rh * ah * dq) / (2.0 * ah * ah);
  double dv2 = dr - dp / (ah * ah);
  double t1 = l1 * dv1, t2 = l2 * dv2, t3 = l2 * rh, t5 = l5 * dv5;
  double fc[5], fd[5];
  fc[0] = 0.5 * (ql * rl + qr * rr) * nm;
  fc[1] = 0.5 * (ql * rl * ul + pl * nx + qr * rr * ur + pr * nx) * nm;
  fc[2] = 0.5 * (ql * rl * vl + pl * ny + qr * rr * vr + pr * ny) * nm;
  fc[3] = 0.5 * (ql * rl * wl + pl * nz + qr * rr * wr + pr * nz) * nm;
  fc[4] = 0.5 * (ql * rl * Hl + pl * fs + qr * rr * Hr + pr * fs) * nm;
  double df = r->dissFact;
  fd[0] = 0.5 * df * (t1 + t2 + t5) * nm;
  fd[1] = 0.5 * df * (t1 * (uh - nx * ah) + t2 * uh + t3 * (du - nx * dq) + t5 * (uh + nx * ah)) * nm;
  fd[2] = 0.5 * df * (t1 * (vh - ny * ah) + t2 * vh + t3 * (de - ny * dq) + t5 * (vh + ny * ah)) * nm;
  fd[3] = 0.5 * df * (t1 * (wh - nz * ah) + t2 * wh + t3 * (dw - nz * dq) + t5 * (wh + nz * ah)) * nm;
  fd[4] = 0.5 * df * (t1 * (Hh - qh * ah) + t2 * sh + t3 * (uh * du + vh * de + wh * dw - qh * dq) +
                      t5 * (Hh + qh * ah)) * nm;
  for (int k = 0; k < 5; ++k) flx[k] = fc[k] - fd[k];
}

// HLLC, RFLU_ModHLLCFlux.F90:2296-2409.  irl/irr are the reciprocal *cell*
// densities (before reconstruction), which the reference uses in Hl/Hr.
void hllc_states(const orc_region_t *r, const double L[5], const double R[5], double irl,
                 double irr, const double n[4], double fs, double flx[5]) {
  double g = r->refGamma;
  double nx = n[0], ny = n[1], nz = n[2], nm = n[3];
  double rl = L[0], ul = L[1], vl = L[2], wl = L[3], pl = L[4];
  double rr = R[0], ur = R[1], vr = R[2], wr = R[3], pr = R[4];
  double el = Eo_DGPUVW(rl, g, pl, ul, vl, wl, KSG);
  double al = C_DGP(rl, g, pl);
  double ql = ul * nx + vl * ny + wl * nz - fs;
  double Hl = el + irl * pl;
  double er = Eo_DGPUVW(rr, g, pr, ur, vr, wr, KSG);
  double ar = C_DGP(rr, g, pr);
  double qr = ur * nx + vr * ny + wr * nz - fs;
  double Hr = er + irr * pr;
  double wt1 = std::sqrt(rr / rl);
  double wt2 = 1.0 / (1.0 + wt1);
  double us = wt2 * (ul + wt1 * ur);
  double vs = wt2 * (vl + wt1 * vr);
  double ws = wt2 * (wl + wt1 * wr);
  double qs = wt2 * (ql + wt1 * qr);
  double Hs = wt2 * (Hl + wt1 * Hr);
  double Vms = us * us + vs * vs + ws * ws;
  double as = C_GHoVm2(g, Hs, Vms);
  double sl = fmin_f(ql - al, qs - as);
  double sr = fmax_f(qr + ar, qs + as);
  if (sl > 0.0) {
    flx[0] = ql * rl * nm;
    flx[1] = (ql * rl * ul + pl * nx) * nm;
    flx[2] = (ql * rl * vl + pl * ny) * nm;
    flx[3] = (ql * rl * wl + pl * nz) * nm;
    flx[4] = (ql * (rl * el + pl) + pl * fs) * nm;
  } else if (sr < 0.0) {
    flx[0] = qr * rr * nm;
    flx[1] = (qr * rr * ur + pr * nx) * nm;
    flx[2] = (qr * rr * vr + pr * ny) * nm;
    flx[3] = (qr * rr * wr + pr * nz) * nm;
    flx[4] = (qr * (rr * er + pr) + pr * fs) * nm;
  } else {
    double sm = (rr * qr * (sr - qr) - rl * ql * (sl - ql) - pr + pl) / (rr * (sr - qr) - rl * (sl - ql));
    double ps = pl + rl * (ql - sl) * (ql - sm);
    double rs, rus, rvs, rws, res, term;
    if (sm > 0.0) {
      term = 1.0 / (sl - sm);
      rs = term * (sl - ql) * rl;
      rus = term * ((sl - ql) * rl * ul + (ps - pl) * nx);
      rvs = term * ((sl - ql) * rl * vl + (ps - pl) * ny);
      rws = term * ((sl - ql) * rl * wl + (ps - pl) * nz);
      res = term * ((sl - ql) * rl * el + (ps * sm - pl * ql));
    } else {
      term = 1.0 / (sr - sm);
      rs = term * (sr - qr) * rr;
      rus = term * ((sr - qr) * rr * ur + (ps - pr) * nx);
      rvs = term * ((sr - qr) * rr * vr + (ps - pr) * ny);
      rws = term * ((sr - qr) * rr * wr + (ps - pr) * nz);
      res = term * ((sr - qr) * rr * er + (ps * sm - pr * qr));
    }
    flx[0] = sm * rs * nm;
    flx[1] = (sm * rus + ps * nx) * nm;
    flx[2] = (sm * rvs + ps * ny) * nm;
    flx[3] = (sm * rws + ps * nz) * nm;
    flx[4] = (sm * (res + ps) - ps * fs) * nm;
  }
}

// RFLU_AUSMPlusUp_FluxFunction2 (modflu/RFLU_ModAUSMPlusUpFlux.F90:469-588)
// on given states with their total enthalpies and sound speeds; vFracF = 1
// (no particles).  The routine computes a blending factor from the mean Mach
// number and then overwrites it with 1, so alpha = 3/16 as in AUSM+.
void ausmup_flux(double sigma, double kp, double ku, double nx, double ny, double nz, double nm,
                 double fs, double rl, double ul, double vl, double wl, double pl, double Hl,
                 double al, double rr, double ur, double vr, double wr, double pr, double Hr,
                 double ar, double flx[5]) {
  double ql = ul * nx + vl * ny + wl * nz - fs;
  double qr = ur * nx + vr * ny + wr * nz - fs;
  double af = 0.5 * (al + ar);
  double ml = ql / af, mla = std::fabs(ml);
  double mr = qr / af, mra = std::fabs(mr);
  double mbarsq = 0.5 * (ml * ml + mr * mr);
  double fa = 1.0;
  double alpha = 0.1875 * (5 * fa * fa - 4);
  double mlp, wtl, mrm, wtr;
  if (mla <= 1.0) {
    mlp = 0.25 * (ml + 1.0) * (ml + 1.0) + 0.125 * (ml * ml - 1.0) * (ml * ml - 1.0);
    wtl = 0.25 * (ml + 1.0) * (ml + 1.0) * (2.0 - ml) + alpha * ml * (ml * ml - 1.0) * (ml * ml - 1.0);
  } else {
    mlp = 0.5 * (ml + mla);
    wtl = 0.5 * (1.0 + ml / mla);
  }
  if (mra <= 1.0) {
    mrm = -0.25 * (mr - 1.0) * (mr - 1.0) - 0.125 * (mr * mr - 1.0) * (mr * mr - 1.0);
    wtr = 0.25 * (mr - 1.0) * (mr - 1.0) * (2.0 + mr) - alpha * mr * (mr * mr - 1.0) * (mr * mr - 1.0);
  } else {
    mrm = 0.5 * (mr - mra);
    wtr = 0.5 * (1.0 - mr / mra);
  }
  double rf = 0.5 * (rl + rr);
  double sigmabar = 1.0 - sigma * mbarsq;
  double mp = (-(kp * fmax_f(sigmabar, 0.0) * (pr - pl))) / (fa * rf * af * af);
  double pu = -(ku * wtl * wtr * fa * af * (rl + rr) * (qr - ql));
  double mf = mlp + mrm + mp;
  double mfa = std::fabs(mf);
  double mfp = 0.5 * (mf + mfa), mfm = 0.5 * (mf - mfa);
  double pf = wtl * pl + wtr * pr + pu;
  const double vFracF = 1.0;
  flx[0] = (af * vFracF * (mfp * rl + mfm * rr)) * nm;
  flx[1] = (af * vFracF * (mfp * rl * ul + mfm * rr * ur) + pf * nx) * nm;
  flx[2] = (af * vFracF * (mfp * rl * vl + mfm * rr * vr) + pf * ny) * nm;
  flx[3] = (af * vFracF * (mfp * rl * wl + mfm * rr * wr) + pf * nz) * nm;
  flx[4] = (af * vFracF * (mfp * rl * Hl + mfm * rr * Hr) + pf * fs) * nm;
}

// ---- per-face fluxes on the region ----------------------------------------

struct Ctx {
  const orc_region_t *r;
  const double *cv, *dv, *grad;
};

// Left/right states of *_ComputeFlux2_TCP: cell values from the conserved
// vector (u = rhou * (1/rho)), p from dv, then rho,u,v,w,p += grad . (fc - cofg).
inline void recon(const Ctx &c, int icg1, const double *fcx, double S[5], double *ir_out,
                  bool second) {
  const double *cv = c.cv + 5 * (size_t)(icg1 - 1);
  double rl = cv[0];
  double irl = 1.0 / rl;
  S[0] = rl;
  S[1] = cv[1] * irl;
  S[2] = cv[2] * irl;
  S[3] = cv[3] * irl;
  S[4] = c.dv[3 * (size_t)(icg1 - 1)];
  *ir_out = irl;
  if (!second) return;
  const double *cg = c.r->cofg + 3 * (size_t)(icg1 - 1);
  double dx = fcx[0] - cg[0], dy = fcx[1] - cg[1], dz = fcx[2] - cg[2];
  const double *gr = c.grad + 15 * (size_t)(icg1 - 1);
  for (int v = 0; v < 5; ++v)
    S[v] = S[v] + gr[3 * v + 0] * dx + gr[3 * v + 1] * dy + gr[3 * v + 2] * dz;
}

void interior_flux(const Ctx &c, int ifg, double flx[5]) {
  const orc_region_t *r = c.r;
  int c1 = r->f2c[2 * (size_t)ifg], c2 = r->f2c[2 * (size_t)ifg + 1];
  const double *n = r->fn + 4 * (size_t)ifg;
  const double *fcx = r->fc + 3 * (size_t)ifg;
  const double fs = 0.0;  // gs(indGs*ifg) with a static grid
  bool second = r->spaceOrder > 1;
  double L[5], R[5], irl, irr;
  recon(c, c1, fcx, L, &irl, second);
  recon(c, c2, fcx, R, &irr, second);
  if (r->spaceDiscr == DISCR_UPW_AUSMPLUSUP) {
    double Hl, al, Hr, ar;
    if (second) {  // RFLU_AUSMPlusUp_ComputeFlux2_TCP (:3255-3632)
      double cp = r->refCp, g = r->refGamma, gc = cp - cp / g;  // MixtPerf_R_CpG
      double tl = L[4] / (L[0] * gc), tr = R[4] / (R[0] * gc);  // MixtPerf_T_DPR
      al = std::sqrt(g * gc * tl);
      Hl = cp * tl + 0.5 * (L[1] * L[1] + L[2] * L[2] + L[3] * L[3]) + KSG;
      ar = std::sqrt(g * gc * tr);
      Hr = cp * tr + 0.5 * (R[1] * R[1] + R[2] * R[2] + R[3] * R[3]) + KSG;
    } else {       // RFLU_AUSMPlusUp_ComputeFlux1 (:894-1366): E/rho + p/rho, dv(SOUN)
      const double *cv1 = c.cv + 5 * (size_t)(c1 - 1), *cv2 = c.cv + 5 * (size_t)(c2 - 1);
      al = c.dv[3 * (size_t)(c1 - 1) + 2];
      Hl = cv1[4] * irl + L[4] / L[0];
      ar = c.dv[3 * (size_t)(c2 - 1) + 2];
      Hr = cv2[4] * irr + R[4] / R[0];
    }
    ausmup_flux(r->ausmSigma, r->ausmKp, r->ausmKu, n[0], n[1], n[2], n[3], fs, L[0], L[1],
                L[2], L[3], L[4], Hl, al, R[0], R[1], R[2], R[3], R[4], Hr, ar, flx);
    return;
  }
  switch (r->spaceDiscr) {
    case DISCR_UPW_AUSMPLUS: ausm_states(r, L, R, n, fs, flx); break;
    case DISCR_UPW_ROE: roe_states(r, L, R, n, fs, flx); break;
    default: hllc_states(r, L, R, irl, irr, n, fs, flx); break;
  }
}

// libfloflu/BcondOutflowPerf.F90:88-160.  The reference leaves ksg an
// uninitialised local on the subsonic branch; it is zero here.
void bcond_outflow_perf(int bcOpt, double pout, double sxn, double syn, double szn, double cpgas,
                        double mol, double rho, double rhou, double rhov, double rhow, double rhoe,
                        double press, double *rhob, double *rhoub, double *rhovb, double *rhowb,
                        double *rhoeb) {
  double rgas = R_M(mol);
  double gamma = G_CpR(cpgas, rgas);
  double u = rhou / rho, v = rhov / rho, w = rhow / rho;
  double csound = C_DGP(rho, gamma, press);
  double mach = std::sqrt(u * u + v * v + w * w) / csound;
  if (mach < 1.0 && (bcOpt == BCOPT_SUBSONIC || bcOpt == BCOPT_MIXED)) {
    double rrhoc = 1.0 / (rho * csound);
    double deltp = press - pout;
    *rhob = rho - deltp / (csound * csound);
    double ub = u + sxn * deltp * rrhoc;
    double vb = v + syn * deltp * rrhoc;
    double wb = w + szn * deltp * rrhoc;
    double vnd = ub * sxn + vb * syn + wb * szn;
    if (vnd < 0.0) {
      ub = std::copysign(1.0, u) * fmax_f(std::fabs(ub), std::fabs(u));
      vb = std::copysign(1.0, v) * fmax_f(std::fabs(vb), std::fabs(v));
      wb = std::copysign(1.0, w) * fmax_f(std::fabs(wb), std::fabs(w));
    }
    *rhoub = *rhob * ub;
    *rhovb = *rhob * vb;
    *rhowb = *rhob * wb;
    *rhoeb = *rhob * Eo_DGPUVW(*rhob, gamma, pout, ub, vb, wb, KSG);
  } else {
    *rhob = rho;
    *rhoub = rhou;
    *rhovb = rhov;
    *rhowb = rhow;
    *rhoeb = rhoe;
  }
}

// RFLU_SetRindStateFarfieldPerf (modflu/RFLU_ModRindStates.F90:249-421),
// TCPERF, no lift correction (corrFlag false), ksg = 0.
void rind_farfield_perf(double cpGas, double mmGas, double nx, double ny, double nz,
                        double machInf, double pInf, double tInf, double alphaInf,
                        double betaInf, double rl, double rul, double rvl, double rwl, double rel,
                        double *rr, double *rur, double *rvr, double *rwr, double *rer,
                        double *pr) {
  double rGas = R_M(mmGas);
  double gGas = G_CpR(cpGas, rGas);
  double ul = rul / rl, vl = rvl / rl, wl = rwl / rl;
  double ql = ul * nx + vl * ny + wl * nz;
  double el = rel / rl;
  double sl2 = ul * ul + vl * vl + wl * wl;
  double pl = (gGas - 1.0) * rl * (el - 0.5 * sl2 - KSG);  // MixtPerf_P_DEoGVm2
  double ri = pInf / (rGas * tInf);                        // MixtPerf_D_PRT
  double pi = pInf;
  double qi = machInf * std::sqrt(gGas * rGas * tInf);     // MixtPerf_C_GRT
  double ui = qi * std::cos(alphaInf) * std::cos(betaInf);
  double vi = qi * std::sin(alphaInf) * std::cos(betaInf);
  double wi = qi * std::sin(betaInf);
  if (machInf < 1.0) {
    double al = C_DGP(rl, gGas, pl);
    double pb, rb, ub, vb, wb;
    if (ql < 0.0) {
      pb = 0.5 * (pi + pl - rl * al * ((ui - ul) * nx + (vi - vl) * ny + (wi - wl) * nz));
      rb = ri - (pi - pb) / (al * al);
      ub = ui - nx * (pi - pb) / (rl * al);
      vb = vi - ny * (pi - pb) / (rl * al);
      wb = wi - nz * (pi - pb) / (rl * al);
    } else {
      pb = pi;
      rb = rl - (pl - pi) / (al * al);
      ub = ul + nx * (pl - pi) / (rl * al);
      vb = vl + ny * (pl - pi) / (rl * al);
      wb = wl + nz * (pl - pi) / (rl * al);
    }
    *rr = rb;
    *rur = rb * ub;
    *rvr = rb * vb;
    *rwr = rb * wb;
    *rer = rb * Eo_DGPUVW(rb, gGas, pb, ub, vb, wb, KSG);
    *pr = pb;
  } else if (ql < 0.0) {
    *rr = ri;
    *rur = ri * ui;
    *rvr = ri * vi;
    *rwr = ri * wi;
    *rer = ri * (pi / (ri * (gGas - 1.0)) + 0.5 * qi * qi + KSG);  // MixtPerf_Eo_DGPVm
    *pr = pi;
  } else {
    *rr = rl;
    *rur = rul;
    *rvr = rvl;
    *rwr = rwl;
    *rer = rel;
    *pr = pl;
  }
}

// libfloflu/BcondInflowPerf.F90:93-272, TCPERF.  The reference leaves ksg
// unset on the supersonic branch, and all outputs unset for a SUBSONIC patch
// whose interior normal velocity is supersonic; ksg = 0 here, and the
// interior state in the latter case.
void bcond_inflow_perf(int bcOptType, int bcOptFixed, double ptot, double ttot, double betah,
                       double betav, double mach, double sxn, double syn, double szn,
                       double cpgas, double mm, double rl, double rul, double rvl, double rwl,
                       double rel, double pl, double *rr, double *rur, double *rvr, double *rwr,
                       double *rer, double *pr) {
  double rgas = R_M(mm);
  double g = G_CpR(cpgas, rgas);
  bool prescribed = bcOptType == BCOPT_SUPERSONIC;
  if (!prescribed) {
    double gm1 = g - 1.0;
    double ul = rul / rl, vl = rvl / rl, wl = rwl / rl;
    double a02 = g * rgas * ttot;                                                 // C2_GRT
    double al = std::sqrt(a02 - 0.5 * (g - 1.0) * (ul * ul + vl * vl + wl * wl));  // C_Co2GUVW
    double ql = ul * sxn + vl * syn + wl * szn;
    if (std::fabs(ql) < al) {
      double sl = std::sqrt(ul * ul + vl * vl + wl * wl);
      double eta = -1.0;
      if (bcOptFixed == BCOPT_FIXED_NO && sl > 1.0e-6) eta = ql / sl;
      double Rm = al - 0.5 * gm1 * ql;
      double disc = 0.5 * gm1 * (eta * eta) * (a02 / (Rm * Rm) * (1.0 + 0.5 * gm1 * (eta * eta)) - 1.0);
      double ar, tr, sr;
      if (disc < 0.0) {
        ar = std::sqrt(a02);
        tr = ttot;
        *pr = ptot;
        sr = 0.0;
      } else {
        ar = Rm / (1.0 + 0.5 * gm1 * eta * eta) * (1.0 + std::sqrt(disc));
        tr = ar * ar / (g * rgas);                                  // T_CGR
        *pr = ptot * std::pow(tr / ttot, g / (g - 1.0));            // P_GPoTTo
        double c2 = ar * ar;
        sr = a02 > c2 ? std::sqrt(2.0 / (g - 1.0) * (a02 - c2)) : 0.0;  // Vm_C2Co2G
      }
      *rr = *pr / (rgas * tr);
      double ur = sr * std::cos(betah) * std::cos(betav);
      double vr = sr * std::sin(betah);
      double wr = sr * std::cos(betah) * std::sin(betav);
      *rer = *rr * (*pr / (*rr * (g - 1.0)) + 0.5 * sr * sr + KSG);  // Eo_DGPVm
      *rur = *rr * ur;
      *rvr = *rr * vr;
      *rwr = *rr * wr;
      return;
    }
    prescribed = bcOptType == BCOPT_MIXED;
  }
  if (prescribed) {
    double p = ptot / (std::pow(1.0 + 0.5 * (g - 1.0) * mach * mach, g / (g - 1.0)));  // P_GMaPo
    double t = ttot / (1.0 + 0.5 * (g - 1.0) * mach * mach);                          // T_GMaTo
    double r = p / (rgas * t);
    double ar = std::sqrt(g * rgas * t);
    double ur = mach * ar * std::cos(betah) * std::cos(betav);
    double vr = mach * ar * std::sin(betah);
    double wr = mach * ar * std::cos(betah) * std::sin(betav);
    *rr = r;
    *rur = r * ur;
    *rvr = r * vr;
    *rwr = r * wr;
    *rer = r * Eo_DGPUVW(r, g, p, ur, vr, wr, KSG);
    *pr = p;
  } else {
    *rr = rl;
    *rur = rul;
    *rvr = rvl;
    *rwr = rwl;
    *rer = rel;
    *pr = pl;
  }
}

// Boundary face flux: rocflu/RFLU_CentralSecondPatch.F90:638-1351 (ORDER 2)
// and rocflu/RFLU_CentralFirstPatch.F90:575-1133 (ORDER 1): slip wall,
// outflow, farfield and injection.  Slip walls leave the mass residual
// untouched (flx[0] unused, returns false for it).
void patch_flux(const Ctx &c, const orc_patch_t &p, int ifl, double flx[5], bool *hasMass) {
  const orc_region_t *r = c.r;
  int c1 = p.bf2c[ifl];
  const double *n = p.fn + 4 * (size_t)ifl;
  double nx = n[0], ny = n[1], nz = n[2], nm = n[3];
  const double *fcx = p.fc + 3 * (size_t)ifl;
  const double fs = 0.0;
  const double *cv = c.cv + 5 * (size_t)(c1 - 1);
  double pdv = c.dv[3 * (size_t)(c1 - 1)];
  if (p.bcType == BC_SLIPWALL) {
    double pl;
    if (p.spaceOrder == 2) {
      double S[5], ir;
      recon(c, c1, fcx, S, &ir, true);
      pl = S[4];
    } else {
      pl = pdv;
    }
    flx[0] = 0.0;
    flx[1] = pl * nx * nm;
    flx[2] = pl * ny * nm;
    flx[3] = pl * nz * nm;
    flx[4] = pl * fs * nm;
    *hasMass = false;
    return;
  }
  const int nData = p.nData > 0 ? p.nData : 1;
  const double *vals = p.vals ? p.vals + (size_t)nData * (p.distrib ? ifl : 0) : nullptr;
  double cp = r->gvCp, mm = r->gvMol;
  if (p.bcType == BC_INJECTION && vals[0] > 0.0) {
    // burning surface: RFLU_SetRindStateInjectPerf (RFLU_ModRindStates.F90:460-505)
    double pl;
    if (p.spaceOrder == 2) {
      double S[5], ir;
      recon(c, c1, fcx, S, &ir, true);
      pl = S[4];
    } else {
      pl = pdv;
    }
    double minj = vals[0], tinj = vals[1];
    double rGas = R_M(mm);
    double rl = pl / (rGas * tinj);                              // MixtPerf_D_PRT
    double ql = -minj / rl + fs;
    double ul = ql * nx, vl = ql * ny, wl = ql * nz;
    double Hl = cp * tinj + 0.5 * (ul * ul + vl * vl + wl * wl) + 0.0;  // MixtPerf_Ho_CpTUVW
    flx[0] = -minj * nm;
    flx[1] = (-minj * ul + pl * nx) * nm;
    flx[2] = (-minj * vl + pl * ny) * nm;
    flx[3] = (-minj * wl + pl * nz) * nm;
    flx[4] = (-minj * Hl + pl * fs) * nm;
    *hasMass = true;
    return;
  }
  // outflow, farfield, injection surface not burning
  double rl, rul, rvl, rwl, rel, pl;
  if (p.spaceOrder == 2) {
    double S[5], ir;
    recon(c, c1, fcx, S, &ir, true);
    rl = S[0];
    pl = S[4];
    rul = rl * S[1];
    rvl = rl * S[2];
    rwl = rl * S[3];
    double rgas = R_M(mm);
    double g = G_CpR(cp, rgas);
    rel = rl * Eo_DGPUVW(rl, g, pl, S[1], S[2], S[3], KSG);
  } else {
    rl = cv[0];
    rul = cv[1];
    rvl = cv[2];
    rwl = cv[3];
    rel = cv[4];
    pl = pdv;
  }
  if (p.bcType == BC_INJECTION) {
    // RFLU_SetRindStateSlipWallPerf (RFLU_ModRindStates.F90:539-588)
    double rGas = R_M(mm);
    double gGas = G_CpR(cp, rGas);
    double irl = 1.0 / rl;
    double ul = irl * rul, vl = irl * rvl, wl = irl * rwl;
    double ql = ul * nx + vl * ny + wl * nz - fs;
    double al = C_DGP(rl, gGas, pl);
    if (ql < 0.0) {
      double term = 1.0 + 0.5 * (gGas - 1.0) * ql / al;
      pl = pl * std::pow(term, 2.0 * gGas / (gGas - 1.0));
    } else {
      double term = (gGas + 1.0) / 4.0;
      pl = pl + term * rl * ql * (ql + std::sqrt(al * al + term * term * ql * ql) / term);
    }
    flx[0] = 0.0;
    flx[1] = pl * nx * nm;
    flx[2] = pl * ny * nm;
    flx[3] = pl * nz * nm;
    flx[4] = pl * fs * nm;
    *hasMass = true;
    return;
  }
  double pr = pl;
  double rr, rur, rvr, rwr, rer;
  if (p.bcType == BC_FARFIELD) {
    rind_farfield_perf(cp, mm, nx, ny, nz, vals[0], vals[3], vals[4], vals[1], vals[2], rl, rul,
                       rvl, rwl, rel, &rr, &rur, &rvr, &rwr, &rer, &pr);
  } else if (p.bcType == BC_INFLOW_TOTANG) {
    double mach = p.bcOptType != BCOPT_SUBSONIC ? vals[4] : 0.0;
    bcond_inflow_perf(p.bcOptType, p.bcOptFixed, vals[0], vals[1], vals[2], vals[3], mach, nx, ny,
                      nz, cp, mm, rl, rul, rvl, rwl, rel, pl, &rr, &rur, &rvr, &rwr, &rer, &pr);
  } else if (p.bcType == BC_INFLOW_VELTEMP) {
    double rgas = R_M(mm);
    double g = G_CpR(cp, rgas);
    double ur = vals[0], vr = vals[1], wr = vals[2], tr = vals[3];
    if (p.bcOptType != BCOPT_SUBSONIC) {
      pr = vals[4];
      rr = pr / (rgas * tr);  // D_PRT
    } else {
      rr = rl;
      pr = rr * rgas * tr;    // P_DRT
    }
    rer = rr * Eo_DGPUVW(rr, g, pr, ur, vr, wr, KSG);
    rur = rr * ur;
    rvr = rr * vr;
    rwr = rr * wr;
  } else {
    if (p.bcOptType != BCOPT_SUPERSONIC) pr = vals[0];
    bcond_outflow_perf(p.bcOptType, pr, nx, ny, nz, cp, mm, rl, rul, rvl, rwl, rel, pl, &rr,
                       &rur, &rvr, &rwr, &rer);
  }
  double ql = (rul * nx + rvl * ny + rwl * nz) / rl - fs;
  double qr = (rur * nx + rvr * ny + rwr * nz) / rr - fs;
  flx[0] = 0.5 * (ql * rl + qr * rr) * nm;
  flx[1] = 0.5 * (ql * rul + pl * nx + qr * rur + pr * nx) * nm;
  flx[2] = 0.5 * (ql * rvl + pl * ny + qr * rvr + pr * ny) * nm;
  flx[3] = 0.5 * (ql * rwl + pl * nz + qr * rwr + pr * nz) * nm;
  flx[4] = 0.5 * (ql * (rel + pl) + pl * fs + qr * (rer + pr) + pr * fs) * nm;
  *hasMass = true;
}

// ---- cell passes ------------------------------------------------------------

// RFLU_ConvertCvCons2Prim, DUVWP branch (modflu/RFLU_ModConvertCv.F90:221-231)
void cons2prim(const orc_region_t *r, double *cv, const double *dv, long b, long e) {
  (void)r;
  for (long i = b; i < e; ++i) {
    double *q = cv + 5 * i;
    double ir = 1.0 / q[0];
    q[1] = ir * q[1];
    q[2] = ir * q[2];
    q[3] = ir * q[3];
    q[4] = dv[3 * i];
  }
}

// RFLU_ConvertCvPrim2Cons, TCPERF, no program burn (RFLU_ModConvertCv.F90:556-592)
void prim2cons(const orc_region_t *r, double *cv, const double *dv, long b, long e) {
  double gc = R_M(r->gvMol);
  double g = G_CpR(r->gvCp, gc);
  for (long i = b; i < e; ++i) {
    double *q = cv + 5 * i;
    double rr = q[0], u = q[1], v = q[2], w = q[3], p = dv[3 * i];
    q[1] = rr * u;
    q[2] = rr * v;
    q[3] = rr * w;
    q[4] = rr * Eo_DGPUVW(rr, g, p, u, v, w, KSG);
  }
}

// RFLU_ComputeGradCellsFast_3D (modflu/RFLU_ModDifferentiationCells.F90:1021-1149)
void gradients(const orc_region_t *r, const double *var, double *grad, long b, long e) {
  for (long icg = b; icg < e; ++icg) {
    const double *mo = r->xyzMoms + 10 * icg;
    double r11 = mo[0], r12 = mo[1], r22 = mo[2], r13 = mo[3], r23 = mo[4], r33 = mo[5];
    double c11 = 1.0 / r11, c22 = 1.0 / r22, c33 = 1.0 / r33;
    double c12 = -c11 * r12;
    double c13 = -(c11 * r13 + c12 * c22 * r23);
    double c23 = -c22 * r23;
    double c1111 = c11 * c11, c2222 = c22 * c22, c3333 = c33 * c33;
    double *gr = grad + 15 * icg;
    for (int k = 0; k < 15; ++k) gr[k] = 0.0;
    const double *x0 = r->cofg + 3 * icg;
    const double *v0 = var + 5 * icg;
    for (int s = r->csOff[icg]; s < r->csOff[icg + 1]; ++s) {
      long icg2 = r->csMem[s] - 1;
      const double *x2 = r->cofg + 3 * icg2;
      double dx = x2[0] - x0[0], dy = x2[1] - x0[1], dz = x2[2] - x0[2];
      double term = 1.0 / std::sqrt(dx * dx + dy * dy + dz * dz);
      dx = term * dx;
      dy = term * dy;
      dz = term * dz;
      double term1 = c1111 * (dx);
      double term2 = c2222 * (dy + c12 * dx);
      double term3 = c3333 * (dz + c23 * dy + c13 * dx);
      double wtx = term * (term1 + c12 * term2 + c13 * term3);
      double wty = term * (term2 + c23 * term3);
      double wtz = term * (term3);
      const double *v2 = var + 5 * icg2;
      for (int v = 0; v < 5; ++v) {
        double dVar = v2[v] - v0[v];
        gr[3 * v + 0] = gr[3 * v + 0] + wtx * dVar;
        gr[3 * v + 1] = gr[3 * v + 1] + wty * dVar;
        gr[3 * v + 2] = gr[3 * v + 2] + wtz * dVar;
      }
    }
  }
}

// One face term of RFLU_ComputeLimiterVenkat (RFLU_ModLimiters.F90:482-504).
// The reference adds TINY = 1e-12 to a denominator that has the sign of d2;
// for d2 < 0 with |denom| near 1e-12 the sum cancels and phi -> -inf, which
// then wins the MIN and flips and amplifies the gradient.  guard = 1 selects
// the labelled extension that adds TINY with the sign of the denominator.
inline void venkat_term(double d2, double dmax, double dmin, double epsq, double *lim, int guard) {
  const double TINY = 1.0e-12;
  if (d2 > 0.0) {
    double numer = (dmax * dmax + epsq) * d2 + 2.0 * d2 * d2 * dmax;
    double denom = d2 * (dmax * dmax + 2.0 * d2 * d2 + dmax * d2 + epsq);
    double term = numer / (denom + TINY);
    *lim = fmin_f(term, *lim);
  } else if (d2 < 0.0) {
    double numer = (dmin * dmin + epsq) * d2 + 2.0 * d2 * d2 * dmin;
    double denom = d2 * (dmin * dmin + 2.0 * d2 * d2 + dmin * d2 + epsq);
    double term = numer / (denom + (guard ? -TINY : TINY));
    *lim = fmin_f(term, *lim);
  }
}

// RFLU_ComputeLimiterVenkat + RFLU_LimitGradCells (modflu/RFLU_ModLimiters.F90:339-532,707-760)
inline long n_tot(const orc_region_t *r) { return r->nCellsTot > 0 ? r->nCellsTot : r->nCells; }

void venkat(const orc_region_t *r, const double *var, double *grad) {
  const long nC = n_tot(r);
  const double THRD = 1.0 / 3.0;
  std::vector<double> vmin(var, var + 5 * nC), vmax(var, var + 5 * nC), lim(5 * nC, 1.0);
  for (long f = 0; f < r->nFaces; ++f) {
    long c1 = r->f2c[2 * f] - 1, c2 = r->f2c[2 * f + 1] - 1;
    for (int v = 0; v < 5; ++v) {
      double var1 = var[5 * c1 + v], var2 = var[5 * c2 + v];
      vmin[5 * c1 + v] = fmin_f(vmin[5 * c1 + v], var2);
      vmin[5 * c2 + v] = fmin_f(vmin[5 * c2 + v], var1);
      vmax[5 * c1 + v] = fmax_f(vmax[5 * c1 + v], var2);
      vmax[5 * c2 + v] = fmax_f(vmax[5 * c2 + v], var1);
    }
  }
  for (long f = 0; f < r->nFaces; ++f) {
    long c1 = r->f2c[2 * f] - 1, c2 = r->f2c[2 * f + 1] - 1;
    const double *fcx = r->fc + 3 * f;
    double dx1 = r->cofg[3 * c1] - fcx[0], dy1 = r->cofg[3 * c1 + 1] - fcx[1],
           dz1 = r->cofg[3 * c1 + 2] - fcx[2];
    double dx2 = r->cofg[3 * c2] - fcx[0], dy2 = r->cofg[3 * c2 + 1] - fcx[1],
           dz2 = r->cofg[3 * c2 + 2] - fcx[2];
    double ds1 = std::pow(r->vol[c1], THRD), ds2 = std::pow(r->vol[c2], THRD);
    double epsq1 = ds1 * ds1 * ds1, epsq2 = ds2 * ds2 * ds2;  // (K*ds)^3 with K = 1
    for (int v = 0; v < 5; ++v) {
      double var1 = var[5 * c1 + v], var2 = var[5 * c2 + v];
      double d1min1 = vmin[5 * c1 + v] - var1, d1max1 = vmax[5 * c1 + v] - var1;
      double d1min2 = vmin[5 * c2 + v] - var2, d1max2 = vmax[5 * c2 + v] - var2;
      const double *g1 = grad + 15 * c1 + 3 * v, *g2 = grad + 15 * c2 + 3 * v;
      double d21 = g1[0] * dx1 + g1[1] * dy1 + g1[2] * dz1;
      double d22 = g2[0] * dx2 + g2[1] * dy2 + g2[2] * dz2;
      venkat_term(d21, d1max1, d1min1, epsq1, &lim[5 * c1 + v], r->venkatGuard);
      venkat_term(d22, d1max2, d1min2, epsq2, &lim[5 * c2 + v], r->venkatGuard);
    }
  }
  for (long c = 0; c < nC; ++c)
    for (int v = 0; v < 5; ++v)
      for (int d = 0; d < 3; ++d) grad[15 * c + 3 * v + d] = lim[5 * c + v] * grad[15 * c + 3 * v + d];
}

// RFLU_WENOGradCellsXYZFast_3D (modflu/RFLU_ModWENO.F90:1402-1588), the 3-D
// branch RFLU_WENOGradCellsXYZWrapper takes (:1615-1668), for cell c: every
// gradient component becomes the average of the cell's and its stencil
// members' components weighted by s = 1/(g^2 + 1e-15), the cell first, the
// members in stored order, sum(s g) / sum(s).  g0 holds every cell's
// unweighted gradients (the reference writes gradENO, then copies).
void weno_cell(const orc_region_t *r, const double *g0, double *grad, long c) {
  for (int k = 0; k < 15; ++k) {
    const double t = g0[15 * c + k];
    double ssum = 1.0 / (t * t + 1.0E-15);
    double acc = ssum * t;
    for (int s = r->csOff[c]; s < r->csOff[c + 1]; ++s) {
      const double tm = g0[15 * (long)(r->csMem[s] - 1) + k];
      const double sm = 1.0 / (tm * tm + 1.0E-15);
      ssum = ssum + sm;
      acc = acc + sm * tm;
    }
    grad[15 * c + k] = acc / ssum;
  }
}

// Faces of every cell (interior, then boundary as (patch, face) pairs), for
// RFLU_LimitGradCellsSimple, which walks a cell's faces through tet2f / hex2f /
// pri2f / pyr2f; its result does not depend on the order.
struct CellFaces {
  std::vector<long> off, item;  // item >= 0: interior face; < 0: -(boundary slot + 1)
  std::vector<const double *> bfc;
};
// In a partitioned region the virtual cells' lists also hold the faces
// between two virtual cells and to cells outside the region (nFaces ..
// nFacesAll, outside side 0) and the patches' faces on virtual cells
// (nBFaces .. nBFacesTot).
CellFaces cell_faces(const orc_region_t *r) {
  const long nC = n_tot(r);
  const long nFA = r->nFacesAll > 0 ? r->nFacesAll : r->nFaces;
  auto nbt = [](const orc_patch_t &p) { return p.nBFacesTot > 0 ? p.nBFacesTot : p.nBFaces; };
  auto in = [&](int c) { return c >= 1 && c <= nC; };
  CellFaces cf;
  cf.off.assign(nC + 1, 0);
  for (long f = 0; f < nFA; ++f)
    for (int k = 0; k < 2; ++k)
      if (in(r->f2c[2 * f + k])) cf.off[r->f2c[2 * f + k]]++;
  for (int ip = 0; ip < r->nPatches; ++ip)
    for (int i = 0; i < nbt(r->patches[ip]); ++i) cf.off[r->patches[ip].bf2c[i]]++;
  for (long c = 0; c < nC; ++c) cf.off[c + 1] += cf.off[c];
  cf.item.resize(cf.off[nC]);
  std::vector<long> fill(cf.off.begin(), cf.off.end() - 1);
  for (long f = 0; f < nFA; ++f)
    for (int k = 0; k < 2; ++k)
      if (in(r->f2c[2 * f + k])) cf.item[fill[r->f2c[2 * f + k] - 1]++] = f;
  for (int ip = 0; ip < r->nPatches; ++ip)
    for (int i = 0; i < nbt(r->patches[ip]); ++i) {
      cf.item[fill[r->patches[ip].bf2c[i] - 1]++] = -(long)cf.bfc.size() - 1;
      cf.bfc.push_back(r->patches[ip].fc + 3 * i);
    }
  return cf;
}

// RFLU_LimitGradCellsSimple (modflu/RFLU_ModLimiters.F90:793-921) for cell c:
// the gradient of a positive variable (density and pressure,
// libflu/RFLU_SetVarInfo.F90:140-144) is set to zero when its reconstruction
// var + grad . (fc - xc) at one of the cell's faces is not positive.
void limit_simple_cell(const orc_region_t *r, const CellFaces &cf, const double *var,
                       double *grad, long c) {
  const double xc = r->cofg[3 * c], yc = r->cofg[3 * c + 1], zc = r->cofg[3 * c + 2];
  for (int v = 0; v < 5; v += 4) {
    const double varc = var[5 * c + v];
    double *g = grad + 15 * c + 3 * v;
    for (long e = cf.off[c]; e < cf.off[c + 1]; ++e) {
      const long it = cf.item[e];
      const double *fcx = it >= 0 ? r->fc + 3 * it : cf.bfc[-it - 1];
      const double dx = fcx[0] - xc, dy = fcx[1] - yc, dz = fcx[2] - zc;
      const double varf = varc + g[0] * dx + g[1] * dy + g[2] * dz;
      if (varf <= 0.0) {
        g[0] = 0.0;
        g[1] = 0.0;
        g[2] = 0.0;
        break;
      }
    }
  }
}

void weno_simple(const orc_region_t *r, const double *var, double *grad) {
  const long nC = n_tot(r);
  std::vector<double> g0(grad, grad + 15 * nC);
  for (long c = 0; c < nC; ++c) weno_cell(r, g0.data(), grad, c);
  CellFaces cf = cell_faces(r);
  for (long c = 0; c < nC; ++c) limit_simple_cell(r, cf, var, grad, c);
}

// CellGradientsMP (libfloflu/CellGradientsMP.F90:158-253), in place on cv
void cell_gradients(const orc_region_t *r, double *cv, const double *dv, double *grad) {
  if (r->spaceOrder <= 1) return;
  cons2prim(r, cv, dv, 0, n_tot(r));
  gradients(r, cv, grad, 0, n_tot(r));
  if (r->reconst == RECONST_LIM_VENKAT) venkat(r, cv, grad);
  if (r->reconst == RECONST_WENO_XYZ) weno_simple(r, cv, grad);
  prim2cons(r, cv, dv, 0, n_tot(r));
}

// ConvectiveFluxes (libfloflu/ConvectiveFluxes.F90:133-159) with diss = 0:
// rhs = -diss, interior faces in order, then patches in order.
void convective_fluxes(const orc_region_t *r, const double *cv, const double *dv,
                       const double *grad, double *rhs) {
  for (long i = 0; i < 5L * n_tot(r); ++i) rhs[i] = -0.0;
  Ctx c{r, cv, dv, grad};
  double flx[5];
  for (long f = 0; f < r->nFaces; ++f) {
    interior_flux(c, (int)f, flx);
    long c1 = r->f2c[2 * f] - 1, c2 = r->f2c[2 * f + 1] - 1;
    for (int k = 0; k < 5; ++k) rhs[5 * c1 + k] = rhs[5 * c1 + k] + flx[k];
    for (int k = 0; k < 5; ++k) rhs[5 * c2 + k] = rhs[5 * c2 + k] - flx[k];
  }
  for (int ip = 0; ip < r->nPatches; ++ip) {
    const orc_patch_t &p = r->patches[ip];
    for (int ifl = 0; ifl < p.nBFaces; ++ifl) {
      bool hasMass;
      patch_flux(c, p, ifl, flx, &hasMass);
      long c1 = p.bf2c[ifl] - 1;
      for (int k = hasMass ? 0 : 1; k < 5; ++k) rhs[5 * c1 + k] = rhs[5 * c1 + k] + flx[k];
    }
  }
  // ZeroDummyCellsMP (libfloflu/RungeKuttaMP.F90:232): virtual cells carry no residual
  for (long i = 5L * r->nCells; i < 5L * n_tot(r); ++i) rhs[i] = 0.0;
}

// RkUpdateGeneric, static grid (libfloflu/RkUpdateGeneric.F90:229-314),
// coefficients from libflu/RFLU_DerivedInputValues.F90:340-389
void rk_coeffs(int scheme, double ark[5], double grk[5], int *nSteps) {
  for (int i = 0; i < 5; ++i) ark[i] = grk[i] = 0.0;
  if (scheme == RK_SCHEME_4_CLASSICAL) {
    ark[0] = 0.5; ark[1] = 0.5; ark[2] = 1.0; ark[3] = 1.0 / 6.0;
    grk[0] = 1.0; grk[1] = 2.0; grk[2] = 2.0; grk[3] = 1.0;
    *nSteps = 4;
  } else if (scheme == RK_SCHEME_3_WRAY) {
    ark[0] = 8.0 / 15.0; ark[1] = 5.0 / 12.0; ark[2] = 0.75;
    grk[0] = 0.0; grk[1] = 17.0 / 25.0; grk[2] = 5.0 / 9.0;
    *nSteps = 3;
  } else {
    ark[0] = 1.0; grk[0] = 1.0;
    *nSteps = 1;
  }
}

void rk_update_cell(int scheme, int istage, int nSteps, double fac, double vol, double *cv,
                    const double *cvOld, const double *rhs, double *rhsSum, const double grk[5]) {
  double adtv = fac / vol;
  for (int iv = 0; iv < 5; ++iv) {
    if (scheme == RK_SCHEME_4_CLASSICAL) {
      if (istage == 1) {
        cv[iv] = cvOld[iv] - adtv * rhs[iv];
        rhsSum[iv] = rhs[iv];
      } else if (istage == nSteps) {
        cv[iv] = cvOld[iv] - adtv * (rhs[iv] + rhsSum[iv]);
      } else {
        cv[iv] = cvOld[iv] - adtv * rhs[iv];
        rhsSum[iv] = rhsSum[iv] + grk[istage - 1] * rhs[iv];
      }
    } else if (scheme == RK_SCHEME_3_WRAY) {
      if (istage == 1) {
        cv[iv] = cvOld[iv] - adtv * rhs[iv];
        rhsSum[iv] = rhs[iv];
      } else if (istage == 2) {
        cv[iv] = cvOld[iv] - adtv * (rhs[iv] - grk[istage - 1] * rhsSum[iv]);
        rhsSum[iv] = rhs[iv];
      } else {
        cv[iv] = cvOld[iv] - adtv * (rhs[iv] - grk[istage - 1] * rhsSum[iv]);
      }
    } else {
      cv[iv] = cvOld[iv] - adtv * rhs[iv];
    }
  }
}

// RFLU_SetDependentVars, TCPERF (libflu/RFLU_SetDependentVars.F90:256-287)
inline void set_dv_cell(double gc, double g, const double *q, double *d) {
  double rr = q[0];
  double ir = 1.0 / rr;
  double Eo = ir * q[4];
  double Vm2 = ir * ir * (q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  d[0] = P_DEoGVm2(rr, Eo, g, Vm2, 0.0);
  d[1] = T_DPR(rr, d[0], gc);
  d[2] = C_GRT(g, gc, d[1]);
}

// AfterUpdateMP checks for one cell (libfloflu/AfterUpdateMP.F90:134-136):
// RFLU_CheckValidity, RFLU_EnforceBounds (libflu/RFLU_EnforceBounds.F90:163-232)
// and RFLU_CheckPositivity (libflu/RFLU_CheckPositivity.F90).
inline int after_update_cell(double gc, double g, double *q, double *d) {
  int st = 0;
  {  // CheckValidity
    double rho = q[0], rrho = 1.0 / rho;
    double u = rrho * q[1], v = rrho * q[2], w = rrho * q[3];
    if (std::isnan(rho) || std::isnan(u) || std::isnan(v) || std::isnan(w) || std::isnan(d[0]) ||
        std::isnan(d[1]))
      st |= ORC_ST_NAN;
  }
  {  // EnforceBounds
    const double pTol = 1.0e-12;
    double rr = q[0], ir = 1.0 / rr;
    double u = ir * q[1], v = ir * q[2], w = ir * q[3], Eo = ir * q[4];
    double Vm2 = u * u + v * v + w * w;
    double p = P_DEoGVm2(rr, Eo, g, Vm2, KSG);
    if (p <= 0.0 && std::fabs(p) <= pTol) {
      p = pTol;
      q[4] = rr * Eo_DGPUVW(rr, g, p, u, v, w, KSG);
      st |= ORC_ST_PCLAMP;
    }
  }
  {  // CheckPositivity
    double rho = q[0], rrho = 1.0 / rho;
    double u = rrho * q[1], v = rrho * q[2], w = rrho * q[3];
    double Vm2 = u * u + v * v + w * w;
    double p = d[0];
    if (p <= 0.0) {
      double Eo = 1.0e4 + 0.5 * Vm2 + KSG;
      p = P_DEoGVm2(rho, Eo, g, Vm2, KSG);
      double t = T_DPR(rho, p, gc);
      d[0] = p;
      d[1] = t;
      q[4] = rho * Eo;
      st |= ORC_ST_PFLOOR;
    }
    if (rho <= 0.0 || p <= 0.0) st |= ORC_ST_NEGPOS;
  }
  return st;
}

}  // namespace

extern "C" {

void orc_set_dv(const orc_region_t *r, const double *cv, double *dv) {
  double gc = R_M(r->gvMol), g = G_CpR(r->gvCp, gc);
  for (long i = 0; i < n_tot(r); ++i) set_dv_cell(gc, g, cv + 5 * i, dv + 3 * i);
}

void orc_set_dv_range(const orc_region_t *r, const double *cv, double *dv, long first, long last) {
  double gc = R_M(r->gvMol), g = G_CpR(r->gvCp, gc);
  for (long i = first; i < last; ++i) set_dv_cell(gc, g, cv + 5 * i, dv + 3 * i);
}

int orc_rk_stage(const orc_region_t *r, int istage, double dtMin, double *cv, double *dv,
                 double *cvOld, double *rhs, double *rhsSum, double *grad) {
  const long nC = r->nCells;
  double ark[5], grk[5];
  int nSteps;
  rk_coeffs(r->rkScheme, ark, grk, &nSteps);
  // RKInitMP (libfloflu/RkInitGeneric.F90:128-150)
  if (r->rkScheme != RK_SCHEME_4_CLASSICAL || istage == 1) std::memcpy(cvOld, cv, sizeof(double) * 5 * nC);
  cell_gradients(r, cv, dv, grad);
  convective_fluxes(r, cv, dv, grad, rhs);
  // SourceTermsMP round trip (libfloflu/SourceTermsMP.F90:138,182), all cells
  cons2prim(r, cv, dv, 0, n_tot(r));
  prim2cons(r, cv, dv, 0, n_tot(r));
  // RKUpdateMP
  double fac = ark[istage - 1] * dtMin;
  for (long i = 0; i < nC; ++i)
    rk_update_cell(r->rkScheme, istage, nSteps, fac, r->vol[i], cv + 5 * i, cvOld + 5 * i,
                   rhs + 5 * i, rhsSum + 5 * i, grk);
  // RFLU_SetVarsContWrapper(1,nCells) then AfterUpdateMP
  double gc = R_M(r->gvMol), g = G_CpR(r->gvCp, gc);
  int st = 0;
  for (long i = 0; i < nC; ++i) set_dv_cell(gc, g, cv + 5 * i, dv + 3 * i);
  for (long i = 0; i < nC; ++i) st |= after_update_cell(gc, g, cv + 5 * i, dv + 3 * i);
  return st;
}

void orc_residual(const orc_region_t *r, const double *cv, const double *dv, double *rhs,
                  double *grad) {
  std::vector<double> q(cv, cv + 5 * (size_t)n_tot(r));
  std::vector<double> g;
  if (!grad) {
    g.assign(15 * (size_t)n_tot(r), 0.0);
    grad = g.data();
  }
  cell_gradients(r, q.data(), dv, grad);
  convective_fluxes(r, q.data(), dv, grad, rhs);
}

// Cell -> face lists of the OpenMP stage and time step, built once per
// region: for every cell its signed interior faces ascending (+(f+1) where the
// cell is f2c(1,f), -(f+1) where it is f2c(2,f)), then its boundary faces
// patch by patch (nF + 1 + the face's index over all patches).  That is the
// order in which the serial face loops add into the cell.
// The plan also holds the stage's scratch (face fluxes, limiter values), so
// that repeated stages neither allocate nor first-touch them again.
struct orc_omp_plan_s {
  long nF = 0, nT = 0;
  std::vector<long> off, lst, poff;
  std::vector<double> ff, bf, lim;
  std::vector<char> bm;
};

orc_omp_plan_t orc_omp_plan_create(const orc_region_t *r) {
  auto *pl = new orc_omp_plan_s;
  const long nF = r->nFaces, nT = n_tot(r);
  pl->nF = nF;
  pl->nT = nT;
  pl->poff.assign(r->nPatches + 1, 0);
  for (int ip = 0; ip < r->nPatches; ++ip) pl->poff[ip + 1] = pl->poff[ip] + r->patches[ip].nBFaces;
  std::vector<long> &off = pl->off;
  off.assign(nT + 1, 0);
  for (long f = 0; f < nF; ++f) {
    off[r->f2c[2 * f]]++;
    off[r->f2c[2 * f + 1]]++;
  }
  for (int ip = 0; ip < r->nPatches; ++ip)
    for (int ifl = 0; ifl < r->patches[ip].nBFaces; ++ifl) off[r->patches[ip].bf2c[ifl]]++;
  for (long i = 0; i < nT; ++i) off[i + 1] += off[i];
  pl->lst.resize(off[nT]);
  std::vector<long> fill(off.begin(), off.end() - 1);
  for (long f = 0; f < nF; ++f) {
    pl->lst[fill[r->f2c[2 * f] - 1]++] = f + 1;
    pl->lst[fill[r->f2c[2 * f + 1] - 1]++] = -(f + 1);
  }
  for (int ip = 0; ip < r->nPatches; ++ip)
    for (int ifl = 0; ifl < r->patches[ip].nBFaces; ++ifl)
      pl->lst[fill[r->patches[ip].bf2c[ifl] - 1]++] = nF + 1 + pl->poff[ip] + ifl;
  pl->ff.resize(5 * nF);
  pl->bf.resize(5 * pl->poff[r->nPatches]);
  pl->bm.resize(pl->poff[r->nPatches]);
  pl->lim.resize(5 * nT);
  return pl;
}

void orc_omp_plan_destroy(orc_omp_plan_t pl) { delete pl; }

static void set_threads(int nThreads) {
#ifdef _OPENMP
  if (nThreads > 0) omp_set_num_threads(nThreads);
#else
  (void)nThreads;
#endif
}

int orc_rk_stage_omp(const orc_region_t *r, int istage, double dtMin, double *cv, double *dv,
                     double *cvOld, double *rhs, double *rhsSum, double *grad, int nThreads) {
  orc_omp_plan_t pl = orc_omp_plan_create(r);
  const int st = orc_rk_stage_omp_plan(r, pl, istage, dtMin, cv, dv, cvOld, rhs, rhsSum, grad, nThreads);
  orc_omp_plan_destroy(pl);
  return st;
}

int orc_rk_stage_omp_plan(const orc_region_t *r, orc_omp_plan_t pl, int istage, double dtMin,
                          double *cv, double *dv, double *cvOld, double *rhs, double *rhsSum,
                          double *grad, int nThreads) {
  set_threads(nThreads);
  const long nC = r->nCells, nF = r->nFaces, nT = n_tot(r);
  const std::vector<long> &off = pl->off, &lst = pl->lst, &poff = pl->poff;
  double ark[5], grk[5];
  int nSteps;
  rk_coeffs(r->rkScheme, ark, grk, &nSteps);
  if (r->rkScheme != RK_SCHEME_4_CLASSICAL || istage == 1) {
#pragma omp parallel for schedule(static)
    for (long i = 0; i < 5 * nC; ++i) cvOld[i] = cv[i];
  }
  if (r->spaceOrder > 1) {
#pragma omp parallel for schedule(static)
    for (long i = 0; i < nT; ++i) cons2prim(r, cv, dv, i, i + 1);
#pragma omp parallel for schedule(static, 256)
    for (long i = 0; i < nT; ++i) gradients(r, cv, grad, i, i + 1);
    if (r->reconst == RECONST_LIM_VENKAT) {
      // per-cell gather form of the limiter: min/max and min over the cell's
      // interior faces are order independent, so this equals the face loop
      const double THRD = 1.0 / 3.0;
      std::vector<double> &lim = pl->lim;
#pragma omp parallel for schedule(static, 256)
      for (long c = 0; c < nT; ++c) {
        double vmin[5], vmax[5];
        for (int v = 0; v < 5; ++v) vmin[v] = vmax[v] = cv[5 * c + v];
        for (long e = off[c]; e < off[c + 1]; ++e) {
          if (lst[e] > nF) continue;  // boundary faces come last
          long f = (lst[e] > 0 ? lst[e] : -lst[e]) - 1;
          long o = (r->f2c[2 * f] - 1 == c) ? r->f2c[2 * f + 1] - 1 : r->f2c[2 * f] - 1;
          for (int v = 0; v < 5; ++v) {
            vmin[v] = fmin_f(vmin[v], cv[5 * o + v]);
            vmax[v] = fmax_f(vmax[v], cv[5 * o + v]);
          }
        }
        double ds = std::pow(r->vol[c], THRD);
        double epsq = ds * ds * ds;
        double l[5] = {1.0, 1.0, 1.0, 1.0, 1.0};
        for (long e = off[c]; e < off[c + 1]; ++e) {
          if (lst[e] > nF) continue;
          long f = (lst[e] > 0 ? lst[e] : -lst[e]) - 1;
          const double *fcx = r->fc + 3 * f;
          double dx = r->cofg[3 * c] - fcx[0], dy = r->cofg[3 * c + 1] - fcx[1],
                 dz = r->cofg[3 * c + 2] - fcx[2];
          for (int v = 0; v < 5; ++v) {
            const double *g1 = grad + 15 * c + 3 * v;
            double d2 = g1[0] * dx + g1[1] * dy + g1[2] * dz;
            venkat_term(d2, vmax[v] - cv[5 * c + v], vmin[v] - cv[5 * c + v], epsq, &l[v], r->venkatGuard);
          }
        }
        for (int v = 0; v < 5; ++v) lim[5 * c + v] = l[v];
      }
#pragma omp parallel for schedule(static)
      for (long c = 0; c < nT; ++c)
        for (int v = 0; v < 5; ++v)
          for (int d = 0; d < 3; ++d) grad[15 * c + 3 * v + d] = lim[5 * c + v] * grad[15 * c + 3 * v + d];
    }
    if (r->reconst == RECONST_WENO_XYZ) {
      std::vector<double> g0(grad, grad + 15 * nT);
#pragma omp parallel for schedule(static, 256)
      for (long c = 0; c < nT; ++c) weno_cell(r, g0.data(), grad, c);
      CellFaces cf = cell_faces(r);
#pragma omp parallel for schedule(static, 256)
      for (long c = 0; c < nT; ++c) limit_simple_cell(r, cf, cv, grad, c);
    }
#pragma omp parallel for schedule(static)
    for (long i = 0; i < nT; ++i) prim2cons(r, cv, dv, i, i + 1);
  }
  // face fluxes, then per-cell gather in reference order
  std::vector<double> &ff = pl->ff;
  Ctx ctx{r, cv, dv, grad};
#pragma omp parallel for schedule(static, 1024)
  for (long f = 0; f < nF; ++f) interior_flux(ctx, (int)f, &ff[5 * f]);
  std::vector<double> &bf = pl->bf;
  std::vector<char> &bm = pl->bm;
  for (int ip = 0; ip < r->nPatches; ++ip) {
#pragma omp parallel for schedule(static, 1024)
    for (int ifl = 0; ifl < r->patches[ip].nBFaces; ++ifl) {
      bool hm;
      patch_flux(ctx, r->patches[ip], ifl, &bf[5 * (poff[ip] + ifl)], &hm);
      bm[poff[ip] + ifl] = hm;
    }
  }
  // per-cell gather over the plan's lists: the reference's accumulation order
  double fac = ark[istage - 1] * dtMin;
  double gc = R_M(r->gvMol), g = G_CpR(r->gvCp, gc);
  int st = 0;
#pragma omp parallel for schedule(static, 256) reduction(| : st)
  for (long c = 0; c < nC; ++c) {
    double acc[5] = {-0.0, -0.0, -0.0, -0.0, -0.0};
    for (long e = off[c]; e < off[c + 1]; ++e) {
      long t = lst[e];
      if (t > nF) {
        long b = t - nF - 1;
        for (int k = bm[b] ? 0 : 1; k < 5; ++k) acc[k] = acc[k] + bf[5 * b + k];
      } else if (t > 0) {
        for (int k = 0; k < 5; ++k) acc[k] = acc[k] + ff[5 * (t - 1) + k];
      } else {
        for (int k = 0; k < 5; ++k) acc[k] = acc[k] - ff[5 * (-t - 1) + k];
      }
    }
    for (int k = 0; k < 5; ++k) rhs[5 * c + k] = acc[k];
    // cv holds the round-tripped state; the update starts from cvOld
    rk_update_cell(r->rkScheme, istage, nSteps, fac, r->vol[c], cv + 5 * c, cvOld + 5 * c,
                   rhs + 5 * c, rhsSum + 5 * c, grk);
    set_dv_cell(gc, g, cv + 5 * c, dv + 3 * c);
    st |= after_update_cell(gc, g, cv + 5 * c, dv + 3 * c);
  }
  // virtual cells: ZeroDummyCellsMP, and the SourceTermsMP round trip the
  // serial stage applies to every cell (the update overwrites it elsewhere)
  for (long c = nC; c < nT; ++c) {
    for (int k = 0; k < 5; ++k) rhs[5 * c + k] = 0.0;
    cons2prim(r, cv, dv, c, c + 1);
    prim2cons(r, cv, dv, c, c + 1);
  }
  return st;
}

static double minimum_time_step(double dtMin, double cfl, double dtImposed, double dtMinLimit,
                                double currentTime);

double orc_dt(const orc_region_t *r, const double *cv, const double *dv, double cfl,
              double dtImposed, double dtMinLimit, double currentTime) {
  const long nC = r->nCells;  // RFLU_TimeStepInviscid: minimum over the actual cells
  std::vector<double> dt(n_tot(r), 0.0);
  const double fsu = 0.0;
  for (long f = 0; f < r->nFaces; ++f) {
    long c1 = r->f2c[2 * f] - 1, c2 = r->f2c[2 * f + 1] - 1;
    const double *n = r->fn + 4 * f;
    double ir1 = 1.0 / cv[5 * c1], ir2 = 1.0 / cv[5 * c2];
    double u1 = cv[5 * c1 + 1] * ir1, v1 = cv[5 * c1 + 2] * ir1, w1 = cv[5 * c1 + 3] * ir1;
    double a1 = dv[3 * c1 + 2];
    double u2 = cv[5 * c2 + 1] * ir2, v2 = cv[5 * c2 + 2] * ir2, w2 = cv[5 * c2 + 3] * ir2;
    double a2 = dv[3 * c2 + 2];
    double vc = 0.5 * ((u1 + u2) * n[0] + (v1 + v2) * n[1] + (w1 + w2) * n[2]);
    double as = 0.5 * (a1 + a2);
    double srad = (std::fabs(vc - fsu) + as) * n[3];
    dt[c1] = dt[c1] + srad;
    dt[c2] = dt[c2] + srad;
  }
  for (int ip = 0; ip < r->nPatches; ++ip) {
    const orc_patch_t &p = r->patches[ip];
    for (int ifl = 0; ifl < p.nBFaces; ++ifl) {
      long c1 = p.bf2c[ifl] - 1;
      const double *n = p.fn + 4 * (size_t)ifl;
      double ir1 = 1.0 / cv[5 * c1];
      double u1 = cv[5 * c1 + 1] * ir1, v1 = cv[5 * c1 + 2] * ir1, w1 = cv[5 * c1 + 3] * ir1;
      double a1 = dv[3 * c1 + 2];
      double vc = u1 * n[0] + v1 * n[1] + w1 * n[2];
      dt[c1] = dt[c1] + (std::fabs(vc - fsu) + a1) * n[3];
    }
  }
  double dtMin = 0.0;
  for (long c = 0; c < nC; ++c) {
    dt[c] = r->vol[c] / dt[c];
    if (c == 0 || dt[c] < dtMin) dtMin = dt[c];
  }
  return minimum_time_step(dtMin, cfl, dtImposed, dtMinLimit, currentTime);
}

// rocflu/RFLU_TimeStepInviscid.F90 over the OpenMP plan: the spectral radius
// of every face in parallel, then each cell's sum in the serial loops' order
// (interior faces ascending, then patches), so dt equals orc_dt bit for bit.
double orc_dt_omp(const orc_region_t *r, orc_omp_plan_t pl, const double *cv, const double *dv,
                  double cfl, double dtImposed, double dtMinLimit, double currentTime,
                  int nThreads) {
  set_threads(nThreads);
  const long nC = r->nCells, nF = r->nFaces;
  const std::vector<long> &off = pl->off, &lst = pl->lst, &poff = pl->poff;
  const double fsu = 0.0;
  std::vector<double> sr(nF + poff[r->nPatches]);
#pragma omp parallel for schedule(static, 1024)
  for (long f = 0; f < nF; ++f) {
    long c1 = r->f2c[2 * f] - 1, c2 = r->f2c[2 * f + 1] - 1;
    const double *n = r->fn + 4 * f;
    double ir1 = 1.0 / cv[5 * c1], ir2 = 1.0 / cv[5 * c2];
    double u1 = cv[5 * c1 + 1] * ir1, v1 = cv[5 * c1 + 2] * ir1, w1 = cv[5 * c1 + 3] * ir1;
    double a1 = dv[3 * c1 + 2];
    double u2 = cv[5 * c2 + 1] * ir2, v2 = cv[5 * c2 + 2] * ir2, w2 = cv[5 * c2 + 3] * ir2;
    double a2 = dv[3 * c2 + 2];
    double vc = 0.5 * ((u1 + u2) * n[0] + (v1 + v2) * n[1] + (w1 + w2) * n[2]);
    double as = 0.5 * (a1 + a2);
    sr[f] = (std::fabs(vc - fsu) + as) * n[3];
  }
  for (int ip = 0; ip < r->nPatches; ++ip) {
    const orc_patch_t &p = r->patches[ip];
#pragma omp parallel for schedule(static, 1024)
    for (int ifl = 0; ifl < p.nBFaces; ++ifl) {
      long c1 = p.bf2c[ifl] - 1;
      const double *n = p.fn + 4 * (size_t)ifl;
      double ir1 = 1.0 / cv[5 * c1];
      double u1 = cv[5 * c1 + 1] * ir1, v1 = cv[5 * c1 + 2] * ir1, w1 = cv[5 * c1 + 3] * ir1;
      double a1 = dv[3 * c1 + 2];
      double vc = u1 * n[0] + v1 * n[1] + w1 * n[2];
      sr[nF + poff[ip] + ifl] = (std::fabs(vc - fsu) + a1) * n[3];
    }
  }
  // the serial minimum starts from cell 1 and skips NaN after it
  double first = 0.0, dtMin = 0.0;
  bool any = false;
#pragma omp parallel
  {
    double m = 0.0;
    bool have = false;
#pragma omp for schedule(static, 1024)
    for (long c = 0; c < nC; ++c) {
      double acc = 0.0;
      for (long e = off[c]; e < off[c + 1]; ++e) {
        const long t = lst[e];
        acc = acc + sr[t > nF ? t - 1 : (t > 0 ? t : -t) - 1];
      }
      const double d = r->vol[c] / acc;
      if (c == 0) first = d;
      if (!have || d < m) {
        if (!std::isnan(d)) {
          m = d;
          have = true;
        }
      }
    }
#pragma omp critical
    if (have && (!any || m < dtMin)) {
      dtMin = m;
      any = true;
    }
  }
  if (nC > 0 && (std::isnan(first) || !any)) dtMin = first;
  return minimum_time_step(dtMin, cfl, dtImposed, dtMinLimit, currentTime);
}

static double minimum_time_step(double dtMin, double cfl, double dtImposed, double dtMinLimit,
                                double currentTime) {
  // rocflu/RFLU_MinimumTimeStep.F90:131-146,235-241
  dtMin = cfl * dtMin;
  double wtdtImposed = 0.0, wtdtComputed = 0.0;
  if (currentTime <= 1.0e-08) wtdtImposed = 1.0; else wtdtComputed = 1.0;
  dtMin = wtdtImposed / dtImposed + wtdtComputed / dtMin;
  dtMin = 1.0 / dtMin;
  if (dtMin <= 0.0) dtMin = 6.0e-12;
  dtMin = fmax_f(dtMin, dtMinLimit);
  return dtMin;
}

void orc_face_flux(const orc_region_t *r, const double *left, const double *right,
                   const double *n, double *flux) {
  double L[5], R[5];
  for (int k = 0; k < 5; ++k) {
    L[k] = left[k];
    R[k] = right[k];
  }
  switch (r->spaceDiscr) {
    case DISCR_UPW_AUSMPLUS: ausm_states(r, L, R, n, 0.0, flux); break;
    case DISCR_UPW_ROE: roe_states(r, L, R, n, 0.0, flux); break;
    case DISCR_UPW_AUSMPLUSUP: {  // second-order state set-up
      double cp = r->refCp, g = r->refGamma, gc = cp - cp / g;
      double tl = L[4] / (L[0] * gc), tr = R[4] / (R[0] * gc);
      double al = std::sqrt(g * gc * tl), ar = std::sqrt(g * gc * tr);
      double Hl = cp * tl + 0.5 * (L[1] * L[1] + L[2] * L[2] + L[3] * L[3]) + KSG;
      double Hr = cp * tr + 0.5 * (R[1] * R[1] + R[2] * R[2] + R[3] * R[3]) + KSG;
      ausmup_flux(r->ausmSigma, r->ausmKp, r->ausmKu, n[0], n[1], n[2], n[3], 0.0, L[0], L[1],
                  L[2], L[3], L[4], Hl, al, R[0], R[1], R[2], R[3], R[4], Hr, ar, flux);
      break;
    }
    default: hllc_states(r, L, R, 1.0 / L[0], 1.0 / R[0], n, 0.0, flux); break;
  }
}

}  // extern "C"
