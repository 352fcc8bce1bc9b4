// rfgpu_kernels.cuh - residual / RK-stage kernels, templated on the working
// precision R of reconstruction, limiter and flux arithmetic.  Included by
// rfgpu_fp64.cu (R = double, built with --fmad=false so every expression
// rounds exactly like the unfused reference expression) and rfgpu_mixed.cu
// (R = float).  On the FP64 path residual accumulation, RK update, EOS and
// time step are FP64 in the reference's operation order; on the mixed path
// they are FP32 with compensation (TwoSum residual sums, a float-float
// conserved state, gather_update_mixed below).
//
// Every kernel walks a tile list (region, first item); a tile is blockDim.x
// consecutive cells / faces / boundary faces of one region, so one launch
// covers one region or a whole batch of regions.  Grids smaller than the tile
// count walk the list persistently.
#pragma once

#include "rfgpu_internal.h"

namespace rfgpu {

template <typename R> __device__ __forceinline__ R rmin(R a, R b) { return b < a ? b : a; }
template <typename R> __device__ __forceinline__ R rmax(R a, R b) { return b > a ? b : a; }

// ---- perfect-gas relations (libfloflu/MixtPerf_*.F90) ----------------------
template <typename R>
__device__ __forceinline__ R eo_dgpuvw(R D, R G, R P, R U, R V, R W) {
  return P / (D * (G - R(1))) + R(0.5) * (U * U + V * V + W * W) + R(0);
}

// Physical constants in the working precision: the FP64 values on the FP64
// path, their FP32 copies on the mixed path (no per-thread conversions).
template <typename R> struct PC;
template <> struct PC<double> {
  const Phys &p;
  __device__ double cp() const { return p.refCp; }
  __device__ double g() const { return p.refGamma; }
  __device__ double gc() const { return p.gcRef; }
  __device__ double gvG() const { return p.gvG; }
  __device__ double eps() const { return p.epsentr; }
  __device__ double diss() const { return p.dissFact; }
};
template <> struct PC<float> {
  const Phys &p;
  __device__ float cp() const { return p.refCpF; }
  __device__ float g() const { return p.refGammaF; }
  __device__ float gc() const { return p.gcRefF; }
  __device__ float gvG() const { return p.gvGF; }
  __device__ float eps() const { return p.epsentrF; }
  __device__ float diss() const { return p.dissFactF; }
};

// ---- flux functions on reconstructed states ----------------------------------

// AUSM+ (modflu/RFLU_ModAUSMFlux.F90:282-367 with the state set-up of :2787-2846)
template <typename R>
__device__ __forceinline__ void ausm_flux(const Phys &ph, const R L[5], const R Rt[5],
                                          R nx, R ny, R nz, R nm, R flx[5]) {
  const PC<R> k{ph};
  const R cp = k.cp(), g = k.g(), gc = k.gc(), fs = R(0);
  R rl = L[0], ul = L[1], vl = L[2], wl = L[3], pl = L[4];
  R rr = Rt[0], ur = Rt[1], vr = Rt[2], wr = Rt[3], pr = Rt[4];
  R tl = pl / (rl * gc);
  R al = sqrt(g * gc * tl);
  R Hl = cp * tl + R(0.5) * (ul * ul + vl * vl + wl * wl) + R(0);
  R tr = pr / (rr * gc);
  R ar = sqrt(g * gc * tr);
  R Hr = cp * tr + R(0.5) * (ur * ur + vr * vr + wr * wr) + R(0);
  R ql = ul * nx + vl * ny + wl * nz - fs;
  R qr = ur * nx + vr * ny + wr * nz - fs;
  R af = R(0.5) * (al + ar);
  R ml = ql / af, mla = fabs(ml);
  R mr = qr / af, mra = fabs(mr);
  R mlp, wtl, mrm, wtr;
  if (mla <= R(1)) {
    mlp = R(0.25) * (ml + R(1)) * (ml + R(1)) + R(0.125) * (ml * ml - R(1)) * (ml * ml - R(1));
    wtl = R(0.25) * (ml + R(1)) * (ml + R(1)) * (R(2) - ml) +
          R(0.1875) * ml * (ml * ml - R(1)) * (ml * ml - R(1));
  } else {
    mlp = R(0.5) * (ml + mla);
    wtl = R(0.5) * (R(1) + ml / mla);
  }
  if (mra <= R(1)) {
    mrm = -(R(0.25) * (mr - R(1)) * (mr - R(1))) - R(0.125) * (mr * mr - R(1)) * (mr * mr - R(1));
    wtr = R(0.25) * (mr - R(1)) * (mr - R(1)) * (R(2) + mr) -
          R(0.1875) * mr * (mr * mr - R(1)) * (mr * mr - R(1));
  } else {
    mrm = R(0.5) * (mr - mra);
    wtr = R(0.5) * (R(1) - mr / mra);
  }
  R mf = mlp + mrm, mfa = fabs(mf);
  R mfp = R(0.5) * (mf + mfa), mfm = R(0.5) * (mf - mfa);
  R pf = wtl * pl + wtr * pr;
  flx[0] = (af * (mfp * rl + mfm * rr)) * nm;
  flx[1] = (af * (mfp * rl * ul + mfm * rr * ur) + pf * nx) * nm;
  flx[2] = (af * (mfp * rl * vl + mfm * rr * vr) + pf * ny) * nm;
  flx[3] = (af * (mfp * rl * wl + mfm * rr * wr) + pf * nz) * nm;
  flx[4] = (af * (mfp * rl * Hl + mfm * rr * Hr) + pf * fs) * nm;
}

// AUSM+up, RFLU_AUSMPlusUp_FluxFunction2 (modflu/RFLU_ModAUSMPlusUpFlux.F90:
// 469-588) with vFracF = 1 (no particles): AUSM+ split Mach numbers and
// pressures plus the pressure-diffusion (kp, sigma) and velocity-diffusion
// (ku) terms; the routine's blending factor is overwritten with 1, so
// alpha = 3/16.  H and a of both sides come from the caller (they are set up
// differently at first and second order).
template <typename R>
__device__ __forceinline__ void ausmup_flux(R sigma, R kp, R ku, const R L[5], const R Rt[5],
                                            R Hl, R al, R Hr, R ar, R nx, R ny, R nz, R nm,
                                            R flx[5]) {
  const R fs = R(0);
  const R rl = L[0], ul = L[1], vl = L[2], wl = L[3], pl = L[4];
  const R rr = Rt[0], ur = Rt[1], vr = Rt[2], wr = Rt[3], pr = Rt[4];
  R ql = ul * nx + vl * ny + wl * nz - fs;
  R qr = ur * nx + vr * ny + wr * nz - fs;
  R af = R(0.5) * (al + ar);
  R ml = ql / af, mla = fabs(ml);
  R mr = qr / af, mra = fabs(mr);
  R mbarsq = R(0.5) * (ml * ml + mr * mr);
  const R fa = R(1);
  const R alpha = R(0.1875) * (R(5) * fa * fa - R(4));
  R mlp, wtl, mrm, wtr;
  if (mla <= R(1)) {
    mlp = R(0.25) * (ml + R(1)) * (ml + R(1)) + R(0.125) * (ml * ml - R(1)) * (ml * ml - R(1));
    wtl = R(0.25) * (ml + R(1)) * (ml + R(1)) * (R(2) - ml) +
          alpha * ml * (ml * ml - R(1)) * (ml * ml - R(1));
  } else {
    mlp = R(0.5) * (ml + mla);
    wtl = R(0.5) * (R(1) + ml / mla);
  }
  if (mra <= R(1)) {
    mrm = -(R(0.25) * (mr - R(1)) * (mr - R(1))) - R(0.125) * (mr * mr - R(1)) * (mr * mr - R(1));
    wtr = R(0.25) * (mr - R(1)) * (mr - R(1)) * (R(2) + mr) -
          alpha * mr * (mr * mr - R(1)) * (mr * mr - R(1));
  } else {
    mrm = R(0.5) * (mr - mra);
    wtr = R(0.5) * (R(1) - mr / mra);
  }
  R rf = R(0.5) * (rl + rr);
  R sigmabar = R(1) - sigma * mbarsq;
  R mp = (-(kp * (sigmabar > R(0) ? sigmabar : R(0)) * (pr - pl))) / (fa * rf * af * af);
  R pu = -(ku * wtl * wtr * fa * af * (rl + rr) * (qr - ql));
  R mf = mlp + mrm + mp, mfa = fabs(mf);
  R mfp = R(0.5) * (mf + mfa), mfm = R(0.5) * (mf - mfa);
  R pf = wtl * pl + wtr * pr + pu;
  const R vFracF = R(1);
  flx[0] = (af * vFracF * (mfp * rl + mfm * rr)) * nm;
  flx[1] = (af * vFracF * (mfp * rl * ul + mfm * rr * ur) + pf * nx) * nm;
  flx[2] = (af * vFracF * (mfp * rl * vl + mfm * rr * vr) + pf * ny) * nm;
  flx[3] = (af * vFracF * (mfp * rl * wl + mfm * rr * wr) + pf * nz) * nm;
  flx[4] = (af * vFracF * (mfp * rl * Hl + mfm * rr * Hr) + pf * fs) * nm;
}

template <typename R>
__device__ __forceinline__ R entropy_fix(R l, R d) {  // RFLU_ModEntropyFixes.F90:95-106
  return (l > d) ? l : (l * l + d * d) / (R(2) * d);
}

// Roe with the Harten-Hyman entropy fix (modflu/RFLU_ModRoeFlux.F90:2725-2855)
template <typename R>
__device__ __forceinline__ void roe_flux(const Phys &ph, const R L[5], const R Rt[5], R nx,
                                         R ny, R nz, R nm, R flx[5]) {
  const PC<R> k{ph};
  const R cp = k.cp(), g = k.g(), gc = k.gc(), fs = R(0);
  R rl = L[0], ul = L[1], vl = L[2], wl = L[3], pl = L[4];
  R rr = Rt[0], ur = Rt[1], vr = Rt[2], wr = Rt[3], pr = Rt[4];
  R tl = pl / (rl * gc);
  R Hl = cp * tl + R(0.5) * (ul * ul + vl * vl + wl * wl) + R(0);
  R ql = ul * nx + vl * ny + wl * nz - fs;
  R tr = pr / (rr * gc);
  R Hr = cp * tr + R(0.5) * (ur * ur + vr * vr + wr * wr) + R(0);
  R qr = ur * nx + vr * ny + wr * nz - fs;
  R rh = sqrt(rl * rr);
  R wt = rl / (rl + rh);
  R uh = wt * ul + (R(1) - wt) * ur;
  R vh = wt * vl + (R(1) - wt) * vr;
  R wh = wt * wl + (R(1) - wt) * wr;
  R Hh = wt * Hl + (R(1) - wt) * Hr;
  R qh = uh * nx + vh * ny + wh * nz - fs;
  R sh = R(0.5) * (uh * uh + vh * vh + wh * wh);
  R ah = sqrt((g - R(1)) * (Hh - R(0.5) * (R(2) * sh)));
  R l1 = fabs(qh - ah), l2 = fabs(qh), l5 = fabs(qh + ah);
  R efc = k.eps() * l5;
  l1 = entropy_fix(l1, efc);
  l2 = entropy_fix(l2, efc);
  l5 = entropy_fix(l5, efc);
  R dr = rr - rl, du = ur - ul, de = vr - vl, dw = wr - wl, dp = pr - pl;
  R dq = du * nx + de * ny + dw * nz;
  R dv1 = (dp - rh * ah * dq) / (R(2) * ah * ah);
  R dv5 = (dp + rh * ah * dq) / (R(2) * ah * ah);
  R dv2 = dr - dp / (ah * ah);
  R t1 = l1 * dv1, t2 = l2 * dv2, t3 = l2 * rh, t5 = l5 * dv5;
  R df = k.diss();
  flx[0] = R(0.5) * (ql * rl + qr * rr) * nm - R(0.5) * df * (t1 + t2 + t5) * nm;
  flx[1] = R(0.5) * (ql * rl * ul + pl * nx + qr * rr * ur + pr * nx) * nm -
           R(0.5) * df * (t1 * (uh - nx * ah) + t2 * uh + t3 * (du - nx * dq) + t5 * (uh + nx * ah)) * nm;
  flx[2] = R(0.5) * (ql * rl * vl + pl * ny + qr * rr * vr + pr * ny) * nm -
           R(0.5) * df * (t1 * (vh - ny * ah) + t2 * vh + t3 * (de - ny * dq) + t5 * (vh + ny * ah)) * nm;
  flx[3] = R(0.5) * (ql * rl * wl + pl * nz + qr * rr * wr + pr * nz) * nm -
           R(0.5) * df * (t1 * (wh - nz * ah) + t2 * wh + t3 * (dw - nz * dq) + t5 * (wh + nz * ah)) * nm;
  flx[4] = R(0.5) * (ql * rl * Hl + pl * fs + qr * rr * Hr + pr * fs) * nm -
           R(0.5) * df * (t1 * (Hh - qh * ah) + t2 * sh + t3 * (uh * du + vh * de + wh * dw - qh * dq) +
                          t5 * (Hh + qh * ah)) * nm;
}

// HLLC (modflu/RFLU_ModHLLCFlux.F90:2296-2409); irl/irr are the reciprocal
// cell densities before reconstruction, as the reference uses in Hl/Hr.
template <typename R>
__device__ __forceinline__ void hllc_flux(const Phys &ph, const R L[5], const R Rt[5], R irl,
                                          R irr, R nx, R ny, R nz, R nm, R flx[5]) {
  const R g = PC<R>{ph}.g(), fs = R(0);
  R rl = L[0], ul = L[1], vl = L[2], wl = L[3], pl = L[4];
  R rr = Rt[0], ur = Rt[1], vr = Rt[2], wr = Rt[3], pr = Rt[4];
  R el = eo_dgpuvw(rl, g, pl, ul, vl, wl);
  R al = sqrt(g * pl / rl);
  R ql = ul * nx + vl * ny + wl * nz - fs;
  R Hl = el + irl * pl;
  R er = eo_dgpuvw(rr, g, pr, ur, vr, wr);
  R ar = sqrt(g * pr / rr);
  R qr = ur * nx + vr * ny + wr * nz - fs;
  R Hr = er + irr * pr;
  R wt1 = sqrt(rr / rl);
  R wt2 = R(1) / (R(1) + wt1);
  R us = wt2 * (ul + wt1 * ur);
  R vs = wt2 * (vl + wt1 * vr);
  R ws = wt2 * (wl + wt1 * wr);
  R qs = wt2 * (ql + wt1 * qr);
  R Hs = wt2 * (Hl + wt1 * Hr);
  R Vms = us * us + vs * vs + ws * ws;
  R as = sqrt((g - R(1)) * (Hs - R(0.5) * Vms));
  R sl = rmin(ql - al, qs - as);
  R sr = rmax(qr + ar, qs + as);
  if (sl > R(0)) {
    flx[0] = ql * rl * nm;
    flx[1] = (ql * rl * ul + pl * nx) * nm;
    flx[2] = (ql * rl * vl + pl * ny) * nm;
    flx[3] = (ql * rl * wl + pl * nz) * nm;
    flx[4] = (ql * (rl * el + pl) + pl * fs) * nm;
  } else if (sr < R(0)) {
    flx[0] = qr * rr * nm;
    flx[1] = (qr * rr * ur + pr * nx) * nm;
    flx[2] = (qr * rr * vr + pr * ny) * nm;
    flx[3] = (qr * rr * wr + pr * nz) * nm;
    flx[4] = (qr * (rr * er + pr) + pr * fs) * nm;
  } else {
    R sm = (rr * qr * (sr - qr) - rl * ql * (sl - ql) - pr + pl) / (rr * (sr - qr) - rl * (sl - ql));
    R ps = pl + rl * (ql - sl) * (ql - sm);
    R rs, rus, rvs, rws, res, term;
    if (sm > R(0)) {
      term = R(1) / (sl - sm);
      rs = term * (sl - ql) * rl;
      rus = term * ((sl - ql) * rl * ul + (ps - pl) * nx);
      rvs = term * ((sl - ql) * rl * vl + (ps - pl) * ny);
      rws = term * ((sl - ql) * rl * wl + (ps - pl) * nz);
      res = term * ((sl - ql) * rl * el + (ps * sm - pl * ql));
    } else {
      term = R(1) / (sr - sm);
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

// ---- vector access to AoS records --------------------------------------------
// Records are 32-byte aligned, so one record row of 8 floats (or 4 doubles) is
// a single 256-bit access: one request per warp touching each 32-byte sector
// once, where two 128-bit halves would issue two requests over the same
// sectors.  ld8/ld4 read through the non-coherent path and are for data no
// thread writes during the kernel; ld8_rw is the coherent form for a thread's
// own record that the same kernel rewrites.
// Read-once streams (per-face and per-cell arrays a pass reads exactly once):
// with H = 1 loaded L1::evict_first so L1 keeps the gathered records the pass
// reuses; H = 0 plain loads.  lds_rw is the coherent form for data the same
// kernel later overwrites (the thread's own state rows).
// Measured on the 128^3 tet box (mixed): update pass 0.650 -> 0.636 ms with
// its hint, gradient pass 1.928 -> 1.925 ms, face pass unchanged (0.636 ms;
// 0.631 ms with and without it once the gradient rows are prefetched), so the
// face pass keeps plain loads.
// Update face loop: the first RF_UPD_PRE face codes loaded together ahead of
// the flux gathers (measured: update pass 0.636 -> 0.596 ms with 4, 0.598 ms
// with 6).
#ifndef RF_UPD_PRE
#define RF_UPD_PRE 6
#endif
// RECONST 2 pass, mixed path: gradient rows gathered together per group and
// the weights from the hardware reciprocal.  Measured on the 128^3 tet box:
// exact division 4.95 ms (2 rows: 5.80, 4 rows: 6.62, the division code's
// registers), reciprocal 4.08 ms, with 2 rows 3.61 ms, with 4 rows 3.48 ms.
// The FP64 path keeps the IEEE division and one row at a time.
#ifndef RF_WENO_U
#define RF_WENO_U 4
#endif
#ifndef RF_WENO_FASTRCP
#define RF_WENO_FASTRCP 1
#endif
// Face pass: both cells' gradient rows prefetched into L1 as soon as the
// face's cells are known (measured 0.640 -> 0.631 ms).
#ifndef RF_FACE_PF
#define RF_FACE_PF 1
#endif
#ifndef RF_HINT_G
#define RF_HINT_G 1   // gradient pass: cell->face lists, WLSQ factor terms
#endif
#ifndef RF_HINT_F
#define RF_HINT_F 0   // face pass: f2c, normals, reconstruction offsets
#endif
#ifndef RF_HINT_U
#define RF_HINT_U 1   // update pass: face codes, state rows, increments, 1/vol
#endif
template <int H>
__device__ __forceinline__ int lds(const int *__restrict__ p) {
  if constexpr (H) {
    int v;
    asm("ld.global.nc.L1::evict_first.s32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
  } else {
    return *p;
  }
}
template <int H>
__device__ __forceinline__ float lds(const float *__restrict__ p) {
  if constexpr (H) {
    float v;
    asm("ld.global.nc.L1::evict_first.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
  } else {
    return *p;
  }
}
template <int H>
__device__ __forceinline__ double lds(const double *__restrict__ p) {
  if constexpr (H) {
    double v;
    asm("ld.global.nc.L1::evict_first.f64 %0, [%1];" : "=d"(v) : "l"(p));
    return v;
  } else {
    return *p;
  }
}
template <int H>
__device__ __forceinline__ float lds_rw(const float *p) {
  if constexpr (H) {
    float v;
    asm volatile("ld.global.L1::evict_first.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
  } else {
    return *p;
  }
}
template <int H>
__device__ __forceinline__ double lds_rw(const double *p) {
  if constexpr (H) {
    double v;
    asm volatile("ld.global.L1::evict_first.f64 %0, [%1];" : "=d"(v) : "l"(p));
    return v;
  } else {
    return *p;
  }
}

// The stencil-index stream of the mixed gradient pass: each index is read
// once, so it is loaded L1::evict_first and leaves L1 to the neighbour records
// the member gathers reuse (measured 1.955 -> 1.924 ms per pass on the
// 128^3 tet box; evict_last on the record gathers themselves changed nothing).
__device__ __forceinline__ int ld_index(const int *__restrict__ p) {
  int v;
  asm("ld.global.nc.L1::evict_first.s32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ void ld8(const float *__restrict__ p, float v[8]) {
  asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]),
        "=f"(v[7])
      : "l"(p));
}
__device__ __forceinline__ void ld4(const double *__restrict__ p, double v[4]) {
  asm("ld.global.nc.v4.f64 {%0,%1,%2,%3}, [%4];"
      : "=d"(v[0]), "=d"(v[1]), "=d"(v[2]), "=d"(v[3])
      : "l"(p));
}
__device__ __forceinline__ void ld8(const double *__restrict__ p, double v[8]) {
  ld4(p, v);
  ld4(p + 4, v + 4);
}
__device__ __forceinline__ void ld8_rw(const float *p, float v[8]) {
  asm volatile("ld.global.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]),
                 "=f"(v[6]), "=f"(v[7])
               : "l"(p)
               : "memory");
}
__device__ __forceinline__ void ld8_rw(const double *p, double v[8]) {
#pragma unroll
  for (int i = 0; i < 2; ++i)
    asm volatile("ld.global.v4.f64 {%0,%1,%2,%3}, [%4];"
                 : "=d"(v[4 * i]), "=d"(v[4 * i + 1]), "=d"(v[4 * i + 2]), "=d"(v[4 * i + 3])
                 : "l"(p + 4 * i)
                 : "memory");
}
__device__ __forceinline__ void ld4(const float *__restrict__ p, float v[4]) {
  float4 a = *reinterpret_cast<const float4 *>(p);
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
}
template <int H>
__device__ __forceinline__ void ld4s(const float *__restrict__ p, float v[4]) {
  if constexpr (H)
    asm("ld.global.nc.L1::evict_first.v4.f32 {%0,%1,%2,%3}, [%4];"
        : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]) : "l"(p));
  else
    ld4(p, v);
}
template <int H>
__device__ __forceinline__ void ld4s(const double *__restrict__ p, double v[4]) {
  if constexpr (H)
    asm("ld.global.nc.L1::evict_first.v4.f64 {%0,%1,%2,%3}, [%4];"
        : "=d"(v[0]), "=d"(v[1]), "=d"(v[2]), "=d"(v[3]) : "l"(p));
  else
    ld4(p, v);
}
__device__ __forceinline__ void st8(float *p, const float v[8]) {
  asm volatile("st.global.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"l"(p), "f"(v[0]), "f"(v[1]),
               "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7])
               : "memory");
}
__device__ __forceinline__ void st8(double *p, const double v[8]) {
#pragma unroll
  for (int i = 0; i < 2; ++i)
    asm volatile("st.global.v4.f64 [%0], {%1,%2,%3,%4};" ::"l"(p + 4 * i), "d"(v[4 * i]),
                 "d"(v[4 * i + 1]), "d"(v[4 * i + 2]), "d"(v[4 * i + 3])
                 : "memory");
}
template <typename R>
__device__ __forceinline__ void ld16(const R *__restrict__ p, R v[16]) {
  ld8(p, v);
  ld8(p + 8, v + 8);
}
template <typename R>
__device__ __forceinline__ void st16(R *p, const R v[16]) {
  st8(p, v);
  st8(p + 8, v + 8);
}

// Cell-centre values the *_ComputeFlux2_TCP loops start from: rho, u = rhou *
// (1/rho) with rhou the conserved momentum as CellGradientsMP's Prim2Cons
// left it (rho * u_prim), p from dv.  On the mixed path the FP32 primitive
// state is used directly.  rc = the cell's record.
template <typename R>
__device__ __forceinline__ void cell_values(const RegionDev<R> &g, int c, const R rc[8], R S[5],
                                            R &ir) {
  const int N = g.nCells;
  R rho = rc[0];
  ir = R(1) / rho;
  S[0] = rho;
  if (sizeof(R) == 8) {
    if (g.ph.spaceOrder > 1) {
      S[1] = (rho * rc[1]) * ir;
      S[2] = (rho * rc[2]) * ir;
      S[3] = (rho * rc[3]) * ir;
    } else {
      S[1] = R(g.cv[N + c]) * ir;
      S[2] = R(g.cv[2 * N + c]) * ir;
      S[3] = R(g.cv[3 * N + c]) * ir;
    }
  } else {
    S[1] = rc[1];
    S[2] = rc[2];
    S[3] = rc[3];
  }
  S[4] = rc[4];
}

template <typename R>
__device__ __forceinline__ void reconstruct(const R G[16], R dx, R dy, R dz, R S[5]) {
#pragma unroll
  for (int v = 0; v < 5; ++v) S[v] = S[v] + G[3 * v] * dx + G[3 * v + 1] * dy + G[3 * v + 2] * dz;
}

// One face term of RFLU_ComputeLimiterVenkat (modflu/RFLU_ModLimiters.F90:482-504).
// guard = 0 keeps the reference's denom + TINY; guard = 1 adds TINY with the
// sign of denom (for d2 < 0 the reference sum can cancel).
// Mixed path: the quotient is the hardware approximate division
// (__fdividef, within 2 ulp for denominators below 2^126; the terms here stay
// far below), measured on the 128^3 tet box: gradient pass 1.838 -> 1.814 ms;
// the FP64 path keeps IEEE division.
#ifndef RF_LIM_FASTDIV
#define RF_LIM_FASTDIV 1
#endif
template <typename R>
__device__ __forceinline__ R venkat_div(R a, R b) {
  if constexpr (sizeof(R) == 4 && RF_LIM_FASTDIV) return __fdividef(a, b);
  else return a / b;
}
// One Venkatakrishnan face term (modflu/RFLU_ModLimiters.F90:482-504): for d2 > 0
// the bound dmax = max - q and +TINY, for d2 < 0 the bound dmin = min - q and
// +TINY (the reference) or -TINY (guard 1, the signed extension); d2 = 0 or
// NaN leaves lim alone.  Written as one path with the bound and the TINY
// selected by the sign, not as two branches: the lanes of a warp whose d2
// differ in sign then run it once (gradient pass 1.803 -> 1.721 ms on the
// 128^3 tet box); every operation and its order is the reference's.
template <typename R>
__device__ __forceinline__ void venkat_term(R d2, R dmax, R dmin, R epsq, R &lim, int guard) {
  const R TINY = R(1.0e-12);
  if (d2 > R(0) || d2 < R(0)) {
    const bool pos = d2 > R(0);
    const R dm = pos ? dmax : dmin;
    R numer = (dm * dm + epsq) * d2 + R(2) * d2 * d2 * dm;
    R denom = d2 * (dm * dm + R(2) * d2 * d2 + dm * d2 + epsq);
    R term = venkat_div(numer, denom + ((pos || !guard) ? TINY : -TINY));
    lim = rmin(term, lim);
  }
}

// ---- kernels ------------------------------------------------------------------

// Bulk prefetch into L2 of the 16-byte-aligned part of [p, p + bytes): one
// instruction per contiguous range, issued by one lane.
__device__ __forceinline__ void prefetch_l1(const void *p) {
  asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}
__device__ __forceinline__ void prefetch_l2(const void *p, size_t bytes) {
  if (p == nullptr) return;  // an array this region does not hold
  const size_t a = ((size_t)p + 15) & ~(size_t)15, e = ((size_t)p + bytes) & ~(size_t)15;
  if (e > a)
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a), "r"((unsigned)(e - a))
                 : "memory");
}

// Tile prefetches.  The streamed index and geometry arrays a tile reads
// (SELL slices of stencil members and cell->face lists, face tables, own-cell
// rows) are pulled into L2 in bulk, so the block does not wait on DRAM for
// each index before the gather it feeds can issue: the gradient pass at the
// start of its own tile, the face and update passes one wave of blocks
// ahead.  Lane 0 of each warp issues its 32-cell slice; thread 0 issues the
// per-tile face rows.
template <typename R>
__device__ __forceinline__ void prefetch_grad_tile(const RegionDev<R> &g, int first, bool faces) {
  if ((threadIdx.x & 31) != 0) return;
  const int N = g.nCells;
  const int sl = (first >> 5) + (threadIdx.x >> 5);
  if (sl * kSlice >= N) return;
  const long long s0 = g.stOff[sl], s1 = g.stOff[sl + 1];
  prefetch_l2(g.stIdx + s0, (size_t)(s1 - s0) * sizeof(int));
  if (sizeof(R) == 8)
    for (int k = 0; k < 3; ++k) prefetch_l2(g.stW + k * g.stTotal + s0, (size_t)(s1 - s0) * sizeof(R));
  if (faces) {
    const long long f0 = g.cfOff[sl], f1 = g.cfOff[sl + 1];
    const size_t nb = (size_t)(f1 - f0);
    prefetch_l2(g.cfCode + f0, nb * sizeof(int));
    prefetch_l2(g.cfNb + f0, nb * sizeof(int));
    for (int k = 0; k < 3; ++k) prefetch_l2(g.cfD + k * g.cfTotal + f0, nb * sizeof(R));
  }
}

template <typename R>
__device__ __forceinline__ void prefetch_face_tile(const RegionDev<R> &g, int first, int count) {
  if (threadIdx.x != 0) return;
  const int F = g.nFaces;
  if (first >= F) return;
  const size_t n = (size_t)(F - first < count ? F - first : count);
  prefetch_l2(g.f2c + first, n * sizeof(int));
  prefetch_l2(g.f2c + F + first, n * sizeof(int));
  prefetch_l2(g.fnA + 4 * (size_t)first, n * 4 * sizeof(R));
  for (int k = 0; k < 3; ++k) {
    prefetch_l2(g.fdl + (size_t)k * F + first, n * sizeof(R));
    prefetch_l2(g.fdr + (size_t)k * F + first, n * sizeof(R));
  }
}

// The update's per-slice ranges (17 on the mixed path) go out from as many
// lanes at once, lane j taking range j (its pointer picked by selects, so the
// warp runs the prefetch code once instead of once per range on one lane:
// update pass 0.600 -> 0.583 ms at config 2; the gradient and face passes,
// with 6 and 9 ranges, measured faster with one lane).
template <typename R>
__device__ __forceinline__ void prefetch_update_tile(const RegionDev<R> &g, int first) {
  const int N = g.nCells;
  const int j = threadIdx.x & 31;
  const int sl = (first >> 5) + (threadIdx.x >> 5);
  if (sl * kSlice >= N) return;
  const int c0 = sl * kSlice, nc = N - c0 < kSlice ? N - c0 : kSlice;
  // mixed: cvF rows 0-9, rhsSumF 10-14, 1/vol 15; split: cv rows 0-4, rhsSum
  // 5-9, 1/vol 10; FP64: cv rows 0-4; then the slice's cell->face codes
  const bool ff = sizeof(R) == 4 && g.cvF != nullptr;
  const int nrow = ff ? 16 : (sizeof(R) == 4 ? 11 : 5);
  if (j > nrow) return;
  const void *p;
  size_t bytes;
  if (j == nrow) {
    const long long f0 = g.cfOff[sl], f1 = g.cfOff[sl + 1];
    p = g.cfCode + f0;
    bytes = (size_t)(f1 - f0) * sizeof(int);
  } else if (ff) {
    const float *b = j < 10 ? g.cvF + (size_t)j * N : (j < 15 ? g.rhsSumF + (size_t)(j - 10) * N : g.ivolF);
    p = b + c0;
    bytes = (size_t)nc * sizeof(float);
  } else {
    const double *b = j < 5 ? g.cv + (size_t)j * N : (j < 10 ? g.rhsSum + (size_t)(j - 5) * N : g.ivol);
    p = b + c0;
    bytes = (size_t)nc * sizeof(double);
  }
  prefetch_l2(p, bytes);
}

// Calls pf(tile) for the tile a block works on now when it is in the first
// wave, and for the tile `dist` ahead (the one a block of the next wave, or
// this block in its next persistent iteration, will take).
template <typename PF>
__device__ __forceinline__ void prefetch_ahead(int t, int nTiles, int dist, PF pf) {
  if (t < dist) pf(t);
  if (t + dist < nTiles) pf(t + dist);
}

#define RF_TILE_LOOP(tiles, nTiles)                                   \
  for (int t_ = blockIdx.x; t_ < (nTiles); t_ += gridDim.x)

// Cons2Prim (modflu/RFLU_ModConvertCv.F90:221-231) of one cell's FP64 state
// into its record, and optionally the EOS first (libflu/RFLU_SetDependentVars.F90:
// 256-287).  The record's centroid slots are kept.  FP64 path.
template <typename R>
__device__ __forceinline__ void set_vars_cell(const RegionDev<R> &g, int c, int computeDv) {
  const int N = g.nCells;
  double q0 = g.cv[c], q1 = g.cv[N + c], q2 = g.cv[2 * N + c], q3 = g.cv[3 * N + c],
         q4 = g.cv[4 * N + c];
  double ir = 1.0 / q0;
  if (computeDv) {
    double gc = g.ph.gvR, gg = g.ph.gvG;
    double Eo = ir * q4;
    double Vm2 = ir * ir * (q1 * q1 + q2 * q2 + q3 * q3);
    double p = (gg - 1.0) * q0 * (Eo - 0.5 * Vm2 - 0.0);
    double T = p / (q0 * gc);
    g.dv[c] = p;
    g.dv[N + c] = T;
    g.dv[2 * N + c] = sqrt(gg * gc * T);
  }
  R r[8];
  ld8_rw(g.rec + 8 * (size_t)c, r);
  r[0] = R(q0);
  r[1] = R(ir * q1);
  r[2] = R(ir * q2);
  r[3] = R(ir * q3);
  r[4] = R(g.dv[c]);
  st8(g.rec + 8 * (size_t)c, r);
}

// Mixed path: the record (rho, u, v, w, p) of a cell from its float-float
// conserved state, in FP32 (the total energy keeps its low part, so p loses
// only the kinetic term's rounding).  The one state-to-record map of the mixed
// path: the update, the upload and the border receive all use it.
__device__ __forceinline__ void record_from_pairs(const Phys &ph, const float qh[5],
                                                  const float ql[5], float r[5]) {
  const float rf = qh[0];
  const float irf = 1.0f / rf;
  r[0] = rf;
  r[1] = qh[1] * irf;
  r[2] = qh[2] * irf;
  r[3] = qh[3] * irf;
  const float kin = 0.5f * (qh[1] * qh[1] + qh[2] * qh[2] + qh[3] * qh[3]) * irf;
  r[4] = (ph.gvGF - 1.0f) * ((qh[4] - kin) + ql[4]);
}

// Pressure of RFLU_SetDependentVars (libflu/RFLU_SetDependentVars.F90:256-287,
// libfloflu/MixtPerf_P.F90:78) from an FP64 conserved vector, in the
// reference's operation order; ir = 1/rho is returned for the velocities.
__device__ __forceinline__ double eos_p(const Phys &ph, const double q[5], double &ir) {
  const double rr = q[0];
  ir = 1.0 / rr;
  const double Eo = ir * q[4];
  const double Vm2 = ir * ir * (q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  return (ph.gvG - 1.0) * rr * (Eo - 0.5 * Vm2 - 0.0);
}

// Split path: the FP32 record of a cell from its FP64 conserved state and
// FP64 pressure (velocities u = (1/rho) rhou as Cons2Prim forms them).
__device__ __forceinline__ void record_from_fp64(const double q[5], double ir, double p,
                                                 float r[8]) {
  r[0] = float(q[0]);
  r[1] = float(ir * q[1]);
  r[2] = float(ir * q[2]);
  r[3] = float(ir * q[3]);
  r[4] = float(p);
}

// Mixed path: a cell's state from an FP64 conserved vector (upload, border
// receive): float-float split, then the record from the pairs, with p from dv
// when given.  FP64 work is the split alone (GB300's FP64 rate bounds these
// conversions).  Split path (no pairs): the FP64 rows, and the record from
// the FP64 EOS (p from dv when given).
__device__ __forceinline__ void state_from_fp64_split(const RegionDev<float> &g, int c,
                                                      const double q[5], const double *pGiven) {
  const int N = g.nCells;
#pragma unroll
  for (int j = 0; j < 5; ++j) g.cv[(size_t)j * N + c] = q[j];
  double ir;
  const double p = eos_p(g.ph, q, ir);
  float r[8];
  ld8_rw(g.rec + 8 * (size_t)c, r);
  record_from_fp64(q, ir, pGiven ? *pGiven : p, r);
  st8(g.rec + 8 * (size_t)c, r);
}
__device__ __forceinline__ void state_from_fp64_ff(const RegionDev<float> &g, int c,
                                                   const double q[5], const double *pGiven) {
  const int N = g.nCells;
  float qh[5], ql[5];
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    qh[j] = (float)q[j];
    ql[j] = (float)(q[j] - (double)qh[j]);
    g.cvF[(size_t)j * N + c] = qh[j];
    g.cvF[(size_t)(5 + j) * N + c] = ql[j];
  }
  float r[8];
  ld8_rw(g.rec + 8 * (size_t)c, r);
  record_from_pairs(g.ph, qh, ql, r);
  if (pGiven) r[4] = float(*pGiven);
  st8(g.rec + 8 * (size_t)c, r);
}
__device__ __forceinline__ void state_from_fp64(const RegionDev<float> &g, int c, const double q[5],
                                                const double *pGiven) {
  if (g.cvF)
    state_from_fp64_ff(g, c, q, pGiven);
  else
    state_from_fp64_split(g, c, q, pGiven);
}

// The double of a float (IEEE widening, always exact) assembled from its bit
// fields with integer operations: the download join is FP64-pipe bound on
// GB300, and this keeps the conversion off that pipe.  Zeros are assembled
// too; subnormals, infinities and NaNs take the conversion instruction.
__device__ __forceinline__ double widen_f32(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
  if (e == 0xffu || (e == 0u && m != 0u)) return (double)f;
  const unsigned long long s = (unsigned long long)(u & 0x80000000u) << 32;
  // exponent bias 127 -> 1023 (+896), 23 -> 52 fraction bits (<< 29)
  const unsigned long long b =
      e ? (s | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)m << 29)) : s;
  return __longlong_as_double((long long)b);
}

// Conserved state of a cell as FP64 (the float-float pair joined on the
// mixed path).
template <typename R>
__device__ __forceinline__ void cons_fp64(const RegionDev<R> &g, int c, double q[5]) {
  const int N = g.nCells;
  if (sizeof(R) == 4 && g.cvF) {
#pragma unroll
    for (int j = 0; j < 5; ++j)
      q[j] = (double)g.cvF[(size_t)j * N + c] + (double)g.cvF[(size_t)(5 + j) * N + c];
  } else {
#pragma unroll
    for (int j = 0; j < 5; ++j) q[j] = g.cv[(size_t)j * N + c];
  }
}

// Uploaded state -> records (and dv).
template <typename R>
__global__ void k_prim(const RegionDev<R> *__restrict__ regs, const Tile *__restrict__ tiles,
                       int nTiles, int computeDv) {
  RF_TILE_LOOP(tiles, nTiles) {
    const Tile tl = tiles[t_];
    const RegionDev<R> &g = regs[tl.region];
    const int c = tl.first + threadIdx.x;
    if (c >= g.nCells) continue;
    set_vars_cell(g, c, computeDv);
  }
}

// ---- halo exchange ---------------------------------------------------------------
// One received virtual cell: RFLU_MPI_CopyCellData (modflu/RFLU_ModMPI.F90:
// 332-390) of cv, then RFLU_SetVarsContWrapper of the cell
// (libfloflu/RungeKuttaMP.F90:381-396): FP64 path, dv and the record rebuilt
// from the copied cv with the EOS every cell uses; mixed path, the
// float-float pair and the sender's record slots copied (the record is a
// function of the pair and of the gas constants, which coupled regions share).
// The source cell's state is read through L2 (__ldcg): in a persistent stage
// launch other blocks updated it earlier in the same kernel.
template <typename R>
__device__ __forceinline__ void halo_cell(const RegionDev<R> &gs, int cs, const RegionDev<R> &gd,
                                          int cd) {
  const int Ns = gs.nCells, Nd = gd.nCells;
  if constexpr (sizeof(R) == 8) {
#pragma unroll
    for (int j = 0; j < 5; ++j) gd.cv[(size_t)j * Nd + cd] = __ldcg(gs.cv + (size_t)j * Ns + cs);
    set_vars_cell(gd, cd, 1);
  } else {
    if (gd.cvF) {
#pragma unroll
      for (int j = 0; j < 10; ++j) gd.cvF[(size_t)j * Nd + cd] = __ldcg(gs.cvF + (size_t)j * Ns + cs);
    } else {  // split path: the FP64 rows
#pragma unroll
      for (int j = 0; j < 5; ++j) gd.cv[(size_t)j * Nd + cd] = __ldcg(gs.cv + (size_t)j * Ns + cs);
    }
    R a[8], b[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = __ldcg(gs.rec + 8 * (size_t)cs + k);
    ld8_rw(gd.rec + 8 * (size_t)cd, b);
#pragma unroll
    for (int k = 0; k < 5; ++k) b[k] = a[k];
    st8(gd.rec + 8 * (size_t)cd, b);
  }
}

template <typename R>
__global__ void k_halo(const RegionDev<R> *__restrict__ regs, const HaloLink *__restrict__ links,
                       int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const HaloLink l = links[i];
  halo_cell(regs[l.srcRegion], l.srcCell, regs[l.dstRegion], l.dstCell);
}

template <typename R>
__global__ void k_halo_pair(const RegionDev<R> *__restrict__ src, const RegionDev<R> *__restrict__ dst,
                            const int *__restrict__ srcCells, const int *__restrict__ dstCells,
                            int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  halo_cell(*src, srcCells[i], *dst, dstCells[i]);
}

// sendBuff(5,n) = cv(:,cells) (RFLU_MPI_ISendWrapper's packing)
template <typename R>
__global__ void k_border_pack(const RegionDev<R> *__restrict__ gp, const int *__restrict__ cells,
                              int n, double *__restrict__ buf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double q[5];
  cons_fp64(*gp, cells[i], q);
#pragma unroll
  for (int j = 0; j < 5; ++j) buf[5 * (size_t)i + j] = q[j];
}

// cv(:,cells) = recvBuff(5,n), then the cells' dv and records
// (RFLU_MPI_RecvWrapper + RFLU_SetVarsContWrapper(nCells+1,nCellsTot))
template <typename R>
__global__ void k_border_unpack(const RegionDev<R> *__restrict__ gp, const int *__restrict__ cells,
                                int n, const double *__restrict__ buf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const RegionDev<R> &g = *gp;
  const int c = cells[i];
  double q[5];
#pragma unroll
  for (int j = 0; j < 5; ++j) q[j] = buf[5 * (size_t)i + j];
  if constexpr (sizeof(R) == 8) {
#pragma unroll
    for (int j = 0; j < 5; ++j) g.cv[(size_t)j * g.nCells + c] = q[j];
    set_vars_cell(g, c, 1);
  } else {
    state_from_fp64(g, c, q, nullptr);
  }
}

// WLSQ gradients of (rho,u,v,w,p) (RFLU_ComputeGradCellsFast_3D,
// modflu/RFLU_ModDifferentiationCells.F90:1021-1149) fused with the
// Venkatakrishnan limiter and RFLU_LimitGradCells (modflu/RFLU_ModLimiters.F90:
// 339-532, 707-760).  One thread per cell; stencil members in stored order
// (the reference's summation order).  The limiter of a cell needs only its own
// unlimited gradient and its face neighbours' values, and min/max and the MIN
// over faces do not depend on the face order, so the per-cell gather equals
// the reference's two face loops.  FP64 path: precomputed weights (bitwise the
// reference's); mixed path: weights rebuilt in FP32 from the records'
// centroids and the cell's WLSQ factor terms.
template <typename R>
__device__ __forceinline__ void dt_block_min(unsigned long long bits, unsigned long long *smin,
                                             unsigned long long *dst) {
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long x = __shfl_down_sync(0xffffffffu, bits, o);
    bits = x < bits ? x : bits;
  }
  if ((threadIdx.x & 31) == 0) smin[threadIdx.x >> 5] = bits;
  __syncthreads();
  if (threadIdx.x < 32) {
    unsigned long long v = threadIdx.x < (blockDim.x >> 5) ? smin[threadIdx.x] : 0x7FF0000000000000ull;
    for (int o = 16; o > 0; o >>= 1) {
      unsigned long long x = __shfl_down_sync(0xffffffffu, v, o);
      v = x < v ? x : v;
    }
    if (threadIdx.x == 0) atomicMin(dst, v);
  }
  __syncthreads();
}

// The per-face terms of cell_dt, shared with the gradient pass that folds the
// time step into its limiter face loop.
template <typename R>
__device__ __forceinline__ R dt_sound(const RegionDev<R> &g, int c, const R r[8]) {
  const R gg = PC<R>{g.ph}.gvG();
  return sizeof(R) == 8 ? R(g.dv[2 * g.nCells + c]) : R(sqrtf(float(gg * r[4] / r[0])));
}
template <typename R>
__device__ __forceinline__ void dt_interior_term(const RegionDev<R> &g, int code, const R r0[8],
                                                 R a0, int nb, const R rn[8], R &acc) {
  R nrm[4];
  ld4(g.fnA + 4 * (size_t)(code >> 1), nrm);
  const R an = dt_sound(g, nb, rn);
  // the face's c1 values first, as in the reference
  const bool first = (code & 1) == 0;
  const R u1 = first ? r0[1] : rn[1], u2 = first ? rn[1] : r0[1];
  const R v1 = first ? r0[2] : rn[2], v2 = first ? rn[2] : r0[2];
  const R w1 = first ? r0[3] : rn[3], w2 = first ? rn[3] : r0[3];
  const R a1 = first ? a0 : an, a2 = first ? an : a0;
  R vc = R(0.5) * ((u1 + u2) * nrm[0] + (v1 + v2) * nrm[1] + (w1 + w2) * nrm[2]);
  R as = R(0.5) * (a1 + a2);
  acc = acc + (fabs(vc - R(0)) + as) * nrm[3];
}
template <typename R>
__device__ __forceinline__ void dt_boundary_term(const RegionDev<R> &g, int code, const R r0[8],
                                                 R a0, R &acc) {
  R nrm[4];
  ld4(g.bfnA + 4 * (size_t)(-code - 1), nrm);
  R vc = r0[1] * nrm[0] + r0[2] * nrm[1] + r0[3] * nrm[2];
  acc = acc + (fabs(vc - R(0)) + a0) * nrm[3];
}
template <typename R>
__device__ __forceinline__ double dt_of(const RegionDev<R> &g, int c, R acc) {
  return sizeof(R) == 8 ? double(R(g.vol[c]) / acc) : double(float(g.vol[c]) / float(acc));
}

// Local time-step sum of RFLU_TimeStepInviscid (rocflu/RFLU_TimeStepInviscid.F90:
// 165-297) for one cell, as a gather over its faces in the reference order:
// sum of (|v_n| + a) * area with face-averaged velocity and sound speed
// (interior faces) or the cell's own (boundary faces).  u = rhou*(1/rho) is
// the record's velocity; a is dv(SOUN) on the FP64 path and sqrt(g p/rho) in
// FP32 on the mixed path.  Returns dt(c) = vol / sum.
template <typename R>
__device__ __forceinline__ double cell_dt(const RegionDev<R> &g, int c, const R r0[8]) {
  const R a0 = dt_sound(g, c, r0);
  R acc = R(0);
  const long long e0 = g.cfOff[c >> 5] + (c & 31);
  const int n = g.cfCnt[c];
  for (int k = 0; k < n; ++k) {
    const long long e = e0 + (long long)k * kSlice;
    const int code = g.cfCode[e];
    if (code >= 0) {
      const int nb = g.cfNb[e];
      R rn[8];
      ld8(g.rec + 8 * (size_t)nb, rn);
      dt_interior_term(g, code, r0, a0, nb, rn, acc);
    } else {
      dt_boundary_term(g, code, r0, a0, acc);
    }
  }
  return dt_of(g, c, acc);
}

// WLSQ gradients of (rho,u,v,w,p) (RFLU_ComputeGradCellsFast_3D,
// modflu/RFLU_ModDifferentiationCells.F90:1021-1149) fused with the
// Venkatakrishnan limiter and RFLU_LimitGradCells (modflu/RFLU_ModLimiters.F90:
// 339-532, 707-760).  One thread per cell; stencil members in stored order
// (the reference's summation order); the stencil indices are read from the
// SELL slice (coalesced across the warp) and the record gathers of
// consecutive members are issued together.  The limiter of a cell needs only its
// own unlimited gradient and its face neighbours' values, and min/max and the
// MIN over faces do not depend on the face order, so the per-cell gather
// equals the reference's two face loops.  FP64 path: precomputed weights
// (bitwise the reference's); mixed path: weights rebuilt in FP32 from the
// records' centroids and the cell's WLSQ factor terms.  With fuseDt the pass
// also reduces the time step (stage 1 of a step).
// Record gathers issued together in the mixed member loop (software-pipelined
// with the next group's index loads).  Measured on the 128^3 tet box: 4 ->
// 1.923 ms, 6 -> 1.893, 7 -> 1.897, 8 -> 1.880, 10 -> 2.033 (spills), 12 ->
// 2.052; without the index pipeline 8 -> 1.904, 12 -> 1.929.
// Limiter face loop: codes and neighbours of the first RF_LIM_PRE faces loaded
// ahead of the records (measured: gradient pass 1.881 -> 1.835 ms with 4,
// 1.830 ms with 6; keeping the six codes live for the second face loop instead
// of reading them again: 1.981 ms).
#ifndef RF_LIM_PRE
#define RF_LIM_PRE 6
#endif
#ifndef RF_GRAD_UNROLL
#define RF_GRAD_UNROLL 8
#endif
// Resident 128-thread blocks per SM requested for the gradient pass (mixed
// path).  Measured on the 128^3 tet box with the loop above: 7 -> 1.878 ms
// (72 registers), 8 -> 1.830 ms (64), 9 -> 2.075 ms (56, spills).
#ifndef RF_GRAD_MINB
#define RF_GRAD_MINB 8
#endif
#ifndef RF_GRAD_MINB_DT
#define RF_GRAD_MINB_DT 8  // the same for the stage-1 pass that also reduces the time step
#endif
// BS threads per block (one cell each, a tile of BS cells); the requested
// residency keeps the same number of resident threads per SM for every BS.
// One tile of the gradient pass (every thread of the block, one cell each).
template <typename R, int FUSE_DT>
__device__ __forceinline__ void grad_tile(const RegionDev<R> *__restrict__ regs,
                                          const Tile *__restrict__ tiles, int t_,
                                          unsigned long long *smin) {
  constexpr bool fuseDt = FUSE_DT != 0;
  {
    const Tile tl = tiles[t_];
    const RegionDev<R> &g = regs[tl.region];
    const int c = tl.first + threadIdx.x;
    const int N = g.nCells;
    const bool valid = c < N;
    // own tile only: prefetching a wave ahead measured slower here (the
    // prefetched slices push the neighbour records the gathers reuse out of L2)
    prefetch_grad_tile(g, tl.first, fuseDt || g.ph.reconst == 11);
    const long long base = valid ? g.stOff[c >> 5] + (c & 31) : 0;
    const int *__restrict__ sidx = g.stIdx + base;
    unsigned long long dtbits = 0x7FF0000000000000ull;
    if (valid) {
      const R *__restrict__ rec = g.rec;
      R r0[8];
      ld8(rec + 8 * (size_t)c, r0);
      R acc[15];
#pragma unroll
      for (int k = 0; k < 15; ++k) acc[k] = R(0);
      const int n = g.stCnt[c];
      // members accumulated in stored order; loads of consecutive members are
      // issued together so their gathers overlap
      if (sizeof(R) == 8) {
        const long long T = g.stTotal;
        auto member = [&](const R rn[8], long long ee) {
          const R wx = g.stW[ee], wy = g.stW[T + ee], wz = g.stW[2 * T + ee];
#pragma unroll
          for (int v = 0; v < 5; ++v) {
            R dVar = rn[v] - r0[v];
            acc[3 * v] = acc[3 * v] + wx * dVar;
            acc[3 * v + 1] = acc[3 * v + 1] + wy * dVar;
            acc[3 * v + 2] = acc[3 * v + 2] + wz * dVar;
          }
        };
        int k = 0;
        for (; k + 2 <= n; k += 2) {
          R ra[8], rb[8];
          ld8(rec + 8 * (size_t)sidx[k * kSlice], ra);
          ld8(rec + 8 * (size_t)sidx[(k + 1) * kSlice], rb);
          member(ra, base + (long long)k * kSlice);
          member(rb, base + (long long)(k + 1) * kSlice);
        }
        for (; k < n; ++k) {
          R ra[8];
          ld8(rec + 8 * (size_t)sidx[k * kSlice], ra);
          member(ra, base + (long long)k * kSlice);
        }
      } else {
        // The reference's weight of member m is w = A d/|d|^2 with d the
        // centroid offset and A the cell's symmetric inverse-moment matrix
        // built from its WLSQ factor (c11^2 + c12^2 c22^2 + c13^2 c33^2, ...).
        // A is the same for every member, so the member loop accumulates
        // S_v = sum (q_v,m - q_v,0) d/|d|^2 and the gradient is A S_v: the
        // reference's sum reassociated, about a quarter fewer operations per
        // member.
        auto member = [&](const R rn[8]) {
          R dx = rn[5] - r0[5], dy = rn[6] - r0[6], dz = rn[7] - r0[7];
          R t = rsqrtf(float(dx * dx + dy * dy + dz * dz));
          t = t * t;
          dx = t * dx;
          dy = t * dy;
          dz = t * dz;
#pragma unroll
          for (int v = 0; v < 5; ++v) {
            R dVar = rn[v] - r0[v];
            acc[3 * v] = acc[3 * v] + dx * dVar;
            acc[3 * v + 1] = acc[3 * v + 1] + dy * dVar;
            acc[3 * v + 2] = acc[3 * v + 2] + dz * dVar;
          }
        };
        // software pipeline: the next group's stencil indices are loaded while
        // this group's records are in flight (same members, same order)
        constexpr int U = RF_GRAD_UNROLL;
        const int nFull = n - n % U;
        int nx[U];
#pragma unroll
        for (int u = 0; u < U; ++u) nx[u] = u < n ? ld_index(sidx + u * kSlice) : 0;
        for (int k = 0; k < nFull; k += U) {
          R ra[U][8];
#pragma unroll
          for (int u = 0; u < U; ++u) ld8(rec + 8 * (size_t)nx[u], ra[u]);
#pragma unroll
          for (int u = 0; u < U; ++u)
            nx[u] = k + U + u < n ? ld_index(sidx + (k + U + u) * kSlice) : 0;
#pragma unroll
          for (int u = 0; u < U; ++u) member(ra[u]);
        }
#pragma unroll
        for (int u = 0; u < U - 1; ++u) {
          if (nFull + u < n) {
            R ra[8];
            ld8(rec + 8 * (size_t)nx[u], ra);
            member(ra);
          }
        }
        const R axx = lds<RF_HINT_G>(g.cwt + c), axy = lds<RF_HINT_G>(g.cwt + N + c),
                axz = lds<RF_HINT_G>(g.cwt + 2 * N + c);
        const R ayy = lds<RF_HINT_G>(g.cwt + 3 * N + c), ayz = lds<RF_HINT_G>(g.cwt + 4 * N + c),
                azz = lds<RF_HINT_G>(g.cwt + 5 * N + c);
#pragma unroll
        for (int v = 0; v < 5; ++v) {
          const R sx = acc[3 * v], sy = acc[3 * v + 1], sz = acc[3 * v + 2];
          acc[3 * v] = axx * sx + axy * sy + axz * sz;
          acc[3 * v + 1] = axy * sx + ayy * sy + ayz * sz;
          acc[3 * v + 2] = axz * sx + ayz * sy + azz * sz;
        }
      }
      if (g.ph.reconst == 11) {
        R vmin[5], vmax[5], lim[5];
#pragma unroll
        for (int v = 0; v < 5; ++v) {
          vmin[v] = r0[v];
          vmax[v] = r0[v];
          lim[v] = R(1);
        }
        const long long T = g.cfTotal;
        const long long e0 = g.cfOff[c >> 5] + (c & 31);
        const int nf = g.cfCnt[c];
        // stage 1: the time-step sum rides on this face loop (same faces, same
        // order and arithmetic as cell_dt)
        R dtacc = R(0), a0 = R(0);
        if constexpr (fuseDt) a0 = dt_sound(g, c, r0);
        auto face_minmax = [&](int code, int nb) {
          if (code < 0) {
            if constexpr (fuseDt) dt_boundary_term(g, code, r0, a0, dtacc);
            return;
          }
          R rn[8];
          ld8(rec + 8 * (size_t)nb, rn);
#pragma unroll
          for (int v = 0; v < 5; ++v) {
            vmin[v] = rmin(vmin[v], rn[v]);
            vmax[v] = rmax(vmax[v], rn[v]);
          }
          if constexpr (fuseDt) dt_interior_term(g, code, r0, a0, nb, rn, dtacc);
        };
        // the first faces' codes and neighbours are loaded together, ahead of
        // their records (same faces, same order); six covers every cell type
        constexpr int MF = RF_LIM_PRE;
        int cc[MF], nn[MF];
#pragma unroll
        for (int k = 0; k < MF; ++k) {
          const long long ee = e0 + (long long)k * kSlice;
          cc[k] = k < nf ? g.cfCode[ee] : -1;
          nn[k] = k < nf ? lds<RF_HINT_G>(g.cfNb + ee) : -1;
        }
#pragma unroll
        for (int k = 0; k < MF; ++k)
          if (k < nf) face_minmax(cc[k], nn[k]);
        for (int k = MF; k < nf; ++k) {
          const long long ee = e0 + (long long)k * kSlice;
          const int code = g.cfCode[ee];
          face_minmax(code, code < 0 ? -1 : lds<RF_HINT_G>(g.cfNb + ee));
        }
        if constexpr (fuseDt) {
          dtbits = (unsigned long long)__double_as_longlong(dt_of(g, c, dtacc));
          if (c >= g.nAct) dtbits = 0x7FF0000000000000ull;  // actual cells only
        }
        const R epsq = lds<RF_HINT_G>(g.epsq + c);
        const int guard = g.ph.venkatGuard;
        auto face_lim = [&](long long ee) {
          const R dx = lds<RF_HINT_G>(g.cfD + ee), dy = lds<RF_HINT_G>(g.cfD + T + ee),
                  dz = lds<RF_HINT_G>(g.cfD + 2 * T + ee);
#pragma unroll
          for (int v = 0; v < 5; ++v) {
            R d2 = acc[3 * v] * dx + acc[3 * v + 1] * dy + acc[3 * v + 2] * dz;
            venkat_term(d2, vmax[v] - r0[v], vmin[v] - r0[v], epsq, lim[v], guard);
          }
        };
        for (int k = 0; k < nf; ++k) {
          const long long ee = e0 + (long long)k * kSlice;
          if (lds<RF_HINT_G>(g.cfCode + ee) >= 0) face_lim(ee);  // its last read
        }
#pragma unroll
        for (int v = 0; v < 5; ++v)
#pragma unroll
          for (int d = 0; d < 3; ++d) acc[3 * v + d] = lim[v] * acc[3 * v + d];
      }
      R out[16];
#pragma unroll
      for (int k = 0; k < 15; ++k) out[k] = acc[k];
      out[15] = R(0);
      if (!g.gradRaw) {
        st16(g.grad + 16 * (size_t)c, out);
      } else if constexpr (sizeof(R) == 8) {
        // RECONST 2, FP64: the WENO weight of each component and its product,
        // as RFLU_WENOGradCellsXYZFast_3D forms them (same operations), once
        // per cell instead of once per stencil visit
        R w[16];
#pragma unroll
        for (int k = 0; k < 15; ++k) w[k] = R(1) / (out[k] * out[k] + R(1.0E-15));
        w[15] = R(0);
        st16(g.gradRaw + 32 * (size_t)c, w);
#pragma unroll
        for (int k = 0; k < 15; ++k) w[k] = w[k] * out[k];
        st16(g.gradRaw + 32 * (size_t)c + 16, w);
      } else {
        st16(g.gradRaw + 16 * (size_t)c, out);  // RECONST 2, mixed: weighted next
      }
      if constexpr (fuseDt) {
        if (g.ph.reconst != 11) {  // no limiter face loop to ride on
          dtbits = (unsigned long long)__double_as_longlong(cell_dt(g, c, r0));
          if (c >= regs[tl.region].nAct) dtbits = 0x7FF0000000000000ull;
        }
      }
    }
    if constexpr (fuseDt) dt_block_min<R>(dtbits, smin, g.dtBits);
  }
}

template <typename R, int FUSE_DT, int BS>
__global__ void __launch_bounds__(BS, ((sizeof(R) == 4) ? (FUSE_DT ? RF_GRAD_MINB_DT : RF_GRAD_MINB)
                                                        : 4) * 128 / BS)
    k_grad_lim(const RegionDev<R> *__restrict__ regs, const Tile *__restrict__ tiles, int nTiles) {
  __shared__ unsigned long long smin[32];
  RF_TILE_LOOP(tiles, nTiles) grad_tile<R, FUSE_DT>(regs, tiles, t_, smin);
}

// Riemann flux of one interior face on its (reconstructed) states, by DISCR.
// AUSM+up sets up H and a as its face loops do: at second order from the
// reconstructed state with refCp/refGamma (T = p/(rho R), a = sqrt(g R T),
// H = cp T + |v|^2/2; RFLU_AUSMPlusUp_ComputeFlux2_TCP :3255-3632), at first
// order from the cells (H = E/rho + p/rho, a = dv(SOUN); ComputeFlux1
// :894-1366, FP32 sound speed sqrt(g p/rho) on the mixed path).
template <typename R>
__device__ __forceinline__ void face_riemann(const RegionDev<R> &g, int c1, int c2, const R L[5],
                                             const R Rt[5], R irl, R irr, const R nrm[4],
                                             R flx[8]) {
  const int sd = g.ph.spaceDiscr;
  if (sd == 4) {
    ausm_flux(g.ph, L, Rt, nrm[0], nrm[1], nrm[2], nrm[3], flx);
  } else if (sd == 1) {
    roe_flux(g.ph, L, Rt, nrm[0], nrm[1], nrm[2], nrm[3], flx);
  } else if (sd == 5) {
    const PC<R> k{g.ph};
    R Hl, al, Hr, ar;
    if (g.ph.spaceOrder > 1) {
      const R cp = k.cp(), gm = k.g(), gc = k.gc();
      const R tl = L[4] / (L[0] * gc), tr = Rt[4] / (Rt[0] * gc);
      al = sqrt(gm * gc * tl);
      Hl = cp * tl + R(0.5) * (L[1] * L[1] + L[2] * L[2] + L[3] * L[3]) + R(0);
      ar = sqrt(gm * gc * tr);
      Hr = cp * tr + R(0.5) * (Rt[1] * Rt[1] + Rt[2] * Rt[2] + Rt[3] * Rt[3]) + R(0);
    } else if (sizeof(R) == 8) {
      const int N = g.nCells;
      al = R(g.dv[2 * N + c1]);
      Hl = R(g.cv[4 * N + c1]) * irl + L[4] / L[0];
      ar = R(g.dv[2 * N + c2]);
      Hr = R(g.cv[4 * N + c2]) * irr + Rt[4] / Rt[0];
    } else {
      const R gv = k.gvG();
      al = sqrt(gv * L[4] / L[0]);
      Hl = eo_dgpuvw(L[0], gv, L[4], L[1], L[2], L[3]) + L[4] / L[0];
      ar = sqrt(gv * Rt[4] / Rt[0]);
      Hr = eo_dgpuvw(Rt[0], gv, Rt[4], Rt[1], Rt[2], Rt[3]) + Rt[4] / Rt[0];
    }
    const R sig = sizeof(R) == 8 ? R(g.ph.ausmSigma) : R(g.ph.ausmSigmaF);
    const R kp = sizeof(R) == 8 ? R(g.ph.ausmKp) : R(g.ph.ausmKpF);
    const R ku = sizeof(R) == 8 ? R(g.ph.ausmKu) : R(g.ph.ausmKuF);
    ausmup_flux(sig, kp, ku, L, Rt, Hl, al, Hr, ar, nrm[0], nrm[1], nrm[2], nrm[3], flx);
  } else {
    hllc_flux(g.ph, L, Rt, irl, irr, nrm[0], nrm[1], nrm[2], nrm[3], flx);
  }
}

// Interior face fluxes, *_ComputeFlux2_TCP face loops (AUSM+ :2726-2846,
// Roe :2646-2855, HLLC :2239-2409), written to the face flux buffer.  A tile
// is BS * FPT consecutive faces; thread i of the block takes faces i, i + BS,
// ... of it (FPT faces per thread).
template <typename R>
__device__ __forceinline__ void face_flux_one(const RegionDev<R> &g, int f) {
  const int F = g.nFaces;
  {
    const int c1 = lds<RF_HINT_F>(g.f2c + f), c2 = lds<RF_HINT_F>(g.f2c + F + f);
#if RF_FACE_PF
    if (g.ph.spaceOrder > 1) {  // both gradient rows on their way while the records arrive
      prefetch_l1(g.grad + 16 * (size_t)c1);
      prefetch_l1(g.grad + 16 * (size_t)c2);
    }
#endif
    R nrm[4];
    ld4s<RF_HINT_F>(g.fnA + 4 * (size_t)f, nrm);
    R r1[8], r2[8];
    ld8(g.rec + 8 * (size_t)c1, r1);
    ld8(g.rec + 8 * (size_t)c2, r2);
    R L[5], Rt[5], irl, irr;
    cell_values(g, c1, r1, L, irl);
    cell_values(g, c2, r2, Rt, irr);
    if (g.ph.spaceOrder > 1) {
      R G[16];
      ld16(g.grad + 16 * (size_t)c1, G);
      reconstruct(G, lds<RF_HINT_F>(g.fdl + f), lds<RF_HINT_F>(g.fdl + F + f),
                  lds<RF_HINT_F>(g.fdl + 2 * F + f), L);
      ld16(g.grad + 16 * (size_t)c2, G);
      reconstruct(G, lds<RF_HINT_F>(g.fdr + f), lds<RF_HINT_F>(g.fdr + F + f),
                  lds<RF_HINT_F>(g.fdr + 2 * F + f), Rt);
    }
    R flx[8];
    face_riemann(g, c1, c2, L, Rt, irl, irr, nrm, flx);
    flx[5] = flx[6] = flx[7] = R(0);
    st8(g.flux + 8 * (size_t)f, flx);
  }
}

template <typename R, int BS, int FPT>
__device__ __forceinline__ void face_tile(const RegionDev<R> *__restrict__ regs,
                                          const Tile *__restrict__ tiles, int nTiles, int t_,
                                          int dist) {
  const Tile tl = tiles[t_];
  const RegionDev<R> &g = regs[tl.region];
  prefetch_ahead(t_, nTiles, dist, [&](int t) {
    const Tile tp = tiles[t];
    prefetch_face_tile(regs[tp.region], tp.first, BS * FPT);
  });
#pragma unroll
  for (int k = 0; k < FPT; ++k) {
    const int f = tl.first + threadIdx.x + k * BS;
    if (f < g.nFaces) face_flux_one(g, f);
  }
}

template <typename R, int BS, int FPT>
__global__ void __launch_bounds__(BS) k_face_flux(const RegionDev<R> *__restrict__ regs,
                                                  const Tile *__restrict__ tiles, int nTiles,
                                                  int pfDist) {
  const int dist = (int)gridDim.x < nTiles ? (int)gridDim.x : pfDist;
  RF_TILE_LOOP(tiles, nTiles) face_tile<R, BS, FPT>(regs, tiles, nTiles, t_, dist);
}

// Farfield rind state, RFLU_SetRindStateFarfieldPerf
// (modflu/RFLU_ModRindStates.F90:249-421) without the airfoil lift
// correction; fd = (ri, pi, qi, ui, vi, wi, machInf) of the face, evaluated
// on the host.  Subsonic: characteristic combination of the interior and
// free-stream states; supersonic: free stream in, interior out.
template <typename R>
__device__ __forceinline__ void farfield_rind(const R *fd, R gGas, R nx, R ny, R nz, R rl, R rul,
                                              R rvl, R rwl, R rel, R &rr, R &rur, R &rvr, R &rwr,
                                              R &rer, R &pr) {
  const R ri = fd[0], pi = fd[1], qi = fd[2], ui = fd[3], vi = fd[4], wi = fd[5], machInf = fd[6];
  const R ul = rul / rl, vl = rvl / rl, wl = rwl / rl;
  const R ql = ul * nx + vl * ny + wl * nz;
  const R el = rel / rl;
  const R sl2 = ul * ul + vl * vl + wl * wl;
  const R pl = (gGas - R(1)) * rl * (el - R(0.5) * sl2 - R(0));
  if (machInf < R(1)) {
    const R al = sqrt(gGas * pl / rl);
    R pb, rb, ub, vb, wb;
    if (ql < R(0)) {
      pb = R(0.5) * (pi + pl - rl * al * ((ui - ul) * nx + (vi - vl) * ny + (wi - wl) * nz));
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
    rr = rb;
    rur = rb * ub;
    rvr = rb * vb;
    rwr = rb * wb;
    rer = rb * eo_dgpuvw(rb, gGas, pb, ub, vb, wb);
    pr = pb;
  } else if (ql < R(0)) {
    rr = ri;
    rur = ri * ui;
    rvr = ri * vi;
    rwr = ri * wi;
    rer = ri * (pi / (ri * (gGas - R(1))) + R(0.5) * qi * qi + R(0));  // MixtPerf_Eo_DGPVm
    pr = pi;
  } else {
    rr = rl;
    rur = rul;
    rvr = rvl;
    rwr = rwl;
    rer = rel;
    pr = pl;
  }
}

// Total-pressure / total-temperature inflow state, libfloflu/BcondInflowPerf.F90:
// 93-272 (ksg = 0).  d = (ptot, ttot, a02, cos betah, sin betah, cos betav,
// sin betav, fixed, supersonic-branch state rr, rur, rvr, rwr, rer, pr).  A
// SUBSONIC patch whose interior normal velocity is supersonic leaves the
// reference's outputs unset; the interior state is used here.
template <typename R>
__device__ __forceinline__ void inflow_totang(const R *d, int opt, R g, R rgas, R nx, R ny, R nz,
                                              R rl, R rul, R rvl, R rwl, R rel, R pl, R &rr,
                                              R &rur, R &rvr, R &rwr, R &rer, R &pr) {
  const R ptot = d[0], ttot = d[1], a02 = d[2], cbh = d[3], sbh = d[4], cbv = d[5], sbv = d[6];
  const bool fixed = d[7] != R(0);
  bool prescribed = opt == 0;  // BCOPT_SUPERSONIC
  if (!prescribed) {
    const R gm1 = g - R(1);
    const R ul = rul / rl, vl = rvl / rl, wl = rwl / rl;
    const R al = sqrt(a02 - R(0.5) * (g - R(1)) * (ul * ul + vl * vl + wl * wl));  // C_Co2GUVW
    const R ql = ul * nx + vl * ny + wl * nz;
    if (fabs(ql) < al) {
      const R sl = sqrt(ul * ul + vl * vl + wl * wl);
      R eta = R(-1);
      if (!fixed && sl > R(1.0e-6)) eta = ql / sl;
      const R Rm = al - R(0.5) * gm1 * ql;
      const R disc =
          R(0.5) * gm1 * (eta * eta) * (a02 / (Rm * Rm) * (R(1) + R(0.5) * gm1 * (eta * eta)) - R(1));
      R ar, tr, sr;
      if (disc < R(0)) {
        ar = sqrt(a02);
        tr = ttot;
        pr = ptot;
        sr = R(0);
      } else {
        ar = Rm / (R(1) + R(0.5) * gm1 * eta * eta) * (R(1) + sqrt(disc));
        tr = ar * ar / (g * rgas);                          // MixtPerf_T_CGR
        pr = ptot * pow(tr / ttot, g / (g - R(1)));         // MixtPerf_P_GPoTTo
        const R c2 = ar * ar;
        sr = a02 > c2 ? sqrt(R(2) / (g - R(1)) * (a02 - c2)) : R(0);  // MixtPerf_Vm_C2Co2G
      }
      rr = pr / (rgas * tr);
      const R ur = sr * cbh * cbv, vr = sr * sbh, wr = sr * cbh * sbv;
      rer = rr * (pr / (rr * (g - R(1))) + R(0.5) * sr * sr + R(0));  // MixtPerf_Eo_DGPVm
      rur = rr * ur;
      rvr = rr * vr;
      rwr = rr * wr;
      return;
    }
    prescribed = opt == 2;  // BCOPT_MIXED
  }
  if (prescribed) {
    rr = d[8];
    rur = d[9];
    rvr = d[10];
    rwr = d[11];
    rer = d[12];
    pr = d[13];
  } else {
    rr = rl;
    rur = rul;
    rvr = rvl;
    rwr = rwl;
    rer = rel;
    pr = pl;
  }
}

// Outflow boundary state, libfloflu/BcondOutflowPerf.F90:88-160 (ksg = 0).
template <typename R>
__device__ __forceinline__ void bcond_outflow(int bcOpt, R pout, R sxn, R syn, R szn, R gamma,
                                              R rho, R rhou, R rhov, R rhow, R rhoe, R press,
                                              R &rhob, R &rhoub, R &rhovb, R &rhowb, R &rhoeb) {
  R u = rhou / rho, v = rhov / rho, w = rhow / rho;
  R csound = sqrt(gamma * press / rho);
  R mach = sqrt(u * u + v * v + w * w) / csound;
  if (mach < R(1) && (bcOpt == 1 || bcOpt == 2)) {
    R rrhoc = R(1) / (rho * csound);
    R deltp = press - pout;
    rhob = rho - deltp / (csound * csound);
    R ub = u + sxn * deltp * rrhoc;
    R vb = v + syn * deltp * rrhoc;
    R wb = w + szn * deltp * rrhoc;
    R vnd = ub * sxn + vb * syn + wb * szn;
    if (vnd < R(0)) {
      ub = copysign(R(1), u) * rmax(fabs(ub), fabs(u));
      vb = copysign(R(1), v) * rmax(fabs(vb), fabs(v));
      wb = copysign(R(1), w) * rmax(fabs(wb), fabs(w));
    }
    rhoub = rhob * ub;
    rhovb = rhob * vb;
    rhowb = rhob * wb;
    rhoeb = rhob * eo_dgpuvw(rhob, gamma, pout, ub, vb, wb);
  } else {
    rhob = rho;
    rhoub = rhou;
    rhovb = rhov;
    rhowb = rhow;
    rhoeb = rhoe;
  }
}

// Boundary face fluxes: slip wall and outflow patches of
// rocflu/RFLU_CentralSecondPatch.F90:638-1013 (ORDER 2) and
// rocflu/RFLU_CentralFirstPatch.F90:575-946 (ORDER 1).  Slip walls store -0.0
// as mass flux, the exact additive identity, since the reference leaves the
// mass residual untouched there.
template <typename R>
__device__ __forceinline__ void bface_tile(const RegionDev<R> *__restrict__ regs,
                                           const Tile *__restrict__ tiles, int t_) {
  {
    const Tile tl = tiles[t_];
    const RegionDev<R> &g = regs[tl.region];
    const int b = tl.first + threadIdx.x;
    const int B = g.nBFaces;
    if (b >= B) return;
    const int N = g.nCells;
    const int c = g.bf2c[b];
    const int kind = g.bkind[b];
    const int type = kind & 15, order = (kind >> 4) & 15, opt = kind >> 8;
    R nrm[4];
    ld4(g.bfnA + 4 * (size_t)b, nrm);
    const R nx = nrm[0], ny = nrm[1], nz = nrm[2], nm = nrm[3];
    const R fs = R(0);
    R flx[8];
    R rc[8];
    ld8(g.rec + 8 * (size_t)c, rc);
    R S[5], ir;
    cell_values(g, c, rc, S, ir);
    if (order == 2) {
      R G[16];
      ld16(g.grad + 16 * (size_t)c, G);
      reconstruct(G, g.bfd[b], g.bfd[B + b], g.bfd[2 * B + b], S);
    }
    const R gvG = PC<R>{g.ph}.gvG();
    if (type == BK_SLIP) {
      R pl = S[4];
      flx[0] = R(-0.0);
      flx[1] = pl * nx * nm;
      flx[2] = pl * ny * nm;
      flx[3] = pl * nz * nm;
      flx[4] = pl * fs * nm;
    } else if (type == BK_INJECTION && g.bdat[kBData * (size_t)b] > R(0)) {
      // burning surface (RFLU_CentralSecondPatch.F90:1237-1351 / FirstPatch
      // :1049-1133 with RFLU_SetRindStateInjectPerf, RFLU_ModRindStates.F90:460-505)
      const R minj = g.bdat[kBData * (size_t)b], tinj = g.bdat[kBData * (size_t)b + 1];
      const R rGas = R(g.ph.gvR), cpGas = R(g.ph.gvCp);
      const R pl = S[4];
      const R rl = pl / (rGas * tinj);
      const R ql = -minj / rl + fs;
      const R ul = ql * nx, vl = ql * ny, wl = ql * nz;
      const R Hl = cpGas * tinj + R(0.5) * (ul * ul + vl * vl + wl * wl) + R(0);
      flx[0] = -minj * nm;
      flx[1] = (-minj * ul + pl * nx) * nm;
      flx[2] = (-minj * vl + pl * ny) * nm;
      flx[3] = (-minj * wl + pl * nz) * nm;
      flx[4] = (-minj * Hl + pl * fs) * nm;
    } else {
      R rl, rul, rvl, rwl, rel, pl;
      if (order == 2) {
        rl = S[0];
        pl = S[4];
        rul = rl * S[1];
        rvl = rl * S[2];
        rwl = rl * S[3];
        rel = rl * eo_dgpuvw(rl, gvG, pl, S[1], S[2], S[3]);
      } else {
        rl = rc[0];
        pl = rc[4];
        if (sizeof(R) == 8 && g.ph.spaceOrder == 1) {  // no conversion round trip
          rul = R(g.cv[N + c]);
          rvl = R(g.cv[2 * N + c]);
          rwl = R(g.cv[3 * N + c]);
          rel = R(g.cv[4 * N + c]);
        } else {  // cv as CellGradientsMP's Prim2Cons left it
          R u = rc[1], v = rc[2], w = rc[3];
          rul = rl * u;
          rvl = rl * v;
          rwl = rl * w;
          rel = rl * eo_dgpuvw(rl, gvG, pl, u, v, w);
        }
      }
      if (type == BK_INJECTION) {
        // surface not burning: slip-wall rind pressure (RFLU_SetRindStateSlipWallPerf,
        // RFLU_ModRindStates.F90:539-588); the mass flux is a +0 contribution
        const R irl = R(1) / rl;
        const R ul = irl * rul, vl = irl * rvl, wl = irl * rwl;
        const R ql = ul * nx + vl * ny + wl * nz - fs;
        const R al = sqrt(gvG * pl / rl);
        if (ql < R(0)) {
          const R term = R(1) + R(0.5) * (gvG - R(1)) * ql / al;
          pl = pl * pow(term, R(2) * gvG / (gvG - R(1)));
        } else {
          const R term = (gvG + R(1)) / R(4);
          pl = pl + term * rl * ql * (ql + sqrt(al * al + term * term * ql * ql) / term);
        }
        flx[0] = R(0);
        flx[1] = pl * nx * nm;
        flx[2] = pl * ny * nm;
        flx[3] = pl * nz * nm;
        flx[4] = pl * fs * nm;
      } else {
        R pr, rr, rur, rvr, rwr, rer;
        if (type == BK_FARFIELD) {
          farfield_rind(g.bdat + kBData * (size_t)b, gvG, nx, ny, nz, rl, rul, rvl, rwl, rel, rr, rur,
                        rvr, rwr, rer, pr);
        } else if (type == BK_INFLOW_TA) {
          inflow_totang(g.bdat + kBData * (size_t)b, opt, gvG, R(g.ph.gvR), nx, ny, nz, rl, rul, rvl,
                        rwl, rel, pl, rr, rur, rvr, rwr, rer, pr);
        } else if (type == BK_INFLOW_VT) {
          const R *d = g.bdat + kBData * (size_t)b;
          const R ur = d[0], vr = d[1], wr = d[2], tr = d[3], rGas = R(g.ph.gvR);
          if (opt != 1) {  // BCOPT_SUBSONIC
            pr = d[4];
            rr = pr / (rGas * tr);  // MixtPerf_D_PRT
          } else {
            rr = rl;
            pr = rr * rGas * tr;    // MixtPerf_P_DRT
          }
          rer = rr * eo_dgpuvw(rr, gvG, pr, ur, vr, wr);
          rur = rr * ur;
          rvr = rr * vr;
          rwr = rr * wr;
        } else {
          pr = (opt != 0) ? R(g.bpout[b]) : pl;
          bcond_outflow(opt, pr, nx, ny, nz, gvG, rl, rul, rvl, rwl, rel, pl, rr, rur, rvr, rwr,
                        rer);
        }
        R ql = (rul * nx + rvl * ny + rwl * nz) / rl - fs;
        R qr = (rur * nx + rvr * ny + rwr * nz) / rr - fs;
        flx[0] = R(0.5) * (ql * rl + qr * rr) * nm;
        flx[1] = R(0.5) * (ql * rul + pl * nx + qr * rur + pr * nx) * nm;
        flx[2] = R(0.5) * (ql * rvl + pl * ny + qr * rvr + pr * ny) * nm;
        flx[3] = R(0.5) * (ql * rwl + pl * nz + qr * rwr + pr * nz) * nm;
        flx[4] = R(0.5) * (ql * (rel + pl) + pl * fs + qr * (rer + pr) + pr * fs) * nm;
      }
    }
    flx[5] = flx[6] = flx[7] = R(0);
    st8(g.bflux + 8 * (size_t)b, flx);
  }
}

template <typename R>
__global__ void __launch_bounds__(128) k_bface_flux(const RegionDev<R> *__restrict__ regs,
                                                    const Tile *__restrict__ tiles, int nTiles) {
  RF_TILE_LOOP(tiles, nTiles) bface_tile<R>(regs, tiles, t_);
}

// AfterUpdateMP checks for one cell (libfloflu/AfterUpdateMP.F90:134-136):
// RFLU_CheckValidity, RFLU_EnforceBounds (libflu/RFLU_EnforceBounds.F90:163-232),
// RFLU_CheckPositivity (libflu/RFLU_CheckPositivity.F90).  Returns status bits.
__device__ __forceinline__ unsigned after_update(double gc, double gg, double q[5], double d[3]) {
  unsigned st = 0;
  {
    double rho = q[0], rrho = 1.0 / rho;
    double u = rrho * q[1], v = rrho * q[2], w = rrho * q[3];
    if (isnan(rho) || isnan(u) || isnan(v) || isnan(w) || isnan(d[0]) || isnan(d[1])) st |= 1u;
  }
  {
    const double pTol = 1.0e-12;
    double rr = q[0], ir = 1.0 / rr;
    double u = ir * q[1], v = ir * q[2], w = ir * q[3], Eo = ir * q[4];
    double Vm2 = u * u + v * v + w * w;
    double p = (gg - 1.0) * rr * (Eo - 0.5 * Vm2 - 0.0);
    if (p <= 0.0 && fabs(p) <= pTol) {
      p = pTol;
      q[4] = rr * (p / (rr * (gg - 1.0)) + 0.5 * (u * u + v * v + w * w) + 0.0);
      st |= 8u;
    }
  }
  {
    double rho = q[0], rrho = 1.0 / rho;
    double u = rrho * q[1], v = rrho * q[2], w = rrho * q[3];
    double Vm2 = u * u + v * v + w * w;
    double p = d[0];
    if (p <= 0.0) {
      double Eo = 1.0e4 + 0.5 * Vm2 + 0.0;
      p = (gg - 1.0) * rho * (Eo - 0.5 * Vm2 - 0.0);
      d[0] = p;
      d[1] = p / (rho * gc);
      q[4] = rho * Eo;
      st |= 4u;
    }
    if (rho <= 0.0 || p <= 0.0) st |= 2u;
  }
  return st;
}

// Error-free transformation of a + b (Knuth's TwoSum); lo collects the
// rounding errors, so hi + lo carries about twice the FP32 significand.
__device__ __forceinline__ void two_sum_acc(float &hi, float &lo, float x) {
  float s = hi + x;
  float bb = s - hi;
  float err = (hi - (s - bb)) + (x - bb);
  hi = s;
  lo += err;
}

// (hi, lo) - d for a float-float pair: TwoSum of hi and -d, the low part and
// the rounding error added, then renormalised with TwoSum.  Additions only, so
// no contraction into FMA can change it.
__device__ __forceinline__ void ff_sub(float &hi, float &lo, float d) {
  const float s = hi - d;
  const float bb = s - hi;
  const float e = (hi - (s - bb)) + (-d - bb);
  const float t = lo + e;
  const float h2 = s + t;
  const float b2 = h2 - s;
  lo = (s - (h2 - b2)) + (t - b2);
  hi = h2;
}

// Mixed-path gather + update.  The FP32 face fluxes are summed with
// compensated (TwoSum) accumulation, so the residual is the FP32-rounded exact
// sum of the fluxes regardless of cancellation; the RK increment
// dU = a*dt/V (rhs - g rhsSum) is formed in FP32 and subtracted from the
// float-float conserved state exactly (ff_sub), so the state carries about 48
// significand bits without FP64 arithmetic (GB300's FP64 rate is a small
// fraction of its FP32 rate).  The pressure for the cell record is
// (g-1)((E_hi - |m|^2/(2 rho)) + E_lo) in FP32: the total energy keeps its low
// part and only the kinetic term is rounded.  Cells whose density or pressure
// is not clearly positive take the exact FP64 checks of AfterUpdateMP on the
// joined state.  dv (p, T, a) is evaluated in FP64 on download.
__device__ __forceinline__ void gather_update_mixed(const RegionDev<float> &g, int c,
                                                    const StepArgs &a) {
  const int N = g.nCells;
  const Phys &ph = g.ph;
  const int is = a.istage;
  const float *cvF = g.cvF;
  // own-cell loads first: they are independent of the flux gathers below
  float qh[5], ql[5];
  float rsOld[5];
  float r[8];
  float ivol = 0.f;
  if (a.update) {
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      qh[j] = lds_rw<RF_HINT_U>(cvF + (size_t)j * N + c);
      ql[j] = lds_rw<RF_HINT_U>(cvF + (size_t)(5 + j) * N + c);
    }
#pragma unroll
    for (int j = 0; j < 5; ++j)
      rsOld[j] = (is > 1) ? lds_rw<RF_HINT_U>(g.rhsSumF + j * N + c) : 0.f;
    ld8_rw(g.rec + 8 * (size_t)c, r);  // the non-coherent path measured the same (0.598 ms)
    ivol = lds<RF_HINT_U>(g.ivolF + c);
  }
  float hi[5] = {0.f, 0.f, 0.f, 0.f, 0.f}, lo[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  const long long e0 = g.cfOff[c >> 5] + (c & 31);
  const int n = g.cfCnt[c];
  auto face = [&](int code) {
    float fl[8];
    if (code >= 0) {
      ld8(g.flux + 8 * (size_t)(code >> 1), fl);
      const float sg = (code & 1) ? -1.f : 1.f;
#pragma unroll
      for (int j = 0; j < 5; ++j) two_sum_acc(hi[j], lo[j], sg * fl[j]);
    } else {
      ld8(g.bflux + 8 * (size_t)(-code - 1), fl);
#pragma unroll
      for (int j = 0; j < 5; ++j) two_sum_acc(hi[j], lo[j], fl[j]);
    }
  };
  // the first faces' codes loaded together, ahead of their flux gathers
  constexpr int MF = RF_UPD_PRE;
  int cc[MF];
#pragma unroll
  for (int k = 0; k < MF; ++k)
    cc[k] = k < n ? lds<RF_HINT_U>(g.cfCode + e0 + (long long)k * kSlice) : 0;
#pragma unroll
  for (int k = 0; k < MF; ++k)
    if (k < n) face(cc[k]);
  for (int k = MF; k < n; ++k) face(lds<RF_HINT_U>(g.cfCode + e0 + (long long)k * kSlice));
  if (a.writeRhs) {
#pragma unroll
    for (int j = 0; j < 5; ++j) g.rhs[j * N + c] = double(hi[j]) + double(lo[j]);
  }
  if (!a.update) return;
  float rhs[5];
#pragma unroll
  for (int j = 0; j < 5; ++j) rhs[j] = hi[j] + lo[j];
  // the device time step is read through L2 (__ldcg): in a persistent stage
  // launch another block wrote it earlier in the same kernel
  const float fac = a.useDeviceDt ? float(__ldcg(g.scal + 3 + is - 1)) : float(ph.ark[is - 1] * a.dtHost);
  const float adtv = fac * ivol;
  const float grk = ph.grkF[is - 1];
  float oh[5], ol[5];
  if (ph.rkScheme == 1) {
    if (is == 1) {
#pragma unroll
      for (int j = 0; j < 5; ++j) {
        oh[j] = qh[j];
        ol[j] = ql[j];
        g.cvOldF[(size_t)j * N + c] = qh[j];
        g.cvOldF[(size_t)(5 + j) * N + c] = ql[j];
      }
    } else {
#pragma unroll
      for (int j = 0; j < 5; ++j) {
        oh[j] = g.cvOldF[(size_t)j * N + c];
        ol[j] = g.cvOldF[(size_t)(5 + j) * N + c];
      }
    }
  } else {
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      oh[j] = qh[j];
      ol[j] = ql[j];
    }
  }
  float *rs = g.rhsSumF;
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    float dU;
    if (ph.rkScheme == 2) {
      if (is == 1) {
        dU = adtv * rhs[j];
        rs[j * N + c] = rhs[j];
      } else if (is == 2) {
        dU = adtv * (rhs[j] - grk * rsOld[j]);
        rs[j * N + c] = rhs[j];
      } else {
        dU = adtv * (rhs[j] - grk * rsOld[j]);
      }
    } else if (ph.rkScheme == 1) {
      if (is == 1) {
        dU = adtv * rhs[j];
        rs[j * N + c] = rhs[j];
      } else if (is == ph.nSteps) {
        dU = adtv * (rhs[j] + rsOld[j]);
      } else {
        dU = adtv * rhs[j];
        rs[j * N + c] = rsOld[j] + grk * rhs[j];
      }
    } else {
      dU = adtv * rhs[j];
    }
    qh[j] = oh[j];
    ql[j] = ol[j];
    ff_sub(qh[j], ql[j], dU);
  }
  // EOS of the new state in FP32 from the pairs
  float rr[5];
  record_from_pairs(ph, qh, ql, rr);
  const float rf = rr[0], uf = rr[1], vf = rr[2], wf = rr[3];
  float pf = rr[4];
  if (!(rf > 0.f) || !(pf > 1.0e-12f) || isnan(uf) || isnan(vf) || isnan(wf)) {
    // exact FP64 checks and bounds of AfterUpdateMP on the joined state
    const double gg = ph.gvG;
    double q[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) q[j] = double(qh[j]) + double(ql[j]);
    const double m2 = fma(q[3], q[3], fma(q[2], q[2], q[1] * q[1]));
    double d[3];
    d[0] = (gg - 1.0) * (q[4] - 0.5 * m2 / q[0]);
    d[1] = d[0] / (q[0] * ph.gvR);
    d[2] = 0.0;
    unsigned st = after_update(ph.gvR, gg, q, d);
    if (st) atomicOr(g.status, st);
    pf = float(d[0]);
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      qh[j] = float(q[j]);
      ql[j] = float(q[j] - double(qh[j]));
    }
  }
  float *cvW = g.cvF;
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    cvW[(size_t)j * N + c] = qh[j];
    cvW[(size_t)(5 + j) * N + c] = ql[j];
  }
  r[0] = rf;
  r[1] = uf;
  r[2] = vf;
  r[3] = wf;
  r[4] = pf;
  st8(g.rec + 8 * (size_t)c, r);
}

// FP64 sum of a cell's face fluxes in the reference accumulation order
// (ConvectiveFluxes' scatter restated as a gather: +flux where the cell is the
// face's first cell, -flux where it is the second, boundary faces added),
// starting from -0.0 as the FP64 path does.  The first RF_UPD_PRE face codes
// are loaded together ahead of the flux gathers.
template <typename R>
__device__ __forceinline__ void face_sum64(const RegionDev<R> &g, const R *__restrict__ flux,
                                           int c, double acc[5]) {
  const long long e0 = g.cfOff[c >> 5] + (c & 31);
  const int n = g.cfCnt[c];
#pragma unroll
  for (int j = 0; j < 5; ++j) acc[j] = -0.0;
  auto face = [&](int code) {
    R fl[8];
    if (code >= 0) {
      ld8(flux + 8 * (size_t)(code >> 1), fl);
      if (code & 1) {
#pragma unroll
        for (int j = 0; j < 5; ++j) acc[j] = acc[j] - double(fl[j]);
      } else {
#pragma unroll
        for (int j = 0; j < 5; ++j) acc[j] = acc[j] + double(fl[j]);
      }
    } else {
      ld8(g.bflux + 8 * (size_t)(-code - 1), fl);
#pragma unroll
      for (int j = 0; j < 5; ++j) acc[j] = acc[j] + double(fl[j]);
    }
  };
  constexpr int MF = RF_UPD_PRE;
  int cc[MF];
#pragma unroll
  for (int k = 0; k < MF; ++k)
    cc[k] = k < n ? lds<RF_HINT_U>(g.cfCode + e0 + (long long)k * kSlice) : 0;
#pragma unroll
  for (int k = 0; k < MF; ++k)
    if (k < n) face(cc[k]);
  for (int k = MF; k < n; ++k) face(lds<RF_HINT_U>(g.cfCode + e0 + (long long)k * kSlice));
}

// Split-path gather + update: the FP32 face fluxes summed in FP64, the RK
// update of the FP64 conserved state (libfloflu/RkUpdateGeneric.F90:229-314)
// and the EOS (libflu/RFLU_SetDependentVars.F90:256-287) in FP64, with the
// reference's operation order except that a*dt/V is a*dt times the stored
// 1/V.  The FP32 record (rho, u, v, w, p) for the next stage's gathers is
// rounded from the FP64 values.  AfterUpdateMP's checks
// (libfloflu/AfterUpdateMP.F90:134-136) change nothing and set no bit when
// rho > 0, p > 0 and the velocities are not NaN, so only other cells run them.
__device__ __forceinline__ void gather_update_split(const RegionDev<float> &g, int c,
                                                    const StepArgs &a) {
  const int N = g.nCells;
  const Phys &ph = g.ph;
  const int is = a.istage;
  double q[5], rsOld[5];
  float r[8];
  double ivol = 0.0;
  if (a.update) {  // own-cell loads first: independent of the flux gathers
#pragma unroll
    for (int j = 0; j < 5; ++j) q[j] = lds_rw<RF_HINT_U>(g.cv + (size_t)j * N + c);
    const bool hist = is > 1 && ph.rkScheme != 3;
#pragma unroll
    for (int j = 0; j < 5; ++j) rsOld[j] = hist ? lds_rw<RF_HINT_U>(g.rhsSum + (size_t)j * N + c) : 0.0;
    ld8_rw(g.rec + 8 * (size_t)c, r);
    ivol = lds<RF_HINT_U>(g.ivol + c);
  }
  double acc[5];
  face_sum64(g, g.flux, c, acc);
  if (a.writeRhs) {
#pragma unroll
    for (int j = 0; j < 5; ++j) g.rhs[(size_t)j * N + c] = acc[j];
  }
  if (!a.update) return;
  const double fac = a.useDeviceDt ? __ldcg(g.scal + 3 + is - 1) : ph.ark[is - 1] * a.dtHost;
  const double adtv = fac * ivol;
  const double grk = ph.grk[is - 1];
  double old[5];
  if (ph.rkScheme == 1) {  // RK4: cvOld saved at stage 1 only
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      if (is == 1) {
        old[j] = q[j];
        g.cvOld[(size_t)j * N + c] = q[j];
      } else {
        old[j] = g.cvOld[(size_t)j * N + c];
      }
    }
  } else {  // Wray / Euler: cvOld = cv at every stage start
#pragma unroll
    for (int j = 0; j < 5; ++j) old[j] = q[j];
  }
  double *rs = g.rhsSum;
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    const double rhs = acc[j];
    if (ph.rkScheme == 2) {
      if (is == 1) {
        q[j] = old[j] - adtv * rhs;
        rs[(size_t)j * N + c] = rhs;
      } else if (is == 2) {
        q[j] = old[j] - adtv * (rhs - grk * rsOld[j]);
        rs[(size_t)j * N + c] = rhs;
      } else {
        q[j] = old[j] - adtv * (rhs - grk * rsOld[j]);
      }
    } else if (ph.rkScheme == 1) {
      if (is == 1) {
        q[j] = old[j] - adtv * rhs;
        rs[(size_t)j * N + c] = rhs;
      } else if (is == ph.nSteps) {
        q[j] = old[j] - adtv * (rhs + rsOld[j]);
      } else {
        q[j] = old[j] - adtv * rhs;
        rs[(size_t)j * N + c] = rsOld[j] + grk * rhs;
      }
    } else {
      q[j] = old[j] - adtv * rhs;
    }
  }
  double ir;
  double p = eos_p(ph, q, ir);
  if (!(q[0] > 0.0 && p > 0.0) || isnan(ir * q[1]) || isnan(ir * q[2]) || isnan(ir * q[3])) {
    double d[3];
    d[0] = p;
    d[1] = p / (q[0] * ph.gvR);
    d[2] = 0.0;
    const unsigned st = after_update(ph.gvR, ph.gvG, q, d);
    if (st) atomicOr(g.status, st);
    p = d[0];
    ir = 1.0 / q[0];
  }
#pragma unroll
  for (int j = 0; j < 5; ++j) g.cv[(size_t)j * N + c] = q[j];
  record_from_fp64(q, ir, p, r);
  st8(g.rec + 8 * (size_t)c, r);
}

// Face->cell residual gather in the reference accumulation order, then the
// RK update (libfloflu/RkUpdateGeneric.F90:229-314), EOS
// (libflu/RFLU_SetDependentVars.F90:256-287), AfterUpdate checks and
// Cons2Prim of the new state for the next stage.  With update = 0 only the
// residual is written (rfgpu_residual).
// SPLIT selects the split path's update at compile time (a run-time branch
// between the two FP32-flux updates costs the mixed path registers).
template <typename R, int SPLIT>
__device__ __forceinline__ void update_tile(const RegionDev<R> *__restrict__ regs,
                                            const Tile *__restrict__ tiles, int nTiles, int t_,
                                            const StepArgs &a, int dist) {
  {
    const Tile tl = tiles[t_];
    const RegionDev<R> &g = regs[tl.region];
    prefetch_ahead(t_, nTiles, dist, [&](int t) {
      const Tile tp = tiles[t];
      prefetch_update_tile(regs[tp.region], tp.first);
    });
    const int c = tl.first + threadIdx.x;
    const int N = g.nCells;
    if (c >= N) return;
    if (c >= g.nAct) {  // virtual cell: ZeroDummyCellsMP, no update
      if (a.writeRhs) {
#pragma unroll
        for (int j = 0; j < 5; ++j) g.rhs[j * N + c] = 0.0;
      }
      return;
    }
    if constexpr (sizeof(R) == 4) {
      if constexpr (SPLIT)
        gather_update_split(g, c, a);
      else
        gather_update_mixed(g, c, a);
      return;
    }
    double acc[5] = {-0.0, -0.0, -0.0, -0.0, -0.0};
    const long long e0 = g.cfOff[c >> 5] + (c & 31);
    const int n = g.cfCnt[c];
    for (int k = 0; k < n; ++k) {
      const int code = g.cfCode[e0 + (long long)k * kSlice];
      R fl[8];
      if (code >= 0) {
        ld8(g.flux + 8 * (size_t)(code >> 1), fl);
        if (code & 1) {
#pragma unroll
          for (int j = 0; j < 5; ++j) acc[j] = acc[j] - double(fl[j]);
        } else {
#pragma unroll
          for (int j = 0; j < 5; ++j) acc[j] = acc[j] + double(fl[j]);
        }
      } else {
        ld8(g.bflux + 8 * (size_t)(-code - 1), fl);
#pragma unroll
        for (int j = 0; j < 5; ++j) acc[j] = acc[j] + double(fl[j]);
      }
    }
    if (a.writeRhs) {
#pragma unroll
      for (int j = 0; j < 5; ++j) g.rhs[j * N + c] = acc[j];
    }
    if (!a.update) return;
    const Phys &ph = g.ph;
    const int is = a.istage;
    const double fac = a.useDeviceDt ? __ldcg(g.scal + 3 + is - 1) : ph.ark[is - 1] * a.dtHost;
    const double adtv = fac / g.vol[c];
    double q[5], old[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) q[j] = g.cv[j * N + c];
    if (ph.rkScheme == 1) {  // RK4: cvOld saved at stage 1 only
      if (is == 1) {
#pragma unroll
        for (int j = 0; j < 5; ++j) {
          old[j] = q[j];
          g.cvOld[j * N + c] = q[j];
        }
      } else {
#pragma unroll
        for (int j = 0; j < 5; ++j) old[j] = g.cvOld[j * N + c];
      }
    } else {  // Wray / Euler: cvOld = cv at every stage start
#pragma unroll
      for (int j = 0; j < 5; ++j) old[j] = q[j];
    }
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      const double rhs = acc[j];
      if (ph.rkScheme == 2) {
        if (is == 1) {
          q[j] = old[j] - adtv * rhs;
          g.rhsSum[j * N + c] = rhs;
        } else if (is == 2) {
          q[j] = old[j] - adtv * (rhs - ph.grk[is - 1] * g.rhsSum[j * N + c]);
          g.rhsSum[j * N + c] = rhs;
        } else {
          q[j] = old[j] - adtv * (rhs - ph.grk[is - 1] * g.rhsSum[j * N + c]);
        }
      } else if (ph.rkScheme == 1) {
        if (is == 1) {
          q[j] = old[j] - adtv * rhs;
          g.rhsSum[j * N + c] = rhs;
        } else if (is == ph.nSteps) {
          q[j] = old[j] - adtv * (rhs + g.rhsSum[j * N + c]);
        } else {
          q[j] = old[j] - adtv * rhs;
          g.rhsSum[j * N + c] = g.rhsSum[j * N + c] + ph.grk[is - 1] * rhs;
        }
      } else {
        q[j] = old[j] - adtv * rhs;
      }
    }
    // EOS
    const double gc = ph.gvR, gg = ph.gvG;
    double d[3];
    {
      double rr = q[0];
      double ir = 1.0 / rr;
      double Eo = ir * q[4];
      double Vm2 = ir * ir * (q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
      d[0] = (gg - 1.0) * rr * (Eo - 0.5 * Vm2 - 0.0);
      d[1] = d[0] / (rr * gc);
      d[2] = sqrt(gg * gc * d[1]);
    }
    unsigned st = after_update(gc, gg, q, d);
    if (st) atomicOr(g.status, st);
#pragma unroll
    for (int j = 0; j < 5; ++j) g.cv[j * N + c] = q[j];
    g.dv[c] = d[0];
    g.dv[N + c] = d[1];
    g.dv[2 * N + c] = d[2];
    const double ir = 1.0 / q[0];
    R r[8];
    ld8_rw(g.rec + 8 * (size_t)c, r);
    r[0] = R(q[0]);
    r[1] = R(ir * q[1]);
    r[2] = R(ir * q[2]);
    r[3] = R(ir * q[3]);
    r[4] = R(d[0]);
    st8(g.rec + 8 * (size_t)c, r);
  }
}

template <typename R, int BS, int SPLIT>
__global__ void __launch_bounds__(BS) k_gather_update(const RegionDev<R> *__restrict__ regs,
                                                      const Tile *__restrict__ tiles,
                                                      int nTiles, StepArgs a, int pfDist) {
  const int dist = (int)gridDim.x < nTiles ? (int)gridDim.x : pfDist;
  RF_TILE_LOOP(tiles, nTiles) update_tile<R, SPLIT>(regs, tiles, nTiles, t_, a, dist);
}

// Mixed path transfers: the host's Fortran images cv(5,N) / dv(3,N), copied
// by DMA into device staging buffers, are converted in one pass per direction
// and chunk, fusing the numbering, layout and precision conversions (upload:
// cons -> record with the EOS of k_prim, float-float split; download:
// float-float join, FP64 dv).  One thread per device cell of the chunk's list
// (its cells in ascending device order), so the device-side state is read and
// written coalesced and the Fortran images are addressed by host cell; one
// thread per host cell scattered the state's ten SoA rows instead.  Kernels
// reading or writing page-locked host memory directly over the CPU-GPU link
// were measured slower than the DMA copies (32 against 20 ms per end-to-end
// step).
template <typename R, int SPLIT>
__global__ void k_upload_list(const RegionDev<R> *__restrict__ regs, const int *__restrict__ list,
                              int n, const double *__restrict__ cvH, const double *__restrict__ dvH) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const RegionDev<R> &g = regs[0];
  const int c = list[i];
  const int h = g.cellOld ? g.cellOld[c] : c;
  double q[5];
#pragma unroll
  for (int j = 0; j < 5; ++j) q[j] = cvH[5 * (size_t)h + j];
  if constexpr (sizeof(R) == 4) {
    if constexpr (SPLIT)
      state_from_fp64_split(g, c, q, dvH ? dvH + 3 * (size_t)h : nullptr);
    else
      state_from_fp64_ff(g, c, q, dvH ? dvH + 3 * (size_t)h : nullptr);
  }
}

template <typename R, int SPLIT>
__global__ void k_download_list(const RegionDev<R> *__restrict__ regs, const int *__restrict__ list,
                                int n, double *__restrict__ cvH, double *__restrict__ dvH) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const RegionDev<R> &g = regs[0];
  const int c = list[i];
  const int h = g.cellOld ? g.cellOld[c] : c;
  const int N = g.nCells;
  double q[5];
  if constexpr (SPLIT) {
#pragma unroll
    for (int j = 0; j < 5; ++j) q[j] = g.cv[(size_t)j * N + c];
  } else {
#pragma unroll
    for (int j = 0; j < 5; ++j)
      q[j] = widen_f32(g.cvF[(size_t)j * N + c]) + widen_f32(g.cvF[(size_t)(5 + j) * N + c]);
  }
  if (cvH) {
#pragma unroll
    for (int j = 0; j < 5; ++j) cvH[5 * (size_t)h + j] = q[j];
  }
  if (dvH && SPLIT) {  // split path: the EOS of its update
    const double gc = g.ph.gvR, gg = g.ph.gvG;
    double ir;
    const double p = eos_p(g.ph, q, ir);
    const double T = p / (q[0] * gc);
    dvH[3 * (size_t)h] = p;
    dvH[3 * (size_t)h + 1] = T;
    dvH[3 * (size_t)h + 2] = sqrt(gg * gc * T);
  } else if (dvH) {
    // FP64 EOS of the joined pairs with one division (by rho) instead of two:
    // the conversion is FP64-pipe bound
    const double gc = g.ph.gvR, gg = g.ph.gvG;
    const double m2 = fma(q[3], q[3], fma(q[2], q[2], q[1] * q[1]));
    const double ir = 1.0 / q[0];
    const double p = (gg - 1.0) * (q[4] - 0.5 * m2 * ir);
    const double T = p * ir * g.ph.gvRinv;
    dvH[3 * (size_t)h] = p;
    dvH[3 * (size_t)h + 1] = T;
    dvH[3 * (size_t)h + 2] = sqrt(gg * gc * T);
  }
}

// ---- time step (standalone pass): per-cell gather of cell_dt, block minimum,
// then an atomic minimum on the bit pattern (dt > 0: the IEEE order equals
// the unsigned integer order).
template <typename R>
__global__ void __launch_bounds__(128) k_dt_cell(const RegionDev<R> *__restrict__ regs,
                                                 const Tile *__restrict__ tiles, int nTiles) {
  __shared__ unsigned long long smin[32];
  RF_TILE_LOOP(tiles, nTiles) {
    const Tile tl = tiles[t_];
    const RegionDev<R> &g = regs[tl.region];
    const int c = tl.first + threadIdx.x;
    unsigned long long bits = 0x7FF0000000000000ull;  // +inf
    if (c < g.nAct) {
      R r0[8];
      ld8(g.rec + 8 * (size_t)c, r0);
      bits = (unsigned long long)__double_as_longlong(cell_dt(g, c, r0));
    }
    dt_block_min<R>(bits, smin, g.dtBits);
  }
}

// RFLU_MinimumTimeStep (rocflu/RFLU_MinimumTimeStep.F90:131-146,235-241) and the
// end-time clip of rocflu/RFLU_TimeStepping.F90:490-493 for one region, from
// the minimum local time step `raw` (bit pattern).
template <typename R>
__device__ __forceinline__ void dt_finalize_region(const RegionDev<R> &g, unsigned long long raw,
                                                   const DtArgs &a) {
  double dtMin = __longlong_as_double((long long)raw);
  const double t = a.useDeviceTime ? __ldcg(g.scal + 1) : a.timeHost;
  dtMin = a.cfl * dtMin;
  double wI = 0.0, wC = 0.0;
  if (t <= 1.0e-08) wI = 1.0; else wC = 1.0;
  dtMin = wI / a.dtImposed + wC / dtMin;
  dtMin = 1.0 / dtMin;
  if (dtMin <= 0.0) dtMin = 6.0e-12;
  dtMin = (a.dtMinLimit > dtMin) ? a.dtMinLimit : dtMin;
  double tNew = t + dtMin;
  if (a.endTime > 0.0 && t + dtMin > a.endTime) {
    dtMin = a.endTime - t;
    tNew = a.endTime;
  }
  if (a.endTime > 0.0 && t >= a.endTime) {  // finished: later stages leave cv as is
    dtMin = 0.0;
    tNew = t;
  }
  g.scal[0] = dtMin;
  g.scal[2] = dtMin;
  for (int i = 0; i < 5; ++i) g.scal[3 + i] = g.ph.ark[i] * dtMin;  // fac of RkUpdateGeneric
  if (a.useDeviceTime) g.scal[1] = tNew;
}

// One thread per independent region.
template <typename R>
__global__ void k_dt_finalize(const RegionDev<R> *__restrict__ regs, int nRegions, DtArgs a) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nRegions) return;
  const RegionDev<R> &g = regs[r];
  const unsigned long long raw = *g.dtBits;
  *g.dtBits = 0x7FF0000000000000ull;
  dt_finalize_region(g, raw, a);
}

// Coupled regions (one block): the minimum over all regions first, as the
// reference's MIN over local regions and MPI_Allreduce(MPI_MIN)
// (RFLU_MinimumTimeStep.F90:148-208), then every region finalizes it.  The
// per-region steps of RFLU_MinimumTimeStep (cfl scaling, imposed/computed
// weighting, floor, dtMinLimit) are monotone non-decreasing, so applying them
// to the minimum gives the reference's minimum of the per-region results.
template <typename R>
__global__ void k_dt_finalize_coupled(const RegionDev<R> *__restrict__ regs, int nRegions,
                                      DtArgs a) {
  __shared__ unsigned long long smin[32];
  unsigned long long v = 0x7FF0000000000000ull;
  for (int r = threadIdx.x; r < nRegions; r += blockDim.x) {
    const unsigned long long x = *regs[r].dtBits;
    v = x < v ? x : v;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_down_sync(0xffffffffu, v, o);
    v = x < v ? x : v;
  }
  if ((threadIdx.x & 31) == 0) smin[threadIdx.x >> 5] = v;
  __syncthreads();
  unsigned long long raw = smin[0];
  for (int w = 1; w < (int)(blockDim.x >> 5); ++w) raw = smin[w] < raw ? smin[w] : raw;
  for (int r = threadIdx.x; r < nRegions; r += blockDim.x) {
    *regs[r].dtBits = 0x7FF0000000000000ull;
    dt_finalize_region(regs[r], raw, a);
  }
}

// The time-step finalisation of a whole Work by one block (the persistent
// stage launch): per region, or the coupled minimum over all regions first,
// as k_dt_finalize / k_dt_finalize_coupled do; the raw minima are read
// through L2, other blocks reduced them earlier in the same kernel.
template <typename R>
__device__ __forceinline__ void dt_finalize_block(const RegionDev<R> *__restrict__ regs,
                                                  const Work &w, const DtArgs &a,
                                                  unsigned long long *smin) {
  if (!w.coupled) {
    for (int r = threadIdx.x; r < w.nRegions; r += blockDim.x) {
      const RegionDev<R> &g = regs[r];
      const unsigned long long raw = __ldcg(g.dtBits);
      *g.dtBits = 0x7FF0000000000000ull;
      dt_finalize_region(g, raw, a);
    }
    return;
  }
  unsigned long long v = 0x7FF0000000000000ull;
  for (int r = threadIdx.x; r < w.nRegions; r += blockDim.x) {
    const unsigned long long x = __ldcg(regs[r].dtBits);
    v = x < v ? x : v;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_down_sync(0xffffffffu, v, o);
    v = x < v ? x : v;
  }
  if ((threadIdx.x & 31) == 0) smin[threadIdx.x >> 5] = v;
  __syncthreads();
  unsigned long long raw = smin[0];
  for (int k = 1; k < (int)(blockDim.x >> 5); ++k) raw = smin[k] < raw ? smin[k] : raw;
  __syncthreads();
  for (int r = threadIdx.x; r < w.nRegions; r += blockDim.x) {
    *regs[r].dtBits = 0x7FF0000000000000ull;
    dt_finalize_region(regs[r], raw, a);
  }
}

template <typename R>
void launch_dt_finalize(const RegionDev<R> *regs, const Work &w, const DtArgs &a,
                        cudaStream_t s) {
  if (w.coupled)
    k_dt_finalize_coupled<R><<<1, 256, 0, s>>>(regs, w.nRegions, a);
  else
    k_dt_finalize<R><<<(w.nRegions + 127) / 128, 128, 0, s>>>(regs, w.nRegions, a);
}

// ---- launchers ----------------------------------------------------------------

template <typename R>
void launch_prim(const RegionDev<R> *regs, const Work &w, int computeDv, cudaStream_t s) {
  int grid = w.grid > 0 && w.grid < w.nCellTiles ? w.grid : w.nCellTiles;
  if (grid > 0) k_prim<R><<<grid, w.block, 0, s>>>(regs, w.cellTiles, w.nCellTiles, computeDv);
}

#define RF_MARK(kind, phase) \
  if (prof) prof->mark(prof->ctx, (kind), (phase), s)

// Blocks of `kernel` (`threads` per block) resident on the whole device at
// once: the prefetch distance in tiles.
template <typename K>
int resident_blocks(K kernel, int threads = 128) {
  int dev = 0, nsm = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, 0);
  return per > 0 && nsm > 0 ? per * nsm : 1;
}

template <typename R>
void launch_weno_xyz(const RegionDev<R> *regs, const Work &w, cudaStream_t s);

// ---- tuned launches: block size (and faces per thread) picked at run time
// from the Work's launch shapes, one template instance per shape -------------
inline int grid_for(int cap, int nTiles) { return cap > 0 && cap < nTiles ? cap : nTiles; }

template <typename R, int F, int BS>
void grad_launch(const RegionDev<R> *regs, const Tile *tiles, int nTiles, int cap, cudaStream_t s) {
  const int grid = grid_for(cap, nTiles);
  if (grid > 0) k_grad_lim<R, F, BS><<<grid, BS, 0, s>>>(regs, tiles, nTiles);
}

template <typename R>
void launch_grad_tuned(const RegionDev<R> *regs, const Work &w, int fuseDt, cudaStream_t s) {
  const bool tuned = w.gradTiles != nullptr;
  const Tile *t = tuned ? w.gradTiles : w.cellTiles;
  const int n = tuned ? w.nGradTiles : w.nCellTiles;
  const int bs = tuned ? w.gradBlock : 128;
  if (bs == 64) {
    if (fuseDt) grad_launch<R, 1, 64>(regs, t, n, w.grid, s);
    else grad_launch<R, 0, 64>(regs, t, n, w.grid, s);
  } else if (bs == 256) {
    if (fuseDt) grad_launch<R, 1, 256>(regs, t, n, w.grid, s);
    else grad_launch<R, 0, 256>(regs, t, n, w.grid, s);
  } else {
    if (fuseDt) grad_launch<R, 1, 128>(regs, t, n, w.grid, s);
    else grad_launch<R, 0, 128>(regs, t, n, w.grid, s);
  }
}

template <typename R, int BS, int FPT>
void face_launch(const RegionDev<R> *regs, const Work &w, cudaStream_t s) {
  static const int pf = resident_blocks(k_face_flux<R, BS, FPT>, BS);
  const int grid = grid_for(w.grid, w.nFaceTiles);
  if (grid > 0) k_face_flux<R, BS, FPT><<<grid, BS, 0, s>>>(regs, w.faceTiles, w.nFaceTiles, pf);
}

template <typename R>
void launch_faces_tuned(const RegionDev<R> *regs, const Work &w, cudaStream_t s) {
  const int bs = w.faceBlock ? w.faceBlock : 128, fpt = w.facesPerThread ? w.facesPerThread : 1;
  if (bs == 64) {
    if (fpt == 2) face_launch<R, 64, 2>(regs, w, s);
    else face_launch<R, 64, 1>(regs, w, s);
  } else if (bs == 256) {
    if (fpt == 2) face_launch<R, 256, 2>(regs, w, s);
    else face_launch<R, 256, 1>(regs, w, s);
  } else {
    if (fpt == 2) face_launch<R, 128, 2>(regs, w, s);
    else face_launch<R, 128, 1>(regs, w, s);
  }
}

template <typename R, int BS, int SPLIT>
void update_launch_k(const RegionDev<R> *regs, const Tile *tiles, int nTiles, int cap,
                     const StepArgs &a, cudaStream_t s) {
  static const int pf = resident_blocks(k_gather_update<R, BS, SPLIT>, BS);
  const int grid = grid_for(cap, nTiles);
  if (grid > 0) k_gather_update<R, BS, SPLIT><<<grid, BS, 0, s>>>(regs, tiles, nTiles, a, pf);
}
template <typename R, int BS>
void update_launch(const RegionDev<R> *regs, const Tile *tiles, int nTiles, int cap,
                   const StepArgs &a, int split, cudaStream_t s) {
  if (sizeof(R) == 4 && split)
    update_launch_k<R, BS, 1>(regs, tiles, nTiles, cap, a, s);
  else
    update_launch_k<R, BS, 0>(regs, tiles, nTiles, cap, a, s);
}

template <typename R>
void launch_update_tuned(const RegionDev<R> *regs, const Work &w, const StepArgs &a,
                         cudaStream_t s) {
  const bool tuned = w.updTiles != nullptr;
  const Tile *t = tuned ? w.updTiles : w.cellTiles;
  const int n = tuned ? w.nUpdTiles : w.nCellTiles;
  const int bs = tuned ? w.cellBlock : 128;
  if (bs == 64) update_launch<R, 64>(regs, t, n, w.grid, a, w.split, s);
  else if (bs == 256) update_launch<R, 256>(regs, t, n, w.grid, a, w.split, s);
  else update_launch<R, 128>(regs, t, n, w.grid, a, w.split, s);
}

// ---- one launch per RK stage ---------------------------------------------------
template <typename R>
__device__ __forceinline__ void weno_tile(const RegionDev<R> *__restrict__ regs,
                                          const Tile *__restrict__ tiles, int t_);

// Grid-wide barrier of the persistent stage kernel, a cooperative launch (so
// every block is resident).  Thread 0 of each block arrives; the last arrival
// clears the count and releases the others by advancing the generation.  Every
// wait is bounded by `spin` SM clock cycles: one that runs out sets bit 0 of
// err, and every block returns as soon as it sees err set after a barrier, so
// the kernel ends and the host reads RFGPU_ERR_TIMEOUT.
__device__ __forceinline__ bool grid_sync(GridBar *b, unsigned expect, long long spin) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned *vgen = &b->gen;
    const unsigned g0 = *vgen;
    __threadfence();
    if (atomicAdd(&b->count, 1u) + 1u == expect) {
      atomicExch(&b->count, 0u);
      __threadfence();
      atomicAdd(&b->gen, 1u);
    } else {
      const long long t0 = clock64();
      while (*vgen == g0) {
        if (clock64() - t0 > spin) {
          atomicOr(&b->err, 1u);
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return *(volatile unsigned *)&b->err == 0;
}

// A whole RK stage of a Work (one region or a batch) in one launch: the
// gradient pass over every cell tile, the WENO-XYZ pass (RECONST 2), the
// time-step finalisation (stage 1 of a step), the interior and boundary face
// passes, the gather + update, and for a coupled batch the halo exchange,
// separated by grid-wide barriers.  The per-tile work is the device code the
// one-pass-per-launch kernels run.  Arrays one phase writes and a later one
// gathers through the read-only path (gradients, face fluxes) are first read
// after the barrier that follows their writes, so no stale copy can be cached;
// scalars and halo sources are read through L2.
#ifndef RF_COOP_MINB
#define RF_COOP_MINB 6  // resident blocks per SM requested for the persistent stage kernel
#endif
template <typename R, int SPLIT>
__global__ void __launch_bounds__(128, (sizeof(R) == 4) ? RF_COOP_MINB : 4)
    k_stage_coop(const RegionDev<R> *__restrict__ regs, Work w, StepArgs a, int grad, int weno) {
  __shared__ unsigned long long smin[32];
  const unsigned expect = gridDim.x + (unsigned)w.barExtra;
  GridBar *bar = w.bar;
  const long long spin = w.barSpin;
  if (grad) {
    for (int t = blockIdx.x; t < w.nCellTiles; t += gridDim.x) {
      if (a.fuseDt)
        grad_tile<R, 1>(regs, w.cellTiles, t, smin);
      else
        grad_tile<R, 0>(regs, w.cellTiles, t, smin);
    }
    if (!grid_sync(bar, expect, spin)) return;
    if (weno) {
      for (int t = blockIdx.x; t < w.nCellTiles; t += gridDim.x) weno_tile<R>(regs, w.cellTiles, t);
      if (!grid_sync(bar, expect, spin)) return;
    }
    if (a.fuseDt) {
      if (blockIdx.x == 0) dt_finalize_block<R>(regs, w, a.dt, smin);
      if (!grid_sync(bar, expect, spin)) return;
    }
  }
  for (int t = blockIdx.x; t < w.nFaceTiles; t += gridDim.x)
    face_tile<R, 128, 1>(regs, w.faceTiles, w.nFaceTiles, t, gridDim.x);
  for (int t = blockIdx.x; t < w.nBFaceTiles; t += gridDim.x) bface_tile<R>(regs, w.bfaceTiles, t);
  if (!grid_sync(bar, expect, spin)) return;
  for (int t = blockIdx.x; t < w.nCellTiles; t += gridDim.x)
    update_tile<R, SPLIT>(regs, w.cellTiles, w.nCellTiles, t, a, gridDim.x);
  if (w.nHalo > 0 && a.update) {
    if (!grid_sync(bar, expect, spin)) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.nHalo; i += gridDim.x * blockDim.x) {
      const HaloLink l = w.halo[i];
      halo_cell(regs[l.srcRegion], l.srcCell, regs[l.dstRegion], l.dstCell);
    }
  }
}

template <typename R, int SPLIT>
void coop_launch(const RegionDev<R> *regs, const Work &w, const StepArgs &a, int grad, int weno,
                 cudaStream_t s) {
  static const int resident = resident_blocks(k_stage_coop<R, SPLIT>, 128);
  int grid = w.nCellTiles > w.nFaceTiles ? w.nCellTiles : w.nFaceTiles;
  if (w.nBFaceTiles > grid) grid = w.nBFaceTiles;
  if (w.grid > 0 && w.grid < grid) grid = w.grid;
  if (grid > resident) grid = resident;
  if (grid < 1) grid = 1;
  cudaMemsetAsync(w.bar, 0, 2 * sizeof(unsigned), s);  // count and generation; err stays
  Work wc = w;
  StepArgs ac = a;
  void *args[] = {(void *)&regs, (void *)&wc, (void *)&ac, (void *)&grad, (void *)&weno};
  cudaLaunchCooperativeKernel((const void *)k_stage_coop<R, SPLIT>, dim3(grid), dim3(128), args, 0,
                              s);
}

template <typename R>
void launch_stage(const RegionDev<R> *regs, const Work &w, const StepArgs &a, cudaStream_t s,
                  long long *launches, int spaceOrder, int reconst, const Prof *prof,
                  int parts) {
  if (w.coop && parts == SP_ALL && w.bar) {
    const int grad = spaceOrder > 1 && w.nCellTiles > 0;
    const int weno = grad && reconst == 2;
    RF_MARK(KP_STAGE, 0);
    if (sizeof(R) == 4 && w.split)
      coop_launch<R, 1>(regs, w, a, grad, weno, s);
    else
      coop_launch<R, 0>(regs, w, a, grad, weno, s);
    RF_MARK(KP_STAGE, 1);
    if (launches) *launches += 1;
    return;
  }
  auto gsz = [&](int nt) { return w.grid > 0 && w.grid < nt ? w.grid : nt; };
  long long n = 0;
  const bool hasGrad = spaceOrder > 1 && w.nCellTiles > 0;
  const bool grad = hasGrad && (parts & SP_GRADIENT);
  const bool flux = parts & SP_FLUX, upd = parts & SP_UPDATE;
  if (grad) {
    RF_MARK(KP_GRADIENT, 0);
    launch_grad_tuned<R>(regs, w, a.fuseDt, s);
    RF_MARK(KP_GRADIENT, 1);
    ++n;
  }
  if (hasGrad && flux && reconst == 2) {  // after every cell's gradient
    RF_MARK(KP_LIMITER, 0);
    launch_weno_xyz<R>(regs, w, s);
    RF_MARK(KP_LIMITER, 1);
    ++n;
  }
  if (a.fuseDt && hasGrad && flux) {
    RF_MARK(KP_DT_FINAL, 0);
    launch_dt_finalize<R>(regs, w, a.dt, s);
    RF_MARK(KP_DT_FINAL, 1);
    ++n;
  }
  if (flux && !(parts & SP_NOFACE) && w.nFaceTiles > 0) {
    RF_MARK(KP_FACE_FLUX, 0);
    launch_faces_tuned<R>(regs, w, s);
    RF_MARK(KP_FACE_FLUX, 1);
    ++n;
  }
  if (flux && w.nBFaceTiles > 0) {
    RF_MARK(KP_BFACE_FLUX, 0);
    k_bface_flux<R><<<gsz(w.nBFaceTiles), w.block, 0, s>>>(regs, w.bfaceTiles, w.nBFaceTiles);
    RF_MARK(KP_BFACE_FLUX, 1);
    ++n;
  }
  if (upd && w.nCellTiles > 0) {
    RF_MARK(KP_GATHER_UPDATE, 0);
    launch_update_tuned<R>(regs, w, a, s);
    RF_MARK(KP_GATHER_UPDATE, 1);
    ++n;
  }
  if (upd && w.nHalo > 0 && a.update) {  // coupled regions: virtual cells from their owners
    RF_MARK(KP_HALO, 0);
    k_halo<R><<<(w.nHalo + 127) / 128, 128, 0, s>>>(regs, w.halo, w.nHalo);
    RF_MARK(KP_HALO, 1);
    ++n;
  }
  if (launches) *launches += n;
}

template <typename R>
void launch_dt(const RegionDev<R> *regs, const Work &w, const DtArgs &a, cudaStream_t s,
               long long *launches, const Prof *prof) {
  auto gsz = [&](int nt) { return w.grid > 0 && w.grid < nt ? w.grid : nt; };
  long long n = 0;
  if (w.nCellTiles > 0) {
    RF_MARK(KP_DT_CELL, 0);
    k_dt_cell<R><<<gsz(w.nCellTiles), w.block, 0, s>>>(regs, w.cellTiles, w.nCellTiles);
    RF_MARK(KP_DT_CELL, 1);
    ++n;
  }
  RF_MARK(KP_DT_FINAL, 0);
  launch_dt_finalize<R>(regs, w, a, s);
  RF_MARK(KP_DT_FINAL, 1);
  ++n;
  if (launches) *launches += n;
}

template <typename R>
void launch_step(const RegionDev<R> *regs, const Work &w, const DtArgs &da, int nStages,
                 cudaStream_t s, long long *launches, int spaceOrder, int reconst,
                 const Prof *prof) {
  const bool fuse = spaceOrder > 1 && w.nCellTiles > 0;
  if (!fuse) launch_dt<R>(regs, w, da, s, launches, prof);
  for (int is = 1; is <= nStages; ++is) {
    StepArgs sa{is, 1, 0.0, 0, 1, (fuse && is == 1) ? 1 : 0, da};
    launch_stage<R>(regs, w, sa, s, launches, spaceOrder, reconst, prof);
  }
}

// RECONST 2 (CellGradientsMP.F90:217-222): RFLU_WENOGradCellsXYZFast_3D
// (modflu/RFLU_ModWENO.F90:1402-1588, the 3-D branch of the wrapper at
// :1615-1668) then RFLU_LimitGradCellsSimple (modflu/RFLU_ModLimiters.F90:
// 793-921), one thread per cell.  Every gradient component becomes the
// average of the cell's and its stencil members' unweighted components
// (gradRaw) weighted by s = 1/(g^2 + 1e-15), the cell first and the members in
// stored order, sum(s g) / sum(s); then the gradient of density and pressure
// (the positive variables, libflu/RFLU_SetVarInfo.F90:140-144) is zeroed when
// var + grad . (fc - xc) is not positive at one of the cell's faces, interior
// or boundary (the result does not depend on the face order).  Regions that
// do not use RECONST 2 skip their tiles.
template <typename R>
__device__ __forceinline__ void weno_tile(const RegionDev<R> *__restrict__ regs,
                                          const Tile *__restrict__ tiles, int t_) {
  {
    const Tile tl = tiles[t_];
    const RegionDev<R> &g = regs[tl.region];
    if (!g.gradRaw) return;
    const int c = tl.first + threadIdx.x;
    if (c >= g.nCells) return;
    const R eps = R(1.0E-15);
    // the weight 1/(g^2 + 1e-15): IEEE division on the FP64 path; on the
    // mixed path optionally the hardware reciprocal (it only weights an average)
    auto weight = [&](R t) -> R {
      if constexpr (sizeof(R) == 4 && RF_WENO_FASTRCP) return __fdividef(1.0f, t * t + eps);
      else return R(1) / (t * t + eps);
    };
    R ss[15], acc[15];
    const long long base = g.stOff[c >> 5] + (c & 31);
    const int n = g.stCnt[c];
    if constexpr (sizeof(R) == 8) {
      // weights and products precomputed by the gradient pass: sums only
      R w[16];
      ld16(g.gradRaw + 32 * (size_t)c, w);
#pragma unroll
      for (int k = 0; k < 15; ++k) ss[k] = w[k];
      ld16(g.gradRaw + 32 * (size_t)c + 16, w);
#pragma unroll
      for (int k = 0; k < 15; ++k) acc[k] = w[k];
      for (int m = 0; m < n; ++m) {
        const R *row = g.gradRaw + 32 * (size_t)g.stIdx[base + (long long)m * kSlice];
        ld16(row, w);
#pragma unroll
        for (int k = 0; k < 15; ++k) ss[k] = ss[k] + w[k];
        ld16(row + 16, w);
#pragma unroll
        for (int k = 0; k < 15; ++k) acc[k] = acc[k] + w[k];
      }
    } else {
      {
        R g0[16];
        ld16(g.gradRaw + 16 * (size_t)c, g0);
#pragma unroll
        for (int k = 0; k < 15; ++k) {
          const R t = g0[k];
          ss[k] = weight(t);
          acc[k] = ss[k] * t;
        }
      }
      auto member = [&](const R gm[16]) {
#pragma unroll
        for (int k = 0; k < 15; ++k) {
          const R t = gm[k];
          const R sm = weight(t);
          ss[k] = ss[k] + sm;
          acc[k] = acc[k] + sm * t;
        }
      };
      {
        // members in stored order, RF_WENO_U gathers issued together with the
        // next group's indices loaded while they are in flight
        constexpr int U = RF_WENO_U;
        const int nFull = n - n % U;
        int nx[U];
#pragma unroll
        for (int u = 0; u < U; ++u) nx[u] = u < n ? ld_index(g.stIdx + base + (long long)u * kSlice) : 0;
        for (int m = 0; m < nFull; m += U) {
          R gm[U][16];
#pragma unroll
          for (int u = 0; u < U; ++u) ld16(g.gradRaw + 16 * (size_t)nx[u], gm[u]);
#pragma unroll
          for (int u = 0; u < U; ++u)
            nx[u] = m + U + u < n ? ld_index(g.stIdx + base + (long long)(m + U + u) * kSlice) : 0;
#pragma unroll
          for (int u = 0; u < U; ++u) member(gm[u]);
        }
#pragma unroll
        for (int u = 0; u < U - 1; ++u) {
          if (nFull + u < n) {
            R gm[16];
            ld16(g.gradRaw + 16 * (size_t)nx[u], gm);
            member(gm);
          }
        }
      }
    }
    R out[16];
#pragma unroll
    for (int k = 0; k < 15; ++k) out[k] = acc[k] / ss[k];
    out[15] = R(0);
    // positivity of the face reconstructions of density (0) and pressure (4)
    R r0[8];
    ld8(g.rec + 8 * (size_t)c, r0);
    if (c >= g.nAct && g.vposOff) {  // a virtual cell of a partitioned region: all its faces
      const long long b0 = g.vposOff[c - g.nAct], b1 = g.vposOff[c - g.nAct + 1];
      const long long P = g.vposTotal;
#pragma unroll
      for (int v = 0; v < 5; v += 4) {
        for (long long e = b0; e < b1; ++e) {
          const R dx = g.vposD[e], dy = g.vposD[P + e], dz = g.vposD[2 * P + e];
          const R varf = r0[v] + out[3 * v] * dx + out[3 * v + 1] * dy + out[3 * v + 2] * dz;
          if (varf <= R(0)) {
            out[3 * v] = out[3 * v + 1] = out[3 * v + 2] = R(0);
            break;
          }
        }
      }
      st16(g.grad + 16 * (size_t)c, out);
      return;
    }
    const long long T = g.cfTotal;
    const long long e0 = g.cfOff[c >> 5] + (c & 31);
    const int nf = g.cfCnt[c];
    const int B = g.nBFaces;
#pragma unroll
    for (int v = 0; v < 5; v += 4) {
      for (int k = 0; k < nf; ++k) {
        const long long e = e0 + (long long)k * kSlice;
        const int code = g.cfCode[e];
        R dx, dy, dz;
        if (code >= 0) {  // the stored offset is xc - fc
          dx = -g.cfD[e];
          dy = -g.cfD[T + e];
          dz = -g.cfD[2 * T + e];
        } else {          // boundary: fc - xc
          const int b = -code - 1;
          dx = g.bfd[b];
          dy = g.bfd[B + b];
          dz = g.bfd[2 * B + b];
        }
        const R varf = r0[v] + out[3 * v] * dx + out[3 * v + 1] * dy + out[3 * v + 2] * dz;
        if (varf <= R(0)) {
          out[3 * v] = out[3 * v + 1] = out[3 * v + 2] = R(0);
          break;
        }
      }
    }
    st16(g.grad + 16 * (size_t)c, out);
  }
}

// The WENO-XYZ pass.  The mixed path's kernel asks for 7 resident blocks of
// 128 per SM (72 registers): the compiler's own choice, 78 registers and 6
// blocks, measured 3.48 against 3.14 ms per launch on the 128^3 tet box (8
// blocks spill, 3.45 ms).  The FP64 kernel keeps the compiler's choice.
#ifndef RF_WENO_MINB
#define RF_WENO_MINB 7
#endif
template <typename R>
__global__ void __launch_bounds__(128) k_weno_xyz(const RegionDev<R> *__restrict__ regs,
                                                  const Tile *__restrict__ tiles, int nTiles) {
  RF_TILE_LOOP(tiles, nTiles) weno_tile<R>(regs, tiles, t_);
}
template <int MINB>
__global__ void __launch_bounds__(128, MINB)
    k_weno_xyz_f32(const RegionDev<float> *__restrict__ regs, const Tile *__restrict__ tiles,
                   int nTiles) {
  RF_TILE_LOOP(tiles, nTiles) weno_tile<float>(regs, tiles, t_);
}

template <typename R>
void launch_weno_xyz(const RegionDev<R> *regs, const Work &w, cudaStream_t s) {
  if (w.nCellTiles <= 0) return;
  const int grid = w.grid > 0 && w.grid < w.nCellTiles ? w.grid : w.nCellTiles;
  if constexpr (sizeof(R) == 4)
    k_weno_xyz_f32<RF_WENO_MINB><<<grid, w.block, 0, s>>>(regs, w.cellTiles, w.nCellTiles);
  else
    k_weno_xyz<R><<<grid, w.block, 0, s>>>(regs, w.cellTiles, w.nCellTiles);
}

template <typename R>
void launch_grad_tiles(const RegionDev<R> *regs, const Work &w, const Tile *tiles, int nTiles,
                       int fuseDt, cudaStream_t s) {
  // the phase tile lists hold 128-cell tiles
  if (fuseDt)
    grad_launch<R, 1, 128>(regs, tiles, nTiles, w.grid, s);
  else
    grad_launch<R, 0, 128>(regs, tiles, nTiles, w.grid, s);
}

template <typename R>
void launch_face_tiles(const RegionDev<R> *regs, const Work &w, const Tile *tiles, int nTiles,
                       cudaStream_t s) {
  // the phase lists hold 128-face tiles, one face per thread
  static const int pf = resident_blocks(k_face_flux<R, 128, 1>, 128);
  const int grid = grid_for(w.grid, nTiles);
  if (grid > 0) k_face_flux<R, 128, 1><<<grid, 128, 0, s>>>(regs, tiles, nTiles, pf);
}

template <typename R>
void launch_update_tiles(const RegionDev<R> *regs, const Work &w, const Tile *tiles, int nTiles,
                         const StepArgs &a, cudaStream_t s) {
  update_launch<R, 128>(regs, tiles, nTiles, w.grid, a, w.split, s);  // 128-cell phase tiles
}

// The transfer chunk a host cell travels in.
__device__ __forceinline__ int host_chunk(const ChunkMap &m, int hostCell) {
  const int t = hostCell / m.block;
  int k = 0;
  while (k < m.nk - 1 && t >= m.tEnd[k]) ++k;
  return k;
}

// Per cell tile: the last chunk holding a record its gradient pass reads (the
// cell's own, its stencil members', its face neighbours') and the first chunk
// among its own cells.  Runs once per region.
template <typename R>
__global__ void k_tile_phases(const RegionDev<R> *__restrict__ regs, const Tile *__restrict__ tiles,
                              int nTiles, ChunkMap m, int *__restrict__ tileLast,
                              int *__restrict__ tileFirst) {
  RF_TILE_LOOP(tiles, nTiles) {
    const Tile tl = tiles[t_];
    const RegionDev<R> &g = regs[tl.region];
    const int c = tl.first + threadIdx.x;
    if (c >= g.nCells) continue;
    auto chunk = [&](int d) { return host_chunk(m, g.cellOld ? g.cellOld[d] : d); };
    const int own = chunk(c);
    int last = own;
    if (g.stOff) {
      const long long b = g.stOff[c >> 5] + (c & 31);
      const int n = g.stCnt[c];
      for (int k = 0; k < n; ++k) last = max(last, chunk(g.stIdx[b + (long long)k * kSlice]));
    }
    const long long e0 = g.cfOff[c >> 5] + (c & 31);
    const int nf = g.cfCnt[c];
    for (int k = 0; k < nf; ++k) {
      const long long e = e0 + (long long)k * kSlice;
      if (g.cfCode[e] >= 0) last = max(last, chunk(g.cfNb[e]));
    }
    atomicMax(tileLast + t_, last);
    atomicMin(tileFirst + t_, own);
  }
}

// The earliest phase any cell of a tile reads a record from: the minimum
// over its cells, their stencil members and face neighbours of the phase of
// the update tile (tilePhase, per 128-cell tile) that rewrites that record.
// A gradient tile of the last stage must run no later than that phase.
template <typename R>
__global__ void k_member_phase(const RegionDev<R> *__restrict__ regs, const Tile *__restrict__ tiles,
                               int nTiles, const int *__restrict__ tilePhase, int block,
                               int *__restrict__ out) {
  RF_TILE_LOOP(tiles, nTiles) {
    const Tile tl = tiles[t_];
    const RegionDev<R> &g = regs[tl.region];
    const int c = tl.first + threadIdx.x;
    if (c >= g.nCells) continue;
    int v = tilePhase[c / block];
    if (g.stOff) {
      const long long b = g.stOff[c >> 5] + (c & 31);
      const int n = g.stCnt[c];
      for (int k = 0; k < n; ++k) v = min(v, tilePhase[g.stIdx[b + (long long)k * kSlice] / block]);
    }
    const long long e0 = g.cfOff[c >> 5] + (c & 31);
    const int nf = g.cfCnt[c];
    for (int k = 0; k < nf; ++k) {
      const long long e = e0 + (long long)k * kSlice;
      if (g.cfCode[e] >= 0) v = min(v, tilePhase[g.cfNb[e] / block]);
    }
    atomicMin(out + t_, v);
  }
}

template <typename R>
void launch_member_phase(const RegionDev<R> *regs, const Work &w, const int *tilePhase, int *out,
                         cudaStream_t s) {
  if (w.nCellTiles > 0)
    k_member_phase<R><<<w.nCellTiles, w.block, 0, s>>>(regs, w.cellTiles, w.nCellTiles, tilePhase,
                                                       w.block, out);
}

template <typename R>
void launch_bface_tiles(const RegionDev<R> *regs, const Work &w, const Tile *tiles, int nTiles,
                        cudaStream_t s) {
  const int grid = grid_for(w.grid, nTiles);
  if (grid > 0) k_bface_flux<R><<<grid, w.block, 0, s>>>(regs, tiles, nTiles);
}

template <typename R>
void launch_tile_phases(const RegionDev<R> *regs, const Work &w, const ChunkMap &m,
                        int *tileLast, int *tileFirst, cudaStream_t s) {
  if (w.nCellTiles > 0)
    k_tile_phases<R><<<w.nCellTiles, w.block, 0, s>>>(regs, w.cellTiles, w.nCellTiles, m,
                                                       tileLast, tileFirst);
}

template <typename R>
void launch_upload_list(const RegionDev<R> *regs, const int *list, int n, const double *cvH,
                        const double *dvH, int split, cudaStream_t s) {
  if (n <= 0) return;
  if (split)
    k_upload_list<R, 1><<<(n + 255) / 256, 256, 0, s>>>(regs, list, n, cvH, dvH);
  else
    k_upload_list<R, 0><<<(n + 255) / 256, 256, 0, s>>>(regs, list, n, cvH, dvH);
}
template <typename R>
void launch_download_list(const RegionDev<R> *regs, const int *list, int n, double *cvH,
                          double *dvH, int split, cudaStream_t s) {
  if (n <= 0) return;
  if (split)
    k_download_list<R, 1><<<(n + 255) / 256, 256, 0, s>>>(regs, list, n, cvH, dvH);
  else
    k_download_list<R, 0><<<(n + 255) / 256, 256, 0, s>>>(regs, list, n, cvH, dvH);
}

// ---- residual without device allocation ---------------------------------------
// Variant of the face-flux and residual-gather passes for rfgpu_residual_noalloc:
// the face fluxes go to a caller-supplied scratch area (the library's static
// device array) and the residual to the same area, in the Fortran layout
// rhs(5,nCells), instead of the region's own buffers.  The region is passed by
// value, so no device-side descriptor has to be written.
template <typename R>
__global__ void __launch_bounds__(128) k_face_flux_scratch(const RegionDev<R> g,
                                                           R *__restrict__ flux) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  const int F = g.nFaces;
  if (f >= F) return;
  const int c1 = g.f2c[f], c2 = g.f2c[F + f];
  R nrm[4];
  ld4(g.fnA + 4 * (size_t)f, nrm);
  R r1[8], r2[8];
  ld8(g.rec + 8 * (size_t)c1, r1);
  ld8(g.rec + 8 * (size_t)c2, r2);
  R L[5], Rt[5], irl, irr;
  cell_values(g, c1, r1, L, irl);
  cell_values(g, c2, r2, Rt, irr);
  if (g.ph.spaceOrder > 1) {
    R G[16];
    ld16(g.grad + 16 * (size_t)c1, G);
    reconstruct(G, g.fdl[f], g.fdl[F + f], g.fdl[2 * F + f], L);
    ld16(g.grad + 16 * (size_t)c2, G);
    reconstruct(G, g.fdr[f], g.fdr[F + f], g.fdr[2 * F + f], Rt);
  }
  R flx[8];
  face_riemann(g, c1, c2, L, Rt, irl, irr, nrm, flx);
  flx[5] = flx[6] = flx[7] = R(0);
  st8(flux + 8 * (size_t)f, flx);
}

template <typename R>
__global__ void __launch_bounds__(128) k_gather_rhs_scratch(const RegionDev<R> g,
                                                            const R *__restrict__ flux,
                                                            double *__restrict__ rhs) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.nCells) return;
  const long long e0 = g.cfOff[c >> 5] + (c & 31);
  const int n = g.cfCnt[c];
  const size_t hc = g.cellOld ? (size_t)g.cellOld[c] : (size_t)c;  // host numbering
  if (c >= g.nAct) {  // virtual cell: ZeroDummyCellsMP
#pragma unroll
    for (int j = 0; j < 5; ++j) rhs[5 * hc + j] = 0.0;
    return;
  }
  bool sum64 = true;  // FP64 and split paths: FP64 sums
  if constexpr (sizeof(R) == 4) sum64 = !g.cvF;
  if (sum64) {
    double acc[5];
    face_sum64(g, flux, c, acc);
#pragma unroll
    for (int j = 0; j < 5; ++j) rhs[5 * hc + j] = acc[j];
    return;
  }
  if constexpr (sizeof(R) == 4) {
    float hi[5] = {0.f, 0.f, 0.f, 0.f, 0.f}, lo[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    for (int k = 0; k < n; ++k) {
      const int code = g.cfCode[e0 + (long long)k * kSlice];
      float fl[8];
      if (code >= 0) {
        ld8(flux + 8 * (size_t)(code >> 1), fl);
        const float sg = (code & 1) ? -1.f : 1.f;
#pragma unroll
        for (int j = 0; j < 5; ++j) two_sum_acc(hi[j], lo[j], sg * fl[j]);
      } else {
        ld8(g.bflux + 8 * (size_t)(-code - 1), fl);
#pragma unroll
        for (int j = 0; j < 5; ++j) two_sum_acc(hi[j], lo[j], fl[j]);
      }
    }
#pragma unroll
    for (int j = 0; j < 5; ++j) rhs[5 * hc + j] = double(hi[j]) + double(lo[j]);
  }
}

// Gradients (the region's own pass), face fluxes into `flux`, boundary fluxes,
// residual into `rhs`; all on stream s.
template <typename R>
void launch_residual_scratch(const RegionDev<R> *regs, const RegionDev<R> &g, const Work &w,
                             int spaceOrder, R *flux, double *rhs, cudaStream_t s) {
  if (spaceOrder > 1 && w.nCellTiles > 0) {
    grad_launch<R, 0, 128>(regs, w.cellTiles, w.nCellTiles, 0, s);
    if (g.gradRaw) launch_weno_xyz<R>(regs, w, s);
  }
  if (g.nFaces > 0) k_face_flux_scratch<R><<<(g.nFaces + 127) / 128, 128, 0, s>>>(g, flux);
  if (w.nBFaceTiles > 0)
    k_bface_flux<R><<<w.nBFaceTiles, w.block, 0, s>>>(regs, w.bfaceTiles, w.nBFaceTiles);
  k_gather_rhs_scratch<R><<<(g.nCells + 127) / 128, 128, 0, s>>>(g, flux, rhs);
}

template <typename R>
void launch_halo(const RegionDev<R> *regs, const HaloLink *links, int n, cudaStream_t s) {
  if (n > 0) k_halo<R><<<(n + 127) / 128, 128, 0, s>>>(regs, links, n);
}
template <typename R>
void launch_halo_pair(const RegionDev<R> *src, const RegionDev<R> *dst, const int *srcCells,
                      const int *dstCells, int n, cudaStream_t s) {
  if (n > 0) k_halo_pair<R><<<(n + 127) / 128, 128, 0, s>>>(src, dst, srcCells, dstCells, n);
}
template <typename R>
void launch_border_pack(const RegionDev<R> *g, const int *cells, int n, double *buf,
                        cudaStream_t s) {
  if (n > 0) k_border_pack<R><<<(n + 127) / 128, 128, 0, s>>>(g, cells, n, buf);
}
template <typename R>
void launch_border_unpack(const RegionDev<R> *g, const int *cells, int n, const double *buf,
                          cudaStream_t s) {
  if (n > 0) k_border_unpack<R><<<(n + 127) / 128, 128, 0, s>>>(g, cells, n, buf);
}

#define RFGPU_INSTANTIATE(R)                                                                  \
  template void launch_prim<R>(const RegionDev<R> *, const Work &, int, cudaStream_t);        \
  template void launch_upload_list<R>(const RegionDev<R> *, const int *, int, const double *,  \
                                      const double *, int, cudaStream_t);                     \
  template void launch_download_list<R>(const RegionDev<R> *, const int *, int, double *,     \
                                        double *, int, cudaStream_t);                         \
  template void launch_residual_scratch<R>(const RegionDev<R> *, const RegionDev<R> &,         \
                                           const Work &, int, R *, double *, cudaStream_t);    \
  template void launch_stage<R>(const RegionDev<R> *, const Work &, const StepArgs &,         \
                                cudaStream_t, long long *, int, int, const Prof *, int);      \
  template void launch_tile_phases<R>(const RegionDev<R> *, const Work &, const ChunkMap &,   \
                                      int *, int *, cudaStream_t);                            \
  template void launch_grad_tiles<R>(const RegionDev<R> *, const Work &, const Tile *, int,   \
                                     int, cudaStream_t);                                      \
  template void launch_update_tiles<R>(const RegionDev<R> *, const Work &, const Tile *, int, \
                                       const StepArgs &, cudaStream_t);                       \
  template void launch_face_tiles<R>(const RegionDev<R> *, const Work &, const Tile *, int,   \
                                     cudaStream_t);                                           \
  template void launch_bface_tiles<R>(const RegionDev<R> *, const Work &, const Tile *, int,  \
                                      cudaStream_t);                                          \
  template void launch_member_phase<R>(const RegionDev<R> *, const Work &, const int *, int *, \
                                       cudaStream_t);                                         \
  template void launch_dt<R>(const RegionDev<R> *, const Work &, const DtArgs &, cudaStream_t, \
                             long long *, const Prof *);                                      \
  template void launch_step<R>(const RegionDev<R> *, const Work &, const DtArgs &, int,       \
                               cudaStream_t, long long *, int, int, const Prof *);            \
  template void launch_halo<R>(const RegionDev<R> *, const HaloLink *, int, cudaStream_t);    \
  template void launch_halo_pair<R>(const RegionDev<R> *, const RegionDev<R> *, const int *,  \
                                    const int *, int, cudaStream_t);                          \
  template void launch_border_pack<R>(const RegionDev<R> *, const int *, int, double *,       \
                                      cudaStream_t);                                          \
  template void launch_border_unpack<R>(const RegionDev<R> *, const int *, int,               \
                                        const double *, cudaStream_t);

}  // namespace rfgpu
