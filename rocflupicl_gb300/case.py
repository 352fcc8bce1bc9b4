"""Run configuration mirroring the RocfluMP input keys the engine honours, and
builders for the synthetic workloads (shock tubes, perturbed tet boxes,
mixed-element boxes, batched tubes).

Keyword meanings follow libfloflu/ReadNumericsSection.F90:110-130 and
libflu/RFLU_InitInputValues.F90:151-200; defaults follow the latter and
libflu/RFLU_InitGlobal.F90:353-354 (refCp = 1004.5, refGamma = 1.4).
"""
from __future__ import annotations

from dataclasses import dataclass, field, replace
from typing import List, Optional

import numpy as np

from . import mesh as _mesh

# modfloflu/ModParameters.F90
DISCR_UPW_ROE, DISCR_UPW_HLLC, DISCR_UPW_AUSMPLUS, DISCR_UPW_AUSMPLUSUP = 1, 3, 4, 5
RECONST_NONE, RECONST_WENO_XYZ, RECONST_LIM_VENKAT = 0, 2, 11
RK_SCHEME_4_CLASSICAL, RK_SCHEME_3_WRAY, RK_SCHEME_1_EULER = 1, 2, 3
BC_OUTFLOW, BC_SLIPWALL, BC_FARFIELD, BC_INJECTION = 20, 60, 80, 90
BC_INFLOW_TOTANG, BC_INFLOW_VELTEMP = 10, 11
BCOPT_SUPERSONIC, BCOPT_SUBSONIC, BCOPT_MIXED = 0, 1, 2
# precision modes (rfgpu.h RFGPU_PREC_*): FP64; mixed = FP32 flux with a
# float-float state updated in FP32; split = FP32 flux with FP64 residual sums,
# RK update and EOS
PREC_FP64, PREC_MIXED, PREC_SPLIT = 0, 1, 2

SCHEME_NAMES = {DISCR_UPW_ROE: "roe", DISCR_UPW_HLLC: "hllc", DISCR_UPW_AUSMPLUS: "ausm+",
                DISCR_UPW_AUSMPLUSUP: "ausm+up"}


@dataclass
class Numerics:
    """The NUMERICS / TIMESTEP keys the engine supports (others are refused)."""
    spaceDiscr: int = DISCR_UPW_AUSMPLUS  # DISCR
    spaceOrder: int = 2                  # ORDER
    reconst: int = RECONST_LIM_VENKAT    # RECONST
    rkScheme: int = RK_SCHEME_3_WRAY     # RKSCHEME
    refCp: float = 1004.5
    refGamma: float = 1.4
    epsentr: float = 0.05                # ENTROPY
    dissFact: float = 1.0                # DISSFACT
    cfl: float = 0.5                     # CFL
    precision: int = PREC_FP64
    # 0: Venkatakrishnan term numer/(denom+1e-12) exactly as the reference;
    # 1: labelled extension adding 1e-12 with the sign of denom (d2 < 0 case)
    venkatGuard: int = 0
    # AUSM+up (DISCR 5): SIGMA, KP, KU, MINF of the NUMERICS section
    # (libfloflu/ReadNumericsSection.F90:239-276 defaults)
    ausmSigma: float = 1.0
    ausmKp: float = 0.25
    ausmKu: float = 0.75
    ausmMInf: float = 0.1

    @property
    def gv(self):
        """(cp, M) as RFLU_SetGasVars stores them for TCPERF
        (libflu/RFLU_SetGasVars.F90:173-179): M = 8314.3 / (cp - cp/g)."""
        gc = self.refCp - self.refCp / self.refGamma
        return self.refCp, 8314.3 / gc

    @property
    def gamma_gv(self) -> float:
        """gamma as the EOS recovers it from gv (RFLU_SetDependentVars.F90:257-258)."""
        cp, mol = self.gv
        gc = 8314.3 / mol
        return cp / (cp - gc)


@dataclass
class PatchBC:
    bcType: int = BC_SLIPWALL
    spaceOrder: int = 1          # .bc ORDER; defaults to spaceOrderBFaces = 1
    bcOptType: int = BCOPT_SUPERSONIC
    pout: Optional[np.ndarray] = None  # outflow static pressure (1,) or (nBFaces,)
    # patch data (pPatch%mixt%vals): (nData,) for the whole patch or (nBFaces, nData);
    # farfield (MACH, ATTACK, SLIP, PRESS, TEMP), injection (MFRATE, TEMP)
    vals: Optional[np.ndarray] = None
    bcOptFixed: int = 0          # inflow TOTANG FIXED switch

    def vals_array(self, n_bfaces: int):
        """(vals (rows, nData) contiguous, nData, distrib) as the C ABI takes them."""
        if self.vals is not None:
            v = np.asarray(self.vals, np.float64)
            if v.ndim == 1:
                return np.ascontiguousarray(v.reshape(1, -1)), v.shape[0], 0
            if v.shape[0] != n_bfaces:
                raise ValueError("per-face patch values need one row per boundary face")
            return np.ascontiguousarray(v), v.shape[1], 1
        if self.pout is None:
            return np.zeros((1, 1)), 1, 0
        p = np.atleast_1d(np.asarray(self.pout, np.float64))
        return np.ascontiguousarray(p.reshape(-1, 1)), 1, 1 if p.shape[0] > 1 else 0


@dataclass
class Case:
    name: str
    mesh: _mesh.BoxMesh
    numerics: Numerics
    bcs: List[PatchBC]
    cv: np.ndarray               # (nCells,5) == Fortran cv(5,nCells)
    dv: np.ndarray               # (nCells,3)
    t_end: float = 0.0
    n_steps: int = 0
    meta: dict = field(default_factory=dict)

    def with_numerics(self, **kw) -> "Case":
        return replace(self, numerics=replace(self.numerics, **kw), cv=self.cv.copy(),
                       dv=self.dv.copy())


def eos_dv(num: Numerics, cv: np.ndarray) -> np.ndarray:
    """RFLU_SetDependentVars for TCPERF (libflu/RFLU_SetDependentVars.F90:256-287),
    element by element in the same operation order (NumPy ufuncs are single
    IEEE operations)."""
    cp, mol = num.gv
    gc = 8314.3 / mol
    g = cp / (cp - gc)
    r = cv[:, 0]
    ir = 1.0 / r
    Eo = ir * cv[:, 4]
    Vm2 = (ir * ir) * ((cv[:, 1] * cv[:, 1] + cv[:, 2] * cv[:, 2]) + cv[:, 3] * cv[:, 3])
    p = ((g - 1.0) * r) * ((Eo - 0.5 * Vm2) - 0.0)
    T = p / (r * gc)
    a = np.sqrt((g * gc) * T)
    return np.stack([p, T, a], axis=1)


def prim_to_cv(num: Numerics, r, u, v, w, p) -> np.ndarray:
    """Conserved state from (rho,u,v,w,p) with E = rho*Eo(rho,g,p,u,v,w)."""
    g = num.gamma_gv
    Eo = p / (r * (g - 1.0)) + 0.5 * ((u * u + v * v) + w * w) + 0.0
    return np.stack([r, r * u, r * v, r * w, r * Eo], axis=1).astype(np.float64)


def tube_bcs(order: int = 2) -> List[PatchBC]:
    """Supersonic outflow (extrapolation) at both x ends, slip walls elsewhere."""
    b = [PatchBC(BC_OUTFLOW, order, BCOPT_SUPERSONIC), PatchBC(BC_OUTFLOW, order, BCOPT_SUPERSONIC)]
    b += [PatchBC(BC_SLIPWALL, order) for _ in range(4)]
    return b


def shock_tube(n: int = 1000, ny: int = 2, nz: int = 2, length=(1.0, 0.01, 0.01),
               left=(1.0, 0.0, 1.0), right=(0.125, 0.0, 0.1), x0: float = 0.5,
               numerics: Optional[Numerics] = None, bc_order: int = 2, t_end: float = 0.2,
               threads: int = 0, stencils: str = "host") -> Case:
    """Sod-type tube of n*ny*nz hexes: (rho,u,p) = left for x < x0, right otherwise.
    stencils="device" builds the stencils and moments on the GPU (same output)."""
    num = numerics or Numerics()
    m = _mesh.box(_mesh.HEX, n, ny, nz, hi=length, threads=threads, stencils=stencils)
    x = m.cofg[:, 0]
    L = x < x0 * length[0]
    r = np.where(L, left[0], right[0])
    u = np.where(L, left[1], right[1])
    p = np.where(L, left[2], right[2])
    z = np.zeros_like(r)
    cv = prim_to_cv(num, r, u, z, z, p)
    return Case("shock_tube", m, num, tube_bcs(bc_order), cv, eos_dv(num, cv), t_end=t_end,
                meta={"n": n, "left": left, "right": right, "x0": x0})


def rankine_hugoniot(Ms: float, gamma: float, rho1: float, p1: float):
    """Post-shock state of a normal shock of Mach Ms moving into gas at rest
    (standard normal-shock relations)."""
    g = gamma
    rho_ratio = (g + 1.0) * Ms * Ms / ((g - 1.0) * Ms * Ms + 2.0)
    p_ratio = 1.0 + 2.0 * g / (g + 1.0) * (Ms * Ms - 1.0)
    a1 = np.sqrt(g * p1 / rho1)
    rho2 = rho1 * rho_ratio
    u2 = Ms * a1 * (1.0 - rho1 / rho2)
    return rho2, u2, p1 * p_ratio


def tet_shock_box(n: int = 128, seed: int = 2024, jitter: float = 0.1, Ms: float = 2.0,
                  sigma: float = 0.1, x_shock: float = 0.2, numerics: Optional[Numerics] = None,
                  n_steps: int = 100, threads: int = 0, stencils: str = "host",
                  ny: Optional[int] = None, nz: Optional[int] = None,
                  length=(1.0, 1.0, 1.0)) -> Case:
    """Planar Ms shock over a perturbed tetrahedral box: n*ny*nz hexes (ny, nz
    default n) x 6 Kuhn tets over [0,length], interior vertices jittered by
    U(+-jitter*h); quiescent air rho=1.2, p=1e5 times a per-cell lognormal
    density factor exp(sigma*Z); Rankine-Hugoniot post-shock state for
    x < x_shock.  Slip walls on y/z, supersonic outflow (extrapolation) on the
    x ends."""
    num = numerics or Numerics(spaceDiscr=DISCR_UPW_ROE)
    m = _mesh.box(_mesh.TET, n, ny or n, nz or n, hi=tuple(length), jitter=jitter, seed=seed,
                  threads=threads, stencils=stencils)
    rng = np.random.default_rng(seed)
    rho1, p1 = 1.2, 1.0e5
    r = rho1 * np.exp(sigma * rng.standard_normal(m.nCells))
    p = np.full(m.nCells, p1)
    u = np.zeros(m.nCells)
    rho2, u2, p2 = rankine_hugoniot(Ms, num.refGamma, rho1, p1)
    post = m.cofg[:, 0] < x_shock
    r = np.where(post, rho2, r)
    u = np.where(post, u2, u)
    p = np.where(post, p2, p)
    z = np.zeros_like(r)
    cv = prim_to_cv(num, r, u, z, z, p)
    return Case("tet_shock_box", m, num, tube_bcs(2), cv, eos_dv(num, cv), n_steps=n_steps,
                meta={"n": n, "seed": seed, "Ms": Ms, "sigma": sigma})


def cold_stream_box(n: int = 12, mach: float = 8.0, T: float = 100.0, seed: int = 5,
                    jitter: float = 0.1, sigma: float = 0.1, dp: float = 0.05,
                    numerics: Optional[Numerics] = None) -> Case:
    """A cold supersonic stream along +x through the jittered Kuhn-tet box:
    kinetic energy far above internal energy (1/2 |u|^2 / e = g (g-1) M^2 / 2,
    18 at Mach 8), where recovering p from E - |m|^2/(2 rho) cancels.  rho =
    p/(R T) times a lognormal factor exp(sigma Z) per cell (contacts carried by
    the stream), p times 1 + dp sin(2 pi x) sin(2 pi y) (acoustic waves), u =
    M a of the base state.  Slip walls on y/z, extrapolation on the x ends."""
    num = numerics or Numerics(spaceDiscr=DISCR_UPW_ROE)
    m = _mesh.box(_mesh.TET, n, n, n, jitter=jitter, seed=seed)
    rng = np.random.default_rng(seed)
    g = num.gamma_gv
    R = 8314.3 / num.gv[1]
    p0 = 1.0e5
    rho0 = p0 / (R * T)
    u0 = mach * np.sqrt(g * R * T)
    x, y = m.cofg[:, 0], m.cofg[:, 1]
    p = p0 * (1.0 + dp * np.sin(2.0 * np.pi * x) * np.sin(2.0 * np.pi * y))
    r = rho0 * np.exp(sigma * rng.standard_normal(m.nCells))
    u = np.full(m.nCells, u0)
    z = np.zeros_like(r)
    cv = prim_to_cv(num, r, u, z, z, p)
    return Case("cold_stream_box", m, num, tube_bcs(2), cv, eos_dv(num, cv),
                meta={"n": n, "seed": seed, "mach": mach, "T": T,
                      "kinetic_over_internal": 0.5 * g * (g - 1.0) * mach * mach})


def fourier_state(xyz: np.ndarray, seed: int, n_modes: int = 8):
    """Smooth random field: sum of n_modes seeded Fourier modes per variable,
    affinely rescaled to rho in [0.5,2], p in [0.5e5,2e5], |u_i| <= 300/sqrt(3)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(5):
        k = rng.uniform(1.0, 4.0, size=(n_modes, 3)) * 2.0 * np.pi * rng.choice([-1, 1], size=(n_modes, 3))
        ph = rng.uniform(0.0, 2.0 * np.pi, size=n_modes)
        amp = rng.uniform(0.5, 1.0, size=n_modes)
        f = np.zeros(xyz.shape[0])
        for j in range(n_modes):
            f += amp[j] * np.sin(xyz @ k[j] + ph[j])
        f = (f - f.min()) / max(f.max() - f.min(), 1e-300)  # [0,1]
        out.append(f)
    r = 0.5 + 1.5 * out[0]
    p = 0.5e5 + 1.5e5 * out[4]
    umax = 300.0 / np.sqrt(3.0)
    u, v, w = [(2.0 * o - 1.0) * umax for o in out[1:4]]
    return r, u, v, w, p


def mixed_box(n: int = 96, seed: int = 7, numerics: Optional[Numerics] = None,
              threads: int = 0, stencils: str = "host") -> Case:
    """n^3 box: hexes with x > 0.5 split into 2 prisms, hexes with z > 0.5 into 6
    tets (prism precedence), pyramid transition cubes where tets meet quad faces;
    smooth seeded Fourier state.  Slip walls everywhere (residual benchmark)."""
    num = numerics or Numerics()
    m = _mesh.box(_mesh.MIXED, n, n, n, threads=threads, stencils=stencils)
    r, u, v, w, p = fourier_state(m.cofg, seed)
    cv = prim_to_cv(num, r, u, v, w, p)
    bcs = [PatchBC(BC_SLIPWALL, 2) for _ in range(6)]
    return Case("mixed_box", m, num, bcs, cv, eos_dv(num, cv), meta={"n": n, "seed": seed})


def tube_ensemble(count: int = 256, seed: int = 11, n_min: int = 500, n_max: int = 125000,
                  cross: int = 2, numerics: Optional[Numerics] = None, n_steps: int = 300,
                  threads: int = 0, scale: float = 1.0) -> List[Case]:
    """Independent 3-D shock tubes n x cross x cross hexes, n log-uniform in
    [n_min, n_max] (times `scale` for reduced tests); left/right rho and p
    log-uniform in [0.1,10], u uniform in [-1,1], diaphragm in [0.3,0.7]."""
    num = numerics or Numerics(precision=PREC_MIXED)
    rng = np.random.default_rng(seed)
    cases = []
    for i in range(count):
        n = int(round(np.exp(rng.uniform(np.log(n_min), np.log(n_max))) * scale))
        n = max(n, 4)
        rl, rr, pl, pr = np.exp(rng.uniform(np.log(0.1), np.log(10.0), size=4))
        ul, ur = rng.uniform(-1.0, 1.0, size=2)
        x0 = rng.uniform(0.3, 0.7)
        c = shock_tube(n, cross, cross, length=(1.0, 1.0 / n * cross, 1.0 / n * cross),
                       left=(rl, ul, pl), right=(rr, ur, pr), x0=x0, numerics=num,
                       threads=threads)
        c.name = f"tube{i}"
        c.n_steps = n_steps
        cases.append(c)
    return cases


def from_files(grid_path: str, flow_path: str, bcs: List[PatchBC],
               numerics: Optional[Numerics] = None, binary: bool = False, endian: str = "<",
               threads: int = 0, stencils: str = "host") -> Case:
    """A case from the reference's grid and flow files (.grda/.grd and the v2
    flow file): the mesh is built from the grid by the same builder as the
    synthetic meshes, cv comes from the flow file, dv from the EOS; bcs gives
    each grid patch its boundary condition, in the grid's patch order."""
    from . import rfluio as IO
    num = numerics or Numerics()
    g = IO.read_grid_binary(grid_path, endian) if binary else IO.read_grid_ascii(grid_path)
    fl = IO.read_flow_binary(flow_path, endian) if binary else IO.read_flow_ascii(flow_path)
    m = IO.mesh_of_grid(g, threads=threads, stencils=stencils)
    if fl.cv.shape != (m.nCells, 5):
        raise ValueError(f"flow file holds {fl.cv.shape}, the grid has {m.nCells} cells x 5")
    if len(bcs) != len(m.patches):
        raise ValueError(f"{len(bcs)} boundary conditions for {len(m.patches)} patches")
    cv = np.ascontiguousarray(fl.cv)
    return Case(f"files:{grid_path}", m, num, list(bcs), cv, eos_dv(num, cv),
                meta={"time": fl.time, "grid": grid_path, "flow": flow_path})


def from_case_files(grid_path: str, flow_path: Optional[str], inp_path: str, bc_path: str,
                    binary: bool = False, endian: str = "<", threads: int = 0,
                    stencils: str = "host", strict: bool = True,
                    casename: Optional[str] = None):
    """A case from a RocfluMP case's files: the grid and flow files, the `.inp`
    numerics and the `.bc` boundary conditions (rocflupicl_gb300.rfluinput).
    Without a flow file the initial state is the one rfluinit makes from the
    `.inp` INITFLOW section (initial_cv; the case name defaults to the `.inp`
    file's name, as RocfluMP names a case's files after it).
    Returns (case, CaseInput, unsupported settings); strict raises ValueError
    when the files ask for anything outside the engine's envelope."""
    import os
    from . import rfluinput as RI
    from . import rfluio as IO
    ci = RI.read_inp(inp_path)
    g = IO.read_grid_binary(grid_path, endian) if binary else IO.read_grid_ascii(grid_path)
    bcs, bad_bc = RI.read_bc(bc_path, len(g.patches), ci.order_bfaces)
    bad = ci.unsupported + bad_bc
    if strict and bad:
        raise ValueError("settings outside the engine's envelope: " + "; ".join(bad))
    if flow_path is None:
        name = casename or os.path.splitext(os.path.basename(inp_path))[0]
        num = ci.numerics
        m = IO.mesh_of_grid(g, threads=threads, stencils=stencils)
        if len(bcs) != len(m.patches):
            raise ValueError(f"{len(bcs)} boundary conditions for {len(m.patches)} patches")
        cv = initial_cv(name, m.cofg[:m.nCells], num, ci.raw.get("INITFLOW", {}))
        c = Case(f"files:{grid_path}", m, num, list(bcs), cv, eos_dv(num, cv),
                 meta={"time": 0.0, "grid": grid_path, "casename": name})
    else:
        c = from_files(grid_path, flow_path, bcs, ci.numerics, binary, endian, threads,
                       stencils)
    c.meta["dt_imposed"], c.meta["max_time"] = ci.dt_imposed, ci.max_time
    c.t_end = ci.max_time
    return c, ci, bad


# INITFLOW FLAG values (modfloflu/ModParameters.F90:911-916)
INITFLOW_FROMSCRATCH, INITFLOW_FROMFILE, INITFLOW_FROMHARDCODE = 1, 2, 3
# the hard-coded initial states restated below (perfect gas only)
HARDCODED_CASES = ("rectshktb", "cylds", "st_sod1", "st_sod1_mp2", "st_sod2", "st_sod2_mp2",
                   "stg1d", "stg2d", "gtlin", "gttri")


def hardcoded_prims(casename: str, xyz: np.ndarray, vals: dict):
    """(rho, u, v, w, p) per cell of RFLU_InitFlowHardCode (utilities/init/
    RFLU_InitFlowHardCode.F90) for the perfect-gas branch of the named cases,
    from the cell centroids and the INITFLOW values (RVALn = prepRealValn)."""
    x, y, z = xyz[:, 0], xyz[:, 1], xyz[:, 2]
    zero = np.zeros_like(x)

    def rv(i):
        k = f"RVAL{i}"
        if k not in vals:
            raise ValueError(f"INITFLOW {k} is not defined, case {casename!r} needs it")
        return float(vals[k])

    def split(inner, a, b):
        return tuple(np.where(inner, ai, bi) for ai, bi in zip(a, b))

    if casename in ("rectshktb", "cylds"):  # :760-813
        if casename == "cylds":
            radius, theta = np.sqrt(x ** 2 + y ** 2), np.arctan2(y, x)
            ur, ut = rv(3) * np.cos(theta), rv(3) * np.sin(theta)
        else:
            radius, ur, ut = x, np.full_like(x, rv(3)), zero
        return split(radius < rv(1), (rv(2), ur, ut, zero, rv(4)), (rv(5), zero, zero, zero, rv(6)))
    if casename in ("st_sod1", "st_sod1_mp2"):  # :4274-4300
        return split(x < 0.5, (1.0, zero, zero, zero, 1.0e5), (0.125, zero, zero, zero, 1.0e4))
    if casename in ("st_sod2", "st_sod2_mp2"):  # :4309-4340
        return split(x < 0.0, (1.0, zero, zero, zero, 1.0e5), (0.01, zero, zero, zero, 1.0e3))
    if casename in ("stg1d", "stg2d"):  # :4232-4270
        a = (rv(2), rv(3), zero, zero, rv(4))
        b = (rv(5), rv(6), zero, zero, rv(7))
        c = (rv(12), rv(13), zero, zero, rv(14))
        return split(x < rv(1), a, split(x < rv(11), b, c))
    if casename == "gtlin":  # :2700-2750 with RFLU_SetExactFlowLinear (RFLU_ModExactFlow.F90:1451-1491)
        def lin(iv, X, Y, Z):
            a = 1.0 + (iv - 1) * 2.0       # 1 + (iVar-1)*(ZCOORD-XCOORD)
            return a * X + (a + 1.0) * Y + (a + 2.0) * Z
        dmin, pmin = lin(1, x.min(), y.min(), z.min()), lin(5, x.min(), y.min(), z.min())
        doffs = -2.0 * dmin if dmin < 0.0 else 0.0
        poffs = -2.0 * pmin if pmin < 0.0 else 0.0
        return (lin(1, x, y, z) + doffs, lin(2, x, y, z), lin(3, x, y, z), lin(4, x, y, z),
                lin(5, x, y, z) + poffs)
    if casename == "gttri":  # :2757-2790 with RFLU_SetExactFlowTrig (RFLU_ModExactFlow.F90:1527-1568)
        pi = 4.0 * np.arctan(1.0)
        a, b, c = rv(1) * pi, rv(2) * pi, rv(3) * pi
        var = np.cos(a * x) * np.sin(b * y) * np.cos(c * z)
        return var + 2.0, var, var, var, var + 2.0
    raise ValueError(f"hard-coded initial state {casename!r} is not restated "
                     f"(restated: {', '.join(HARDCODED_CASES)})")


def initial_cv(casename: str, xyz: np.ndarray, num: Numerics, initflow: dict) -> np.ndarray:
    """The initial conserved state of rfluinit for an INITFLOW section: FLAG 1
    a uniform state (RFLU_InitFlowScratch: DENS, VELX/Y/Z, PRESS), FLAG 3 the
    hard-coded state of the case name (hardcoded_prims); E = rho Eo as
    MixtPerf_Eo_DGPUVW forms it."""
    if "FLAG" not in initflow:
        raise ValueError("INITFLOW FLAG is not defined")
    flag = int(round(initflow["FLAG"]))
    n = xyz.shape[0]
    if flag == INITFLOW_FROMSCRATCH:
        need = ["VELX", "VELY", "VELZ", "PRESS", "DENS"]
        missing = [k for k in need if k not in initflow]
        if missing:
            raise ValueError("INITFLOW FLAG 1 without " + ", ".join(missing))
        r, u, v, w, p = (np.full(n, float(initflow[k]))
                         for k in ("DENS", "VELX", "VELY", "VELZ", "PRESS"))
    elif flag == INITFLOW_FROMHARDCODE:
        r, u, v, w, p = (np.broadcast_to(np.asarray(a, np.float64), (n,)).copy()
                         for a in hardcoded_prims(casename, xyz, initflow))
    else:
        raise ValueError(f"INITFLOW FLAG {flag}: the state comes from a flow file")
    return prim_to_cv(num, r, u, v, w, p)


def write_flow(path: str, cv: np.ndarray, time: float = 0.0, binary: bool = False,
               endian: str = "<") -> None:
    """Write a state (nCells, 5) as the reference's v2 flow file."""
    from . import rfluio as IO
    fl = IO.Flow(np.ascontiguousarray(cv, np.float64), time=time)
    if binary:
        IO.write_flow_binary(path, fl, endian)
    else:
        IO.write_flow_ascii(path, fl)
