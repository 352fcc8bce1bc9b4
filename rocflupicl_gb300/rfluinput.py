"""RocfluMP case input files: the numerics, time-stepping, reference, mixture
and initial-flow sections of the `.inp` file and the boundary-condition
sections of the `.bc` file, read the way the reference reads them, mapped onto
the engine's options, with every setting outside the engine's envelope
reported.

Reading rules (libfloflu/ReadInputUtil.F90, ReadSection; the `.bc` sections
follow ReadPatchSection, where a key given twice takes the later value):
a section starts at a line whose trimmed text is its header (`# NUMERICS`) and
ends at the next line starting with `#`; a key matches a line that starts with
the key's text, in key-list order, and each key takes the first value after it
(a list-directed read) and is then defined (a later line does not redefine
it); a line defines at most one key, the first undefined one that matches.
Section and key lists: ReadNumericsSection.F90:110-130,
ReadTimestepSection.F90:108-136, ReadReferenceSection.F90:103-112,
ReadMixtureSection.F90:123-124, ReadFlowSection.F90:105-107,
ReadInitFlowSection.F90:46-102 (its numeric keys; case.initial_cv makes the
state),
modflu/RFLU_ModReadBcInputFile.F90 (BC sections, keys and the degree to
radian conversion of angles).  Defaults where a key is absent:
libflu/RFLU_InitInputValues.F90:181-200, libflu/RFLU_InitGlobal.F90:232-354.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Tuple

import numpy as np

from . import case as K

NUMERICS_KEYS = ["CFL", "DISCR", "ORDER", "ENTROPY", "DISSFACT", "RECONST", "DIMENS",
                 "CRECONSTC", "CRECONSTF", "CRECONSTCW", "CRECONSTFW", "TOLERICT", "SDIMENSC",
                 "SDIMENSF", "SDIMENSBF", "ORDERBF", "AXIFLAG", "SIGMA", "KP", "KU", "MINF"]
TIMESTEP_KEYS = ["FLOWTYPE", "TIMESTEP", "MAXTIME", "WRITIME", "PRNTIME", "MAXITER", "RESTOL",
                 "WRIITER", "PRNITER", "STARTTIME", "STARTITER", "SOLVERTYPE", "ORDER",
                 "MAXSUBITER", "TOLSUBITER", "PREDICTSOL", "DTMINLIMIT", "RKSCHEME", "RUNTIME",
                 "FOMWRITIME", "TOLPC", "TOLHYPRE", "MAXITPC", "MAXITHYPRE", "FOMWRIITER",
                 "HYPRESOLVER", "WALLTIME", "SAFEWRTIME", "PRNTENDTIME"]
REFERENCE_KEYS = ["ABSVEL", "PRESS", "DENS", "CP", "GAMMA", "LENGTH", "RENUM", "PRLAM",
                  "PRTURB", "SCNLAM"]
MIXTURE_KEYS = ["FROZENFLAG", "GASMODEL"]
# libfloflu/ReadInitFlowSection.F90:46-102 (numeric keys, in the reference's order)
INITFLOW_KEYS = (["FLAG", "VELX", "VELY", "VELZ", "PRESS", "DENS", "TEMP"]
                 + [f"IVAL{i}" for i in range(1, 17)] + [f"RVAL{i}" for i in range(1, 21)]
                 + ["DX", "DY", "DZ", "RVAL24", "IVAL17", "IVAL18", "IVAL19", "RVAL25",
                    "RBFLAG"])
FLOWMODEL_KEYS = ["MODEL", "MOVEGRID", "PBAFLAG"]
USED_KEYS = ["USED"]

BC_KEYS = {
    "# BC_SLIPW": ["MVPATCH", "SMGRID", "ORDER"],
    "# BC_OUTFLOW": ["TYPE", "PRESS", "MVPATCH", "SMGRID", "ORDER", "STATS", "MOVEDIR",
                     "COUPLED", "KIND", "REFLECT", "NSCBCK", "THRUSTFLAG"],
    "# BC_FARF": ["CORR", "MACH", "ATTACK", "SLIP", "PRESS", "TEMP", "MVPATCH", "SMGRID",
                  "ORDER", "MOVEDIR", "COUPLED", "KIND", "THRUSTFLAG"],
    "# BC_INJECT": ["MFRATE", "TEMP", "COUPLED", "BFLAG", "MVPATCH", "SMGRID", "MOVEDIR",
                    "STATS", "CRECONST"],
    "# BC_INFLOW_TOTANG": ["TYPE", "FIXED", "PTOT", "TTOT", "BETAH", "BETAV", "MACH", "MVPATCH",
                           "SMGRID", "MOVEDIR", "COUPLED", "KIND", "REFLECT", "THRUSTFLAG",
                           "ORDER"],
    "# BC_INFLOW_VELTEMP": ["TYPE", "VELX", "VELY", "VELZ", "TEMP", "PRESS", "MVPATCH", "SMGRID",
                            "MOVEDIR", "COUPLED", "KIND", "REFLECT", "THRUSTFLAG", "ORDER"],
}
BC_OTHER = ["# BC_INFLOW", "# BC_NOSLIP", "# BC_NOSLIP_HFLUX", "# BC_NOSLIP_TEMP",
            "# BC_PERIODIC", "# BC_SYMMETRY", "# BC_VIRTUAL"]

# global%deg2rad = 1/(180/pi), pi = 4 atan(1) (libflu/RFLU_InitGlobal.F90:333-335)
DEG2RAD = 1.0 / (180.0 / (4.0 * math.atan(1.0)))


def _value(text: str) -> float:
    """The first item of a list-directed read of one real."""
    tok = text.replace(",", " ").split()
    if not tok:
        raise ValueError("key without a value")
    return float(tok[0].rstrip("/").replace("D", "E").replace("d", "e"))


def _read_keys(lines: List[str], keys: List[str]) -> Dict[str, float]:
    """ReadSection (libfloflu/ReadInputUtil.F90): every line against the keys
    not yet defined, in key order; a line defines at most the first key whose
    text begins it (so `RVAL10 5.` defines an undefined RVAL1, reading 0.)."""
    vals: Dict[str, float] = {}
    for line in lines:
        for k in keys:
            if k not in vals and line.startswith(k):
                vals[k] = _value(line[len(k):])
                break
    return vals


def _read_patch_keys(lines: List[str], keys: List[str]) -> Dict[str, float]:
    """ReadPatchSection's value keys (libfloflu/ReadInputUtil.F90): every line
    against every key, with no record of what is defined, so a key given on
    two lines takes the later value."""
    vals: Dict[str, float] = {}
    for line in lines:
        for k in keys:
            if line.startswith(k):
                vals[k] = _value(line[len(k):])
    return vals


def _sections(path: str) -> List[Tuple[str, List[str]]]:
    """(header, body lines) of every `# NAME` section, in file order."""
    out: List[Tuple[str, List[str]]] = []
    cur: Optional[Tuple[str, List[str]]] = None
    with open(path) as f:
        for raw in f:
            line = raw.rstrip("\n")
            if line.startswith("#"):
                if cur is not None:
                    out.append(cur)
                    cur = None
                head = line.strip()
                if head != "#":
                    cur = (head, [])
            elif cur is not None:
                cur[1].append(line)
    if cur is not None:
        out.append(cur)
    return out


@dataclass
class CaseInput:
    """The `.inp` settings the engine uses, and the ones it cannot honour."""
    numerics: K.Numerics
    dt_imposed: float = 1.0e-5        # TIMESTEP (global%dtImposed)
    dt_min_limit: float = 1.0e-10     # DTMINLIMIT
    max_time: float = 1.0e-4          # MAXTIME (end time of an unsteady run)
    order_bfaces: int = 1             # ORDERBF (spaceOrderBFaces, the patches' default ORDER)
    raw: Dict[str, Dict[str, float]] = field(default_factory=dict)
    unsupported: List[str] = field(default_factory=list)


def read_inp(path: str) -> CaseInput:
    secs = dict(_sections(path))
    num = _read_keys(secs.get("# NUMERICS", []), NUMERICS_KEYS)
    ts = _read_keys(secs.get("# TIMESTEP", []), TIMESTEP_KEYS)
    ref = _read_keys(secs.get("# REFERENCE", []), REFERENCE_KEYS)
    mix = _read_keys(secs.get("# MIXTURE", []), MIXTURE_KEYS)
    flow = _read_keys(secs.get("# FLOWMODEL", []), FLOWMODEL_KEYS)
    spec = _read_keys(secs.get("# SPECIES", []), USED_KEYS)
    picl = _read_keys(secs.get("# PICL", []), USED_KEYS)
    init = _read_keys(secs.get("# INITFLOW", []), INITFLOW_KEYS)
    n = K.Numerics(
        spaceDiscr=int(round(num.get("DISCR", K.DISCR_UPW_ROE))),
        spaceOrder=int(round(num.get("ORDER", 1))),
        reconst=int(round(num.get("RECONST", 2))),          # default RECONST_WENO_XYZ
        rkScheme=int(round(ts.get("RKSCHEME", K.RK_SCHEME_4_CLASSICAL))),
        refCp=ref.get("CP", 1004.5), refGamma=ref.get("GAMMA", 1.4),
        epsentr=abs(num.get("ENTROPY", 0.05)), dissFact=abs(num.get("DISSFACT", 1.0)),
        cfl=abs(num.get("CFL", 3.0)),
        ausmSigma=num.get("SIGMA", 1.0), ausmKp=num.get("KP", 0.25), ausmKu=num.get("KU", 0.75),
        ausmMInf=num.get("MINF", 0.1))
    ci = CaseInput(numerics=n, dt_imposed=ts.get("TIMESTEP", 1.0e-5),
                   dt_min_limit=ts.get("DTMINLIMIT", 1.0e-10), max_time=ts.get("MAXTIME", 1.0e-4),
                   order_bfaces=int(round(num.get("ORDERBF", 1))),
                   raw={"NUMERICS": num, "TIMESTEP": ts, "REFERENCE": ref, "MIXTURE": mix,
                        "FLOWMODEL": flow, "SPECIES": spec, "PICL": picl, "INITFLOW": init})
    bad = ci.unsupported
    if n.spaceDiscr not in (K.DISCR_UPW_ROE, K.DISCR_UPW_HLLC, K.DISCR_UPW_AUSMPLUS,
                            K.DISCR_UPW_AUSMPLUSUP):
        bad.append(f"DISCR {n.spaceDiscr}: not one of 1 (Roe), 3 (HLLC), 4 (AUSM+), 5 (AUSM+up)")
    if n.spaceOrder not in (1, 2):
        bad.append(f"ORDER {n.spaceOrder}")
    if n.spaceOrder == 2 and n.reconst not in (K.RECONST_NONE, K.RECONST_WENO_XYZ,
                                               K.RECONST_LIM_VENKAT):
        bad.append(f"RECONST {n.reconst}: the engine reconstructs with WLSQ gradients, "
                   "unlimited (0), WENO-XYZ weighted (2) or Venkatakrishnan-limited (11)")
    for k in ("CRECONSTC", "CRECONSTF"):
        if int(round(num.get(k, 0))) != 0:
            bad.append(f"{k} {int(num[k])}: constrained reconstruction")
    if int(round(num.get("DIMENS", 3))) != 3 or int(round(num.get("AXIFLAG", 0))) != 0:
        bad.append("DIMENS / AXIFLAG: three-dimensional, non-axisymmetric only")
    if n.rkScheme not in (K.RK_SCHEME_4_CLASSICAL, K.RK_SCHEME_3_WRAY, K.RK_SCHEME_1_EULER):
        bad.append(f"RKSCHEME {n.rkScheme}")
    if int(round(ts.get("FLOWTYPE", 0))) != 1:
        bad.append("FLOWTYPE 0: steady flow (local time stepping) is not on the path")
    if int(round(flow.get("MODEL", 0))) != 0:
        bad.append("FLOWMODEL MODEL: Euler only")
    if int(round(flow.get("MOVEGRID", 0))) != 0:
        bad.append("FLOWMODEL MOVEGRID: static grids only")
    if int(round(mix.get("GASMODEL", K_GAS_TCPERF))) != K_GAS_TCPERF:
        bad.append(f"GASMODEL {int(mix['GASMODEL'])}: thermally and calorically perfect gas only")
    if int(round(spec.get("USED", 0))) != 0:
        bad.append("SPECIES USED: species sources are outside the residual engine")
    if int(round(picl.get("USED", 0))) != 0:
        bad.append("PICL USED: particle coupling is outside the residual engine")
    return ci


K_GAS_TCPERF = 1  # GAS_MODEL_TCPERF


def read_bc(path: str, n_patches: int, order_bfaces: int = 1):
    """Boundary conditions of global patches 1..n_patches from a `.bc` file:
    (list of PatchBC in patch order, list of unsupported settings).  A patch
    no section names keeps a slip wall and is reported."""
    bcs: List[Optional[K.PatchBC]] = [None] * n_patches
    bad: List[str] = []
    for head, lines in _sections(path):
        if head in BC_OTHER:
            bad.append(f"{head[2:]}: boundary condition not on the engine's path")
            continue
        if head not in BC_KEYS:
            continue
        keys = BC_KEYS[head]
        p0, p1, distrib, body = 1, 999999, 0, []
        for line in lines:  # ReadPatchSection's own keys first
            if line.startswith("PATCH"):
                t = line[5:].replace(",", " ").split()
                p0, p1 = int(t[0]), int(t[1])
                p0 = 1 if p0 <= 0 else p0
                p1 = 999999 if p1 <= 0 else p1
                p1 = max(p1, p0)
            elif line.startswith("DISTRIB"):
                distrib = min(max(int(_value(line[7:])), 0), 1)
            elif line.startswith("NAME") or line.startswith("FILE"):
                pass
            else:
                body.append(line)
        v = _read_patch_keys(body, keys)
        if distrib:
            bad.append(f"{head[2:]} PATCH {p0} {p1}: distributed values (DISTRIB 1) come from a "
                       "separate file; give them per face through PatchBC.vals")
        order = int(round(v["ORDER"])) if "ORDER" in v else order_bfaces
        order = 2 if order == 2 else 1
        if head == "# BC_SLIPW":
            bc = K.PatchBC(K.BC_SLIPWALL, order)
        elif head == "# BC_OUTFLOW":
            typ = int(round(v.get("TYPE", 0)))
            bc = K.PatchBC(K.BC_OUTFLOW, order, typ,
                           pout=np.array([v["PRESS"]]) if "PRESS" in v else None)
        elif head == "# BC_FARF":
            if int(round(v.get("CORR", 0))) != 0:
                bad.append(f"BC_FARF CORR {int(v['CORR'])}: the airfoil lift correction")
            bc = K.PatchBC(K.BC_FARFIELD, order, 0, vals=np.array(
                [v.get("MACH", 0.0), v.get("ATTACK", 0.0) * DEG2RAD, v.get("SLIP", 0.0) * DEG2RAD,
                 v.get("PRESS", 0.0), v.get("TEMP", 0.0)]))
        elif head == "# BC_INJECT":
            bc = K.PatchBC(K.BC_INJECTION, order, 0,
                           vals=np.array([v.get("MFRATE", 0.0), v.get("TEMP", 0.0)]))
        elif head == "# BC_INFLOW_TOTANG":
            bc = K.PatchBC(K.BC_INFLOW_TOTANG, order, int(round(v.get("TYPE", 0))),
                           vals=np.array([v.get("PTOT", 0.0), v.get("TTOT", 0.0),
                                          v.get("BETAH", 0.0) * DEG2RAD,
                                          v.get("BETAV", 0.0) * DEG2RAD, v.get("MACH", 0.0)]),
                           bcOptFixed=int(round(v.get("FIXED", 0))))
        else:  # BC_INFLOW_VELTEMP
            bc = K.PatchBC(K.BC_INFLOW_VELTEMP, order, int(round(v.get("TYPE", 0))),
                           vals=np.array([v.get("VELX", 0.0), v.get("VELY", 0.0),
                                          v.get("VELZ", 0.0), v.get("TEMP", 0.0),
                                          v.get("PRESS", 0.0)]))
        for ip in range(max(p0, 1), min(p1, n_patches) + 1):
            bcs[ip - 1] = bc
    out = []
    for ip, bc in enumerate(bcs):
        if bc is None:
            bad.append(f"patch {ip + 1}: no boundary condition given (slip wall assumed)")
            bc = K.PatchBC(K.BC_SLIPWALL, order_bfaces)
        out.append(bc)
    return out, bad
