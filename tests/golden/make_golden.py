"""Writes tests/golden/oracle_small.npz: the oracle's residual, limited
gradients and a short trajectory on three small seeded cases (a Sod tube, a
jittered Kuhn-tet shock box, a mixed hex/prism/tet/pyramid box).

The reference itself cannot be built here (Fortran 90 + MPI, no compiler), so
these are not reference outputs: they freeze the oracle - the C++ FP64
restatement every GPU parity test compares against - so that a change to it
shows up as a failed CPU test (tests/test_golden.py) instead of silently
moving both sides of the GPU comparisons.  Run it again only on purpose, after
a reviewed change to the oracle.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from rocflupicl_gb300 import case as K  # noqa: E402

CASES = {
    "sod": lambda: K.shock_tube(40, numerics=K.Numerics(venkatGuard=1)),
    "tet_roe": lambda: K.tet_shock_box(3, seed=11, numerics=K.Numerics(
        spaceDiscr=K.DISCR_UPW_ROE, venkatGuard=1)),
    "tet_hllc_refguard": lambda: K.tet_shock_box(3, seed=12, numerics=K.Numerics(
        spaceDiscr=K.DISCR_UPW_HLLC, venkatGuard=0)),
    "mixed_ausm": lambda: K.mixed_box(3, numerics=K.Numerics(
        spaceDiscr=K.DISCR_UPW_AUSMPLUS, venkatGuard=1)),
    "tet_weno": lambda: K.tet_shock_box(3, seed=13, numerics=K.Numerics(
        spaceDiscr=K.DISCR_UPW_ROE, venkatGuard=1, reconst=K.RECONST_WENO_XYZ)),
}
STEPS = 4


def compute(c):
    from oracle.oracle import Oracle
    o = Oracle(c)
    rhs, grad = o.residual(c.cv.copy(), c.dv.copy())
    cv, dv = c.cv.copy(), c.dv.copy()
    dti = o.dt(cv, dv, c.numerics.cfl, 1.0, 0.0, 1.0)
    t, _, st = o.run(cv, dv, n_steps=STEPS, dt_imposed=dti)
    return {"rhs": rhs, "grad": grad, "cv": cv, "dv": dv, "t": np.array([t]),
            "status": np.array([st]), "cv0": c.cv}


def main():
    out = {}
    for name, make in CASES.items():
        for k, v in compute(make()).items():
            out[f"{name}/{k}"] = v
    np.savez_compressed(os.path.join(HERE, "oracle_small.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
