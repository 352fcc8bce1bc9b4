"""Exact solution of the 1-D Riemann problem for a perfect gas (Toro,
"Riemann Solvers and Numerical Methods for Fluid Dynamics", ch. 4): Newton
iteration on the star pressure, then sampling of the self-similar solution.
The reference has no exact Sod solution of its own; this one is written from
the mathematics and used to check the oracle."""
from __future__ import annotations

import numpy as np


def _f(p, rk, pk, ak, g):
    if p > pk:  # shock
        A = 2.0 / ((g + 1.0) * rk)
        B = (g - 1.0) / (g + 1.0) * pk
        q = np.sqrt(A / (p + B))
        return (p - pk) * q, q * (1.0 - 0.5 * (p - pk) / (B + p))
    pr = p / pk  # rarefaction
    return (2.0 * ak / (g - 1.0)) * (pr ** ((g - 1.0) / (2.0 * g)) - 1.0), \
        1.0 / (rk * ak) * pr ** (-(g + 1.0) / (2.0 * g))


def star_state(left, right, g=1.4):
    rl, ul, pl = left
    rr, ur, pr = right
    al, ar = np.sqrt(g * pl / rl), np.sqrt(g * pr / rr)
    p = max(1e-12, 0.5 * (pl + pr))
    for _ in range(100):
        fl, dfl = _f(p, rl, pl, al, g)
        fr, dfr = _f(p, rr, pr, ar, g)
        dp = (fl + fr + (ur - ul)) / (dfl + dfr)
        pn = max(1e-12, p - dp)
        if abs(pn - p) < 1e-14 * (pn + p):
            p = pn
            break
        p = pn
    fl, _ = _f(p, rl, pl, al, g)
    fr, _ = _f(p, rr, pr, ar, g)
    u = 0.5 * (ul + ur) + 0.5 * (fr - fl)
    return p, u


def sample(x, t, x0, left, right, g=1.4):
    """(rho, u, p) at positions x and time t for a diaphragm at x0."""
    rl, ul, pl = left
    rr, ur, pr = right
    al, ar = np.sqrt(g * pl / rl), np.sqrt(g * pr / rr)
    ps, us = star_state(left, right, g)
    out = np.zeros((len(x), 3))
    for i, xi in enumerate(np.asarray(x)):
        s = (xi - x0) / t
        if s <= us:  # left of contact
            if ps > pl:
                sl = ul - al * np.sqrt((g + 1.0) / (2.0 * g) * ps / pl + (g - 1.0) / (2.0 * g))
                if s <= sl:
                    out[i] = (rl, ul, pl)
                else:
                    rs = rl * ((ps / pl + (g - 1) / (g + 1)) / ((g - 1) / (g + 1) * ps / pl + 1.0))
                    out[i] = (rs, us, ps)
            else:
                shl = ul - al
                als = al * (ps / pl) ** ((g - 1.0) / (2.0 * g))
                stl = us - als
                if s <= shl:
                    out[i] = (rl, ul, pl)
                elif s >= stl:
                    out[i] = (rl * (ps / pl) ** (1.0 / g), us, ps)
                else:
                    c = 2.0 / (g + 1.0) + (g - 1.0) / ((g + 1.0) * al) * (ul - s)
                    out[i] = (rl * c ** (2.0 / (g - 1.0)),
                              2.0 / (g + 1.0) * (al + (g - 1.0) / 2.0 * ul + s),
                              pl * c ** (2.0 * g / (g - 1.0)))
        else:
            if ps > pr:
                sr = ur + ar * np.sqrt((g + 1.0) / (2.0 * g) * ps / pr + (g - 1.0) / (2.0 * g))
                if s >= sr:
                    out[i] = (rr, ur, pr)
                else:
                    rs = rr * ((ps / pr + (g - 1) / (g + 1)) / ((g - 1) / (g + 1) * ps / pr + 1.0))
                    out[i] = (rs, us, ps)
            else:
                shr = ur + ar
                ars = ar * (ps / pr) ** ((g - 1.0) / (2.0 * g))
                str_ = us + ars
                if s >= shr:
                    out[i] = (rr, ur, pr)
                elif s <= str_:
                    out[i] = (rr * (ps / pr) ** (1.0 / g), us, ps)
                else:
                    c = 2.0 / (g + 1.0) - (g - 1.0) / ((g + 1.0) * ar) * (ur - s)
                    out[i] = (rr * c ** (2.0 / (g - 1.0)),
                              2.0 / (g + 1.0) * (-ar + (g - 1.0) / 2.0 * ur + s),
                              pr * c ** (2.0 * g / (g - 1.0)))
    return out
