"""Algorithmic HBM bytes of one RK stage: the compulsory traffic of a
three-pass stage in which every array element is counted once per pass and
no cache re-read is counted, evaluated from the actual cell, face, boundary
face and stencil-member counts.  s is the working-precision size (8 for the
FP64 path, 4 for the mixed path's FP32 primitive state / gradients).

  pass                       per cell                          per member  per int. face  per bnd. face
  P1 prim + WLSQ gradient    cv 40, cofg 24, xyzMoms 48,        CSR idx 4   -              -
                             CSR offset 4; write prim 5s,
                             grad 15s
  P2 Venkatakrishnan         prim 5s, grad 15s, cofg 24,        -           f2c 8, fc 24,  -
                             vol 8, c2f offset 4; write 15s                 c2f 8
  P3 flux + gather + update  prim 5s, grad 15s, cofg 24,        -           f2c 8, fn 32,  bf2c 4, fn 32,
     + EOS                   c2f offset 4, cv 40, rhsSum 40,                fc 24, c2f 8   fc 24, c2f 4
                             vol 8; write cv 40, rhsSum 40,
                             p 8, a 8

Totals per stage: FP64 964 Nc + 4 M + 112 Nf + 64 Nb, mixed 664 Nc + 4 M +
112 Nf + 64 Nb.  The engine's kernels map onto the passes as below; the
per-kernel split of P3 gives the face kernels the per-face columns plus the
cell data they gather (prim, grad, cofg) and the gather/update kernel the
update columns, so the kernel figures add up to the pass totals.  The figures
do not move with design choices (precomputed weights, fused passes).
"""
from __future__ import annotations


def kernel_bytes(nc: int, nf: int, nb: int, m: int, s: int) -> dict:
    """Algorithmic bytes per launch of each stage kernel."""
    grad = nc * (40 + 24 + 48 + 4 + 5 * s + 15 * s) + 4 * m
    lim = nc * (5 * s + 15 * s + 24 + 8 + 4 + 15 * s) + nf * (8 + 24 + 8)
    face = nf * (8 + 32 + 24 + 8) + nc * (5 * s + 15 * s + 24)
    bface = nb * (4 + 32 + 24 + 4)
    upd = nc * (4 + 40 + 40 + 8 + 40 + 40 + 8 + 8)
    return {"gradient": grad, "limiter": lim, "face_flux": face, "bface_flux": bface,
            "gather_update": upd}


def stage_bytes(nc: int, nf: int, nb: int, m: int, s: int) -> int:
    return sum(kernel_bytes(nc, nf, nb, m, s).values())


def engine_kernel_bytes(nc: int, nf: int, nb: int, m: int, s: int) -> dict:
    """Algorithmic bytes per launch of the engine's kernels: the gradient
    kernel fuses the limiter, so it carries P1 + P2."""
    kb = kernel_bytes(nc, nf, nb, m, s)
    return {"gradient": kb["gradient"] + kb["limiter"], "face_flux": kb["face_flux"],
            "bface_flux": kb["bface_flux"], "gather_update": kb["gather_update"]}


def residual_bytes(nc: int, nf: int, nb: int, m: int, s: int) -> int:
    """Single residual evaluation: P1 + P2 + P3 without the update columns
    (cv, rhsSum, vol, p, a)."""
    kb = kernel_bytes(nc, nf, nb, m, s)
    return kb["gradient"] + kb["limiter"] + kb["face_flux"] + kb["bface_flux"] + nc * 4


FLOPS_FP64 = {"member": 50, "face": 300, "limiter_face": 100, "cell": 60}


def stage_flops(nc: int, nf: int, nb: int, m: int) -> int:
    """Rough FP64 flop count of one stage (shows the FP64 path is ALU-bound)."""
    f = FLOPS_FP64
    return f["member"] * m + f["face"] * (nf + nb) + f["limiter_face"] * nf + f["cell"] * nc
