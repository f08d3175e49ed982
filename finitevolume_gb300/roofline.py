"""Algorithmic HBM bytes of the residual-and-update loop (one place).

Counts are per launch, with every array that a kernel must read or write
crossing HBM exactly once (neighbour gathers re-read nothing).  N cells, F
faces, Fb boundary faces, E = 2F - Fb cell-face (CSR) entries; s = 8 bytes
(FP64) or 4 (FP32-flux mode) for the flux-precision arrays (primitive copy
W, gradients G, face fluxes).

Whole residual evaluation, per the survey's per-stage formula (one RK stage
of 2nd-order MUSCL with materialised gradient and limiter arrays):
    B2 = 340 N + 56 F
and first order, forward Euler, local dt:
    B1 = 76 N + 40 F

Per kernel of this implementation, at an RK stage without time-step work
(stages 2 and 3; the limiter is fused into the gradient kernel, so no
limiter array exists; face fluxes are materialised once):
    gradients  W r (4s N) + G w (8s N) + CSR offsets 4N + per-entry
               neighbour 4E + LSQ weights 2s E + face offsets 2s E
               + weight sums 2s N + Venkatakrishnan eps^2 s N
               = 15s N + 4N + (4 + 4s) E
    faces      W r (4s N) + G r (8s N) + normal/length/CFL length 4s F
               + offsets from both centroids 4s F + owner/neighbour 8F
               + fluxes w (4s F)
               = 12s N + (12s + 8) F
    update     fluxes r (4s F) + CSR offsets 4N + entries 4E + U r/w 64N
               + U0 r 32N + W w (4s N) + dt/V r 8N
               = 4s F + 4E + (108 + 4s) N
Arrays an earlier kernel has just written may still sit in the 129 MB L2,
so a measured DRAM figure can come in below these counts.
"""
from __future__ import annotations


def survey_stage_bytes(n: int, f: int) -> float:
    """B2: algorithmic bytes of one 2nd-order RK stage (survey formula)."""
    return 340.0 * n + 56.0 * f


def survey_o1_bytes(n: int, f: int) -> float:
    """B1: first order, forward Euler, local dt."""
    return 76.0 * n + 40.0 * f


def kernel_bytes(kind: str, n: int, f: int, fb: int, fp32: bool = False) -> float:
    s = 4.0 if fp32 else 8.0
    e = 2 * f - fb
    if kind == "gradients":
        return 15 * s * n + 4 * n + (4 + 4 * s) * e
    if kind == "faces":
        return 12 * s * n + (12 * s + 8) * f
    if kind == "update":
        return 4 * s * f + 4 * e + (108 + 4 * s) * n
    raise ValueError(kind)


KERNEL_NAMES = ("gradients", "faces", "update")


# DRAM bytes per cell per launch measured by ncu (dram__bytes_read.sum +
# dram__bytes_write.sum, one launch of each kernel class) on the 968,907-cell
# NACA0012 mixed mesh; the captures are summarised under profiles/.  In
# FP64 the gradient pass writes the per-entry limiter increments that the
# face pass reads (32 B per entry each way), which puts both above their
# algorithmic bytes on purpose: the FP64 kernels are bound by FP64 issue,
# not by DRAM, and the increments save the face pass one multiply-add per
# variable and side.
MEASURED_TRAFFIC_PER_CELL = {"gradients": 382.0, "faces": 401.3, "update": 207.2}
MEASURED_TRAFFIC_PER_CELL_FP32 = {"gradients": 146.3, "faces": 165.1, "update": 147.7}

# FP64-pipe thread instructions per cell and per launch from the same
# captures (smsp__inst_executed_pipe_fp64.sum x 32 / cells).  On GB300 the
# FP64 pipe, not HBM, bounds the FP64 kernels.
MEASURED_FP64_INST_PER_CELL = {"gradients": 236.4, "faces": 232.0, "update": 44.4}


def measured_traffic(kind: str, n_cells: int, fp32: bool = False):
    b = (MEASURED_TRAFFIC_PER_CELL_FP32 if fp32 else MEASURED_TRAFFIC_PER_CELL).get(kind)
    return None if b is None else round(b * n_cells)
