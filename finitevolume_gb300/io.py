"""Run outputs in the reference's formats: checkpoints and the residual CSV.

* :func:`write_checkpoint` / :func:`read_checkpoint` -- the binary layout of
  include/Checkpoint.h:26-46 through the C ABI (``fv_checkpoint_write`` /
  ``fv_checkpoint_read``), so GPU runs resume from and into reference
  checkpoints.
* :class:`ResidualCSV` -- ``step,residual_rho,residual_rho_u,residual_rho_v,
  residual_E`` every ``interval`` steps, flushed on every row
  (src/main.cpp:3474-3515).
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, TextIO, Tuple

import numpy as np

from . import capi

EQUATIONS = {"diffusion": 0, "euler": 1, "advection_diffusion": 2, "navier_stokes": 3, "rans_sa": 4, "rans_sst": 5}
_PER_CELL = {0: 1, 1: 4, 2: 1, 3: 4, 4: 5, 5: 6}


def write_checkpoint(path: str, equation: str, step_index: int, payload: np.ndarray, build_number: int = 0) -> None:
    eq = EQUATIONS[equation]
    p = np.ascontiguousarray(payload, dtype=np.float64)
    cells = p.size // _PER_CELL[eq]
    if cells * _PER_CELL[eq] != p.size:
        raise ValueError("payload size is not a whole number of cells")
    capi.check(capi.lib().fv_checkpoint_write(path.encode(), eq, int(step_index), int(build_number), cells,
                                              capi.dptr(p.reshape(-1))))


def read_checkpoint(path: str, equation: Optional[str], cell_count: int) -> Tuple[np.ndarray, int, int]:
    """(payload, step_index, build_number).  equation=None reads the state
    block of any flow-equation checkpoint (Checkpoint::read_flow_field)."""
    eq = -1 if equation is None else EQUATIONS[equation]
    per = 4 if eq < 0 else _PER_CELL[eq]
    out = np.zeros(cell_count * per)
    step = C.c_int64()
    build = C.c_uint64()
    capi.check(capi.lib().fv_checkpoint_read(path.encode(), eq, int(cell_count), C.byref(step), C.byref(build),
                                             capi.dptr(out)))
    return (out.reshape(cell_count, per) if per > 1 else out), step.value, build.value


class ResidualCSV:
    """Residual history file of the reference's run loop."""

    def __init__(self, path: str, interval: int = 1, precision: int = 6, extra=()):
        self.f: TextIO = open(path, "w")
        self.interval = max(1, int(interval))
        self.precision = precision
        cols = ["residual_rho", "residual_rho_u", "residual_rho_v", "residual_E"] + [f"residual_{x}" for x in extra]
        self.f.write("step," + ",".join(cols) + "\n")
        self.f.flush()

    def record(self, step_index: int, norms) -> None:
        if step_index % self.interval:
            return
        vals = ",".join(f"{float(x):.{self.precision}g}" for x in norms)
        self.f.write(f"{step_index},{vals}\n")
        self.f.flush()

    def close(self) -> None:
        self.f.close()
