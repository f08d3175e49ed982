"""Case-file driver (finitevolume_gb300/case.py).

CPU: the parser reads the reference's case format, and next_cfl follows
src/CflRamp.cpp:7-27 on the reference's own ramp checks (the unit checks
of its --verify-cfl-ramp mode: growth to the ceiling on a falling
residual, shrink to the floor on a rising one, hold when flat, hard reset
on divergence, no change before the window is full).
GPU: a case file runs the Euler solver with the CFL ramp, writes the
residual CSV, stops at the tolerance and resumes from its checkpoint.
"""
import os

import numpy as np
import pytest

from finitevolume_gb300 import case as K
from finitevolume_gb300 import fvmesh, meshgen


def test_next_cfl_follows_the_reference_ramp():
    p = K.CflRampParams(cfl_min=0.05, growth_factor=1.5, shrink_factor=0.5, window=5, divergence_threshold=2.0)
    # window not full: unchanged
    assert K.next_cfl(0.3, 2.0, [1.0, 0.5], p) == 0.3
    # falling: grows, clamped at the ceiling
    cfl = 0.05
    for _ in range(20):
        cfl = K.next_cfl(cfl, 2.0, [1.0, 0.8, 0.6, 0.4, 0.2], p)
    assert cfl == 2.0
    # mildly rising (beyond the 10% dead band, below divergence): shrinks to the floor
    cfl = 1.0
    for _ in range(20):
        cfl = K.next_cfl(cfl, 2.0, [1.0, 1.1, 1.2, 1.3, 1.5], p)
    assert cfl == 0.05
    # flat (within the dead band): holds
    assert K.next_cfl(0.7, 2.0, [1.0, 1.0, 1.0, 1.0, 1.05], p) == 0.7
    # divergent jump: hard reset
    assert K.next_cfl(1.5, 2.0, [1.0, 10.0, 100.0, 1000.0, 1000.0], p) == 0.05


def test_parser_reads_the_reference_format(tmp_path):
    f = tmp_path / "c.case"
    f.write_text("""# comment
equation = euler
mesh_file = og.fvmesh   # trailing comment
nsteps = 40
gamma = 1.4
cfl = 0.8
cfl_mode = ramp
cfl_min = 0.1
cfl_ramp_window = 4
flux_scheme = hllc
euler_init = freestream 1.0 0.5 0.0 0.714285714
boundary airfoil wall
boundary farfield farfield 1.0 0.5 0.0 0.714285714
residual_file = out/res.csv
residual_tolerance_rho = 1e-3
output_file = out/x.vtk
checkpoint_file = out/ck.bin
""")
    c = K.CaseInput.load(str(f))
    assert c.equation == "euler" and c.nsteps == 40 and c.cfl == 0.8 and c.cfl_mode == "ramp"
    assert c.cfl_ramp.cfl_min == 0.1 and c.cfl_ramp.window == 4 and c.flux_scheme == "hllc"
    assert c.mesh_file == os.path.join(str(tmp_path), "og.fvmesh")
    assert c.init["euler_init"] == ("freestream", [1.0, 0.5, 0.0, 0.714285714])
    assert c.boundaries[1] == ("farfield", "farfield", [1.0, 0.5, 0.0, 0.714285714])
    assert c.tolerances == {"rho": 1e-3}
    assert "output_file" in c.ignored


@pytest.mark.gpu
def test_case_runs_ramps_stops_and_resumes(gpu, tmp_path):
    m = meshgen.naca_ogrid(48, 24)
    fvmesh.write_fvmesh(m, str(tmp_path / "og.fvmesh"))
    M = 0.5
    text = f"""equation = euler
mesh_file = og.fvmesh
nsteps = 400
cfl = 0.9
cfl_mode = ramp
cfl_min = 0.1
cfl_ramp_window = 5
euler_init = freestream 1 {M} 0 {1 / 1.4!r}
boundary airfoil wall
boundary farfield farfield 1 {M} 0 {1 / 1.4!r}
residual_file = res.csv
checkpoint_file = ck.bin
"""
    (tmp_path / "a.case").write_text(text)
    c = K.CaseInput.load(str(tmp_path / "a.case"))
    r = K.run_case(c, log=lambda *a: None)
    assert r["outcome"] == "completed" and r["last_step"] == 400 and r["cfl"] == 0.9
    rows = (tmp_path / "res.csv").read_text().splitlines()
    assert rows[0] == "step,residual_rho,residual_rho_u,residual_rho_v,residual_E" and len(rows) == 401
    # resume: nothing left to run at nsteps = 400; with a tolerance the run
    # stops at the first step whose density residual is below it
    rho = np.array([float(x.split(",")[1]) for x in rows[1:]])
    (tmp_path / "b.case").write_text(text.replace("nsteps = 400", "nsteps = 900").replace(
        "checkpoint_file = ck.bin", "checkpoint_file = ck.bin\nresidual_tolerance_rho = " + repr(float(rho[-1] * 0.5))))
    r2 = K.run_case(K.CaseInput.load(str(tmp_path / "b.case")), log=lambda *a: None)
    assert r2["outcome"] in ("converged", "completed") and r2["last_step"] > 400
    if r2["outcome"] == "converged":
        assert r2["residual"][0] < rho[-1] * 0.5


def test_next_cfl_matches_the_compiled_reference():
    """400 seeded residual windows and ramp parameter sets through the
    reference's own next_cfl (fixture tests/golden/cfl_ramp.npz)."""
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "cfl_ramp.npz"))
    for head, h, want in zip(z["heads"], z["hist"], z["out"]):
        p = K.CflRampParams(cfl_min=head[2], growth_factor=head[3], shrink_factor=head[4], window=int(head[6]),
                            divergence_threshold=head[5])
        hist = list(h[:int(head[7])])
        assert K.next_cfl(head[0], head[1], hist, p) == want
