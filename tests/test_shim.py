"""The C++ drop-in headers (include/fvgb300/).

A driver written against the reference's class API (tests/shim/driver.cpp)
must compile unchanged against the drop-in headers -- with the reference's
own UnstructuredMesh.h/EulerState.h/GradientReconstruction.h where the
reference is installed (CPU test), else with stand-in declarations of the
same structs -- link against libfvgb300.so, and on a GPU reproduce the
reference's outputs through EulerFVMSolver, NavierStokesFVMSolver and
UnstructuredFVMSolver.
"""
import os
import subprocess

import numpy as np
import pytest

from finitevolume_gb300 import build, solvers as S
from helpers import case_of, load_golden, parse_ic, poly_of, rel_err

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "tests", "shim")
REF_INCLUDE = os.path.join(build.reference_dir(), "include")


def compile_driver(out_dir, ref_include):
    exe = os.path.join(out_dir, "driver")
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include", "fvgb300"), "-I",
           os.path.join(ROOT, "include"), "-I", ref_include, os.path.join(SHIM, "driver.cpp"), "-L",
           build.LIB_DIR, "-lfvgb300", f"-Wl,-rpath,{build.LIB_DIR}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def write_mesh(mesh, path, patch_specs=None):
    ex = mesh.export()
    fi, cd, off, cf = ex["faces_i32"], ex["cells_f64"], ex["cell_face_off"], ex["cell_faces"]
    nodes = mesh.poly.nodes
    with open(path, "w") as f:
        f.write(f"{nodes.shape[0]}\n")
        f.write("\n".join(f"{x!r} {y!r}" for x, y in nodes.tolist()) + "\n")
        f.write(f"{fi.shape[0]}\n")
        f.write("\n".join(" ".join(map(str, r)) for r in fi.tolist()) + "\n")
        f.write(f"{cd.shape[0]}\n")
        for c in range(cd.shape[0]):
            fl = cf[off[c]:off[c + 1]].tolist()
            f.write(f"{float(cd[c, 0])!r} {float(cd[c, 1])!r} {float(cd[c, 2])!r} {len(fl)} {' '.join(map(str, fl))}\n")
        names = mesh.patch_names
        f.write(f"{len(names)}\n")
        for n in names:
            t, v = (patch_specs or {}).get(n, (0, 0.0))
            f.write(f"{n} {t} {float(v)!r}\n")


def test_driver_compiles_against_reference_headers(tmp_path):
    build.build_library()
    inc = REF_INCLUDE if os.path.isdir(REF_INCLUDE) else os.path.join(SHIM, "ref_decls")
    assert os.path.exists(compile_driver(str(tmp_path), inc))


def test_driver_compiles_against_stand_in_declarations(tmp_path):
    """The GPU test compiles the driver with tests/shim/ref_decls (the
    reference is not installed there): those stand-ins must cover every
    reference type the drop-in headers use."""
    build.build_library()
    assert os.path.exists(compile_driver(str(tmp_path), os.path.join(SHIM, "ref_decls")))


@pytest.mark.parametrize("which", ["reference", "stand-in"])
def test_class_surface_compiles(which):
    """Every member of the reference's solver classes, called with the
    reference's argument types, compiles against the drop-in headers."""
    inc = REF_INCLUDE if which == "reference" and os.path.isdir(REF_INCLUDE) else os.path.join(SHIM, "ref_decls")
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "include", "fvgb300"),
           "-I", os.path.join(ROOT, "include"), "-I", inc, os.path.join(SHIM, "api_surface.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def _run(exe, mesh_txt, case, out):
    with open(out + ".case", "w") as f:
        f.write("\n".join(f"{k} {float(v)!r}" for k, v in case.items()) + "\n")
    subprocess.run([exe, mesh_txt, out + ".case", out], check=True, capture_output=True)
    return np.fromfile(out)


@pytest.mark.gpu
def test_driver_reproduces_reference(gpu, tmp_path):
    exe = compile_driver(str(tmp_path), os.path.join(SHIM, "ref_decls"))
    # Euler, Rusanov
    g = load_golden("naca_og64")
    case = case_of(g)
    ic = parse_ic(case["ic"])
    m = S.Mesh(poly_of(g))
    write_mesh(m, str(tmp_path / "og.txt"))
    out = _run(exe, str(tmp_path / "og.txt"), dict(kind=0, flux=0, cfl=case["cfl"], steps=case["steps"],
                                                   rho=ic["rho"], u=ic["u"], v=ic["v"], p=ic["p"]),
               str(tmp_path / "e.f64"))
    U, res = out[:-4].reshape(-1, 4), out[-4:]
    assert rel_err(U, g["field_rusanov"]) < 1e-10
    np.testing.assert_allclose(res, g["hist_rusanov"][-1], rtol=1e-10)
    # Navier-Stokes, Rusanov + LSQ
    g = load_golden("ns_naca_og64")
    case = case_of(g)
    ic = parse_ic(case["ic"])
    m = S.Mesh(poly_of(g))
    write_mesh(m, str(tmp_path / "ns.txt"))
    out = _run(exe, str(tmp_path / "ns.txt"), dict(kind=1, flux=0, cfl=case["cfl"], steps=case["steps"],
                                                   rho=ic["rho"], u=ic["u"], v=ic["v"], p=ic["p"], R=case["R"],
                                                   mu=case["mu"], Pr=case["Pr"]), str(tmp_path / "n.f64"))
    assert rel_err(out[:-4].reshape(-1, 4), g["field_rusanov_lsq"]) < 1e-10
    # RANS with Spalart-Allmaras, HLLC + LSQ
    g = load_golden("rans_naca_og64")
    case = case_of(g)
    ic = parse_ic(case["ic"])
    m = S.Mesh(poly_of(g))
    write_mesh(m, str(tmp_path / "rans.txt"))
    nut_far = float(case["bc"][1].split(":")[6])
    out = _run(exe, str(tmp_path / "rans.txt"), dict(kind=3, flux=1, cfl=case["cfl"], steps=case["steps"],
                                                     rho=ic["rho"], u=ic["u"], v=ic["v"], p=ic["p"], R=case["R"],
                                                     mu=case["mu"], Pr=case["Pr"], Prt=case["Prt"],
                                                     nut0=case["nut0"], nut_far=nut_far), str(tmp_path / "r.f64"))
    n = m.n_cells
    assert rel_err(out[:4 * n].reshape(-1, 4), g["field_hllc_lsq"]) < 1e-10
    assert rel_err(out[4 * n:5 * n], g["nut_hllc_lsq"]) < 1e-10
    # Diffusion: patch kinds come from mesh.patches, as in the reference
    g = load_golden("diffusion_cart")
    case = case_of(g)
    m = S.Mesh(poly_of(g))
    specs = {}
    for s in case["bc"]:
        n, kind, val = s.split(":")
        specs[n] = (1 if kind == "neumann" else 0, float(val))
    write_mesh(m, str(tmp_path / "d.txt"), specs)
    out = _run(exe, str(tmp_path / "d.txt"), dict(kind=2, alpha=case["alpha"], dt=case["dt"], v0=case["v0"],
                                                  r0=case["r0"], steps=case["steps"], rho=1.0, u=0.0, v=0.0, p=1.0),
               str(tmp_path / "d.f64"))
    assert np.array_equal(out[:-1], g["field"])
