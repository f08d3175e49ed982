"""Generate the golden fixtures of the reference's own outputs.

Runs the reference solver classes (compiled in place by ``oracle/Makefile``
into ``oracle/_ref/fvref``) on small seeded meshes and stores inputs and
outputs as compressed ``.npz`` files in this directory.  The reference
checkout is only needed to regenerate the fixtures; the tests read the
committed ``.npz`` files.

    python tests/golden/make_golden.py [--ref /path/to/reference]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from finitevolume_gb300 import build, fvmesh, meshgen  # noqa: E402

GAMMA = 1.4


def fvref(mode, mesh_path, outdir, **kw):
    args = [os.path.join(ROOT, "oracle", "_ref", "fvref"), mode, f"mesh={mesh_path}", f"out={outdir}"]
    for k, v in kw.items():
        vals = v if isinstance(v, list) else [v]
        args += [f"{k}={x}" for x in vals]
    r = subprocess.run(args, capture_output=True, text=True, check=True)
    return json.loads(r.stdout.strip().splitlines()[-1])


def mesh_arrays(m):
    return dict(nodes=m.nodes, cell_off=m.cell_off, cell_nodes=m.cell_nodes, bedges=m.bedges, bpatch=m.bpatch,
                patch_names=np.array(m.patch_names))


def prim_str(rho, u, v, p):
    return ":".join(repr(float(x)) for x in (rho, u, v, p))


def euler_case(name, mesh, case, tmp, steps):
    path = os.path.join(tmp, name + ".fvmesh")
    fvmesh.write_fvmesh(mesh, path)
    out = os.path.join(tmp, name)
    os.makedirs(out, exist_ok=True)
    res = {}
    for flux in case["fluxes"]:
        fvref("euler", path, out, flux=flux, cfl=case["cfl"], ic=case["ic"], bc=case["bc"], steps=steps,
              gamma=GAMMA)
        res[f"field_{flux}"] = np.fromfile(os.path.join(out, "field.f64")).reshape(-1, 4)
        res[f"hist_{flux}"] = np.fromfile(os.path.join(out, "resid.f64")).reshape(-1, 4)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **mesh_arrays(mesh), **res,
                        case=np.array(json.dumps({**case, "steps": steps})))


def ns_case(name, mesh, case, tmp, steps):
    path = os.path.join(tmp, name + ".fvmesh")
    fvmesh.write_fvmesh(mesh, path)
    out = os.path.join(tmp, name)
    os.makedirs(out, exist_ok=True)
    ref = case["ref"]
    res = {}
    for flux in case["fluxes"]:
        for grad in case["grads"]:
            fvref("ns", path, out, flux=flux, grad=grad, cfl=case["cfl"], ic=case["ic"], bc=case["bc"], steps=steps,
                  gamma=GAMMA, R=case["R"], mu=case["mu"], Pr=case["Pr"], ref_rho=ref[0], ref_u=ref[1], ref_v=ref[2],
                  ref_p=ref[3], ref_len=ref[4], ref_mx=ref[5], ref_my=ref[6])
            tag = f"{flux}_{grad}"
            res[f"field_{tag}"] = np.fromfile(os.path.join(out, "field.f64")).reshape(-1, 4)
            res[f"hist_{tag}"] = np.fromfile(os.path.join(out, "resid.f64")).reshape(-1, 4)
            res[f"forces_{tag}"] = np.fromfile(os.path.join(out, "forces.f64")).reshape(-1, 11)
            res[f"wall_{tag}"] = np.fromfile(os.path.join(out, "wall.f64")).reshape(-1, 3)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **mesh_arrays(mesh), **res,
                        case=np.array(json.dumps({**case, "steps": steps})))


def rans_case(name, mesh, case, tmp, steps):
    path = os.path.join(tmp, name + ".fvmesh")
    fvmesh.write_fvmesh(mesh, path)
    out = os.path.join(tmp, name)
    os.makedirs(out, exist_ok=True)
    ref = case["ref"]
    res = {}
    for flux in case["fluxes"]:
        for grad in case["grads"]:
            fvref("rans", path, out, flux=flux, grad=grad, cfl=case["cfl"], ic=case["ic"], bc=case["bc"], steps=steps,
                  gamma=GAMMA, R=case["R"], mu=case["mu"], Pr=case["Pr"], Prt=case["Prt"], nut0=case["nut0"],
                  ref_rho=ref[0], ref_u=ref[1], ref_v=ref[2], ref_p=ref[3], ref_len=ref[4], ref_mx=ref[5],
                  ref_my=ref[6])
            tag = f"{flux}_{grad}"
            res[f"field_{tag}"] = np.fromfile(os.path.join(out, "field.f64")).reshape(-1, 4)
            res[f"nut_{tag}"] = np.fromfile(os.path.join(out, "nut.f64"))
            res[f"hist_{tag}"] = np.fromfile(os.path.join(out, "history.f64")).reshape(-1, 5)
            res[f"forces_{tag}"] = np.fromfile(os.path.join(out, "forces.f64")).reshape(-1, 11)
    res["walld"] = np.fromfile(os.path.join(out, "walld.f64"))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **mesh_arrays(mesh), **res,
                        case=np.array(json.dumps({**case, "steps": steps})))


def rans_fixtures(tmp):
    """Spalart-Allmaras RANS (RANSTurbulenceSASolver): a no-slip NACA0012 in
    a farfield with freestream nu-tilde = 3 nu, and a channel between an
    isothermal still wall and a moving wall with outflow ends."""
    R = 287.0
    M, aoa = 0.5, np.radians(2.0)
    u, v, p = M * np.cos(aoa), M * np.sin(aoa), 1.0 / GAMMA
    mu = 1e-3
    og = meshgen.naca_ogrid(64, 32)
    rans_case("rans_naca_og64", og, {
        "fluxes": ["rusanov", "hllc"], "grads": ["lsq", "gg"], "cfl": 0.5, "R": R, "mu": mu, "Pr": 0.72,
        "Prt": 0.9, "nut0": 3 * mu, "ic": "free:" + prim_str(1.0, u, v, p),
        "bc": ["airfoil:noslip", "farfield:farfield:" + prim_str(1.0, u, v, p) + ":" + repr(3 * mu)],
        "ref": [1.0, float(u), float(v), float(p), 1.0, 0.25, 0.0]}, tmp, 150)
    T_inf = (1.0 / GAMMA) / R
    ch = meshgen.sod_strip(24, 8, length=2.0, height=1.0, jitter=0.15, seed=3)
    rans_case("rans_channel_tri", ch, {
        "fluxes": ["rusanov"], "grads": ["lsq", "gg"], "cfl": 0.4, "R": R, "mu": 5e-3, "Pr": 0.72, "Prt": 0.9,
        "nut0": 2e-2, "ic": "free:" + prim_str(1.0, 0.05, 0.0, 1.0 / GAMMA),
        "bc": ["bottom:noslip:0:0:" + repr(T_inf), "top:noslip:0.2:0", "left:outflow", "right:outflow"],
        "ref": [1.0, 0.2, 0.0, 1.0 / GAMMA, 2.0, 1.0, 0.5]}, tmp, 200)


def cfl_ramp_fixture(tmp):
    """next_cfl on seeded residual windows: falling, rising, flat, noisy and
    divergent sequences, several ramp parameter sets."""
    rng = np.random.default_rng(5)
    recs, rows = [], []
    for i in range(400):
        window = int(rng.integers(3, 20))
        n = int(rng.integers(1, window + 1)) if i % 7 == 0 else window
        kind = i % 5
        steps = np.arange(n)
        if kind == 0:
            h = 10.0 ** (-0.1 * steps * rng.uniform(0.1, 2.0))
        elif kind == 1:
            h = 10.0 ** (0.01 * steps * rng.uniform(0.5, 20.0))
        elif kind == 2:
            h = np.full(n, rng.uniform(1e-6, 1.0)) * (1.0 + rng.uniform(-0.02, 0.02, n))
        elif kind == 3:
            h = 10.0 ** rng.normal(-3.0, 0.3, n)
        else:
            h = 10.0 ** (0.5 * steps * rng.uniform(0.5, 2.0))
        head = [rng.uniform(0.05, 3.0), rng.uniform(0.5, 5.0), rng.uniform(0.01, 0.2), rng.uniform(1.05, 2.0),
                rng.uniform(0.2, 0.9), rng.uniform(0.5, 3.0), float(window), float(n)]
        recs.append(np.concatenate([head, h]))
        rows.append((head, h))
    path = os.path.join(tmp, "ramp.bin")
    np.concatenate(recs).astype(np.float64).tofile(path)
    out = os.path.join(tmp, "ramp.out")
    subprocess.run([os.path.join(ROOT, "oracle", "_ref", "fvref"), "cflramp", f"in={path}", f"out={out}"],
                   check=True, capture_output=True)
    np.savez_compressed(os.path.join(HERE, "cfl_ramp.npz"), heads=np.array([r[0] for r in rows]),
                        hist=np.array([np.pad(r[1], (0, 20 - len(r[1])), constant_values=np.nan) for r in rows]),
                        out=np.fromfile(out))


def config1_fixture(tmp, steps=3000):
    """The small plain-method configuration at its own size, in the
    reference's mode: NACA0012 O-grid 256 x 128 (32,768 cells), first-order
    Rusanov, forward Euler with the global CFL time step at CFL 0.5, slip
    wall and fixed-state farfield, M 0.5, AoA 2 deg, 3,000 iterations.  The
    field, the residual history and the inviscid wall forces
    (compute_wall_forces) are the reference's; the mesh arrays are stored
    with them, since the generator's trigonometry differs in the last bits
    between host maths libraries."""
    M, aoa = 0.5, np.radians(2.0)
    u, v, p = M * np.cos(aoa), M * np.sin(aoa), 1.0 / GAMMA
    og = meshgen.naca_ogrid(256, 128)
    path = os.path.join(tmp, "og256.fvmesh")
    fvmesh.write_fvmesh(og, path)
    out = os.path.join(tmp, "og256")
    os.makedirs(out, exist_ok=True)
    case = {"flux": "rusanov", "cfl": 0.5, "ic": "free:" + prim_str(1.0, u, v, p),
            "bc": ["airfoil:wall", "farfield:farfield:" + prim_str(1.0, u, v, p)], "mach": M, "aoa_deg": 2.0,
            "ref": [1.0, float(u), float(v), float(p), 1.0, 0.25, 0.0], "steps": steps, "mesh": "naca_ogrid(256, 128)"}
    ref = case["ref"]
    info = fvref("euler", path, out, flux="rusanov", cfl=case["cfl"], ic=case["ic"], bc=case["bc"], steps=steps,
                 gamma=GAMMA, ref_rho=ref[0], ref_u=ref[1], ref_v=ref[2], ref_p=ref[3], ref_len=ref[4],
                 ref_mx=ref[5], ref_my=ref[6])
    np.savez_compressed(os.path.join(HERE, "config1_og256_ref.npz"), **mesh_arrays(og),
                        field=np.fromfile(os.path.join(out, "field.f64")).reshape(-1, 4),
                        hist=np.fromfile(os.path.join(out, "resid.f64")).reshape(-1, 4),
                        forces=np.fromfile(os.path.join(out, "forces.f64")).reshape(-1, 11),
                        case=np.array(json.dumps(case)))
    return info


def adjoint_fd_fixture(tmp, steps=80000, h_mach=1e-4, h_aoa_deg=1e-3):
    """Drag and lift of the reference's own EulerFVMSolver converged to its
    round-off floor at a freestream and at the four central-difference
    neighbours in Mach number and angle of attack: NACA0012 O-grid 64 x 32
    (first spacing 1e-2, farfield at 10 chords), first order, forward Euler,
    global dt at CFL 0.9, slip wall and fixed-state farfield, M 0.5, AoA 2
    deg, Rusanov and HLLC, 80,000 iterations each.  Forces by
    compute_wall_forces with zero viscosity, the freestream as the force
    reference.  The central differences of these drags are the
    reference-solver derivatives the discrete adjoint is checked against."""
    og = meshgen.naca_ogrid(64, 32, first=1e-2, r_far=10.0)
    path = os.path.join(tmp, "og64c.fvmesh")
    fvmesh.write_fvmesh(og, path)
    M0, a0 = 0.5, 2.0
    points = [(M0, a0), (M0 + h_mach, a0), (M0 - h_mach, a0), (M0, a0 + h_aoa_deg), (M0, a0 - h_aoa_deg)]
    res = {}
    for flux in ("rusanov", "hllc"):
        rows, last = [], []
        for (M, ad) in points:
            a = np.radians(ad)
            u, v, p = M * np.cos(a), M * np.sin(a), 1.0 / GAMMA
            out = os.path.join(tmp, f"adj_{flux}_{M}_{ad}")
            os.makedirs(out, exist_ok=True)
            fvref("euler", path, out, flux=flux, cfl=0.9, ic="free:" + prim_str(1.0, u, v, p),
                  bc=["airfoil:wall", "farfield:farfield:" + prim_str(1.0, u, v, p)], steps=steps, gamma=GAMMA,
                  ref_rho=1.0, ref_u=u, ref_v=v, ref_p=p, ref_len=1.0, ref_mx=0.25, ref_my=0.0)
            f = np.fromfile(os.path.join(out, "forces.f64")).reshape(-1, 11)
            tot = f[f[:, 0] == -1][0]
            rows.append([M, ad, tot[8], tot[9]])  # cd_total, cl
            last.append(np.fromfile(os.path.join(out, "resid.f64")).reshape(-1, 4)[-1])
            if M == M0 and ad == a0:
                res[f"field_{flux}"] = np.fromfile(os.path.join(out, "field.f64")).reshape(-1, 4)
        res[f"points_{flux}"] = np.array(rows)
        res[f"final_resid_{flux}"] = np.array(last)
    case = {"mach": M0, "aoa_deg": a0, "h_mach": h_mach, "h_aoa_deg": h_aoa_deg, "cfl": 0.9, "steps": steps,
            "mesh": "naca_ogrid(64, 32, first=1e-2, r_far=10)", "bc": ["airfoil:wall", "farfield:farfield"],
            "columns": ["mach", "aoa_deg", "cd_total", "cl"]}
    np.savez_compressed(os.path.join(HERE, "adjoint_fd_ref.npz"), **mesh_arrays(og), **res,
                        case=np.array(json.dumps(case)))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=build.reference_dir())
    ap.add_argument("--only", choices=["rans", "cfl", "config1", "adjoint"], default=None,
                    help="regenerate one group of fixtures")
    a = ap.parse_args()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={a.ref}"], check=True)
    if a.only == "cfl":
        with tempfile.TemporaryDirectory() as tmp:
            cfl_ramp_fixture(tmp)
        return
    if a.only == "rans":
        with tempfile.TemporaryDirectory() as tmp:
            rans_fixtures(tmp)
        return
    if a.only == "config1":
        with tempfile.TemporaryDirectory() as tmp:
            print(config1_fixture(tmp))
        return
    if a.only == "adjoint":
        with tempfile.TemporaryDirectory() as tmp:
            adjoint_fd_fixture(tmp)
        return
    with tempfile.TemporaryDirectory() as tmp:
        rans_fixtures(tmp)
        cfl_ramp_fixture(tmp)
        config1_fixture(tmp)
        adjoint_fd_fixture(tmp)
        # NACA0012 O-grid, M=0.5, AoA=2 deg, slip wall + fixed farfield.
        M, aoa = 0.5, np.radians(2.0)
        u, v, p = M * np.cos(aoa), M * np.sin(aoa), 1.0 / GAMMA
        og = meshgen.naca_ogrid(64, 32)
        euler_case("naca_og64", og, {
            "fluxes": ["rusanov", "hllc", "exact"], "cfl": 0.5, "ic": "free:" + prim_str(1.0, u, v, p),
            "bc": ["airfoil:wall", "farfield:farfield:" + prim_str(1.0, u, v, p)],
            "mach": M, "aoa_deg": 2.0}, tmp, 200)
        # Sod shock tube on a perturbed triangle strip, walls all round.
        sod = meshgen.sod_strip(100, 4, seed=1)
        euler_case("sod_tri", sod, {
            "fluxes": ["rusanov", "hllc", "exact"], "cfl": 0.5, "ic": "two:1:0:0:1:0.125:0:0:0.1:0.5",
            "bc": ["bottom:wall", "right:outflow", "top:wall", "left:outflow"]}, tmp, 120)
        # Gradients on the wavy (non-affine) quad mesh: linear + quadratic field.
        wavy = meshgen.wavy_quads(8)
        path = os.path.join(tmp, "wavy.fvmesh")
        fvmesh.write_fvmesh(wavy, path)
        res = {}
        for scheme in ("lsq", "gg"):
            for tag, coef in (("lin", "1.5:2:-3:0:0:0"), ("quad", "0.5:1:2:0.7:-1.1:0.4")):
                out = os.path.join(tmp, f"g_{scheme}_{tag}")
                os.makedirs(out)
                fvref("grad", path, out, grad=scheme, phi=coef)
                res[f"grad_{scheme}_{tag}"] = np.fromfile(os.path.join(out, "grad.f64")).reshape(-1, 2)
                res[f"facegrad_{scheme}_{tag}"] = np.fromfile(os.path.join(out, "facegrad.f64")).reshape(-1, 4)
                res[f"coef_{tag}"] = np.array([float(x) for x in coef.split(":")])
        out = os.path.join(tmp, "wavy_mesh")
        os.makedirs(out)
        fvref("mesh", path, out)
        for f in ("faces_i32", "faces_f64", "cells_f64", "cell_face_off", "cell_faces"):
            dt = np.int32 if ("i32" in f or "cell_face" in f) else np.float64
            res["mesh_" + f] = np.fromfile(os.path.join(out, f + ".bin"), dtype=dt)
        np.savez_compressed(os.path.join(HERE, "wavy_grad.npz"), **mesh_arrays(wavy), **res)
        # Navier-Stokes: no-slip NACA0012 at Re_c = 500 (adiabatic wall), and
        # a channel with an isothermal moving top wall (Couette-like).
        R = 287.0
        T_inf = (1.0 / GAMMA) / R
        og = meshgen.naca_ogrid(64, 32)
        ns_case("ns_naca_og64", og, {
            "fluxes": ["rusanov", "hllc"], "grads": ["lsq", "gg"], "cfl": 0.5, "R": R, "mu": 1e-3, "Pr": 0.72,
            "ic": "free:" + prim_str(1.0, u, v, p),
            "bc": ["airfoil:noslip", "farfield:farfield:" + prim_str(1.0, u, v, p)],
            "ref": [1.0, float(u), float(v), float(p), 1.0, 0.25, 0.0]}, tmp, 150)
        ch = meshgen.sod_strip(24, 8, length=2.0, height=1.0, jitter=0.15, seed=3)
        ns_case("ns_channel_tri", ch, {
            "fluxes": ["rusanov"], "grads": ["lsq", "gg"], "cfl": 0.5, "R": R, "mu": 5e-3, "Pr": 0.72,
            "ic": "free:" + prim_str(1.0, 0.05, 0.0, 1.0 / GAMMA),
            "bc": ["bottom:noslip:0:0:" + repr(T_inf), "top:noslip:0.2:0:" + repr(1.1 * T_inf),
                   "left:outflow", "right:outflow"],
            "ref": [1.0, 0.2, 0.0, 1.0 / GAMMA, 2.0, 1.0, 0.5]}, tmp, 200)
        # Scalar diffusion on a Cartesian patch: Dirichlet + Neumann sides.
        cart = meshgen.cartesian(12, 10, 2.0, 1.5)
        cart.nodes -= np.array([1.0, 0.75])
        path = os.path.join(tmp, "cart.fvmesh")
        fvmesh.write_fvmesh(cart, path)
        out = os.path.join(tmp, "diff")
        os.makedirs(out)
        case = {"alpha": 0.3, "dt": 2e-3, "v0": 2.0, "r0": 0.5, "steps": 80,
                "bc": ["bottom:dirichlet:0.25", "right:neumann:-0.5", "top:dirichlet:1.0", "left:neumann:0.0"]}
        fvref("diff", path, out, alpha=case["alpha"], dt=case["dt"], v0=case["v0"], r0=case["r0"],
              steps=case["steps"], bc=case["bc"])
        np.savez_compressed(os.path.join(HERE, "diffusion_cart.npz"), **mesh_arrays(cart),
                            field=np.fromfile(os.path.join(out, "field.f64")),
                            hist=np.fromfile(os.path.join(out, "resid.f64")), case=np.array(json.dumps(case)))
    # Checkpoints written by the reference's Checkpoint::write.
    with tempfile.TemporaryDirectory() as tmp:
        rng = np.random.default_rng(7)
        U = rng.random((10, 4))
        phi = rng.random(7)
        U.tofile(os.path.join(tmp, "U.f64"))
        phi.tofile(os.path.join(tmp, "phi.f64"))
        exe = os.path.join(ROOT, "oracle", "_ref", "fvref")
        subprocess.run([exe, "ckpt", "op=write", f"path={os.path.join(HERE, 'ckpt_euler_ref.bin')}", "eq=1",
                        "step=1234", "build=42", f"in={os.path.join(tmp, 'U.f64')}", "cells=10"], check=True)
        subprocess.run([exe, "ckpt", "op=write", f"path={os.path.join(HERE, 'ckpt_diffusion_ref.bin')}", "eq=0",
                        "step=77", "build=9", f"in={os.path.join(tmp, 'phi.f64')}", "cells=7"], check=True)
        np.savez(os.path.join(HERE, "ckpt_payloads.npz"), euler=U, diffusion=phi)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
