#!/usr/bin/env python3
"""Benchmark of the explicit residual-and-update loop on one GB300.

Workload (the headline configuration): 2nd-order Euler on a ~1M-cell
mixed-polygon mesh -- a NACA0012 O-grid core of 1024 x 512 quads plus a
seeded, Lloyd-relaxed polygonal outer region to 20 chords -- with
least-squares gradients, the Venkatakrishnan limiter (K = 5), the HLLC
flux, SSP-RK3 at CFL 1.2 with local time stepping, slip wall and
characteristic farfield, M = 0.8, AoA = 1.25 deg, FP64.  One step = one
full iteration (three RK stages).  Synthetic, seeded inputs; nothing is
read from disk except the mesh cache this script itself writes.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  ``--impl reference`` times the CPU
restatement of the reference's loop (oracle/, extended to this scheme) on
the host cores instead; the reference itself has no 2nd-order path.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

GAMMA = 1.4
MACH, AOA_DEG, CFL, VENKAT_K = 0.8, 1.25, 1.2, 5.0
MESH_KW = dict(ni=1024, nj=512, first=1e-3, r_core=2.0, r_far=20.0, code="0012", lloyd_iters=4, seed=0)
METRIC = "Mcell-iters/s, 2nd-order HLLC Euler at 1M cells; batched/FP32/adjoint vs plain"
DATA = "synthetic (seeded NACA0012 mixed mesh; freestream + seeded smooth 1% perturbation start)"
# FP64-pipe thread instructions per second of one GB300 (152 SMs at 2070 MHz,
# a dependent-chain-free DFMA loop timed with CUDA events: 1.02 TFLOP/s).
FP64_PIPE_GINST_S = 510.0


def freestream():
    a = np.radians(AOA_DEG)
    return 1.0, MACH * np.cos(a), MACH * np.sin(a), 1.0 / GAMMA


def load_mesh():
    from finitevolume_gb300 import meshgen
    return meshgen.cached("naca_mixed", **MESH_KW)


def make_solver(poly, fp32=False):
    from finitevolume_gb300 import solvers as S
    r, u, v, p = freestream()
    mesh = S.Mesh(poly, reorder="morton")
    bcs = [S.EulerBoundaryCondition(S.EulerBoundaryType.Wall),
           S.EulerBoundaryCondition(S.EulerBoundaryType.CharacteristicFarfield, S.from_primitive(r, u, v, p, GAMMA))]
    ic = S.EulerInitialCondition(S.EulerICMode.Freestream, rho=r, u=u, v=v, p=p)
    s = S.EulerFVMSolver(mesh, bcs, GAMMA, CFL, ic, S.NumericalFluxScheme.HLLC, order=2, rk_stages=3,
                         local_dt=True, gradient=S.GradientScheme.LeastSquares, limiter=S.Limiter.Venkatakrishnan,
                         venkat_k=VENKAT_K, fp32_flux=fp32)
    s.set_field(initial_state(poly))
    return s, mesh


def initial_state(poly):
    """Freestream plus a seeded, smooth 1% perturbation (reference cell order).

    A uniform start leaves most gradients exactly zero for the first
    hundreds of iterations, which skips most of the limiter's work; the
    perturbation gives every cell the cost profile of a developed flow.
    """
    from finitevolume_gb300.fvmesh import cell_centroids
    cxy = cell_centroids(poly)
    rng = np.random.default_rng(1234)
    r, u, v, p = freestream()
    fields = []
    for _ in range(4):
        k = rng.uniform(0.5, 3.0, size=(3, 2))
        ph = rng.uniform(0, 2 * np.pi, size=3)
        fields.append(sum(np.sin(cxy @ k[i] + ph[i]) for i in range(3)) / 3.0)
    rho = r * (1.0 + 0.01 * fields[0])
    uu = u + 0.01 * MACH * fields[1]
    vv = v + 0.01 * MACH * fields[2]
    pp = p * (1.0 + 0.01 * fields[3])
    return np.ascontiguousarray(np.stack([rho, rho * uu, rho * vv, pp / (GAMMA - 1.0) + 0.5 * rho * (uu * uu + vv * vv)],
                                         1))


def port_solver(poly):
    """The oracle port (CPU FP64 restatement of the reference's loop, with
    this build's second-order extensions) configured for the headline
    scheme, starting from the benchmark's initial state."""
    from oracle import port
    r, u, v, p = freestream()
    st = [r, r * u, r * v, p / (GAMMA - 1.0) + 0.5 * r * (u * u + v * v)]
    e = port.OracleEuler(port.OracleMesh(poly), [(0, [0.0] * 4), (3, st)], gamma=GAMMA, cfl=CFL,
                         ic={"mode": "free", "rho": r, "u": u, "v": v, "p": p}, flux=1, order=2, rk=3, local_dt=True,
                         gradient=0, limiter=2, venkat_k=VENKAT_K)
    e.set_field(initial_state(poly))
    return e


def headline_config(n_cells: int, n_faces: int, world: int) -> dict:
    """The ``config`` block of the headline line, the same on both arms."""
    return {"workload": "naca0012_mixed_1M_o2_hllc_lsq_venkat_rk3", "cells": n_cells, "faces": n_faces,
            "mach": MACH, "aoa_deg": AOA_DEG, "cfl": CFL,
            "l2": "inputs larger than L2 (working set > 400 MB), no flush",
            "parallelism": f"replicas{world}" if world > 1 else "single"}


def force_ref():
    r, u, v, p = freestream()
    return (r, u, v, p, 1.0, 0.25, 0.0)


# --------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        except OSError:
            pass
        finally:
            if self.path and os.path.exists(self.path):
                os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# --------------------------------------------------------------------------
# Replicas (N GPUs, one independent solve each; the path has no exchange step)
def max_over_ranks(x: float, world: int, device: str) -> float:
    """The slowest rank's value (timed regions end at a barrier)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())


def replica_rate(n_cells: int, steps: int, max_ms: float, world: int) -> float:
    """Whole-job Mcell-iters/s: every rank advanced its own n_cells for
    ``steps`` iterations within the slowest rank's time."""
    return world * n_cells * steps / (max_ms / 1e3) / 1e6


# --------------------------------------------------------------------------
# Batched steady solves: 256 NACA 4-digit O-grids (camber 0-6%, thickness
# 8-18%, 4k-64k cells log-uniform), M 0.3-0.85, AoA -4..8 deg, 2nd-order
# HLLC + LSQ/Venkatakrishnan, SSP-RK3, local dt at CFL 1.2.
def batch_workload(n: int, seed: int = 0):
    from finitevolume_gb300 import meshgen, solvers as S
    cases = meshgen.batch_cases(n, seed)
    meshes = [S.Mesh(meshgen.naca_ogrid(c["ni"], c["nj"], shape=c["shape"]), reorder="morton") for c in cases]
    fss = []
    for c in cases:
        a = np.radians(c["aoa_deg"])
        fss.append((1.0, c["mach"] * np.cos(a), c["mach"] * np.sin(a), 1.0 / GAMMA))
    return cases, meshes, fss


def _plain_solver(mesh, fs, fp32):
    from finitevolume_gb300 import solvers as S
    bcs = [S.EulerBoundaryCondition(S.EulerBoundaryType.Wall),
           S.EulerBoundaryCondition(S.EulerBoundaryType.CharacteristicFarfield, S.from_primitive(*fs, GAMMA))]
    ic = S.EulerInitialCondition(S.EulerICMode.Freestream, rho=fs[0], u=fs[1], v=fs[2], p=fs[3])
    return S.EulerFVMSolver(mesh, bcs, GAMMA, CFL, ic, S.NumericalFluxScheme.HLLC, order=2, rk_stages=3,
                            local_dt=True, gradient=S.GradientScheme.LeastSquares, limiter=S.Limiter.Venkatakrishnan,
                            venkat_k=VENKAT_K, fp32_flux=fp32)


def _batch_solver(meshes, fss, fp32, tol=-1.0):
    from finitevolume_gb300 import solvers as S
    return S.BatchSolver(meshes, [S.EulerBoundaryType.Wall, S.EulerBoundaryType.CharacteristicFarfield], fss,
                         GAMMA, CFL, S.NumericalFluxScheme.HLLC, venkat_k=VENKAT_K, fp32_flux=fp32, tol=tol)


def batch_throughput(meshes, fss, fp32: bool, iters: int):
    """Fixed-iteration rate of the batch vs the same instances one by one.

    Returns (batched Mcell-iters/s, sequential Mcell-iters/s); both timed
    on the host around direct solver calls ending in a device sync.
    """
    import torch
    from finitevolume_gb300 import capi
    cells = sum(m.n_cells for m in meshes)
    b = _batch_solver(meshes, fss, fp32)
    b.autotune(steps=2, cache=False)
    b.run(3)
    b.status()
    t0 = time.perf_counter()
    b.run(iters)
    b.status()
    tb = time.perf_counter() - t0
    del b
    ts = 0.0
    for m, fs in zip(meshes, fss):
        s = _plain_solver(m, fs, fp32)
        try:
            s.run(3)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s.run(iters)  # fv_step returns after its stream has drained
        except capi.FVError:  # a diverged instance: timed up to the raise
            pass
        ts += time.perf_counter() - t0
        del s
    return cells * iters / tb / 1e6, cells * iters / ts / 1e6


def batch_converged_newton(meshes, fss, tol: float = 1e-8, warm: int = 200, max_newton: int = 80,
                           n_seq: int = 12, seed: int = 1, cd_tol: float = 1e-5, fp32_max_iter: int = 3000,
                           fp32_chunk: int = 250, round_steps: int = 20) -> dict:
    """Converged steady solves per second of a batch of the steady family,
    every solve to its own L2 density residual below ``tol`` within
    ``max_newton`` Newton steps (the same cap for every path).

    The steady solver: ``warm`` SSP-RK3 iterations, the limiter frozen at
    the state they reach, then Newton-Krylov on the frozen-limiter residual
    (the explicit iteration alone limit-cycles on the transonic half).
    - FP64 batched: all instances in one batch, one block-diagonal Newton
      solve with per-instance CFL numbers and early exit, in rounds of
      ``round_steps`` Newton steps after which the unconverged instances
      are repacked into a smaller batch.
    - sequential: the same procedure, one plain solver per instance, for a
      seeded sample of ``n_seq`` instances, each timed in full to
      convergence; solves/s over that sample.  Twice: with the Newton
      preconditioner in FP64 (the plain FP64 GPU path) and with its blocks
      in FP32 (mixed precision, the default; the residual, the
      Jacobian-vector products and the solution stay FP64).
    - FP32-flux batched (mixed precision; FP32 flux and gradients, FP64
      accumulation, update and norms): the same warm-up, then explicit
      SSP-RK3 with agglomeration multigrid; an instance counts
      as converged once |CD - CD_fp64| <= ``cd_tol`` against its converged
      FP64 drag at two consecutive checkpoints (every ``fp32_chunk``
      iterations) and is then frozen; at most ``fp32_max_iter`` iterations.
      Its limiter is frozen at the FP64 batch's values, so both precisions
      solve the same discrete scheme.
    All wall times are host-side around the solver calls, ending in a
    device synchronisation.
    """
    import torch
    from finitevolume_gb300 import capi
    n = len(meshes)
    refs = [(fs[0], fs[1], fs[2], fs[3], 1.0, 0.25, 0.0) for fs in fss]
    out = {"instances": n, "tol_l2_density": tol, "warm_rk3_iterations": warm,
           "cells_total": int(sum(m.n_cells for m in meshes))}
    # FP64 batched, in rounds: after each round the instances still
    # unconverged are repacked into a smaller batch (their states and frozen
    # limiter values carried over), so the shared Newton steps stop paying
    # for instances that are done.
    b = _batch_solver(meshes, fss, False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b.run(warm)
    b.freeze_limiter(True)
    psi64 = np.concatenate([b.limiter_values(i) for i in range(n)], 0)
    off = np.cumsum([0] + [m.n_cells for m in meshes])
    steps = np.full(n, -1, np.int64)
    cd64 = np.full(n, np.nan)
    live = np.arange(n)
    done_steps, rounds = 0, []
    while live.size and done_steps < max_newton:
        k = min(round_steps, max_newton - done_steps)
        # later rounds restart the CFL ramp higher (the controller halves it
        # again where that is too much)
        _, it = b.newton(max_newton=k, tol=tol, **({} if not rounds else {"cfl0": 200.0}))
        st = b.last_newton_instance_steps.copy()
        fld = b.field_all()
        loff = np.cumsum([0] + [meshes[i].n_cells for i in live])
        for j, i in enumerate(live):
            if st[j] >= 0:
                steps[i] = done_steps + st[j]
                cd64[i] = b.wall_forces(j, *refs[i])["cd_total"]
        rounds.append({"instances": int(live.size), "newton_steps": int(it), "converged": int((st >= 0).sum())})
        done_steps += k
        keep = st < 0
        if not keep.any() or done_steps >= max_newton:
            break
        nxt = live[keep]
        U = np.concatenate([fld[loff[j]:loff[j + 1]] for j in np.nonzero(keep)[0]], 0)
        P = np.concatenate([psi64[off[i]:off[i + 1]] for i in nxt], 0)
        del b
        b = _batch_solver([meshes[i] for i in nxt], [fss[i] for i in nxt], False)
        b.set_field(U)
        b.set_limiter_values(P)
        live = nxt
    del b
    torch.cuda.synchronize()
    tb = time.perf_counter() - t0
    conv = steps >= 0
    out["f64_batched"] = {"solves_per_s": round(int(conv.sum()) / tb, 4), "seconds": round(tb, 2),
                          "converged": int(conv.sum()), "rounds": rounds, "preconditioner": "FP32 blocks",
                          "instance_newton_steps_median": float(np.median(steps[conv])) if conv.any() else None}
    # plain solver per instance, seeded sample, each solve timed in full:
    # all-FP64 (FP64 preconditioner, the plain FP64 GPU path) and mixed
    # (FP32 preconditioner blocks, the default; the same FP64 residual,
    # Jacobian-vector products and converged solution)
    rng = np.random.default_rng(seed)
    sample = np.sort(rng.choice(n, size=min(n_seq, n), replace=False))
    for tag, kind in (("f64_sequential", 1), ("mixed_sequential", 2)):
        ts, nconv, dcd = 0.0, 0, []
        for i in sample:
            s = _plain_solver(meshes[i], fss[i], False)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ok = False
            try:
                s.run(warm)
                s.freeze_limiter(True)
                s.newton(max_newton=max_newton, tol=tol, precond_kind=kind)
                ok = bool(s.last_newton_instance_steps[0] >= 0)
            except capi.FVError:
                pass
            torch.cuda.synchronize()
            ts += time.perf_counter() - t0
            if ok:
                nconv += 1
                if conv[i]:
                    dcd.append(abs(s.wall_forces(*refs[i])["cd_total"] - cd64[i]))
            del s
        out[tag] = {"solves_per_s": round(nconv / ts, 4), "seconds": round(ts, 2), "converged": nconv,
                    "preconditioner": "FP64 blocks" if kind == 1 else "FP32 blocks",
                    "sample": [int(i) for i in sample],
                    "max_abs_dCD_vs_batched": float(max(dcd)) if dcd else None}
    base = max(out["f64_sequential"]["solves_per_s"], 1e-30)
    out["f64_batched"]["speedup_vs_f64_sequential"] = round(out["f64_batched"]["solves_per_s"] / base, 2)
    out["mixed_sequential"]["speedup_vs_f64_sequential"] = round(out["mixed_sequential"]["solves_per_s"] / base, 2)
    # FP32-flux batched, drag criterion against the converged FP64 drag
    b = _batch_solver(meshes, fss, True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b.run(warm)
    b.set_limiter_values(psi64)  # the same frozen-limiter scheme as the FP64 solves
    b.multigrid()
    hits = np.zeros(n, np.int64)
    conv32 = np.zeros(n, bool)
    done = warm
    while done < fp32_max_iter:
        b.run(fp32_chunk)
        done += fp32_chunk
        for i in np.nonzero(conv & ~conv32)[0]:
            cd = b.wall_forces(int(i), *refs[i])["cd_total"]
            hits[i] = hits[i] + 1 if abs(cd - cd64[i]) <= cd_tol else 0
            if hits[i] >= 2:
                conv32[i] = True
                b.set_active(int(i), False)
        if conv32[conv].all():
            break
    torch.cuda.synchronize()
    t32 = time.perf_counter() - t0
    del b
    out["fp32_flux_batched"] = {"solves_per_s": round(int(conv32.sum()) / t32, 4), "seconds": round(t32, 2),
                                "converged": int(conv32.sum()), "iterations": int(done),
                                "criterion": f"|CD - CD_fp64| <= {cd_tol} at two consecutive checkpoints",
                                "solver": "explicit SSP-RK3 + 4-level agglomeration multigrid, frozen limiter"}
    out["fp32_flux_batched"]["speedup_vs_f64_sequential"] = round(out["fp32_flux_batched"]["solves_per_s"] / base, 2)
    return out


def adjoint_cost(iters: int = 200, warm: int = 300):
    """Discrete adjoint against the primal on the 500k-cell NACA0012 O-grid
    (1024 x 488), M 0.75, AoA 2 deg, 2nd-order HLLC + LSQ/Venkatakrishnan,
    SSP-RK3 at CFL 1.2: wall time per primal iteration, per adjoint
    iteration (frozen and full limiter) and of the linearisation.  The
    adjoint iteration is the transposed linearised primal iteration, so it
    converges at the primal's asymptotic rate and the cost of a converged
    adjoint relative to a converged primal is the ratio at equal iteration
    counts."""
    import torch
    from finitevolume_gb300 import meshgen, solvers as S
    M, aoa = 0.75, 2.0
    a = np.radians(aoa)
    fs = (1.0, M * np.cos(a), M * np.sin(a), 1.0 / GAMMA)
    mesh = S.Mesh(meshgen.cached("naca_ogrid", ni=1024, nj=488), reorder="morton")
    s = _plain_solver(mesh, fs, False)
    s.run(warm)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s.run(iters)
    tp = (time.perf_counter() - t0) / iters
    ref = np.array([1.0, fs[1], fs[2], fs[3], 1.0, 0.25, 0.0])
    out = {"workload": "naca0012 O-grid 1024x488, M 0.75, AoA 2, 2nd-order HLLC, Venkatakrishnan K=5",
           "cells": mesh.n_cells, "primal_ms_per_iter": round(tp * 1e3, 4), "iterations_timed": iters}
    for full in (False, True):
        adj = S.DiscreteAdjoint(s, full_limiter=full)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        adj.forward()
        tl = time.perf_counter() - t0
        _, g = S.force_gradient(s, S.Objective.Drag, ref)
        adj.solve(g, 3, 0.0)  # warm-up
        t0 = time.perf_counter()
        adj.solve(g, iters, 0.0)
        ta = (time.perf_counter() - t0) / iters
        key = "full_limiter" if full else "frozen_limiter"
        out[key] = {"adjoint_ms_per_iter": round(ta * 1e3, 4), "linearise_ms": round(tl * 1e3, 2),
                    "cost_vs_primal_per_iter": round(ta / tp, 3),
                    "cost_vs_primal_1000_iters": round((tl + 1000 * ta) / (1000 * tp), 3)}
        del adj
    # Converged: the primal to 1e-11 (SSP-RK3 warm-up from this state on,
    # limiter frozen, Newton-Krylov), then the frozen-limiter drag adjoint
    # to a relative residual of 1e-10 by pseudo-transient iterations on the
    # transposed Newton system; wall times from the start of the primal.
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s2 = _plain_solver(mesh, fs, False)
    s2.run(warm)
    s2.freeze_limiter()
    hp, kp = s2.newton(max_newton=400, tol=1e-11)
    torch.cuda.synchronize()
    tprim = time.perf_counter() - t0
    adj = S.DiscreteAdjoint(s2, full_limiter=False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    gd = adj.freestream_gradient(S.Objective.Drag, M, aoa, [1], max_iter=40000, tol=1e-10, method="krylov")
    torch.cuda.synchronize()
    tadj = time.perf_counter() - t0
    out["converged"] = {"primal_seconds": round(tprim, 2), "primal_residual": float(hp[-1, 0]),
                        "primal_newton_steps": int(kp), "primal_warm_rk3_iterations": warm,
                        "adjoint_seconds": round(tadj, 2), "adjoint_matvecs": gd["iterations"],
                        "adjoint_residual": gd["adjoint_residual"], "dCD_dM": gd["dJ_dM"],
                        "adjoint_vs_converged_primal": round(tadj / tprim, 3)}
    del adj, s2, s
    return out


def adjoint_check(n_dirs: int = 16, h: float = 1e-6, h_small: float = 1e-8, tol: float = 1e-11, warm: int = 300,
                  max_newton: int = 600,
                  fd_tol: float = 1e-13, fd_max_newton: int = 200, sweeps: int = 8, adj_cfl: float = 3e3,
                  adj_tol: float = 1e-10, adj_max_matvec: int = 40000):
    """Gradients of the 500k-cell NACA0012 O-grid case (1024 x 488, M 0.75,
    AoA 2 deg, 2nd-order HLLC + LSQ/Venkatakrishnan K=5, local dt) from the
    discrete adjoint against central differences of converged primal
    solves: dCD/dM, dCD/dAoA, and dCL/dX along ``n_dirs`` seeded
    wall-normal displacement fields smoothed over 20 wall nodes, at the
    configured step h and at ``h_small``.

    Primal: ``warm`` SSP-RK3 iterations, the limiter frozen there (the
    live limiter limit-cycles near 1e-3 on this transonic case), then
    Newton-Krylov on the frozen-limiter residual to ``tol``.  The
    differences are converged the same way from the base state, to
    ``fd_tol``, with the limiter frozen at the same values, so the
    frozen-limiter adjoint is the exact linearisation of what they
    difference; the full-limiter adjoint differs by the limiter's own
    sensitivity.  Adjoint solves: pseudo-transient iterations on the
    transposed Newton system at CFL ``adj_cfl`` to a relative residual of
    ``adj_tol``.  Reported: relative errors, and the adjoint wall time
    (drag + lift adjoints and the shape gradient) as a multiple of the
    converged primal solve's."""
    import torch
    from finitevolume_gb300 import capi, meshgen, solvers as S
    M, aoa = 0.75, 2.0

    def fs_of(m, al):
        a = np.radians(al)
        return (1.0, m * np.cos(a), m * np.sin(a), 1.0 / GAMMA)

    def ref_of(m, al):
        return np.array([*fs_of(m, al), 1.0, 0.25, 0.0])

    def log(d):
        print(json.dumps(d), file=sys.stderr, flush=True)

    poly = meshgen.cached("naca_ogrid", ni=1024, nj=488)
    mesh = S.Mesh(poly, reorder="morton")
    fs = fs_of(M, aoa)
    out = {"workload": "naca0012 O-grid 1024x488, M 0.75, AoA 2, 2nd-order HLLC, LSQ + Venkatakrishnan K=5, "
                       "local dt; primal: SSP-RK3 warm-up, limiter frozen, Newton-Krylov",
           "cells": mesh.n_cells, "tol_l2_density": tol, "h_shape": h, "directions": n_dirs}
    s = _plain_solver(mesh, fs, False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s.run(warm)
    s.freeze_limiter()
    hp, kp = s.newton(max_newton=max_newton, tol=tol, precond_sweeps=sweeps)
    torch.cuda.synchronize()
    tprimal = time.perf_counter() - t0
    psi = s.limiter_values()
    out["primal"] = {"warm_iterations": warm, "newton_steps": kp, "residual": float(hp[-1, 0]),
                     "seconds": round(tprimal, 2), "cells_limited": int((psi < 1.0).any(axis=1).sum())}
    log({"primal": out["primal"]})
    U0 = s.field()
    f0 = s.wall_forces(*ref_of(M, aoa))
    out["cl"], out["cd"] = f0["cl"], f0["cd_total"]

    dirs = meshgen.wall_normal_directions(poly, n_dirs, seed=0, width=20)
    for full in (False, True):
        key = "full_limiter" if full else "frozen_limiter"
        adj = S.DiscreteAdjoint(s, full_limiter=full)
        adj.krylov_cfl, adj.krylov_sweeps = adj_cfl, sweeps
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        try:
            # the full-limiter system is not the linearisation of the frozen
            # scheme the primal converged; it gets a smaller product budget
            mv = adj_max_matvec if not full else adj_max_matvec // 5
            gd = adj.freestream_gradient(S.Objective.Drag, M, aoa, [1], max_iter=mv, tol=adj_tol, method="krylov")
            _, g = S.force_gradient(s, S.Objective.Lift, ref_of(M, aoa))
            _, _, hist, it = adj.solve(g, mv, adj_tol, method="krylov")
            gl = adj.shape_gradient(S.Objective.Lift, ref_of(M, aoa))
        except capi.FVError as e:
            out[key] = {"error": str(e)}
            log({key: out[key]})
            del adj
            continue
        torch.cuda.synchronize()
        ta = time.perf_counter() - t0
        out[key] = {
            "dCD_dM": gd["dJ_dM"], "dCD_dAoA_deg": gd["dJ_dAoA_deg"], "drag_matvecs": gd["iterations"],
            "drag_adjoint_residual": gd["adjoint_residual"], "lift_matvecs": it,
            "lift_adjoint_rel_residual": float(hist[-1]) if len(hist) else None,
            "dCL_dX_dirs": [float(np.sum(gl * d)) for d in dirs], "seconds": round(ta, 2),
            "seconds_vs_primal": round(ta / tprimal, 3)}
        log({key: out[key]})
        del adj

    def frozen_solve(sp):
        sp.set_field(U0)
        hh, k = sp.newton(max_newton=fd_max_newton, tol=fd_tol, precond_sweeps=sweeps)
        return k, float(hh[-1, 0])

    # central differences, limiter frozen at psi: freestream
    hM, ha = 1e-6, 1e-5
    fd = {}
    for key, (m, al) in {"M+": (M + hM, aoa), "M-": (M - hM, aoa), "a+": (M, aoa + ha), "a-": (M, aoa - ha)}.items():
        sp = _plain_solver(mesh, fs_of(m, al), False)
        sp.set_limiter_values(psi)
        c, r = frozen_solve(sp)
        fd[key] = (sp.wall_forces(*ref_of(m, al))["cd_total"], c, r)
        del sp
    out["fd_freestream"] = {"dCD_dM": (fd["M+"][0] - fd["M-"][0]) / (2 * hM),
                            "dCD_dAoA_deg": (fd["a+"][0] - fd["a-"][0]) / (2 * ha),
                            "h_M": hM, "h_aoa_deg": ha,
                            "newton_steps": [fd[k][1] for k in fd], "residuals": [fd[k][2] for k in fd]}
    log({"fd_freestream": out["fd_freestream"]})
    # shape (one solver, geometry moved on the device), at the configured
    # step h and at h_small: the differenced solves cross the kinks of the
    # discrete scheme (wave-branch switches at sonic faces), so the central
    # difference approaches the derivative only as h shrinks
    sp = _plain_solver(mesh, fs, False)
    sp.set_limiter_values(psi)
    X = poly.nodes.copy()
    fd_by_h = {}
    for hh in (h, h_small):
        fd_cl, steps, resids = [], [], []
        for d in dirs:
            v = {}
            for sgn in (1, -1):
                sp.update_nodes(X + sgn * hh * d)
                c, r = frozen_solve(sp)
                steps.append(c)
                resids.append(r)
                v[sgn] = sp.wall_forces(*ref_of(M, aoa))["cl"]
            fd_cl.append((v[1] - v[-1]) / (2 * hh))
        fd_by_h[hh] = fd_cl
        out[f"fd_shape_h{hh:g}"] = {"h": hh, "dCL_dX_dirs": fd_cl, "newton_steps_median": float(np.median(steps)),
                                    "residual_max": float(np.max(resids))}
        log({f"fd_shape_h{hh:g}": out[f"fd_shape_h{hh:g}"]})
    sp.update_nodes(X)
    for key in ("frozen_limiter", "full_limiter"):
        o = out[key]
        if "error" in o:
            continue
        ad = np.array(o["dCL_dX_dirs"])
        for hh, fd_cl in fd_by_h.items():
            fdv = np.array(fd_cl)
            rel = np.abs(ad - fdv) / np.maximum(np.abs(fdv), 1e-3)
            o[f"shape_rel_err_max_h{hh:g}"] = float(rel.max())
            o[f"shape_rel_err_median_h{hh:g}"] = float(np.median(rel))
        o["dCD_dM_rel_err"] = abs(o["dCD_dM"] - out["fd_freestream"]["dCD_dM"]) / abs(out["fd_freestream"]["dCD_dM"])
        o["dCD_dAoA_rel_err"] = (abs(o["dCD_dAoA_deg"] - out["fd_freestream"]["dCD_dAoA_deg"]) /
                                 abs(out["fd_freestream"]["dCD_dAoA_deg"]))
    return out


def rans_sa_rate(steps: int = 20, warm: int = 3, cpu: bool = True):
    """RANS with the Spalart-Allmaras model on the ~2M-cell NACA4412 hybrid
    mesh (40 wall-clustered quad layers, y+ ~ 1 at Re_c 6e6, growth 1.15,
    seeded random triangles to 30 chords): M 0.15, AoA 4 deg, Re_c 6e6,
    Pr 0.72, Pr_t 0.9, freestream nu-tilde = 3 nu, HLLC with Green-Gauss
    viscous gradients, the reference's forward-Euler global-dt scheme.
    With ``cpu``: the oracle's restatement of RANSTurbulenceSASolver runs
    the same warm + steps iterations from the same start on all host
    threads (the CPU baseline, timed over the steps after the warm-up) and
    its field and nu-tilde are compared with the GPU's (parity)."""
    import torch
    from finitevolume_gb300 import meshgen, solvers as S
    M, aoa, Re = 0.15, 4.0, 6e6
    a = np.radians(aoa)
    rho, u, v, p = 1.0, M * np.cos(a), M * np.sin(a), 1.0 / GAMMA
    mu = rho * M * 1.0 / Re
    R = 287.0
    mesh = S.Mesh(meshgen.cached("naca_hybrid"), reorder="morton")
    far = S.NSBoundaryCondition(S.NSBoundaryType.Farfield, farfield_state=list(S.from_primitive(rho, u, v, p, GAMMA)))
    bcs = [S.RANSBoundaryConditionSA(S.NSBoundaryCondition(S.NSBoundaryType.NoSlipWall)),
           S.RANSBoundaryConditionSA(far, 3.0 * mu / rho)]
    ic = S.EulerInitialCondition(S.EulerICMode.Freestream, rho=rho, u=u, v=v, p=p)
    s = S.RANSTurbulenceSASolver(mesh, bcs, GAMMA, R, mu, 0.72, 0.9, 0.5, ic, 3.0 * mu / rho,
                                 S.NumericalFluxScheme.HLLC, S.GradientScheme.GreenGauss)
    s.run(warm)
    torch.cuda.synchronize()
    ms, launches = s.step_timed(steps)
    t = float(np.sum(ms))
    out = {"workload": "naca4412 hybrid, 40 quad layers + random triangles, M 0.15, AoA 4, Re 6e6, SA-noft2",
           "cells": mesh.n_cells, "faces": mesh.n_faces, "value": round(mesh.n_cells * steps / (t / 1e3) / 1e6, 3),
           "unit": "Mcell-iters/s", "ms_per_step": round(t / steps, 4), "steps": steps,
           "nut_residual": s.nut_residual()}
    if cpu:
        from oracle import port
        poly = mesh.poly
        om = port.OracleMesh(poly)
        st = tuple(S.from_primitive(rho, u, v, p, GAMMA))
        bcs = [{"type": "noslip"}, {"type": "farfield", "state": st, "nut": 3.0 * mu / rho}]
        o = port.OracleRANS(om, bcs, GAMMA, R, mu, 0.72, 0.9, 0.5, {"rho": rho, "u": u, "v": v, "p": p},
                            3.0 * mu / rho, flux=1, gradient=1)
        o.run(warm)
        t0 = time.perf_counter()
        o.run(steps)
        tc = time.perf_counter() - t0
        f_cpu, nut_cpu, _ = o.get()
        del o, om
        out["cpu_baseline"] = {"value": round(mesh.n_cells * steps / tc / 1e6, 3), "unit": "Mcell-iters/s",
                               "cores": port.num_threads(), "kind": "port",
                               "sample": f"{steps} RANSTurbulenceSASolver steps (after {warm} warm-up) of the "
                                         f"oracle restatement on the full mesh, OpenMP over {port.num_threads()} "
                                         f"threads ({tc:.1f} s)"}
        fg, ng = s.field(), s.nut_field()
        out["parity"] = {"against": "oracle port (CPU FP64 RANSTurbulenceSASolver restatement), same start state",
                         "iterations": warm + steps, "tolerance": 1e-10,
                         "max_rel_field_err": float(np.max(np.abs(fg - f_cpu)) / np.max(np.abs(f_cpu))),
                         "max_rel_nut_err": float(np.max(np.abs(ng - nut_cpu)) / np.max(np.abs(nut_cpu)))}
    return out


def sod_layout(nx: int = 1000, ny: int = 500, steps: int = 50):
    """Sod shock tube (rho 1/0.125, p 1/0.1) on a 1M-cell randomly perturbed
    triangle strip, 2nd-order HLLC + LSQ/Venkatakrishnan, SSP-RK3, global
    dt: the fields after ``steps`` steps in identity, Morton and RCM cell
    order must be bit-identical; also the Morton run's rate."""
    from finitevolume_gb300 import meshgen, solvers as S
    poly = meshgen.sod_strip(nx, ny, seed=0)
    out = {"workload": f"sod strip {nx}x{ny}x2 triangles, 2nd-order HLLC, SSP-RK3, global dt",
           "cells": int(poly.n_cells), "steps": steps}
    fields = {}
    for reorder in ("none", "morton", "rcm"):
        mesh = S.Mesh(poly, reorder=reorder)
        bcs = [S.EulerBoundaryCondition(S.EulerBoundaryType.Wall),
               S.EulerBoundaryCondition(S.EulerBoundaryType.Outflow),
               S.EulerBoundaryCondition(S.EulerBoundaryType.Wall),
               S.EulerBoundaryCondition(S.EulerBoundaryType.Outflow)]
        ic = S.EulerInitialCondition(S.EulerICMode.TwoRegion, rho_l=1.0, u_l=0.0, v_l=0.0, p_l=1.0, rho_r=0.125,
                                     u_r=0.0, v_r=0.0, p_r=0.1, x0=0.5)
        sv = S.EulerFVMSolver(mesh, bcs, GAMMA, 0.5, ic, S.NumericalFluxScheme.HLLC, order=2, rk_stages=3,
                              local_dt=False)
        ms, _ = sv.step_timed(steps)
        fields[reorder] = sv.field()
        out[f"{reorder}_Mcell_iters_s"] = round(poly.n_cells * steps / (float(np.sum(ms)) / 1e3) / 1e6, 3)
        del sv
    out["bitwise_identical"] = bool(np.array_equal(fields["none"], fields["morton"]) and
                                    np.array_equal(fields["none"], fields["rcm"]))
    return out


def config1_rate(steps: int = 3000):
    """The reference's own scheme at small scale: NACA0012 O-grid 256 x 128
    (32,768 cells, first spacing 1e-3, farfield at 20 chords), first-order
    Rusanov, forward Euler with local time stepping at CFL 0.5, slip wall
    and characteristic farfield, M 0.5, AoA 2 deg, 3,000 iterations; CL, CD
    and the final density residual.  Timed (wall clock around fv_step, after
    an untimed run that builds the graphs) in three forms: the dataflow form
    of the persistent kernel (the default with local dt), its grid-barrier
    form and the two-kernel path."""
    import torch
    from finitevolume_gb300 import meshgen, solvers as S
    M, aoa = 0.5, 2.0
    a = np.radians(aoa)
    fs = (1.0, M * np.cos(a), M * np.sin(a), 1.0 / GAMMA)
    mesh = S.Mesh(meshgen.naca_ogrid(256, 128), reorder="morton")
    bcs = [S.EulerBoundaryCondition(S.EulerBoundaryType.Wall),
           S.EulerBoundaryCondition(S.EulerBoundaryType.CharacteristicFarfield, S.from_primitive(*fs, GAMMA))]
    ic = S.EulerInitialCondition(S.EulerICMode.Freestream, rho=fs[0], u=fs[1], v=fs[2], p=fs[3])

    def timed(persistent):
        s = S.EulerFVMSolver(mesh, bcs, GAMMA, 0.5, ic, S.NumericalFluxScheme.Rusanov, local_dt=True)
        s.set_persistent(persistent)
        U0 = s.field()
        s.run(steps, history=True)  # graphs and history ring built here
        s.set_field(U0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        h = s.run(steps, history=True)
        return s, h, time.perf_counter() - t0

    s, h, t = timed(True)
    _, h3, t3 = timed("barrier")
    _, h2, t2 = timed(False)
    f = s.wall_forces(fs[0], fs[1], fs[2], fs[3], 1.0, 0.25, 0.0)
    form = {0: "two-kernel", 1: "grid-barrier", 2: "dataflow"}
    out = {"workload": "naca0012 O-grid 256x128, 1st-order Rusanov, forward Euler, local dt, CFL 0.5, M 0.5, AoA 2",
           "cells": mesh.n_cells, "steps": steps, "seconds": round(t, 4),
           "value": round(mesh.n_cells * steps / t / 1e6, 3),
           "unit": "Mcell-iters/s (wall clock around fv_step, persistent kernel)",
           "persistent_form": form[s.persistent()[0]],
           "persistent_grid_blocks": s.persistent()[1],
           "grid_barrier_form": {"seconds": round(t3, 4), "value": round(mesh.n_cells * steps / t3 / 1e6, 3),
                                 "history_equal": bool(np.array_equal(h, h3))},
           "two_kernel_path": {"seconds": round(t2, 4), "value": round(mesh.n_cells * steps / t2 / 1e6, 3)},
           "speedup_vs_two_kernel": round(t2 / t, 3),
           "history_equal_two_kernel_rtol": float(np.max(np.abs(h - h2) / np.abs(h2))),
           "cl": f["cl"], "cd": f["cd_total"], "residual_rho_first": float(h[0, 0]),
           "residual_rho_last": float(h[-1, 0])}
    try:
        out["cpu_baseline"] = config1_cpu_rate(steps)
    except Exception as e:  # an auxiliary figure never breaks the bench line
        out["cpu_baseline"] = {"error": str(e)[:200]}
    return out


def config1_cpu_rate(steps: int = 3000, seconds: float = 3.0) -> dict:
    """The same first-order case on the host cores: the oracle port (the
    reference's first-order loop, here with local time stepping and the
    characteristic farfield), OpenMP over all threads, a bounded sample of
    the iterations."""
    from finitevolume_gb300 import meshgen
    from oracle import port
    M, aoa = 0.5, 2.0
    a = np.radians(aoa)
    r, u, v, p = 1.0, M * np.cos(a), M * np.sin(a), 1.0 / GAMMA
    st = [r, r * u, r * v, p / (GAMMA - 1.0) + 0.5 * r * (u * u + v * v)]
    om = port.OracleMesh(meshgen.naca_ogrid(256, 128))
    e = port.OracleEuler(om, [(0, [0.0] * 4), (3, st)], gamma=GAMMA, cfl=0.5,
                         ic={"mode": "free", "rho": r, "u": u, "v": v, "p": p}, flux=0, order=1, rk=1,
                         local_dt=True)
    t0 = time.perf_counter()
    e.run(10)
    per = (time.perf_counter() - t0) / 10
    n = max(10, min(steps, int(seconds / max(per, 1e-6))))
    t0 = time.perf_counter()
    e.run(n)
    dt = time.perf_counter() - t0
    return {"value": round(om.n_cells * n / dt / 1e6, 3), "unit": "Mcell-iters/s", "cores": port.num_threads(),
            "kind": "port", "sample": f"{n} of the {steps} iterations after 10 warm-up ({dt:.2f} s)"}


def profile_target(target: str, steps: int) -> dict:
    """Profiler targets beside the headline: the adjoint iteration on the
    500k-cell O-grid, the RANS-SA step on the 2M-cell hybrid mesh, config 1
    (``steps`` calls of 100 persistent first-order steps on the 32k O-grid)
    and a multigrid V-cycle on the 1M-cell mixed mesh (direct launches)."""
    import torch
    from finitevolume_gb300 import meshgen, solvers as S
    t0 = time.perf_counter()
    if target == "adjoint":
        M, aoa = 0.75, 2.0
        a = np.radians(aoa)
        fs = (1.0, M * np.cos(a), M * np.sin(a), 1.0 / GAMMA)
        mesh = S.Mesh(meshgen.cached("naca_ogrid", ni=1024, nj=488), reorder="morton")
        s = _plain_solver(mesh, fs, False)
        s.run(20)
        adj = S.DiscreteAdjoint(s)
        adj.forward()
        _, g = S.force_gradient(s, S.Objective.Drag, np.array([1.0, fs[1], fs[2], fs[3], 1.0, 0.25, 0.0]))
        adj.solve(g, steps, 0.0)
    elif target == "rans":
        rans_sa_rate(steps=steps, warm=1, cpu=False)
    elif target == "config1":
        # the 32k O-grid, first-order Rusanov, local dt: one persistent
        # launch per fv_step of up to 256 steps
        M, aoa = 0.5, 2.0
        a = np.radians(aoa)
        fs = (1.0, M * np.cos(a), M * np.sin(a), 1.0 / GAMMA)
        mesh = S.Mesh(meshgen.naca_ogrid(256, 128), reorder="morton")
        bcs = [S.EulerBoundaryCondition(S.EulerBoundaryType.Wall),
               S.EulerBoundaryCondition(S.EulerBoundaryType.CharacteristicFarfield, S.from_primitive(*fs, GAMMA))]
        ic = S.EulerInitialCondition(S.EulerICMode.Freestream, rho=fs[0], u=fs[1], v=fs[2], p=fs[3])
        s = S.EulerFVMSolver(mesh, bcs, GAMMA, 0.5, ic, S.NumericalFluxScheme.Rusanov, local_dt=True)
        for _ in range(steps):
            s.run(100)
    else:
        poly = load_mesh()
        s, _ = make_solver(poly)
        s.multigrid()
        s.run(steps)
    torch.cuda.synchronize()
    return {"steps": steps, "seconds": round(time.perf_counter() - t0, 3)}


def run_batched(args):
    """--batched: converged solves/s of the whole 256-instance family
    (batch_converged_newton over every instance, a 24-instance sequential
    sample, FP64 and mixed-precision preconditioners)."""
    import torch
    torch.cuda.init()
    _, meshes, fss = batch_workload(args.instances)
    out = {"metric": "converged steady solves/s, 256-instance batched Euler (per-instance early exit)",
           "unit": "solves/s", "higher_is_better": True, "n_gpus": 1, "data": "synthetic (seeded NACA family)",
           "config": {"workload": "naca4_family_ogrid_batch", "instances": len(meshes),
                      "cells_total": int(sum(m.n_cells for m in meshes)), "tol_l2_density": args.tol,
                      "max_newton": args.max_newton, "cfl": CFL}}
    out["results"] = batch_converged_newton(meshes, fss, tol=args.tol, max_newton=args.max_newton, n_seq=24)
    print(json.dumps(out), flush=True)


# --------------------------------------------------------------------------
def cpu_port_rate(poly, max_seconds: float, threads: int = 0, keep: dict = None):
    """Time the oracle port (CPU restatement, OpenMP) on the same workload,
    from the benchmark's start state.  ``keep`` (a dict) receives the
    port's field and the number of iterations it took."""
    from oracle import port
    if threads:
        port.set_threads(threads)
    e = port_solver(poly)
    t0 = time.perf_counter()
    e.run(1)  # warm-up iteration (page faults, thread start-up)
    first = time.perf_counter() - t0
    n = max(1, min(200, int(max_seconds / max(first, 1e-3))))
    t0 = time.perf_counter()
    e.run(n)
    dt = time.perf_counter() - t0
    if keep is not None:
        keep["field"], keep["iterations"] = e.field(), n + 1
    return e.n_cells * n / dt / 1e6, n, dt, port.num_threads()


def cpu_baseline_block(poly, seconds: float, seconds_1t: float, keep: dict = None) -> dict:
    """The bench line's cpu_baseline: the oracle port on all host threads,
    plus a single-thread sample of the same scheme on the same mesh."""
    from oracle import port
    all_threads = port.num_threads()
    v, n, dt, cores = cpu_port_rate(poly, seconds, keep=keep)
    out = {"value": round(v, 3), "unit": "Mcell-iters/s", "cores": cores, "kind": "port",
           "sample": f"{n} SSP-RK3 iterations of the same 2nd-order HLLC scheme on the full mesh, "
                     f"OpenMP over {cores} threads ({dt:.1f} s)"}
    if seconds_1t > 0:
        try:
            v1, n1, dt1, _ = cpu_port_rate(poly, seconds_1t, threads=1)
        finally:
            port.set_threads(all_threads)
        out["single_thread"] = {"value": round(v1, 3), "unit": "Mcell-iters/s", "cores": 1,
                                "sample": f"{n1} iterations on one thread ({dt1:.1f} s)"}
    return out


def run_reference(args, rank):
    """--impl reference: the CPU restatement of the reference's loop (the
    oracle port, OpenMP over all host threads) on the same workload, with the
    same config block, warm-up and step count as this build's arm where the
    time budget allows (each step is one full SSP-RK3 iteration)."""
    if rank != 0:
        return
    poly = load_mesh()
    budget = float(os.environ.get("FV_REF_SECONDS", "60"))
    from oracle import port
    e = port_solver(poly)
    w = max(args.warmup, 3)
    t0 = time.perf_counter()
    e.run(1)
    per = time.perf_counter() - t0
    if w > 1:
        e.run(w - 1)
    k = max(1, min(args.steps, int(budget / max(per, 1e-3))))
    t0 = time.perf_counter()
    e.run(k)
    dt = time.perf_counter() - t0
    value = e.n_cells * k / dt / 1e6
    sample = f"{k} of the requested {args.steps} iterations on the full {e.n_cells}-cell mesh after {w} warm-up"
    line = {"metric": METRIC, "value": round(value, 3), "unit": "Mcell-iters/s", "n_gpus": args.gpus,
            "steps": k, "warmup": w, "ms_per_step": round(dt / k * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": DATA,
            "impl": "reference",
            "config": headline_config(e.n_cells, e.mesh.n_faces, args.gpus),
            "cpu_baseline": {"value": round(value, 3), "unit": "Mcell-iters/s", "cores": port.num_threads(),
                             "kind": "port", "sample": sample},
            "e2e": {"value": round(value, 3), "unit": "Mcell-iters/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--profile", action="store_true",
                    help="profiler target: build the workload, run --steps iterations with direct launches, exit")
    ap.add_argument("--fp32", action="store_true", help="with --profile: the FP32-flux variant")
    ap.add_argument("--profile-target", choices=["euler", "adjoint", "rans", "multigrid", "config1"], default="euler",
                    help="with --profile: which kernels to run (profiler target)")
    ap.add_argument("--adjoint-check", action="store_true",
                    help="adjoint gradients of the 500k-cell case against central differences of converged solves")
    ap.add_argument("--batched", action="store_true",
                    help="converged solves/s of the batched airfoil family instead of the headline")
    ap.add_argument("--instances", type=int, default=256)
    ap.add_argument("--tol", type=float, default=1e-8)
    ap.add_argument("--max-newton", type=int, default=120)
    args = ap.parse_args()
    if args.batched:
        run_batched(args)
        return
    if args.adjoint_check:
        import torch
        torch.cuda.init()
        print(json.dumps({"adjoint_check": adjoint_check()}), flush=True)
        return
    if args.profile:
        if args.profile_target == "euler":
            poly = load_mesh()
            s, _ = make_solver(poly, fp32=args.fp32)
            ms, launches = s.step_timed(args.steps)
            print(json.dumps({"profile_steps": args.steps, "kernel_ms": ms.tolist(), "launches": launches.tolist()}))
        else:
            print(json.dumps({"profile": args.profile_target, **profile_target(args.profile_target, args.steps)}))
        return

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        run_reference(args, rank)
        return

    import torch
    import torch.distributed as dist

    torch.cuda.set_device(local_rank)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))

    from finitevolume_gb300 import capi, roofline, __version__  # noqa: F401

    # CPU baseline first (before the first GPU call in this process: OpenMP
    # threads only, no fork).
    poly = load_mesh()
    cpu = None
    port_run = {}
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline_block(poly, float(os.environ.get("FV_CPU_SECONDS", "15")),
                                 float(os.environ.get("FV_CPU_1T_SECONDS", "5")), keep=port_run)

    solver, mesh = make_solver(poly)
    n_cells, n_faces, n_bf = mesh.n_cells, mesh.n_faces, mesh.n_bfaces
    u_ptr, s_ptr = solver.device_state()
    stream = torch.cuda.ExternalStream(s_ptr)

    launch = solver.autotune(steps=3, cache=False)  # launch shapes by timing, state restored
    solver.run(max(args.warmup, 3))  # warm-up through the graph path

    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clk:
        ev0.record(stream)
        ms, launches = solver.step_timed(args.steps)
        ev1.record(stream)
        ev1.synchronize()
    torch.cuda.synchronize()
    elapsed_ms = max_over_ranks(ev0.elapsed_time(ev1), world, "cuda")
    clocks = clk.summary()
    value = replica_rate(n_cells, args.steps, elapsed_ms, world)

    # Roofline of the dominant kernel class (largest summed device time).
    hbm, peak_src = measured_peaks()
    k_dom = int(np.argmax(ms))
    kname = roofline.KERNEL_NAMES[k_dom]
    per_launch_ms = ms[k_dom] / max(launches[k_dom], 1)
    alg = roofline.kernel_bytes(kname, n_cells, n_faces, n_bf)
    achieved = alg / (per_launch_ms / 1e3) / 1e9
    stage_ms = float(np.sum(ms)) / (3 * args.steps)
    stage_alg = roofline.survey_stage_bytes(n_cells, n_faces)
    roof = {"bound": "hbm", "kernel": f"k_{'grad' if kname == 'gradients' else 'face' if kname == 'faces' else 'update'}",
            "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s", "frac": round(achieved / hbm, 4),
            "peak_source": peak_src, "traffic": roofline.measured_traffic(kname, n_cells),
            "algorithmic_bytes_per_launch": alg, "launch_ms": round(per_launch_ms, 4),
            "kernel_ms_per_step": {k: round(m / args.steps, 4) for k, m in zip(roofline.KERNEL_NAMES, ms)},
            "stage": {"survey_bytes_B2": stage_alg, "ms": round(stage_ms, 4),
                      "achieved_GBs": round(stage_alg / (stage_ms / 1e3) / 1e9, 1)}}
    # What actually bounds it: FP64-pipe issue (ncu instruction count per
    # cell of this kernel x cells / live launch time, against the GB300
    # DFMA rate of 0.51e12 thread instructions/s measured on the box).
    inst = roofline.MEASURED_FP64_INST_PER_CELL.get(kname)
    if inst is not None:
        ach_inst = inst * n_cells / (per_launch_ms / 1e3) / 1e9
        roof["fp64_pipe"] = {"inst_per_cell_ncu": inst, "achieved_ginst_s": round(ach_inst, 1),
                             "peak_ginst_s": FP64_PIPE_GINST_S, "frac": round(ach_inst / FP64_PIPE_GINST_S, 4)}
        roof["fp64_pipe_frac"] = roof["fp64_pipe"]["frac"]

    # End to end through the public API with host buffers: every step
    # uploads the state from pinned host memory (set_field), advances one
    # iteration, reads the residual norms and downloads the state (field).
    e2e_steps = min(args.steps, 10)
    host = torch.empty((n_cells, 4), dtype=torch.float64, pin_memory=True).numpy()
    out = torch.empty((n_cells, 4), dtype=torch.float64, pin_memory=True).numpy()
    from finitevolume_gb300 import capi as _c
    L = _c.lib()
    capi.check(L.fv_get_field(solver._h, _c.dptr(host)))
    norms = np.zeros(4)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        capi.check(L.fv_set_field(solver._h, _c.dptr(host)))
        capi.check(L.fv_step(solver._h, 1, None))
        capi.check(L.fv_get_residual(solver._h, _c.dptr(norms)))
        capi.check(L.fv_get_field(solver._h, _c.dptr(out)))
        host, out = out, host
    e2e_s = time.perf_counter() - t0
    e2e = {"value": round(world * n_cells * e2e_steps / e2e_s / 1e6, 3), "unit": "Mcell-iters/s",
           "h2d_bytes_per_step": 32 * n_cells, "d2h_bytes_per_step": 32 * n_cells + 32,
           "steps": e2e_steps, "api": "fv_set_field + fv_step(1) + fv_get_residual + fv_get_field"}

    # Parity of the headline itself: the GPU solver run from the same start
    # state for as many iterations as the CPU baseline's port run took.
    parity = None
    if port_run:
        ps, _ = make_solver(poly)
        ps.run(port_run["iterations"])
        Ug, Uc = ps.field(), port_run["field"]
        parity = {"against": "oracle port (CPU FP64, oracle/fv_oracle.cpp), same start state",
                  "iterations": port_run["iterations"], "tolerance": 1e-10,
                  "max_rel_field_err": float(np.max(np.abs(Ug - Uc)) / np.max(np.abs(Uc)))}
        del ps

    variants = {}
    if not args.no_variants:
        # FP32 flux/gradient arithmetic, FP64 accumulation/update/norms.
        a, _ = make_solver(poly)
        b, _ = make_solver(poly, fp32=True)
        b.autotune(steps=3, cache=False)
        a.run(args.warmup)
        b.run(args.warmup)
        ms32, l32 = b.step_timed(args.steps)
        a.run(args.steps)
        fa, fb = a.wall_forces(*force_ref()), b.wall_forces(*force_ref())
        Ua, Ub = a.field(), b.field()
        v32 = n_cells * args.steps / (float(np.sum(ms32)) / 1e3) / 1e6
        k32 = int(np.argmax(ms32))
        kn32 = roofline.KERNEL_NAMES[k32]
        pl32 = ms32[k32] / max(l32[k32], 1)
        alg32 = roofline.kernel_bytes(kn32, n_cells, n_faces, n_bf, fp32=True)
        variants["fp32_flux"] = {
            "value": round(v32, 3), "unit": "Mcell-iters/s", "speedup_vs_fp64": round(v32 / value * world, 3),
            "kernel_ms_per_step": {k: round(m / args.steps, 4) for k, m in zip(roofline.KERNEL_NAMES, ms32)},
            "roofline": {"bound": "hbm", "kernel": kn32, "launch_ms": round(pl32, 4),
                         "algorithmic_bytes_per_launch": alg32,
                         "achieved": round(alg32 / (pl32 / 1e3) / 1e9, 1), "peak": hbm, "unit": "GB/s",
                         "frac": round(alg32 / (pl32 / 1e3) / 1e9 / hbm, 4),
                         "traffic": roofline.measured_traffic(kn32, n_cells, fp32=True)},
            "dCL": abs(fa["cl"] - fb["cl"]), "dCD": abs(fa["cd_total"] - fb["cd_total"]),
            "state_l2_rel": float(np.linalg.norm(Ua - Ub) / np.linalg.norm(Ua)),
            "iterations_compared": args.warmup + args.steps}
        del a, b
        # Batched steady solves at a fixed iteration count: 256 instances
        # advanced together vs the same instances one after another.
        _, bm, bfs = batch_workload(256)
        it = int(os.environ.get("FV_BATCH_ITERS", "20"))
        for prec, fp32 in (("f64", False), ("fp32_flux", True)):
            rb, rs = batch_throughput(bm, bfs, fp32, it)
            variants[f"batched_256_{prec}"] = {
                "value": round(rb, 3), "unit": "Mcell-iters/s", "sequential": round(rs, 3),
                "speedup_vs_sequential": round(rb / rs, 3), "iterations": it,
                "cells_total": int(sum(m.n_cells for m in bm)),
                "workload": "256 NACA 4-digit O-grids, 4k-64k cells log-uniform, M 0.3-0.85, AoA -4..8"}
        # converged solves/s on a seeded 64-instance subset of the family
        # (the full family's long tail of transonic instances takes
        # minutes), the same subset for every path
        sub = np.sort(np.random.default_rng(5).choice(len(bm), 64, replace=False))
        variants["batched_converged_64"] = batch_converged_newton([bm[i] for i in sub], [bfs[i] for i in sub])
        variants["batched_converged_64"]["subset_of_256"] = [int(i) for i in sub]
        del bm
        variants["adjoint_500k"] = adjoint_cost()
        variants["rans_sa_2M"] = rans_sa_rate()
        variants["sod_layout_1M"] = sod_layout()
        variants["config1_o1_rusanov_32k"] = config1_rate()

    if rank == 0:
        line = {"metric": METRIC, "value": round(value, 3), "unit": "Mcell-iters/s", "n_gpus": world,
                "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": round(elapsed_ms / args.steps, 4),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": DATA, "config": headline_config(n_cells, n_faces, world),
                "launch_threads_per_block": {k: launch[k] for k in ("gradients", "faces", "cells")},
                "roofline": roof, "cpu_baseline": cpu, "parity": parity, "e2e": e2e, "clocks": clocks,
                "gpu_launches": int(np.sum(launches)), "variants": variants}
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
