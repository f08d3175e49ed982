"""The allocation-free step, checked against the regular solver.

fv_step_noalloc serves callers that cannot let the library allocate device
memory (their own device pool, relaxed-mode graph capture elsewhere in the
process, allocation-free real-time loops): they pass the mesh and the state
in their own device buffers -- here torch tensors stand in for the caller's
memory -- and the step runs on a fixed scratch array compiled into the
library.  Two calls in a row must agree with two fv_step calls of a solver
built on the same mesh, within the parity tolerance of the other tests.

This file is collected last on purpose, and it also passes alone in a fresh
process (it creates everything it uses).
"""
import ctypes as C

import numpy as np
import pytest

from finitevolume_gb300 import capi, meshgen, solvers as S

pytestmark = pytest.mark.gpu

TOL = 1e-10
GAMMA = 1.4


def _caller_mesh(mesh, torch):
    """Device arrays of the mesh in reference numbering, in torch memory."""
    ex = mesh.export()
    fi, fd, cd = ex["faces_i32"], ex["faces_f64"], ex["cells_f64"]
    left, right, patch = fi[:, 2].copy(), fi[:, 3].copy(), fi[:, 4].copy()
    vol = cd[:, 0].copy()
    length = np.where(right >= 0, np.minimum(vol[left], vol[np.maximum(right, 0)]), vol[left]) / fd[:, 2]
    geom = np.stack([fd[:, 0], fd[:, 1], fd[:, 2], length], 1).copy()
    off, cf = ex["cell_face_off"], ex["cell_faces"]
    owner_cell = np.repeat(np.arange(mesh.n_cells), np.diff(off))
    entries = ((cf.astype(np.int64) << 1) | (left[cf] == owner_cell)).astype(np.int32)
    dev = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in
           dict(left=left, right=right, patch=patch, geom=geom, off=off, cf=entries, vol=vol).items()}
    desc = capi.NoAllocMesh(mesh.n_cells, mesh.n_faces, dev["left"].data_ptr(), dev["right"].data_ptr(),
                            dev["patch"].data_ptr(), dev["geom"].data_ptr(), dev["off"].data_ptr(),
                            dev["cf"].data_ptr(), dev["vol"].data_ptr())
    return desc, dev


@pytest.mark.parametrize("flux", [S.NumericalFluxScheme.Rusanov, S.NumericalFluxScheme.HLLC])
def test_noalloc_step_matches_solver_twice(gpu, flux):
    torch = pytest.importorskip("torch")
    poly = meshgen.naca_ogrid(64, 32)
    mesh = S.Mesh(poly)
    M, aoa = 0.5, np.radians(2.0)
    r, u, v, p = 1.0, M * np.cos(aoa), M * np.sin(aoa), 1.0 / GAMMA
    fs = S.from_primitive(r, u, v, p, GAMMA)
    bcs = [S.EulerBoundaryCondition(S.EulerBoundaryType.Wall),
           S.EulerBoundaryCondition(S.EulerBoundaryType.Farfield, fs)]
    ic = S.EulerInitialCondition(S.EulerICMode.Freestream, rho=r, u=u, v=v, p=p)
    ref = S.EulerFVMSolver(mesh, bcs, GAMMA, 0.5, ic, flux)

    desc, keep = _caller_mesh(mesh, torch)
    U = torch.from_numpy(ref.field()).cuda()
    bc_arr = (capi.BC * 2)()
    bc_arr[0].type = 0
    bc_arr[1].type = 1
    for k in range(4):
        bc_arr[1].state[k] = float(fs[k])
    norms = np.zeros(4)
    L = capi.lib()
    for _ in range(2):
        capi.check(L.fv_step_noalloc(C.byref(desc), bc_arr, 2, GAMMA, 0.5, int(flux), C.c_void_p(U.data_ptr()),
                                     capi.dptr(norms), None))
        ref.step()
        got = U.cpu().numpy()
        want = ref.field()
        assert np.max(np.abs(got - want)) <= TOL * np.max(np.abs(want))
        np.testing.assert_allclose(norms, ref.residual().as_array(), rtol=TOL)

    # The promise itself: once the first call has loaded the module, further
    # calls take no device memory (free bytes of the device unchanged).
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        capi.check(L.fv_step_noalloc(C.byref(desc), bc_arr, 2, GAMMA, 0.5, int(flux), C.c_void_p(U.data_ptr()),
                                     capi.dptr(norms), None))
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    del keep


def test_noalloc_rejects_patches_outside_the_bc_table(gpu):
    """A boundary face whose patch has no boundary condition is an error
    found on the device before any step kernel runs; the state is left
    untouched."""
    torch = pytest.importorskip("torch")
    mesh = S.Mesh(meshgen.naca_ogrid(32, 16))
    desc, keep = _caller_mesh(mesh, torch)
    U0 = np.tile(np.array([1.0, 0.5, 0.0, 2.5]), (mesh.n_cells, 1))
    U = torch.from_numpy(U0.copy()).cuda()
    bc_arr = (capi.BC * 1)()  # the farfield patch (1) has no entry
    norms = np.zeros(4)
    rc = capi.lib().fv_step_noalloc(C.byref(desc), bc_arr, 1, GAMMA, 0.5, 0, C.c_void_p(U.data_ptr()),
                                    capi.dptr(norms), None)
    assert rc == capi.FV_ERR_BAD_ARG
    assert b"patch" in capi.lib().fv_last_error()
    assert np.array_equal(U.cpu().numpy(), U0)
    del keep


def test_noalloc_rejects_meshes_beyond_the_fixed_scratch(gpu):
    desc = capi.NoAllocMesh(10, capi.NOALLOC_MAX_FACES + 1, 1, 1, 1, 32, 1, 1, 1)
    norms = np.zeros(4)
    rc = capi.lib().fv_step_noalloc(C.byref(desc), None, 0, GAMMA, 0.5, 0, C.c_void_p(32), capi.dptr(norms), None)
    assert rc == capi.FV_ERR_BAD_ARG
    assert b"at most" in capi.lib().fv_last_error()
