/*
 * fv_gb300.h -- C ABI of the GB300-native (sm_103a) explicit
 * residual-and-update loop of FiniteVolume.
 *
 * The reference has no FFI or plugin layer: its solvers are C++ classes
 * linked into one executable.  Each entry point below replaces one method of
 * those classes (cited per function); include/fvgb300/*.hpp re-creates the
 * classes themselves on top of this ABI so a reference-style driver compiles
 * unchanged.  Every function returns an fv_status; fv_last_error() gives the
 * message of the calling thread's last failure.  There is no CPU fallback:
 * without a usable CUDA device every solver entry point fails with
 * FV_ERR_CUDA.
 *
 * Conventions
 *  - Fields cross the ABI as AoS double[4] per cell {rho, rho_u, rho_v, E}
 *    in the caller's (reference) cell order; the device layout is reordered
 *    internally and mapped back on every get/set.
 *  - Indices are 0-based int32; cell counts up to 2^31-1.
 *  - A solver is not re-entrant (same contract as the reference classes).
 */
#ifndef FV_GB300_H
#define FV_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    FV_OK = 0,
    FV_ERR_BAD_ARG = 1,     /* invalid argument / size mismatch              */
    FV_ERR_CUDA = 2,        /* CUDA runtime error or no usable device        */
    FV_ERR_NONFINITE = 3,   /* NaN/Inf detected in the residual norms        */
    FV_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up            */
    FV_ERR_BAD_MESH = 5,    /* untagged boundary face, degenerate geometry.. */
    FV_ERR_UNSUPPORTED = 6  /* option combination not implemented            */
} fv_status;

typedef struct fv_mesh_s* fv_mesh_t;
typedef struct fv_solver_s* fv_solver_t;

/* Thread-local text of the last error returned on this thread. */
const char* fv_last_error(void);
/* ABI version (major*100 + minor). */
int fv_abi_version(void);
/* Number of CUDA devices visible (0 without a GPU); never fails. */
int fv_device_count(void);

/* ------------------------------------------------------------------------
 * Mesh
 * ------------------------------------------------------------------------ */
enum { FV_REORDER_NONE = 0, FV_REORDER_MORTON = 1, FV_REORDER_RCM = 2 };

/*
 * Build a mesh from CCW polygon cells + tagged boundary edges.
 * Replaces MeshReader::read_fvmesh + build_cells_faces_patches
 * (src/MeshReader.cpp:317-456, :825-958): faces are derived by walking each
 * cell's edges in order, the first cell to visit an edge owns it
 * (cell_left) and fixes its node order, so face numbering, orientation and
 * each cell's face order match the reference reader exactly.  Boundary edges
 * that match no cell edge are ignored; an untagged boundary face, a
 * non-positive or non-finite cell area, a zero-length face or a
 * self-intersecting cell fails with FV_ERR_BAD_MESH (validate_mesh_geometry,
 * src/MeshReader.cpp:125-288).
 *   xy          [2*n_nodes]   node coordinates
 *   cell_off    [n_cells+1]   CSR offsets into cell_nodes
 *   cell_nodes  [cell_off[n_cells]]
 *   bedge_nodes [2*n_bedges], bedge_patch [n_bedges] (0..n_patches-1)
 */
int fv_mesh_create_polygons(int32_t n_nodes, const double* xy, int32_t n_cells, const int64_t* cell_off,
                            const int32_t* cell_nodes, int32_t n_bedges, const int32_t* bedge_nodes,
                            const int32_t* bedge_patch, int32_t n_patches, int32_t reorder, fv_mesh_t* out);

/*
 * Build a mesh from an already-derived face topology: the fields of the
 * reference's UnstructuredMesh (include/UnstructuredMesh.h:20-106).
 * Face geometry (midpoint, length, unit normal) is recomputed from the
 * nodes as UnstructuredMesh::compute_geometry does (:89-105); cell volume
 * and centroid are taken as given (the reference reader fills them).
 *   face_nodes [2*n_faces] node1,node2   face_cells [2*n_faces] left,right(-1)
 *   face_patch [n_faces] (-1 = internal)  cell_face_off [n_cells+1], cell_faces
 *   cell_geom  [3*n_cells] volume, x_centroid, y_centroid
 */
int fv_mesh_create_faces(int32_t n_nodes, const double* xy, int32_t n_faces, const int32_t* face_nodes,
                         const int32_t* face_cells, const int32_t* face_patch, int32_t n_cells,
                         const int32_t* cell_face_off, const int32_t* cell_faces, const double* cell_geom,
                         int32_t n_patches, int32_t reorder, fv_mesh_t* out);

/* counts[0..4] = cells, faces, boundary faces, patches, cell-face entries */
int fv_mesh_counts(fv_mesh_t mesh, int64_t counts[5]);

/*
 * Topology and geometry in reference numbering (test/inspection helper).
 * Any pointer may be NULL.  face_i32 [5*F] node1,node2,left,right,patch;
 * face_f64 [5*F] nx,ny,area,x_mid,y_mid; cell_f64 [3*N] volume,cx,cy;
 * cell_face_off [N+1]; cell_faces [entries].
 */
int fv_mesh_export(fv_mesh_t mesh, int32_t* face_i32, double* face_f64, double* cell_f64,
                   int32_t* cell_face_off, int32_t* cell_faces);
/* Device-order permutation: perm[new] = reference cell index. */
int fv_mesh_permutation(fv_mesh_t mesh, int32_t* perm);
/* The partition the persistent first-order kernel's dataflow form makes of
 * this mesh over `blocks` blocks (one per SM on the device; host only;
 * inspection and test helper; no reference counterpart).  patch_types
 * [n_patches] are the FV_BC_* of the solver's patches (warps with a cell on
 * a characteristic farfield face weigh more).  counts[4] receives the block
 * count nb (min(blocks, ceil(N/32))), the lengths of dep_face and dep_cell,
 * and 1 if the plan is used (no block waits for more than 32 blocks in a
 * phase) else 0.  In device numbering: block b owns the cells
 * [cell_off[b], cell_off[b+1]) and the faces faces[face_off[b] ..
 * face_off[b+1]) (boundary faces first); its face phase waits for the
 * blocks dep_face[dep_face_off[b] .. dep_face_off[b+1]), its cell phase for
 * dep_cell[...]; face_cells[2F] the left and right cell (-1: boundary) of
 * each face.  Array sizes: nb+1 for the offsets, F for faces, 2F for
 * face_cells; any array may be NULL (call with NULL arrays to size). */
int fv_mesh_dataflow_plan(fv_mesh_t mesh, const int32_t* patch_types, int32_t blocks, int32_t counts[4],
                          int32_t* cell_off, int32_t* face_off, int32_t* faces, int32_t* dep_face_off,
                          int32_t* dep_face, int32_t* dep_cell_off, int32_t* dep_cell, int32_t* face_cells);
/* The first coarse level that fv_solver_multigrid builds from this mesh
 * (host only; inspection and test helper; no reference counterpart).
 * counts[2] receives the coarse cell and face counts; any other pointer may
 * be NULL: agg [N] the agglomerate of each fine cell (reference
 * numbering), coarse_cell_f64 [3*Nc] volume,cx,cy, coarse_face_i32 [3*Fc]
 * left,right (-1 on boundary),patch (-1 inside), coarse_face_f64 [3*Fc]
 * nx,ny,length (the unit normal and length of the summed n A of the fine
 * faces merged into it, oriented out of `left`).  Call once with NULL
 * arrays to size them; the result is deterministic. */
int fv_mesh_agglomerate(fv_mesh_t mesh, int32_t counts[2], int32_t* agg, double* coarse_cell_f64,
                        int32_t* coarse_face_i32, double* coarse_face_f64);
int fv_mesh_destroy(fv_mesh_t mesh);

/* ------------------------------------------------------------------------
 * Euler / Navier-Stokes solver
 * ------------------------------------------------------------------------ */
enum {
    FV_BC_WALL = 0,          /* slip wall (Euler) -- EulerBoundaryType::Wall      */
    FV_BC_FARFIELD = 1,      /* fixed state -- EulerBoundaryType::Farfield        */
    FV_BC_OUTFLOW = 2,       /* zero gradient -- EulerBoundaryType::Outflow       */
    FV_BC_CHAR_FARFIELD = 3, /* characteristic (Riemann-invariant) farfield; new  */
    FV_BC_NOSLIP = 4         /* no-slip wall (NS) -- NSBoundaryType::NoSlipWall   */
};
enum { FV_FLUX_RUSANOV = 0, FV_FLUX_HLLC = 1, FV_FLUX_EXACT = 2 };
enum { FV_GRAD_LSQ = 0, FV_GRAD_GG = 1 };
enum { FV_LIM_NONE = 0, FV_LIM_BARTH = 1, FV_LIM_VENKAT = 2 };
enum { FV_DT_GLOBAL = 0, FV_DT_LOCAL = 1 };
enum { FV_PREC_FP64 = 0, FV_PREC_FP32_FLUX = 1 };

/* One boundary condition per mesh patch (EulerBoundaryCondition,
 * include/EulerFVMSolver.h:25-29; NSBoundaryCondition,
 * include/NavierStokesFVMSolver.h:25-32). */
typedef struct {
    int32_t type;        /* FV_BC_*                                              */
    int32_t isothermal;  /* NOSLIP: 1 = isothermal at wall_T, 0 = adiabatic     */
    double state[4];     /* FARFIELD / CHAR_FARFIELD: conserved freestream state */
    double wall_u, wall_v, wall_T;
    double nut;          /* RANS-SA, FARFIELD: freestream nu-tilde               */
} fv_bc_t;

/* EulerInitialCondition (include/EulerFVMSolver.h:59-67), primitive form. */
typedef struct {
    int32_t two_region;  /* 0 freestream, 1 left/right split at x0 */
    int32_t pad;
    double rho, u, v, p;
    double rho_l, u_l, v_l, p_l;
    double rho_r, u_r, v_r, p_r;
    double x0;
} fv_ic_t;

typedef struct {
    int32_t flux;          /* FV_FLUX_*                                        */
    int32_t order;         /* 1 = piecewise constant (reference), 2 = MUSCL    */
    int32_t gradient;      /* FV_GRAD_* (order 2 reconstruction, NS viscous)   */
    int32_t limiter;       /* FV_LIM_* (order 2)                               */
    double venkat_k;       /* Venkatakrishnan K                                */
    int32_t rk_stages;     /* 1 forward Euler (reference), 3 SSP-RK3           */
    int32_t dt_mode;       /* FV_DT_GLOBAL (reference) or FV_DT_LOCAL          */
    int32_t precision;     /* FV_PREC_*                                        */
    int32_t strict;        /* 1: IEEE op-for-op with the reference (no FMA)    */
    double exact_tol;      /* exact Riemann Newton relative tolerance          */
    int32_t exact_max_iter;
    int32_t viscous;       /* 1: Navier-Stokes viscous + heat flux; 2: RANS with
                              the Spalart-Allmaras (SA-noft2) model             */
    double gas_constant, mu, prandtl;
    double prandtl_t;      /* RANS: turbulent Prandtl number                   */
    double initial_nut;    /* RANS: uniform initial nu-tilde                   */
    double sa[9];          /* RANS: cb1, cb2, sigma, kappa, cw2, cw3, cv1, cv2, cv3
                              (SAModelConstants, include/SpalartAllmaras.h:13-23) */
} fv_options_t;

/* Fill *opt with the reference's defaults: Rusanov, order 1, forward Euler,
 * global dt, FP64, exact tol 1e-6 / 20 iterations, LSQ, Venkatakrishnan K=5. */
void fv_options_default(fv_options_t* opt);

/*
 * Construct a solver (EulerFVMSolver ctor, include/EulerFVMSolver.h:107-113,
 * src/EulerFVMSolver.cpp:12-38; NavierStokesFVMSolver ctor when
 * opt->viscous, include/NavierStokesFVMSolver.h:118-121).  bcs[] is indexed
 * by patch.  The initial condition is applied from cell centroids exactly as
 * the reference constructors do.  The mesh may be destroyed afterwards.
 */
int fv_solver_create(fv_mesh_t mesh, const fv_bc_t* bcs, int32_t n_bcs, double gamma, double cfl,
                     const fv_ic_t* ic, const fv_options_t* opt, fv_solver_t* out);
int fv_solver_destroy(fv_solver_t s);

/* Use this CUDA stream (cudaStream_t) for all work; NULL = solver-owned. */
int fv_solver_set_stream(fv_solver_t s, void* stream);

/*
 * Advance n steps (EulerFVMSolver::step / run, src/EulerFVMSolver.cpp:58-121).
 * Replayed from a captured CUDA graph.  If history != NULL it receives the
 * n x 4 residual norms (EulerResidualNorms of each step, same definition as
 * the reference: L2 of the un-normalised flux residual, taken before the
 * dt/volume scaling).  Synchronises the stream before returning; returns
 * FV_ERR_NONFINITE if the last step's norms are not finite.
 */
int fv_step(fv_solver_t s, int32_t n, double* history);
/* Enqueue n steps without synchronising (history stays on the device). */
int fv_step_async(fv_solver_t s, int32_t n);
/*
 * Advance n steps with every kernel launched directly (no graph) and a CUDA
 * event recorded on the solver's stream after each launch; synchronises.
 * kernel_ms[k] receives the summed device time and launches[k] the number
 * of launches of each kernel class: 0 gradients + limiter, 1 face fluxes,
 * 2 cell update.  Same results as fv_step.
 */
int fv_step_timed(fv_solver_t s, int32_t n, double kernel_ms[3], int32_t launches[3]);
/* Copy the last n residual-norm rows recorded on the device (n x 4). */
int fv_get_history(fv_solver_t s, int32_t n, double* history);

/* Launch shapes (threads per block of the gradient, face and cell kernels:
 * 128..512, multiples of 32) of the second-order / multi-stage path, and
 * the autotuner that picks them: each kernel class is timed over `steps`
 * steps at 128, 256 and 512 threads per block (CUDA events on the solver's
 * stream), the fastest shape per class is kept, and the solver's state is
 * restored afterwards.  No reference counterpart (the reference's loops are
 * OpenMP). */
int fv_solver_set_launch(fv_solver_t s, const int32_t blocks[3]);
/* Persistent kernel of the first-order forward-Euler FP64 Euler path (the
 * reference's own scheme, EulerFVMSolver::step / compute_dt,
 * src/EulerFVMSolver.cpp:58-162): one cooperative launch runs a chunk of
 * steps, meeting the flux -> update and global-dt dependencies at grid
 * barriers instead of kernel boundaries; same results as the two-kernel
 * path (bit for bit in strict mode).  On by default where the device
 * supports cooperative launch; on = 0 selects the two-kernel path.  With
 * local time stepping the kernel runs in a dataflow form: one block per SM
 * owns a range of cells, and each phase waits only for the blocks it shares
 * faces with instead of for the whole grid (same results again); on = 2
 * keeps the grid-barrier form.  fv_solver_persistent reports the form in
 * use (0 two-kernel path, 1 grid-barrier form, 2 dataflow form) and its
 * grid size (either pointer may be NULL).  No reference counterpart (the
 * reference's loops are OpenMP). */
int fv_solver_set_persistent(fv_solver_t s, int32_t on);
int fv_solver_persistent(fv_solver_t s, int32_t* on, int32_t* grid);
/* Bound on every wait of the persistent kernel (grid barrier, or a
 * neighbour's progress word in the dataflow form), in SM clock cycles
 * (default 2e9, about one second).  A wait that runs out makes the launch
 * end early and fv_step / fv_step_timed return FV_ERR_TIMEOUT (the state is
 * then unspecified).  phantom_arrivals > 0 makes every grid barrier (both
 * forms begin with one) wait for that many arrivals that never come: a
 * check of the timeout path that faults and hangs nothing; set it back to
 * 0 afterwards. */
int fv_solver_set_wait_limit(fv_solver_t s, int64_t cycles, int32_t phantom_arrivals);
/* Limiter freezing (second order with a limiter; a no-op otherwise): on=1
 * evaluates the limiter once at the current state and reuses those values
 * in every later step (the scheme becomes smooth, so steady solves that
 * limit-cycle through the limiter's switching converge to machine
 * precision, and the frozen-limiter adjoint is its exact linearisation);
 * on=0 evaluates the limiter again.  No reference counterpart. */
int fv_solver_freeze_limiter(fv_solver_t s, int32_t on);
/* The frozen limiter values [4 n_cells] (per cell: rho, u, v, p; reference
 * cell order): psi_out (may be NULL) receives them; psi_in (may be NULL,
 * each value in [0, 1]) freezes the limiter at the given values, e.g. those
 * of another solver on the same mesh. */
int fv_solver_limiter_values(fv_solver_t s, double* psi_out, const double* psi_in);
/* Move the mesh nodes (xy [2 n_nodes], the mesh's node numbering) and
 * recompute on the device every geometric quantity the Euler solver uses:
 * face normals, lengths, midpoints and CFL lengths, shoelace cell areas and
 * centroids (UnstructuredMesh::compute_geometry,
 * include/UnstructuredMesh.h:89-105; src/MeshReader.cpp:56-76) and the
 * second-order reconstruction geometry, in place (captured graphs stay
 * valid).  mesh is the mesh the solver was created from (built from cell
 * polygons); the mesh handle itself keeps its original nodes.  Gives the
 * geometry of a solver built on the moved mesh bit for bit (Green-Gauss
 * interpolation weights: to the last bit of hypot). */
int fv_solver_update_nodes(fv_solver_t s, fv_mesh_t mesh, const double* xy);
int fv_solver_autotune(fv_solver_t s, int32_t steps, int32_t blocks[3]);
/* Agglomeration multigrid (full approximation scheme) for steady solves
 * with local time stepping: `levels` coarse levels agglomerated from mesh
 * (the solver's own mesh), first order, SSP-RK3, `smooth` iterations per
 * level per V-cycle, corrections scaled by `relax` (0 < relax <= 1).  Every
 * fv_step is then one smoothing iteration plus one V-cycle; the converged
 * solution is the scheme's own.  levels = 0 turns it off.  No reference
 * counterpart. */
int fv_solver_multigrid(fv_solver_t s, fv_mesh_t mesh, int32_t levels, int32_t smooth, double relax);

/* EulerFVMSolver::field / set_field / residual / set_cfl / gas_gamma
 * (include/EulerFVMSolver.h:121-160). */
int fv_get_field(fv_solver_t s, double* U);
int fv_set_field(fv_solver_t s, const double* U);
int fv_get_residual(fv_solver_t s, double norms[4]);
int fv_set_cfl(fv_solver_t s, double cfl);
/* RANSTurbulenceSASolver::nut_field / set_field(U, nut) / nut_residual
 * (include/RANSTurbulenceSASolver.h): nu-tilde per cell in the caller's
 * order, and the wall distance the SA model uses (compute_wall_distance,
 * include/WallDistance.h:38). */
int fv_get_nut(fv_solver_t s, double* nut);
int fv_set_nut(fv_solver_t s, const double* nut);
int fv_get_nut_residual(fv_solver_t s, double* norm);
int fv_get_wall_distance(fv_solver_t s, double* d);
int fv_get_gamma(fv_solver_t s, double* gamma);
/* Device pointer to the AoS state in device cell order, and the solver's
 * stream (for callers that time or chain work on it). */
int fv_device_state(fv_solver_t s, void** U_dev, void** stream);

/* Wall force integration over every boundary face whose patch is a wall
 * (FV_BC_WALL or FV_BC_NOSLIP): compute_wall_traction + compute_wall_forces
 * (src/WallTraction.cpp:95-217).  Wall pressure is the owner cell's
 * pressure; friction is added for viscous solvers.  ref[7] = rho_ref,
 * u_ref, v_ref, p_ref, length_ref, moment_x, moment_y.  out[11] =
 * friction_drag, pressure_drag, total_drag, lift, moment, cd_friction,
 * cd_pressure, cd_total, cl, cm, n_wall_faces (domain total). */
int fv_wall_forces(fv_solver_t s, const double ref[7], double out[11]);

/* ------------------------------------------------------------------------
 * Batched steady solves (many independent meshes, one launch sequence)
 * ------------------------------------------------------------------------ */
/*
 * No single reference counterpart: the reference solves one case per
 * process.  Concatenates n meshes (same patch count) into one batch mesh;
 * each instance's cells stay contiguous in device order.
 */
int fv_mesh_create_batch(int32_t n, const fv_mesh_t* meshes, int32_t reorder, fv_mesh_t* out);
/*
 * One solver over a batch mesh: the scheme of opt (local time stepping
 * required), shared per-patch boundary types bcs[], and one freestream per
 * instance (inst_freestream [4n], conserved) used by the farfield patches
 * and as each instance's initial state.  fv_step advances every active
 * instance; each instance's residual norms are reduced on its own and the
 * instance is frozen once its density norm falls below the tolerance
 * (per-instance early exit).  fv_get_field returns all instances in order.
 */
int fv_batch_create(fv_mesh_t batch_mesh, const fv_bc_t* bcs, int32_t n_bcs, const double* inst_freestream, double gamma,
                    double cfl, const fv_options_t* opt, fv_solver_t* out);
/* Density-residual tolerance of the early exit (< 0: never freeze). */
int fv_batch_set_tolerance(fv_solver_t s, double tol_rho);
/* Per instance: active flag, iterations taken, last residual norms [4n]. */
int fv_batch_status(fv_solver_t s, int32_t* active, int32_t* iterations, double* norms);
/* fv_wall_forces restricted to one instance's wall faces. */
int fv_batch_wall_forces(fv_solver_t s, int32_t instance, const double ref[7], double out[11]);
/* Freeze (active = 0) or resume (1) one instance, e.g. once the caller's own
 * convergence test (a force coefficient) holds.  Takes effect at the next
 * fv_step. */
int fv_batch_set_active(fv_solver_t s, int32_t instance, int32_t active);

/* ------------------------------------------------------------------------
 * Discrete adjoint of the Euler residual (no reference counterpart: the
 * reference has no adjoint).  The adjoint pair differentiates the residual
 * R(U, fs) that EulerFVMSolver::step drives to zero (the face and cell
 * passes of src/EulerFVMSolver.cpp:61-111, with the MUSCL / limiter /
 * characteristic-farfield extensions of this library), linearised at one
 * state with the limiter values frozen there.  fs is the primitive
 * freestream (rho, u, v, p) of each farfield patch.  Arrays are [4 N] AoS
 * in the caller's (reference) cell order; freestream arrays are
 * [4 n_patches].  FP64 Euler solvers with the Rusanov or HLLC flux (least-
 * squares gradients at second order).  The adjoint object borrows the
 * solver's mesh arrays: destroy it before the solver.
 * --------------------------------------------------------------------- */
typedef struct fv_adjoint_s* fv_adjoint_t;

/* FROZEN: the limiter values are held at the linearisation state (the
 * usual frozen-limiter adjoint); FULL: the limiter is differentiated too,
 * through its active branch (neighbour extreme, face extrapolation extreme,
 * Venkatakrishnan / Barth-Jespersen formula), including its geometric
 * inputs (face offsets, eps^2, boundary extremes) in shape gradients. */
enum { FV_ADJ_FROZEN_LIMITER = 0, FV_ADJ_FULL_LIMITER = 1 };
int fv_adjoint_create(fv_solver_t s, int32_t limiter_mode, fv_adjoint_t* out);
int fv_adjoint_destroy(fv_adjoint_t a);
/* Forward: linearise at U (NULL: the solver's current state) and return
 * R(U) (NULL: not returned). */
int fv_residual_forward(fv_adjoint_t a, const double* U, double* R);
/* Tangent: dR = dR/dU dU + dR/dfs dfs (dfs may be NULL). */
int fv_residual_jvp(fv_adjoint_t a, const double* dU, const double* dfs, double* dR);
/* Backward: Ubar = (dR/dU)^T Rbar, fsbar = (dR/dfs)^T Rbar (fsbar may be NULL). */
int fv_residual_backward(fv_adjoint_t a, const double* Rbar, double* Ubar, double* fsbar);
/* Solve (dR/dU)^T lambda = dJdU by SSP-RK3 pseudo-time iteration at the
 * primal's local time step, until every component of the residual norm is
 * below tol or max_iter iterations; returns lambda, fsbar = (dR/dfs)^T
 * lambda, the norm history [4 * iterations] and the iteration count (each
 * output may be NULL).  Then dJ/dalpha = dJ/dalpha|explicit - fsbar .
 * dfs/dalpha. */
int fv_adjoint_solve(fv_adjoint_t a, const double* dJdU, int32_t max_iter, double tol, double* lambda, double* fsbar,
                     double* history, int32_t* iterations);
/* The same system by restarted GMRES(restart) on the fixed point of that
 * pseudo-time iteration (one pseudo-time iteration per matvec), until the
 * GMRES residual is below rtol times its initial value or max_matvec
 * matvecs: converges where the pseudo-time iteration diverges (a primal
 * whose explicit iteration limit-cycles, a frozen limiter with growing
 * modes).  history [max_matvec]: relative GMRES residual after each
 * matvec; residual[4]: norms of (dR/dU)^T lambda - dJdU at the result.
 * Other outputs as fv_adjoint_solve; each may be NULL. */
int fv_adjoint_solve_gmres(fv_adjoint_t a, const double* dJdU, int32_t restart, int32_t max_matvec, double rtol,
                           double* lambda, double* fsbar, double* history, int32_t* matvecs, double residual[4]);
/* The same adjoint system by pseudo-transient iterations with the Newton
 * solver's linear algebra, for converged transonic states where the explicit
 * pseudo-time iteration is slow: with A = -dR/dU, each outer iteration
 * solves (V/dt + A)^T delta = -dJdU - A^T lambda by one GMRES(restart) cycle
 * (to a relative residual of 1e-2), right-preconditioned by symmetric block
 * Gauss-Seidel sweeps (over a cell colouring, on FP32 copies of the blocks)
 * of the transposed first-order Jacobian plus V/dt, V/dt at the given CFL number (the one the primal
 * Newton iteration reached), and adds delta to lambda.  Stops when
 * |(dR/dU)^T lambda - dJdU| is below rtol |dJdU| or after max_matvec
 * products; history [outer iterations] that relative residual before each
 * outer iteration (at most max_matvec / 2 + 1 entries);
 * residual[4] the norms of (dR/dU)^T lambda - dJdU.  Other outputs as
 * fv_adjoint_solve; each may be NULL. */
int fv_adjoint_solve_krylov(fv_adjoint_t a, const double* dJdU, double cfl, int32_t restart, int32_t max_matvec,
                            double rtol, int32_t precond_sweeps, double* lambda, double* fsbar, double* history,
                            int32_t* matvecs, double residual[4]);
/* Shape gradient dJ/dX [2 n_nodes] (x, y per node, the mesh's node
 * numbering) of the objective the last fv_adjoint_solve was solved for:
 * dJ/dX|explicit - lambda^T dR/dX through face normals, lengths and
 * midpoints, shoelace cell centroids, the least-squares weights and (FULL
 * mode) the limiter values.  mesh is the mesh the solver was created from;
 * it must have been built from cell polygons (fv_mesh_create_polygons). */
int fv_adjoint_shape_gradient(fv_adjoint_t a, fv_mesh_t mesh, int32_t objective, const double ref[7], double* dJdX);
/* Geometric cotangent Xbar = (dR/dX)^T Rbar [2 n_nodes] at the
 * linearisation state (the residual's node sensitivities alone; the same
 * map the shape gradient applies to lambda). */
int fv_residual_shape_vjp(fv_adjoint_t a, fv_mesh_t mesh, const double* Rbar, double* Xbar);
/* ------------------------------------------------------------------------
 * Newton-Krylov steady solves (no reference counterpart: the reference
 * reaches steady states with its explicit loop only).  Drives the same
 * discrete residual R(U) that EulerFVMSolver::step advances
 * (src/EulerFVMSolver.cpp:58-112, with this library's MUSCL / limiter /
 * characteristic-farfield extensions) to zero by pseudo-transient
 * continuation: each step solves (V/dt - dR/dU) dU = R by GMRES with the
 * adjoint's exact Jacobian-vector products, preconditioned on the
 * first-order Jacobian (multicolour symmetric block Gauss-Seidel on FP32 or
 * FP64 blocks, or block Jacobi), then U += alpha dU with alpha <= 1 bounding the relative change
 * of every cell's density and pressure.  The CFL number of V/dt starts at
 * cfl0, grows by cfl_growth after each step that lowers the density
 * residual, was taken in full (alpha = 1) and whose GMRES solve reached a
 * relative residual of 0.7 or less (up to cfl_max); it holds after a rise
 * below 2x and halves after a larger one or after a GMRES solve that ended
 * above 0.9; a step that raises it more than 10x is undone and retried at
 * a quarter of its CFL number.  FP64 Euler solvers with the Rusanov or HLLC
 * flux (least-squares gradients at second order), single or batched: a
 * batch is solved as one block-diagonal system in which every instance has
 * its own residual norms, CFL number, step length and undo decision and
 * stops once its own density residual is below tol; each instance's
 * right-hand side is scaled to unit norm for the GMRES solve, so that every
 * instance's equations weigh alike.
 * --------------------------------------------------------------------- */
typedef struct {
    int32_t limiter_mode;   /* FV_ADJ_FROZEN_LIMITER or FV_ADJ_FULL_LIMITER: the limiter's
                               treatment in the Jacobian (freeze the solver's limiter,
                               fv_solver_freeze_limiter, for an exact Newton method)     */
    int32_t max_newton;     /* Newton steps                                               */
    double tol;             /* stop when the density residual L2 norm is below tol       */
    double cfl0, cfl_max, cfl_growth;
    int32_t krylov_dim;     /* GMRES(m), one cycle per Newton step (1..200)               */
    double krylov_rtol;     /* relative GMRES tolerance                                   */
    int32_t precond_sweeps; /* preconditioner sweeps                                      */
    int32_t precond_kind;   /* 2 multicolour symmetric block Gauss-Seidel on FP32 copies of
                               the blocks (default), 1 the same in FP64, 0 block Jacobi   */
    double max_rel_change;  /* bound on the relative density / pressure change per step   */
} fv_newton_t;
/* Defaults: frozen-limiter Jacobian, 200 steps, tol 1e-11, CFL 10 growing
 * x1.5 up to 1e6, GMRES(40) to 1e-2, 2 symmetric Gauss-Seidel sweeps, 20%
 * change. */
void fv_newton_default(fv_newton_t* opt);
/* Runs from the solver's current state and leaves the result there.
 * history (may be NULL) receives one row of 8 per evaluated state
 * [iterations + 1 rows]: the four residual norms (over all instances), then
 * the largest CFL number, the GMRES iterations, its relative residual and
 * the smallest step length alpha of the step that produced it (zeros in
 * row 0).  instance_steps (may be NULL; one entry per batch instance, or
 * one) receives the Newton step at which each instance converged, -1 where
 * it did not. */
int fv_steady_newton(fv_solver_t s, const fv_newton_t* opt, double* history, int32_t* iterations,
                     int32_t* instance_steps);

/* Wall-force coefficient J (objective 0 drag, 1 lift, 2 moment; pressure
 * part with the owner-cell pressure, ref as fv_wall_forces) at the
 * solver's current state, and dJ/dU (may be NULL). */
int fv_force_gradient(fv_solver_t s, int32_t objective, const double ref[7], double* value, double* dJdU);

/* ------------------------------------------------------------------------
 * Scalar diffusion solver (UnstructuredFVMSolver)
 * ------------------------------------------------------------------------ */
typedef struct fv_diffusion_s* fv_diffusion_t;

/*
 * UnstructuredFVMSolver(mesh, alpha, dt, initial_value, initial_radius)
 * (include/UnstructuredFVMSolver.h:34-35, src/UnstructuredFVMSolver.cpp:6-19).
 * The reference reads each boundary patch's BoundaryType/value from
 * mesh.patches (include/UnstructuredMesh.h:49-60); here they are passed per
 * patch: patch_type 0 = Dirichlet (value at the face midpoint), 1 = Neumann
 * (prescribed flux = value * length).
 */
int fv_diffusion_create(fv_mesh_t mesh, double alpha, double dt, double initial_value, double initial_radius,
                        const int32_t* patch_type, const double* patch_value, fv_diffusion_t* out);
int fv_diffusion_destroy(fv_diffusion_t d);
/* step() x n (src/UnstructuredFVMSolver.cpp:44-92); history[n] receives
 * residual_norm() after each step when non-NULL.  n <= 65536 per call. */
int fv_diffusion_step(fv_diffusion_t d, int32_t n, double* history);
/* field() / set_field() / residual_norm() (include/UnstructuredFVMSolver.h:48-73). */
int fv_diffusion_get_field(fv_diffusion_t d, double* phi);
int fv_diffusion_set_field(fv_diffusion_t d, const double* phi);
int fv_diffusion_residual(fv_diffusion_t d, double* norm);

/* ------------------------------------------------------------------------
 * Gradient reconstruction (GradientCalculator, face_gradient)
 * ------------------------------------------------------------------------ */
typedef struct fv_gradient_s* fv_gradient_t;

/* GradientCalculator(mesh, scheme) (include/GradientReconstruction.h:60,
 * src/GradientReconstruction.cpp:45-80): precomputes the geometry once. */
int fv_gradient_create(fv_mesh_t mesh, int32_t scheme, fv_gradient_t* out);
int fv_gradient_destroy(fv_gradient_t g);
/*
 * GradientCalculator::compute(mesh, phi, boundary_phi)
 * (include/GradientReconstruction.h:73, src/GradientReconstruction.cpp:83-150).
 * phi [N] and boundary_phi [F] (only boundary-face entries are read) in
 * reference numbering; grad [2N] = dphidx, dphidy per cell.  When face_out
 * is non-NULL it receives, per face [4F], face_gradient's corrected normal
 * derivative, corrected_face_gradient_vector's x and y, and
 * face_normal_distance (src/GradientReconstruction.cpp:153-199).
 */
int fv_gradient_compute(fv_gradient_t g, const double* phi, const double* boundary_phi, double* grad,
                        double* face_out);

/* ------------------------------------------------------------------------
 * Checkpoints in the reference's file layout
 * ------------------------------------------------------------------------ */
/* CheckpointEquation (include/Checkpoint.h:11-18). */
enum {
    FV_CKPT_DIFFUSION = 0,
    FV_CKPT_EULER = 1,
    FV_CKPT_ADVECTION_DIFFUSION = 2,
    FV_CKPT_NAVIER_STOKES = 3,
    FV_CKPT_RANS_SA = 4,
    FV_CKPT_RANS_SST = 5
};
/*
 * Checkpoint::write (include/Checkpoint.h:26-46, :72-86): 40-byte header
 * (magic, version 2, equation tag, cell count, step index, build number)
 * then the raw payload: cell_count doubles (Diffusion, AdvectionDiffusion),
 * cell_count x 4 (Euler, NavierStokes), x 5 (RANS_SA: U then nut),
 * x 6 (RANS_SST: U then k then omega).
 */
int fv_checkpoint_write(const char* path, int32_t equation, int64_t step_index, uint64_t build_number,
                        int64_t cell_count, const double* payload);
/*
 * Checkpoint::read / read_flow_field (include/Checkpoint.h:102-142): checks
 * magic, version, equation tag and cell count, fails on a truncated file.
 * expected_equation < 0 accepts any flow equation and reads its state block
 * (cell_count x 4).  FV_ERR_BAD_ARG with a message on any mismatch.
 */
int fv_checkpoint_read(const char* path, int32_t expected_equation, int64_t expected_cell_count, int64_t* step_index,
                       uint64_t* build_number, double* payload);

/* ------------------------------------------------------------------------
 * Allocation-free step
 * ------------------------------------------------------------------------ */
/*
 * No counterpart in the reference.  For callers that cannot let a library
 * allocate device memory: an application that owns the whole device budget
 * and serves it from its own pool, code running while other threads capture
 * CUDA graphs in relaxed mode (allocation is illegal there), or a real-time
 * loop that forbids allocation after start-up.  The caller keeps the mesh
 * and the state in its own device buffers; this entry point performs one
 * first-order step of EulerFVMSolver::step (global CFL dt, the caller's
 * flux) and calls no cudaMalloc, cudaFree or allocating library routine.
 *
 * Its work arrays live in one fixed, file-scope device array of about
 * 4 MiB, held by every GPU that loads the library until the process exits;
 * hence the limits below (larger meshes fail with FV_ERR_BAD_ARG).  Every
 * call resolves that array's device address in the current context; the
 * first call in a context may load the module, so make it before any
 * stream capture.  All calls share the array; calls whose GPU work overlaps
 * race on it and must be serialised by the caller.  The call synchronises
 * `stream`.  Before stepping, a device-side check rejects (FV_ERR_BAD_ARG)
 * a boundary face whose patch is outside [0, n_bcs), a face cell index out
 * of range, and CSR offsets or entries that are not a valid cell-to-face
 * map.
 *
 * Mesh arrays are device pointers in the caller's cell/face numbering:
 *   face_left/face_right [F] (right = -1 on boundary faces), face_patch [F]
 *   (0 <= patch < n_bcs on boundary faces),
 *   face_geom [4F] = nx, ny, length, CFL length (min(V_L, V_R)/length, or
 *   V_L/length on boundary faces), 32-byte aligned,
 *   cell_face_off [N+1], cell_faces [E] = face << 1 | (cell owns the face),
 *   listed in the reference's per-cell face order, cell_volume [N].
 * U: device, AoS double[4] per cell, 32-byte aligned, updated in place.
 * norms: host, receives the step's residual norms (EulerResidualNorms).
 */
#define FV_NOALLOC_MAX_FACES 131072
#define FV_NOALLOC_MAX_CELLS 131072
typedef struct {
    int32_t n_cells, n_faces;
    const int32_t* face_left;
    const int32_t* face_right;
    const int32_t* face_patch;
    const double* face_geom;
    const int32_t* cell_face_off;
    const int32_t* cell_faces;
    const double* cell_volume;
} fv_noalloc_mesh_t;

int fv_step_noalloc(const fv_noalloc_mesh_t* mesh, const fv_bc_t* bcs, int32_t n_bcs, double gamma, double cfl,
                    int32_t flux, double* U, double norms[4], void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FV_GB300_H */
