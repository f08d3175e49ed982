// Internals of the discrete-adjoint object shared by the translation units
// that drive its linearisation: adjoint.cu (the adjoint pair and solves)
// and newton.cu (the Newton-Krylov steady solver, whose Jacobian-vector
// products are the adjoint's tangent map).
#pragma once

#include <vector>

#include "capi_internal.h"
#include "types.h"

namespace adjk {

using fvgb::BCTable;
using fvgb::St;

struct AdjArgs {
    int n_cells, n_faces, n_int_faces, order, flux;
    const int* fl;
    const int* fr;
    const int* fpatch;
    const double4_32a* fgeom;
    const int* cf_off;
    const int* cf;
    const int* cnb;
    const double2* lsq;
    const double2* lsq_sum;
    const double4_32a* frf;
    const int* twin;
    BCTable bc;
    double gamma, igm1, cfl;
    // linearisation state
    const St* W;         // [N] primitives
    const double2* Gu;   // [4N] unlimited gradients
    const double* psi;   // [4N] limiter values
    double* JL;          // [16F] dF/dw_L (boundary: through the ghost state)
    double* JR;          // [16F] dF/dw_R (boundary: dF/d fs)
    double* Gb;          // [32 Fb] 0.5 (I + dghost/dw) | 0.5 dghost/dfs of the gradient's boundary value
    unsigned char* fb;   // [F] bit 0 owner side fell back to the cell value, bit 1 neighbour side
    St* F;               // [F] flux times length
    double* D;           // [N] local dt / V
    // work arrays
    double* wbar;        // [8F]
    St* Wbar;            // [N]
    double2* Gub;        // [4N]
    double* fsb;         // [4 Fb]
    St* dW;              // [N]
    double2* dG;         // [4N]
    St* dF;              // [F]
    const double* dfs;   // [4 * kMaxPatches] primitive freestream tangents
    // full-limiter linearisation (limiter != 0 and full == 1): per cell and
    // variable the active side (0 none, +1 dmax side, -1 dmin side), the
    // entry of the extreme neighbour value (-1: the cell itself), the entry
    // of the extreme face extrapolation, and dpsi/d(d1), dpsi/dy
    int full, limiter;
    const double2* erf;  // [E] face midpoint - centroid
    const double* eps2;  // [N] Venkatakrishnan eps^2
    signed char* lside;  // [4N]
    int* led;            // [4N]
    int* ler;            // [4N]
    double2* lpd;        // [4N] (dpsi/dd1, dpsi/dy)
    double* lpe;         // [4N] dpsi/d eps^2 (Venkatakrishnan; 0 otherwise)
    double* ldb;         // [4N] cotangent of d1 passed to the extreme neighbour
    // batched solvers (Newton only; null otherwise): instance of each cell
    // and each instance's conserved freestream, used by the farfield ghosts
    const int* cell_inst;
    const double* inst_fs;
};

}  // namespace adjk

struct fv_adjoint_s {
    fv_solver_s* solver = nullptr;
    adjk::AdjArgs a{};
    int N = 0, F = 0, Fb = 0, P = 0;
    std::vector<void*> owned;
    fvgb::St *U = nullptr, *W = nullptr, *stage_ref = nullptr, *stage_dev = nullptr, *lam = nullptr, *lam0 = nullptr,
       *rhs = nullptr, *Rdev = nullptr;
    double2 *Gu = nullptr, *G = nullptr;
    double *psi = nullptr, *cs = nullptr, *partials = nullptr, *hist = nullptr, *dfs_dev = nullptr;
    int* counter = nullptr;
    // GMRES work arrays (allocated on first use): restart + 1 basis vectors,
    // the affine part c, the work vector, the iterate, reduction partials
    // and device scalars
    double *kV = nullptr, *kc = nullptr, *kw = nullptr, *kx = nullptr, *kpart = nullptr, *kh = nullptr;
    int k_restart = 0;
    // shape-gradient work arrays (allocated on first use)
    double *geo_face = nullptr, *geo_ab = nullptr, *geo_sb = nullptr, *geo_nbg = nullptr, *geo_er = nullptr,
           *geo_ep = nullptr;
    int hist_cap = 0;
    bool linearised = false;
    bool solved = false;
    ~fv_adjoint_s() {
        for (void* p : owned) cudaFree(p);
        if (hist) cudaFree(hist);
    }
    template <typename T>
    T* alloc(size_t n) {
        void* p = nullptr;
        FV_CUDA(cudaMalloc(&p, sizeof(T) * (n ? n : 1)));
        owned.push_back(p);
        return static_cast<T*>(p);
    }
};

namespace adjh {
// fv_adjoint_create, also for batched solvers when allow_batch (the
// farfield ghosts then take each instance's own freestream; the freestream
// tangents and cotangents of the adjoint pair are not defined there).
void create(fv_solver_t solver, int limiter_mode, bool allow_batch, fv_adjoint_t* out);
// Linearise at A->U (flux Jacobians, limiter values, residual fluxes and
// the local dt at the solver's CFL number).
void linearise(fv_adjoint_s* A);
// a.D = cfl / sum_f lambda_f |f| at the linearisation state.
void lin_dt(fv_adjoint_s* A, double cfl);
// R(U) at the linearisation state, device order.
void residual_dev(fv_adjoint_s* A, fvgb::St* R);
// dR = (dR/dU) dU at the linearisation state (freestream held fixed),
// device order in and out.
void jvp_dev(fv_adjoint_s* A, const fvgb::St* dU, fvgb::St* dR);
// out = (dR/dU)^T lam at the linearisation state, device order; also
// leaves the per-boundary-face freestream cotangents for fsbar().
void vjp_dev(fv_adjoint_s* A, const fvgb::St* lam, fvgb::St* out);
// reference-order host array <-> device-order state
void upload(fv_adjoint_s* A, const double* host_ref, fvgb::St* dev);
void download(fv_adjoint_s* A, const fvgb::St* dev, double* host_ref);
// (dR/dfs)^T lam per patch [4 n_patches] after vjp_dev(lam)
void fsbar(fv_adjoint_s* A, double* out);
}  // namespace adjh
