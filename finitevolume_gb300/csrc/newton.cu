// Newton-Krylov steady solver for the Euler residual (FP64, first or
// second order): pseudo-transient continuation with switched evolution
// relaxation, exact Jacobian-vector products and a block-Jacobi
// preconditioner.
//
// No reference counterpart: the reference advances its steady cases with
// the explicit loop only (EulerFVMSolver::step, src/EulerFVMSolver.cpp:
// 58-112).  The steady state solved for is the same discrete R(U) = 0 that
// loop drives to zero (its face and cell passes, extended to MUSCL in this
// library); only the path to it differs.
//
// Each Newton step, at the current state U:
//   - linearise R (the discrete adjoint's linearisation: per face the flux
//     Jacobians with respect to both reconstructed states, the limiter
//     values frozen or differentiated through their active branch);
//   - solve (V/dt - dR/dU) dU = R(U) by right-preconditioned GMRES(m),
//     with V/dt = sum_f lambda_f |f| / CFL_k (the primal's local time step)
//     and a CFL number that grows by a set factor after every step that
//     lowers the residual (so the iteration becomes Newton's method), holds
//     after a mild rise and halves after a larger one;
//   - the preconditioner works on the first-order part of that matrix:
//     per cell the 4x4 block V/dt I + sum_f +-J_f M_c (J_f the face's flux
//     Jacobian of this cell's side, M_c = dW/dU), inverted once per Newton
//     step, and per face the coupling to the neighbour's block.  It is
//     nu symmetric block Gauss-Seidel sweeps over a colouring of the cells
//     (no two neighbours share a colour, so each colour is one kernel that
//     updates its cells in place), by default on FP32 copies of the blocks
//     formed once per step (the sweeps only approximate the inverse; the
//     residual, the Jacobian-vector products and the Krylov vectors stay
//     FP64), or in FP64, or nu block-Jacobi sweeps;
//   - U += alpha dU, alpha <= 1 the largest step that changes no cell's
//     density or pressure by more than a set fraction (linear estimate).
// A step whose residual comes out more than ten times larger than the one
// before is undone and retried with the CFL number divided by four.
//
// Batched solvers are solved as one block-diagonal system: every instance
// (a contiguous cell range) has its own residual norms, CFL number, step
// length and accept / undo decision, and leaves the iteration once its
// density residual is below the tolerance; a single solver is one instance.
//
// Every reduction is a fixed-grid block sum folded in block order, so runs
// are bit reproducible.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <memory>
#include <string>
#include <vector>

#include "adjoint_internal.h"

#define FV_KNS nk
#include "euler_o1.cuh"
#undef FV_KNS

using fvgb::St;

namespace nk {

constexpr int kB = 256;
constexpr int kGrid = 1024;
inline int blocks(size_t n) { return (int)((n + kB - 1) / kB); }

__device__ __forceinline__ void prim_jac(const St& w, double g, double J[16]) {
    const double ir = 1.0 / w.r, gm1 = g - 1.0;
    const double u = w.ru, v = w.rv;  // W is stored as (rho, u, v, p)
    J[0] = 1.0; J[1] = 0.0; J[2] = 0.0; J[3] = 0.0;
    J[4] = -u * ir; J[5] = ir; J[6] = 0.0; J[7] = 0.0;
    J[8] = -v * ir; J[9] = 0.0; J[10] = ir; J[11] = 0.0;
    J[12] = 0.5 * gm1 * (u * u + v * v); J[13] = -gm1 * u; J[14] = -gm1 * v; J[15] = gm1;
}

// 4x4 inverse by Gauss-Jordan with partial pivoting (row-major).
__device__ __forceinline__ void inv4(double A[16], double X[16]) {
#pragma unroll
    for (int i = 0; i < 16; ++i) X[i] = (i % 5 == 0) ? 1.0 : 0.0;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        int p = c;
        double best = fabs(A[4 * c + c]);
#pragma unroll
        for (int r = c + 1; r < 4; ++r)
            if (fabs(A[4 * r + c]) > best) { best = fabs(A[4 * r + c]); p = r; }
        if (p != c)
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                double t = A[4 * c + k]; A[4 * c + k] = A[4 * p + k]; A[4 * p + k] = t;
                t = X[4 * c + k]; X[4 * c + k] = X[4 * p + k]; X[4 * p + k] = t;
            }
        const double d = 1.0 / A[4 * c + c];
#pragma unroll
        for (int k = 0; k < 4; ++k) { A[4 * c + k] *= d; X[4 * c + k] *= d; }
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            if (r == c) continue;
            const double m = A[4 * r + c];
#pragma unroll
            for (int k = 0; k < 4; ++k) { A[4 * r + k] -= m * A[4 * c + k]; X[4 * r + k] -= m * X[4 * c + k]; }
        }
    }
}

// Per cell: the inverse of V/dt I + sum_owner J_L M_c - sum_neighbour J_R M_c.
__global__ void k_pc_diag(const adjk::AdjArgs a, double* __restrict__ Dinv) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.n_cells) return;
    double S[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) S[i] = 0.0;
    for (int e = a.cf_off[c]; e < a.cf_off[c + 1]; ++e) {
        const int ent = a.cf[e];
        const int f = ent >> 1;
        const bool own = ent & 1;
        const double* J = own ? a.JL + 16 * (size_t)f : a.JR + 16 * (size_t)f;
        const double sg = own ? 1.0 : -1.0;
#pragma unroll
        for (int i = 0; i < 16; ++i) S[i] += sg * J[i];
    }
    double M[16];
    prim_jac(ld_state(a.W, c), a.gamma, M);
    double B[16];
    const double d = 1.0 / a.D[c];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            double t = (i == k) ? d : 0.0;
#pragma unroll
            for (int j = 0; j < 4; ++j) t += S[4 * i + j] * M[4 * j + k];
            B[4 * i + k] = t;
        }
    double X[16];
    inv4(B, X);
    double* o = Dinv + 16 * (size_t)c;
#pragma unroll
    for (int i = 0; i < 16; ++i) o[i] = X[i];
}

// y_c = M_c z_c
__global__ void k_mz(const adjk::AdjArgs a, const St* __restrict__ z, St* __restrict__ y) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.n_cells) return;
    double M[16];
    prim_jac(ld_state(a.W, c), a.gamma, M);
    const St u = ld_state(z, c);
    const double x[4] = {u.r, u.ru, u.rv, u.E};
    double o[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) o[i] = M[4 * i] * x[0] + M[4 * i + 1] * x[1] + M[4 * i + 2] * x[2] + M[4 * i + 3] * x[3];
    st_state(y, c, st_make(o[0], o[1], o[2], o[3]));
}

// One block-Jacobi sweep: z_c = Dinv_c (r_c - sum_nb P_c,nb z_nb) with the
// neighbour couplings P_c,nb = +J_R M_nb (c owns the face) or -J_L M_nb
// (c is its neighbour); Mz = M z of the previous sweep (null: first sweep
// from z = 0).
__global__ void k_jacobi(const adjk::AdjArgs a, const double* __restrict__ Dinv, const St* __restrict__ r,
                         const St* __restrict__ Mz, St* __restrict__ z) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.n_cells) return;
    const St rc = ld_state(r, c);
    double t[4] = {rc.r, rc.ru, rc.rv, rc.E};
    if (Mz) {
        for (int e = a.cf_off[c]; e < a.cf_off[c + 1]; ++e) {
            const int ent = a.cf[e];
            const int f = ent >> 1;
            const int L = a.fl[f], R = a.fr[f];
            if (R < 0) continue;
            const bool own = ent & 1;
            const int nb = own ? R : L;
            const double* J = own ? a.JR + 16 * (size_t)f : a.JL + 16 * (size_t)f;
            const double sg = own ? -1.0 : 1.0;
            const St q = ld_state(Mz, nb);
            const double y[4] = {q.r, q.ru, q.rv, q.E};
#pragma unroll
            for (int i = 0; i < 4; ++i)
                t[i] += sg * (J[4 * i] * y[0] + J[4 * i + 1] * y[1] + J[4 * i + 2] * y[2] + J[4 * i + 3] * y[3]);
        }
    }
    const double* X = Dinv + 16 * (size_t)c;
    double o[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) o[i] = X[4 * i] * t[0] + X[4 * i + 1] * t[1] + X[4 * i + 2] * t[2] + X[4 * i + 3] * t[3];
    st_state(z, c, st_make(o[0], o[1], o[2], o[3]));
}

// One colour of a block Gauss-Seidel sweep, in place: for the cells of
// this colour z_c = Dinv_c (r_c - sum_nb P_c,nb z_nb) with the current z of
// the neighbours (other colours) and M_nb formed from their primitives.
__global__ void k_gs_colour(const adjk::AdjArgs a, const double* __restrict__ Dinv, const St* __restrict__ r,
                            St* __restrict__ z, const int* __restrict__ cells, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = cells[i];
    const St rc = ld_state(r, c);
    double t[4] = {rc.r, rc.ru, rc.rv, rc.E};
    for (int e = a.cf_off[c]; e < a.cf_off[c + 1]; ++e) {
        const int ent = a.cf[e];
        const int f = ent >> 1;
        const int L = a.fl[f], R = a.fr[f];
        if (R < 0) continue;
        const bool own = ent & 1;
        const int nb = own ? R : L;
        const double* J = own ? a.JR + 16 * (size_t)f : a.JL + 16 * (size_t)f;
        const double sg = own ? -1.0 : 1.0;
        double M[16];
        prim_jac(ld_state(a.W, nb), a.gamma, M);
        const St q = ld_state(z, nb);
        const double x[4] = {q.r, q.ru, q.rv, q.E};
        double y[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) y[k] = M[4 * k] * x[0] + M[4 * k + 1] * x[1] + M[4 * k + 2] * x[2] + M[4 * k + 3] * x[3];
#pragma unroll
        for (int k = 0; k < 4; ++k)
            t[k] += sg * (J[4 * k] * y[0] + J[4 * k + 1] * y[1] + J[4 * k + 2] * y[2] + J[4 * k + 3] * y[3]);
    }
    const double* X = Dinv + 16 * (size_t)c;
    double o[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) o[k] = X[4 * k] * t[0] + X[4 * k + 1] * t[1] + X[4 * k + 2] * t[2] + X[4 * k + 3] * t[3];
    st_state(z, c, st_make(o[0], o[1], o[2], o[3]));
}

// One colour of a block Gauss-Seidel sweep of the transposed matrix, in
// place: z_c = Dinv_c^T (r_c - sum_nb (P^T)_c,nb z_nb) with
// (P^T)_c,nb = P_nb,c^T = -M_c^T J_L^T (c owns the face) or M_c^T J_R^T (c
// is its neighbour).
__global__ void k_gs_colour_t(const adjk::AdjArgs a, const double* __restrict__ Dinv, const St* __restrict__ r,
                              St* __restrict__ z, const int* __restrict__ cells, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = cells[i];
    double q[4] = {0.0, 0.0, 0.0, 0.0};
    for (int e = a.cf_off[c]; e < a.cf_off[c + 1]; ++e) {
        const int ent = a.cf[e];
        const int f = ent >> 1;
        const int L = a.fl[f], R = a.fr[f];
        if (R < 0) continue;
        const bool own = ent & 1;
        const int nb = own ? R : L;
        const double* J = own ? a.JL + 16 * (size_t)f : a.JR + 16 * (size_t)f;
        const double sg = own ? 1.0 : -1.0;
        const St zz = ld_state(z, nb);
        const double x[4] = {zz.r, zz.ru, zz.rv, zz.E};
#pragma unroll
        for (int k = 0; k < 4; ++k) q[k] += sg * (J[k] * x[0] + J[4 + k] * x[1] + J[8 + k] * x[2] + J[12 + k] * x[3]);
    }
    double M[16];
    prim_jac(ld_state(a.W, c), a.gamma, M);
    const St rc = ld_state(r, c);
    double t[4] = {rc.r, rc.ru, rc.rv, rc.E};
#pragma unroll
    for (int k = 0; k < 4; ++k) t[k] += M[k] * q[0] + M[4 + k] * q[1] + M[8 + k] * q[2] + M[12 + k] * q[3];
    const double* X = Dinv + 16 * (size_t)c;
    double o[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) o[k] = X[k] * t[0] + X[4 + k] * t[1] + X[8 + k] * t[2] + X[12 + k] * t[3];
    st_state(z, c, st_make(o[0], o[1], o[2], o[3]));
}

// ---- FP32 preconditioner (kind 2) -------------------------------------
// The Gauss-Seidel sweeps only have to approximate the inverse of the
// first-order PTC matrix, so they run on FP32 copies of its blocks: per
// cell-face entry e of cell c (neighbour nb across face f) the coupling
// block B_e = sg J M_nb of the forward sweep (16 floats), per cell Dinv.
// The sweeps then cost one 4x4 float block-vector product per neighbour,
// on the FP32 pipe, instead of forming M_nb and two FP64 products per
// neighbour and sweep; their input and output stay FP64 vectors.

// Per cell: the FP32 coupling blocks of its entries and its Dinv.
__global__ void k_pc_blocks(const adjk::AdjArgs a, const double* __restrict__ Dinv, float* __restrict__ B,
                            float* __restrict__ Dinvf) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.n_cells) return;
    for (int e = a.cf_off[c]; e < a.cf_off[c + 1]; ++e) {
        const int ent = a.cf[e];
        const int f = ent >> 1;
        const int L = a.fl[f], R = a.fr[f];
        float* o = B + 16 * (size_t)e;
        if (R < 0) {
#pragma unroll
            for (int i = 0; i < 16; ++i) o[i] = 0.0f;
            continue;
        }
        const bool own = ent & 1;
        const int nb = own ? R : L;
        const double* J = own ? a.JR + 16 * (size_t)f : a.JL + 16 * (size_t)f;
        const double sg = own ? -1.0 : 1.0;
        double M[16];
        prim_jac(ld_state(a.W, nb), a.gamma, M);
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                double t = 0.0;
#pragma unroll
                for (int j = 0; j < 4; ++j) t += J[4 * i + j] * M[4 * j + k];
                o[4 * i + k] = (float)(sg * t);
            }
    }
#pragma unroll
    for (int i = 0; i < 16; ++i) Dinvf[16 * (size_t)c + i] = (float)Dinv[16 * (size_t)c + i];
}

// One colour of a Gauss-Seidel sweep on the FP32 blocks, in place on the
// float iterate zf: t = r_c + sum_e B_e zf_nb, zf_c = Dinv_c t (TRANS: the
// transposed matrix, t = r_c + sum_e B_twin(e)^T zf_nb, zf_c = Dinv_c^T t).
template <bool TRANS>
__global__ void k_gs_colour_f(const adjk::AdjArgs a, const float* __restrict__ B, const int* __restrict__ twin,
                              const float* __restrict__ Dinvf, const St* __restrict__ r, float4* __restrict__ zf,
                              const int* __restrict__ cells, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = cells[i];
    const St rc = ld_state(r, c);
    float t[4] = {(float)rc.r, (float)rc.ru, (float)rc.rv, (float)rc.E};
    for (int e = a.cf_off[c]; e < a.cf_off[c + 1]; ++e) {
        const int ent = a.cf[e];
        const int f = ent >> 1;
        const int L = a.fl[f], R = a.fr[f];
        if (R < 0) continue;
        const int nb = (ent & 1) ? R : L;
        const float4 z = zf[nb];
        const float x[4] = {z.x, z.y, z.z, z.w};
        if (TRANS) {
            const float* Bt = B + 16 * (size_t)twin[e];
#pragma unroll
            for (int k = 0; k < 4; ++k) t[k] += Bt[k] * x[0] + Bt[4 + k] * x[1] + Bt[8 + k] * x[2] + Bt[12 + k] * x[3];
        } else {
            const float* Be = B + 16 * (size_t)e;
#pragma unroll
            for (int k = 0; k < 4; ++k)
                t[k] += Be[4 * k] * x[0] + Be[4 * k + 1] * x[1] + Be[4 * k + 2] * x[2] + Be[4 * k + 3] * x[3];
        }
    }
    const float* X = Dinvf + 16 * (size_t)c;
    float o[4];
#pragma unroll
    for (int k = 0; k < 4; ++k)
        o[k] = TRANS ? X[k] * t[0] + X[4 + k] * t[1] + X[8 + k] * t[2] + X[12 + k] * t[3]
                     : X[4 * k] * t[0] + X[4 * k + 1] * t[1] + X[4 * k + 2] * t[2] + X[4 * k + 3] * t[3];
    zf[c] = make_float4(o[0], o[1], o[2], o[3]);
}

// z = widened zf
__global__ void k_widen(St* __restrict__ z, const float4* __restrict__ zf, int n) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const float4 v = zf[c];
    st_state(z, c, st_make(v.x, v.y, v.z, v.w));
}

// out = -x
__global__ void k_neg(St* __restrict__ out, const St* __restrict__ x, int n) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const St a = ld_state(x, c);
    st_state(out, c, st_make(-a.r, -a.ru, -a.rv, -a.E));
}

// x += y
__global__ void k_axpy_state(St* __restrict__ x, const St* __restrict__ y, int n) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    st_state(x, c, ld_state(x, c) + ld_state(y, c));
}

// out = a + b
__global__ void k_add_state(St* __restrict__ out, const St* __restrict__ a, const St* __restrict__ b, int n) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    st_state(out, c, ld_state(a, c) + ld_state(b, c));
}

// out = a - b
__global__ void k_sub_state(St* __restrict__ out, const St* __restrict__ a, const St* __restrict__ b, int n) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    st_state(out, c, ld_state(a, c) - ld_state(b, c));
}

// w = x / D - Jx  (the PTC operator applied to x; D = dt / V)
__global__ void k_ptc(const double* __restrict__ D, const St* __restrict__ x, const St* __restrict__ Jx,
                      St* __restrict__ w, int n) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const double d = 1.0 / D[c];
    const St a = ld_state(x, c), b = ld_state(Jx, c);
    st_state(w, c, st_make(d * a.r - b.r, d * a.ru - b.ru, d * a.rv - b.rv, d * a.E - b.E));
}

__device__ __forceinline__ double block_sum(double t) {
    __shared__ double red[kB / 32];
    t = warp_sum(t);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
    __syncthreads();
    double v = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < kB / 32; ++w) v += red[w];
    return v;
}

// partials[i * gridDim.x + block] = block's part of <V_i, w>, i < nv
__global__ void __launch_bounds__(kB) k_mdot(const double* __restrict__ V, int nv, const double* __restrict__ w,
                                            size_t n, double* __restrict__ partials) {
    for (int i = 0; i < nv; ++i) {
        const double* v = V + (size_t)i * n;
        double t = 0.0;
        for (size_t k = blockIdx.x * (size_t)kB + threadIdx.x; k < n; k += (size_t)gridDim.x * kB) t += v[k] * w[k];
        const double s = block_sum(t);
        if (threadIdx.x == 0) partials[(size_t)i * gridDim.x + blockIdx.x] = s;
    }
}

// out[i] (+)= sum of partials row i (one block per row), sqrt when sq
__global__ void __launch_bounds__(kB) k_mfold(const double* __restrict__ partials, int nblk, double* __restrict__ out,
                                             int accumulate, int sq) {
    const int i = blockIdx.x;
    double t = 0.0;
    for (int b = threadIdx.x; b < nblk; b += kB) t += partials[(size_t)i * nblk + b];
    const double s = block_sum(t);
    if (threadIdx.x == 0) {
        const double v = sq ? sqrt(s) : s;
        out[i] = accumulate ? out[i] + v : v;
    }
}

// w -= sum_i h[i] V_i
__global__ void k_mupdate(double* __restrict__ w, const double* __restrict__ V, const double* __restrict__ h, int nv,
                          size_t n) {
    const size_t k = blockIdx.x * (size_t)kB + threadIdx.x;
    if (k >= n) return;
    double t = w[k];
    for (int i = 0; i < nv; ++i) t -= h[i] * V[(size_t)i * n + k];
    w[k] = t;
}

// out = x * s[0]^-1  (s a device scalar)
__global__ void k_scale_inv(double* __restrict__ out, const double* __restrict__ x, const double* __restrict__ s,
                            size_t n) {
    const size_t k = blockIdx.x * (size_t)kB + threadIdx.x;
    if (k < n) out[k] = x[k] / s[0];
}

// out = sum_i y[i] V_i
__global__ void k_combine(double* __restrict__ out, const double* __restrict__ V, const double* __restrict__ y, int nv,
                          size_t n) {
    const size_t k = blockIdx.x * (size_t)kB + threadIdx.x;
    if (k >= n) return;
    double t = 0.0;
    for (int i = 0; i < nv; ++i) t += y[i] * V[(size_t)i * n + k];
    out[k] = t;
}

// Per instance (one block per instance; instances are contiguous cell
// ranges, a single solver is one instance): the four residual L2 norms.
__global__ void __launch_bounds__(kB) k_inst_norm4(const St* __restrict__ R, const int* __restrict__ off,
                                                  double* __restrict__ out) {
    const int i = blockIdx.x;
    double t[4] = {0.0, 0.0, 0.0, 0.0};
    for (int c = off[i] + threadIdx.x; c < off[i + 1]; c += kB) {
        const St r = ld_state(R, c);
        t[0] += r.r * r.r; t[1] += r.ru * r.ru; t[2] += r.rv * r.rv; t[3] += r.E * r.E;
    }
    for (int k = 0; k < 4; ++k) {
        const double v = block_sum(t[k]);
        if (threadIdx.x == 0) out[4 * i + k] = sqrt(v);
    }
}

// Per instance: D *= cfl[i] (D formed at CFL 1), and a zero right-hand side
// for instances that take no step.
__global__ void __launch_bounds__(kB) k_inst_prepare(double* __restrict__ D, St* __restrict__ R,
                                                    const int* __restrict__ off, const double* __restrict__ cfl,
                                                    const int* __restrict__ mask) {
    const int i = blockIdx.x;
    const double k = cfl[i];
    const bool on = mask[i] != 0;
    for (int c = off[i] + threadIdx.x; c < off[i + 1]; c += kB) {
        D[c] *= k;
        if (!on) st_state(R, c, st_make(0.0, 0.0, 0.0, 0.0));
    }
}

// Per instance: the largest alpha <= 1 with no density or pressure of its
// cells falling by more than the fraction frac (linearised).
__global__ void __launch_bounds__(kB) k_inst_alpha(const adjk::AdjArgs a, const St* __restrict__ du,
                                                  const int* __restrict__ off, double frac,
                                                  double* __restrict__ alpha) {
    const int i = blockIdx.x;
    double amin = 1.0;
    for (int c = off[i] + threadIdx.x; c < off[i + 1]; c += kB) {
        const St w = ld_state(a.W, c);
        double M[16];
        prim_jac(w, a.gamma, M);
        const St u = ld_state(du, c);
        const double x[4] = {u.r, u.ru, u.rv, u.E};
        const double dr = x[0];
        const double dp = M[12] * x[0] + M[13] * x[1] + M[14] * x[2] + M[15] * x[3];
        if (dr < 0.0) amin = fmin(amin, frac * w.r / -dr);
        if (dp < 0.0) amin = fmin(amin, frac * w.E / -dp);  // W.E holds the pressure
        if (!isfinite(dr) || !isfinite(dp)) amin = 0.0;
    }
    amin = warp_min(amin);
    __shared__ double red[kB / 32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = amin;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = red[0];
        for (int w = 1; w < kB / 32; ++w) v = fmin(v, red[w]);
        alpha[i] = v;
    }
}

// Per instance: x *= s[i] (inverse: x /= s[i]).
__global__ void __launch_bounds__(kB) k_inst_scale(St* __restrict__ x, const int* __restrict__ off,
                                                  const double* __restrict__ s, int inverse) {
    const int i = blockIdx.x;
    const double k = s[i];
    for (int c = off[i] + threadIdx.x; c < off[i + 1]; c += kB) {
        const St v = ld_state(x, c);
        st_state(x, c, inverse ? st_make(v.r / k, v.ru / k, v.rv / k, v.E / k) : k * v);
    }
}

// Per instance: U += alpha[i] dU where mask[i]; U = Ubak where revert[i].
__global__ void __launch_bounds__(kB) k_inst_update(St* __restrict__ U, const St* __restrict__ du,
                                                   const St* __restrict__ Ubak, const int* __restrict__ off,
                                                   const double* __restrict__ alpha, const int* __restrict__ mask,
                                                   const int* __restrict__ revert) {
    const int i = blockIdx.x;
    const bool step = mask && mask[i], back = revert && revert[i];
    if (!step && !back) return;
    const double al = step ? alpha[i] : 0.0;
    for (int c = off[i] + threadIdx.x; c < off[i + 1]; c += kB) {
        if (back) st_state(U, c, ld_state(Ubak, c));
        else st_state(U, c, ld_state(U, c) + al * ld_state(du, c));
    }
}

}  // namespace nk

namespace {

// Relative GMRES residual of a Newton step's linear solve: at or below
// kRelGrow the CFL number may grow; above kRelFail it is halved.
constexpr double kRelGrow = 0.7;
constexpr double kRelFail = 0.9;
// Relative residual target of the inner GMRES cycle of an adjoint
// pseudo-transient iteration.
constexpr double kInnerRtol = 1e-2;

struct NewtonWork {
    int N = 0, m = 0;
    size_t n = 0;
    std::vector<void*> owned;
    double *V = nullptr, *Dinv = nullptr, *part = nullptr, *h = nullptr, *scal = nullptr;
    St *R = nullptr, *z = nullptr, *z2 = nullptr, *Mz = nullptr, *Jx = nullptr, *w = nullptr, *du = nullptr,
       *Ubak = nullptr, *tmp = nullptr, *zx = nullptr;
    int kind = 2;                   // preconditioner: 0 block Jacobi, 1 multicolour symmetric Gauss-Seidel
                                    // (FP64), 2 the same on FP32 blocks
    float* Bf = nullptr;            // kind 2: coupling blocks [16 E], Dinv [16 N], iterate [N]
    float* Dinvf = nullptr;
    float4* zf = nullptr;
    int* twin = nullptr;            // kind 2, transposed sweeps: the other entry of each entry's face
    int* colour_cells = nullptr;    // cells grouped by colour
    std::vector<int> colour_off;    // [n_colours + 1]
    ~NewtonWork() {
        for (void* p : owned) cudaFree(p);
    }
    template <typename T>
    T* alloc(size_t k) {
        void* p = nullptr;
        FV_CUDA(cudaMalloc(&p, sizeof(T) * (k ? k : 1)));
        owned.push_back(p);
        return static_cast<T*>(p);
    }
};

void check_launch() { FV_CUDA(cudaGetLastError()); }

// Greedy colouring of the cell graph (face neighbours) in device order:
// each cell takes the smallest colour none of its earlier neighbours has.
void colour_cells(const fvgb::Solver& s, NewtonWork& W, cudaStream_t st) {
    const int N = s.N, F = s.F;
    std::vector<int> off(N + 1), fl(F), fr(F);
    FV_CUDA(cudaMemcpyAsync(off.data(), s.dm.cf_off, sizeof(int) * (N + 1), cudaMemcpyDeviceToHost, st));
    FV_CUDA(cudaMemcpyAsync(fl.data(), s.dm.fl, sizeof(int) * F, cudaMemcpyDeviceToHost, st));
    FV_CUDA(cudaMemcpyAsync(fr.data(), s.dm.fr, sizeof(int) * F, cudaMemcpyDeviceToHost, st));
    FV_CUDA(cudaStreamSynchronize(st));
    std::vector<int> cf(off[N]);
    FV_CUDA(cudaMemcpyAsync(cf.data(), s.dm.cf, sizeof(int) * cf.size(), cudaMemcpyDeviceToHost, st));
    FV_CUDA(cudaStreamSynchronize(st));
    std::vector<int> col(N, -1);
    int nc = 0;
    std::vector<char> used;
    for (int c = 0; c < N; ++c) {
        used.assign(nc + 1, 0);
        for (int e = off[c]; e < off[c + 1]; ++e) {
            const int f = cf[e] >> 1;
            if (fr[f] < 0) continue;
            const int nb = fl[f] == c ? fr[f] : fl[f];
            if (col[nb] >= 0) used[col[nb]] = 1;
        }
        int k = 0;
        while (used[k]) ++k;
        col[c] = k;
        nc = std::max(nc, k + 1);
    }
    W.colour_off.assign(nc + 1, 0);
    for (int c = 0; c < N; ++c) ++W.colour_off[col[c] + 1];
    for (int k = 0; k < nc; ++k) W.colour_off[k + 1] += W.colour_off[k];
    std::vector<int> list(N), pos(W.colour_off.begin(), W.colour_off.end() - 1);
    for (int c = 0; c < N; ++c) list[pos[col[c]]++] = c;
    W.colour_cells = W.alloc<int>(N);
    fvgb::h2d_sync(W.colour_cells, list.data(), sizeof(int) * N, st);
}

// z = P^-1 r from z = 0: `sweeps` symmetric Gauss-Seidel sweeps (forward
// then backward over the colours), or `sweeps` block-Jacobi sweeps.
// Kind 2: `sweeps` symmetric Gauss-Seidel sweeps on the FP32 blocks (TRANS:
// of the transposed matrix), from zero, widened into z.
template <bool TRANS>
void precondition_f32(fv_adjoint_s* A, NewtonWork& W, const St* r, St* z, int sweeps, cudaStream_t s) {
    FV_CUDA(cudaMemsetAsync(W.zf, 0, sizeof(float4) * (size_t)W.N, s));
    const int nc = (int)W.colour_off.size() - 1;
    for (int sw = 0; sw < sweeps; ++sw)
        for (int pass = 0; pass < 2; ++pass)
            for (int q = 0; q < nc; ++q) {
                const int k = pass == 0 ? q : nc - 1 - q;
                const int n = W.colour_off[k + 1] - W.colour_off[k];
                if (n == 0) continue;
                nk::k_gs_colour_f<TRANS><<<nk::blocks(n), nk::kB, 0, s>>>(A->a, W.Bf, W.twin, W.Dinvf, r, W.zf,
                                                                          W.colour_cells + W.colour_off[k], n);
            }
    nk::k_widen<<<nk::blocks(W.N), nk::kB, 0, s>>>(z, W.zf, W.N);
    check_launch();
}

// The FP32 blocks of kind 2 (after k_pc_diag has formed Dinv).
void pc_blocks(fv_adjoint_s* A, NewtonWork& W, cudaStream_t s) {
    nk::k_pc_blocks<<<nk::blocks(W.N), nk::kB, 0, s>>>(A->a, W.Dinv, W.Bf, W.Dinvf);
    check_launch();
}

// Storage of kind 2 (and, with transposed sweeps, the entry twins).
void alloc_f32_pc(const fvgb::Solver& s, NewtonWork& W, bool twins, cudaStream_t st) {
    const int N = s.N, F = s.F;
    std::vector<int> off(N + 1);
    FV_CUDA(cudaMemcpyAsync(off.data(), s.dm.cf_off, sizeof(int) * (N + 1), cudaMemcpyDeviceToHost, st));
    FV_CUDA(cudaStreamSynchronize(st));
    const size_t E = (size_t)off[N];
    W.Bf = W.alloc<float>(16 * E);
    W.Dinvf = W.alloc<float>(16 * (size_t)N);
    W.zf = W.alloc<float4>(N);
    if (!twins) return;
    std::vector<int> cf(E), tw(E, -1), first(F, -1);
    FV_CUDA(cudaMemcpyAsync(cf.data(), s.dm.cf, sizeof(int) * E, cudaMemcpyDeviceToHost, st));
    FV_CUDA(cudaStreamSynchronize(st));
    for (size_t e = 0; e < E; ++e) {
        const int f = cf[e] >> 1;
        if (first[f] < 0) first[f] = (int)e;
        else {
            tw[e] = first[f];
            tw[first[f]] = (int)e;
        }
    }
    W.twin = W.alloc<int>(E);
    fvgb::h2d_sync(W.twin, tw.data(), sizeof(int) * E, st);
}

void precondition(fv_adjoint_s* A, NewtonWork& W, const St* r, St* z, int sweeps, cudaStream_t s) {
    if (W.kind == 2) {
        precondition_f32<false>(A, W, r, z, sweeps, s);
        return;
    }
    if (W.kind == 1) {
        FV_CUDA(cudaMemsetAsync(z, 0, sizeof(St) * (size_t)W.N, s));
        const int nc = (int)W.colour_off.size() - 1;
        for (int sw = 0; sw < sweeps; ++sw)
            for (int pass = 0; pass < 2; ++pass)
                for (int q = 0; q < nc; ++q) {
                    const int k = pass == 0 ? q : nc - 1 - q;
                    const int n = W.colour_off[k + 1] - W.colour_off[k];
                    if (n == 0) continue;
                    nk::k_gs_colour<<<nk::blocks(n), nk::kB, 0, s>>>(A->a, W.Dinv, r, z,
                                                                     W.colour_cells + W.colour_off[k], n);
                }
        check_launch();
        return;
    }
    const int nb = nk::blocks(W.N);
    nk::k_jacobi<<<nb, nk::kB, 0, s>>>(A->a, W.Dinv, r, nullptr, z);
    check_launch();
    for (int i = 1; i < sweeps; ++i) {
        nk::k_mz<<<nb, nk::kB, 0, s>>>(A->a, z, W.Mz);
        nk::k_jacobi<<<nb, nk::kB, 0, s>>>(A->a, W.Dinv, r, W.Mz, W.z2);
        check_launch();
        FV_CUDA(cudaMemcpyAsync(z, W.z2, sizeof(St) * (size_t)W.N, cudaMemcpyDeviceToDevice, s));
    }
}

// z = P^-T r from z = 0: `sweeps` symmetric Gauss-Seidel sweeps of the
// transposed matrix over the colours.
void precondition_t(fv_adjoint_s* A, NewtonWork& W, const St* r, St* z, int sweeps, cudaStream_t s) {
    if (W.kind == 2) {
        precondition_f32<true>(A, W, r, z, sweeps, s);
        return;
    }
    FV_CUDA(cudaMemsetAsync(z, 0, sizeof(St) * (size_t)W.N, s));
    const int nc = (int)W.colour_off.size() - 1;
    for (int sw = 0; sw < sweeps; ++sw)
        for (int pass = 0; pass < 2; ++pass)
            for (int q = 0; q < nc; ++q) {
                const int k = pass == 0 ? q : nc - 1 - q;
                const int n = W.colour_off[k + 1] - W.colour_off[k];
                if (n == 0) continue;
                nk::k_gs_colour_t<<<nk::blocks(n), nk::kB, 0, s>>>(A->a, W.Dinv, r, z, W.colour_cells + W.colour_off[k],
                                                                   n);
            }
    check_launch();
}

// out[0..nv) = <V_i, w> (device), folded deterministically
void mdot(NewtonWork& W, const double* V, int nv, const double* w, double* out, bool accumulate, cudaStream_t s) {
    const int grid = (int)std::min<size_t>(nk::kGrid, (W.n + nk::kB - 1) / nk::kB);
    nk::k_mdot<<<grid, nk::kB, 0, s>>>(V, nv, w, W.n, W.part);
    nk::k_mfold<<<nv, nk::kB, 0, s>>>(W.part, grid, out, accumulate ? 1 : 0, 0);
    check_launch();
}

double norm2(NewtonWork& W, const double* x, double* dev_out, cudaStream_t s) {
    const int grid = (int)std::min<size_t>(nk::kGrid, (W.n + nk::kB - 1) / nk::kB);
    nk::k_mdot<<<grid, nk::kB, 0, s>>>(x, 1, x, W.n, W.part);
    nk::k_mfold<<<1, nk::kB, 0, s>>>(W.part, grid, dev_out, 0, 1);
    check_launch();
    double v = 0.0;
    FV_CUDA(cudaMemcpyAsync(&v, dev_out, sizeof(double), cudaMemcpyDeviceToHost, s));
    FV_CUDA(cudaStreamSynchronize(s));
    return v;
}

// Right-preconditioned restarted GMRES on A x = b from the x given (zero
// when x0_zero), at most max_mv applications of A, until the residual is
// below rtol times |b|.  op(z, w): w = A z; pc(v, z): z = P^-1 v.  Returns
// the matvec count; *rel the last relative residual estimate.
template <class Op, class Pc>
int gmres_gen(NewtonWork& W, const St* b, St* x, bool x0_zero, int m, int max_mv, double rtol, double* rel,
              cudaStream_t s, Op op, Pc pc) {
    const size_t n = W.n;
    const int vb = (int)((n + nk::kB - 1) / nk::kB);
    auto V = [&](int i) { return W.V + (size_t)i * n; };
    double* wv = reinterpret_cast<double*>(W.w);
    FV_CUDA(cudaMemcpyAsync(W.tmp, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    const double bnorm = norm2(W, reinterpret_cast<const double*>(W.tmp), W.scal, s);
    *rel = 1.0;
    if (x0_zero) FV_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, s));
    if (!(bnorm > 0.0) || !std::isfinite(bnorm)) {
        FV_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, s));
        return 0;
    }
    std::vector<double> H((size_t)(m + 1) * m, 0.0), cs(m), sn(m), g(m + 1, 0.0), y(m), hc(m + 2);
    int mv = 0;
    bool first = true;
    while (mv < max_mv) {
        // r = b - A x (x = 0 on the first cycle from zero)
        if (first && x0_zero) {
            FV_CUDA(cudaMemcpyAsync(V(0), b, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
        } else {
            op(x, W.Jx);
            ++mv;
            nk::k_sub_state<<<nk::blocks(W.N), nk::kB, 0, s>>>(reinterpret_cast<St*>(V(0)), b, W.Jx, W.N);
            check_launch();
        }
        first = false;
        const double beta = norm2(W, V(0), W.scal, s);
        if (!std::isfinite(beta)) fvgb::raise(FV_ERR_NONFINITE, "GMRES: non-finite residual");
        *rel = beta / bnorm;
        if (*rel <= rtol || mv >= max_mv) break;
        nk::k_scale_inv<<<vb, nk::kB, 0, s>>>(V(0), V(0), W.scal, n);
        check_launch();
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        int k = 0;
        for (int j = 0; j < m && mv < max_mv; ++j) {
            pc(reinterpret_cast<const St*>(V(j)), W.z);
            op(W.z, W.w);
            ++mv;
            // classical Gram-Schmidt, twice
            mdot(W, W.V, j + 1, wv, W.h, false, s);
            nk::k_mupdate<<<vb, nk::kB, 0, s>>>(wv, W.V, W.h, j + 1, n);
            mdot(W, W.V, j + 1, wv, W.h + m + 2, false, s);
            nk::k_mupdate<<<vb, nk::kB, 0, s>>>(wv, W.V, W.h + m + 2, j + 1, n);
            check_launch();
            std::vector<double> h1(j + 1), h2(j + 1);
            FV_CUDA(cudaMemcpyAsync(h1.data(), W.h, sizeof(double) * (j + 1), cudaMemcpyDeviceToHost, s));
            FV_CUDA(cudaMemcpyAsync(h2.data(), W.h + m + 2, sizeof(double) * (j + 1), cudaMemcpyDeviceToHost, s));
            const double hn = norm2(W, wv, W.scal, s);
            for (int i = 0; i <= j; ++i) hc[i] = h1[i] + h2[i];
            hc[j + 1] = hn;
            for (int i = 0; i <= j + 1; ++i)
                if (!std::isfinite(hc[i])) fvgb::raise(FV_ERR_NONFINITE, "GMRES: non-finite Krylov vector");
            if (hn > 0.0) {
                nk::k_scale_inv<<<vb, nk::kB, 0, s>>>(V(j + 1), wv, W.scal, n);
                check_launch();
            }
            for (int i = 0; i < j; ++i) {
                const double t = cs[i] * hc[i] + sn[i] * hc[i + 1];
                hc[i + 1] = -sn[i] * hc[i] + cs[i] * hc[i + 1];
                hc[i] = t;
            }
            const double den = std::hypot(hc[j], hc[j + 1]);
            cs[j] = den > 0.0 ? hc[j] / den : 1.0;
            sn[j] = den > 0.0 ? hc[j + 1] / den : 0.0;
            hc[j] = den;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            for (int i = 0; i <= j; ++i) H[(size_t)i * m + j] = hc[i];
            k = j + 1;
            *rel = std::fabs(g[j + 1]) / bnorm;
            if (*rel <= rtol || !(hn > 0.0)) break;
        }
        for (int i = k - 1; i >= 0; --i) {
            double t = g[i];
            for (int l = i + 1; l < k; ++l) t -= H[(size_t)i * m + l] * y[l];
            y[i] = t / H[(size_t)i * m + i];
        }
        // x += P^-1 (V y)
        FV_CUDA(cudaMemcpyAsync(W.h, y.data(), sizeof(double) * k, cudaMemcpyHostToDevice, s));
        nk::k_combine<<<vb, nk::kB, 0, s>>>(reinterpret_cast<double*>(W.tmp), W.V, W.h, k, n);
        check_launch();
        pc(W.tmp, W.zx);
        nk::k_axpy_state<<<nk::blocks(W.N), nk::kB, 0, s>>>(x, W.zx, W.N);
        check_launch();
        FV_CUDA(cudaStreamSynchronize(s));
        if (*rel <= rtol) break;
    }
    return mv;
}

// One GMRES(m) cycle from x = 0 on the Newton system (V/dt - J) x = b.
int gmres(fv_adjoint_s* A, NewtonWork& W, const St* b, St* x, int m, double rtol, int sweeps, double* rel,
          cudaStream_t s) {
    auto op = [&](const St* z, St* w) {
        adjh::jvp_dev(A, z, W.Jx);
        nk::k_ptc<<<nk::blocks(W.N), nk::kB, 0, s>>>(A->a.D, z, W.Jx, w, W.N);
        check_launch();
    };
    auto pc = [&](const St* v, St* z) { precondition(A, W, v, z, sweeps, s); };
    return gmres_gen(W, b, x, true, m, m, rtol, rel, s, op, pc);
}

}  // namespace

extern "C" {

void fv_newton_default(fv_newton_t* o) {
    if (!o) return;
    o->limiter_mode = FV_ADJ_FROZEN_LIMITER;
    o->max_newton = 200;
    o->tol = 1e-11;
    o->cfl0 = 10.0;
    o->cfl_max = 1e6;
    o->cfl_growth = 1.5;
    o->krylov_dim = 80;
    o->krylov_rtol = 1e-2;
    o->precond_sweeps = 8;
    o->precond_kind = 2;
    o->max_rel_change = 0.2;
}

int fv_steady_newton(fv_solver_t solver, const fv_newton_t* opt, double* history, int32_t* iterations,
                     int32_t* instance_steps) {
    return fvgb::guarded([&] {
        if (!solver || !opt) fvgb::raise(FV_ERR_BAD_ARG, "null argument");
        const fv_newton_t o = *opt;
        if (o.max_newton < 0 || !(o.tol >= 0.0) || !(o.cfl0 > 0.0) || !(o.cfl_max >= o.cfl0) ||
            !(o.cfl_growth >= 1.0) || o.krylov_dim < 1 || o.krylov_dim > 200 || !(o.krylov_rtol > 0.0) ||
            o.precond_sweeps < 1 || o.precond_kind < 0 || o.precond_kind > 2 || !(o.max_rel_change > 0.0))
            fvgb::raise(FV_ERR_BAD_ARG, "fv_steady_newton: bad options");
        fvgb::Solver& s = solver->s;
        fv_adjoint_t Ah = nullptr;
        adjh::create(solver, o.limiter_mode, true, &Ah);
        std::unique_ptr<fv_adjoint_s> A(Ah);
        cudaStream_t st = s.stream;
        NewtonWork W;
        W.N = s.N;
        W.n = 4 * (size_t)s.N;
        W.m = o.krylov_dim;
        W.V = W.alloc<double>((size_t)(o.krylov_dim + 1) * W.n);
        W.Dinv = W.alloc<double>(16 * (size_t)s.N);
        W.part = W.alloc<double>((size_t)nk::kGrid * std::max(o.krylov_dim + 2, 4));
        W.h = W.alloc<double>(2 * (size_t)(o.krylov_dim + 2));
        W.scal = W.alloc<double>(8);
        W.R = W.alloc<St>(s.N);
        W.z = W.alloc<St>(s.N);
        W.z2 = W.alloc<St>(s.N);
        W.Mz = W.alloc<St>(s.N);
        W.Jx = W.alloc<St>(s.N);
        W.w = W.alloc<St>(s.N);
        W.du = W.alloc<St>(s.N);
        W.Ubak = W.alloc<St>(s.N);
        W.tmp = W.alloc<St>(s.N);
        W.zx = W.alloc<St>(s.N);
        W.kind = o.precond_kind;
        if (W.kind >= 1) colour_cells(s, W, st);
        if (W.kind == 2) alloc_f32_pc(s, W, false, st);
        // instances: contiguous cell ranges (a single solver is one)
        const std::vector<int> off = s.batch ? std::vector<int>(s.group_off.begin(), s.group_off.end())
                                             : std::vector<int>{0, s.N};
        const int ni = (int)off.size() - 1;
        int* d_off = W.alloc<int>(ni + 1);
        fvgb::h2d_sync(d_off, off.data(), sizeof(int) * (ni + 1), st);
        double* d_nrm = W.alloc<double>(4 * (size_t)ni);
        double* d_cfl = W.alloc<double>(ni);
        double* d_alpha = W.alloc<double>(ni);
        int* d_mask = W.alloc<int>(ni);
        int* d_revert = W.alloc<int>(ni);
        double* d_scale = W.alloc<double>(ni);
        std::vector<double> scale(ni, 1.0);
        std::vector<double> nr(4 * (size_t)ni), prev(ni, -1.0), cfl(ni, o.cfl0), last_cfl(ni, 0.0), alpha(ni, 0.0);
        std::vector<int> stepped(ni, 0), rejects(ni, 0), mask(ni, 0), revert(ni, 0), conv_at(ni, -1);
        FV_CUDA(cudaStreamSynchronize(st));
        int it = 0;
        double last_rel = 0.0;
        int last_mv = 0;
        for (;;) {
            FV_CUDA(cudaMemcpyAsync(A->U, s.U, sizeof(St) * (size_t)s.N, cudaMemcpyDeviceToDevice, st));
            adjh::linearise(A.get());
            adjh::residual_dev(A.get(), W.R);
            nk::k_inst_norm4<<<ni, nk::kB, 0, st>>>(W.R, d_off, d_nrm);
            check_launch();
            FV_CUDA(cudaMemcpyAsync(nr.data(), d_nrm, sizeof(double) * nr.size(), cudaMemcpyDeviceToHost, st));
            FV_CUDA(cudaStreamSynchronize(st));
            // per instance: accept the last step (adapt its CFL number) or undo it
            bool any_revert = false;
            for (int i = 0; i < ni; ++i) {
                revert[i] = 0;
                const double r = nr[4 * i], e = nr[4 * i + 3];
                if (it == 0 && (!std::isfinite(r) || !std::isfinite(e)))
                    fvgb::raise(FV_ERR_NONFINITE, "fv_steady_newton: non-finite residual at the start");
                if (!stepped[i]) {
                    if (prev[i] < 0.0) prev[i] = r;
                    continue;
                }
                stepped[i] = 0;
                const double ratio = r / prev[i];
                if ((!(ratio <= 10.0) || !std::isfinite(e)) && rejects[i] < 10) {
                    revert[i] = 1;
                    any_revert = true;
                    cfl[i] = std::max(o.cfl0 * 1e-3, 0.25 * last_cfl[i]);
                    ++rejects[i];
                    continue;
                }
                rejects[i] = 0;
                // The CFL number grows only after a step that lowered the
                // residual, was taken in full and came from a linear solve
                // that reduced its residual at least to kRelGrow; a linear
                // solve that made no headway (above kRelFail) halves it, as
                // a large rise does.  Without the linear test the CFL number
                // keeps growing on tiny decreases while GMRES no longer
                // solves the system at all, and the iteration stalls there.
                const bool lin_ok = last_rel <= kRelGrow, lin_fail = last_rel > kRelFail;
                if (ratio < 1.0 && lin_ok && alpha[i] >= 1.0) cfl[i] = std::min(o.cfl_max, last_cfl[i] * o.cfl_growth);
                else if (ratio < 2.0 && !lin_fail) cfl[i] = last_cfl[i];
                else cfl[i] = std::max(o.cfl0 * 1e-3, 0.5 * last_cfl[i]);
                prev[i] = r;
            }
            if (any_revert) {
                // undo those instances' steps and evaluate again
                FV_CUDA(cudaMemcpyAsync(d_revert, revert.data(), sizeof(int) * ni, cudaMemcpyHostToDevice, st));
                nk::k_inst_update<<<ni, nk::kB, 0, st>>>(s.U, W.du, W.Ubak, d_off, d_alpha, nullptr, d_revert);
                check_launch();
                continue;
            }
            // history: norms over all instances, largest CFL, smallest step length
            int active = 0;
            for (int i = 0; i < ni; ++i) {
                mask[i] = prev[i] >= o.tol ? 1 : 0;
                if (!mask[i] && conv_at[i] < 0) conv_at[i] = it;
                active += mask[i];
            }
            if (history) {
                double* row = history + 8 * (size_t)it;
                for (int q = 0; q < 4; ++q) {
                    double t = 0.0;
                    for (int i = 0; i < ni; ++i) t += nr[4 * i + q] * nr[4 * i + q];
                    row[q] = std::sqrt(t);
                }
                double cmax = 0.0, amin = it ? 1.0 : 0.0;
                for (int i = 0; i < ni; ++i) {
                    cmax = std::max(cmax, it ? last_cfl[i] : 0.0);
                    if (it) amin = std::min(amin, alpha[i]);
                }
                row[4] = cmax;
                row[5] = last_mv;
                row[6] = last_rel;
                row[7] = amin;
            }
            if (active == 0 || it >= o.max_newton) break;
            // the step: (V/dt - J) dU = R per instance at its own CFL number
            FV_CUDA(cudaMemcpyAsync(d_cfl, cfl.data(), sizeof(double) * ni, cudaMemcpyHostToDevice, st));
            FV_CUDA(cudaMemcpyAsync(d_mask, mask.data(), sizeof(int) * ni, cudaMemcpyHostToDevice, st));
            adjh::lin_dt(A.get(), 1.0);
            nk::k_inst_prepare<<<ni, nk::kB, 0, st>>>(A->a.D, W.R, d_off, d_cfl, d_mask);
            nk::k_pc_diag<<<nk::blocks(s.N), nk::kB, 0, st>>>(A->a, W.Dinv);
            check_launch();
            if (W.kind == 2) pc_blocks(A.get(), W, st);
            // The system is block diagonal over the instances, so scaling an
            // instance's right-hand side scales only its own solution.  Each
            // is scaled to unit norm before GMRES (and its solution back
            // after): the minimisation then weighs every instance's
            // equations alike instead of being dominated by the instances
            // with the largest residuals.  One instance: a no-op up to
            // rounding.
            for (int i = 0; i < ni; ++i) {
                const double r2 = nr[4 * i] * nr[4 * i] + nr[4 * i + 1] * nr[4 * i + 1] +
                                  nr[4 * i + 2] * nr[4 * i + 2] + nr[4 * i + 3] * nr[4 * i + 3];
                scale[i] = (mask[i] && r2 > 0.0 && std::isfinite(r2)) ? 1.0 / std::sqrt(r2) : 1.0;
            }
            if (ni > 1) {
                FV_CUDA(cudaMemcpyAsync(d_scale, scale.data(), sizeof(double) * ni, cudaMemcpyHostToDevice, st));
                nk::k_inst_scale<<<ni, nk::kB, 0, st>>>(W.R, d_off, d_scale, 0);
                check_launch();
            }
            double rel = 0.0;
            const int mv = gmres(A.get(), W, W.R, W.du, o.krylov_dim, o.krylov_rtol, o.precond_sweeps, &rel, st);
            if (ni > 1) {
                nk::k_inst_scale<<<ni, nk::kB, 0, st>>>(W.du, d_off, d_scale, 1);
                check_launch();
            }
            nk::k_inst_alpha<<<ni, nk::kB, 0, st>>>(A->a, W.du, d_off, o.max_rel_change, d_alpha);
            check_launch();
            FV_CUDA(cudaMemcpyAsync(alpha.data(), d_alpha, sizeof(double) * ni, cudaMemcpyDeviceToHost, st));
            FV_CUDA(cudaMemcpyAsync(W.Ubak, s.U, sizeof(St) * (size_t)s.N, cudaMemcpyDeviceToDevice, st));
            nk::k_inst_update<<<ni, nk::kB, 0, st>>>(s.U, W.du, W.Ubak, d_off, d_alpha, d_mask, nullptr);
            check_launch();
            FV_CUDA(cudaStreamSynchronize(st));
            for (int i = 0; i < ni; ++i) {
                stepped[i] = mask[i];
                if (mask[i]) last_cfl[i] = cfl[i];
            }
            last_rel = rel;
            last_mv = mv;
            ++it;
        }
        if (iterations) *iterations = it;
        if (instance_steps)
            for (int i = 0; i < ni; ++i) instance_steps[i] = conv_at[i];
        s.refresh_primitives();
        FV_CUDA(cudaStreamSynchronize(st));
    });
}

int fv_adjoint_solve_krylov(fv_adjoint_t A, const double* dJdU, double cfl, int32_t restart, int32_t max_matvec,
                            double rtol, int32_t precond_sweeps, double* lambda, double* fsbar, double* history,
                            int32_t* matvecs, double residual[4]) {
    return fvgb::guarded([&] {
        if (!A || !dJdU || !(cfl > 0.0) || restart < 1 || restart > 200 || max_matvec < 1 || !(rtol > 0.0) ||
            precond_sweeps < 1)
            fvgb::raise(FV_ERR_BAD_ARG, "fv_adjoint_solve_krylov: bad argument");
        if (!A->linearised) fvgb::raise(FV_ERR_BAD_ARG, "call fv_residual_forward first");
        fvgb::Solver& s = A->solver->s;
        cudaStream_t st = s.stream;
        NewtonWork W;
        W.N = s.N;
        W.n = 4 * (size_t)s.N;
        W.m = restart;
        W.V = W.alloc<double>((size_t)(restart + 1) * W.n);
        W.Dinv = W.alloc<double>(16 * (size_t)s.N);
        W.part = W.alloc<double>((size_t)nk::kGrid * std::max(restart + 2, 4));
        W.h = W.alloc<double>(2 * (size_t)(restart + 2));
        W.scal = W.alloc<double>(8);
        W.R = W.alloc<St>(s.N);
        W.z = W.alloc<St>(s.N);
        W.z2 = W.alloc<St>(s.N);
        W.Mz = W.alloc<St>(s.N);
        W.Jx = W.alloc<St>(s.N);
        W.w = W.alloc<St>(s.N);
        W.du = W.alloc<St>(s.N);
        W.tmp = W.alloc<St>(s.N);
        W.zx = W.alloc<St>(s.N);
        colour_cells(s, W, st);
        W.kind = 2;
        alloc_f32_pc(s, W, true, st);
        // the preconditioner's pseudo time step; the primal's is restored after
        const double cfl_primal = A->a.cfl;
        adjh::lin_dt(A, cfl);
        nk::k_pc_diag<<<nk::blocks(s.N), nk::kB, 0, st>>>(A->a, W.Dinv);
        check_launch();
        pc_blocks(A, W, st);
        // -(dR/dU)^T lam = -dJ/dU
        adjh::upload(A, dJdU, W.du);
        nk::k_neg<<<nk::blocks(s.N), nk::kB, 0, st>>>(W.R, W.du, s.N);
        check_launch();
        // With A = -dR/dU the adjoint system is A^T lam = b, b = -dJ/dU.
        // Pseudo-transient outer iterations: (V/dt + A)^T delta = b - A^T lam
        // by one GMRES(restart) cycle, lam += delta; the shifted operator is
        // the transpose of the primal Newton system, so the iteration
        // contracts like the primal's steps at the same CFL number.
        auto op = [&](const St* z, St* w) {
            adjh::vjp_dev(A, z, W.Jx);
            nk::k_ptc<<<nk::blocks(W.N), nk::kB, 0, st>>>(A->a.D, z, W.Jx, w, W.N);
            check_launch();
        };
        auto pc = [&](const St* v, St* z) { precondition_t(A, W, v, z, precond_sweeps, st); };
        St* r = W.z2;
        St* delta = W.Mz;
        const double bnorm = norm2(W, reinterpret_cast<const double*>(W.R), W.scal, st);
        double rel = 1.0;
        // history: relative residual |b - A^T lam| / |b| before every outer iteration
        std::vector<double> hh;
        int mv = 0;
        FV_CUDA(cudaMemsetAsync(A->lam, 0, sizeof(St) * (size_t)s.N, st));
        while (bnorm > 0.0) {
            // r = b - A^T lam = b + (dR/dU)^T lam
            adjh::vjp_dev(A, A->lam, W.Jx);
            nk::k_add_state<<<nk::blocks(s.N), nk::kB, 0, st>>>(r, W.R, W.Jx, s.N);
            check_launch();
            ++mv;
            rel = norm2(W, reinterpret_cast<const double*>(r), W.scal, st) / bnorm;
            if (!std::isfinite(rel)) fvgb::raise(FV_ERR_NONFINITE, "fv_adjoint_solve_krylov: non-finite residual");
            hh.push_back(rel);
            if (rel <= rtol || mv >= max_matvec) break;
            double rin = 1.0;
            const int k = gmres_gen(W, r, delta, true, restart, std::min(restart, max_matvec - mv), kInnerRtol, &rin,
                                    st, op, pc);
            mv += k;
            nk::k_axpy_state<<<nk::blocks(s.N), nk::kB, 0, st>>>(A->lam, delta, s.N);
            check_launch();
            if (k == 0) break;
        }
        adjh::lin_dt(A, cfl_primal);
        // residual of (dR/dU)^T lam - dJ/dU, per component
        adjh::vjp_dev(A, A->lam, W.Jx);
        nk::k_sub_state<<<nk::blocks(s.N), nk::kB, 0, st>>>(W.z, W.Jx, W.du, s.N);
        int* d_off = W.alloc<int>(2);
        const int off[2] = {0, s.N};
        fvgb::h2d_sync(d_off, off, sizeof(off), st);
        nk::k_inst_norm4<<<1, nk::kB, 0, st>>>(W.z, d_off, W.scal);
        check_launch();
        double r4[4];
        FV_CUDA(cudaMemcpyAsync(r4, W.scal, sizeof(r4), cudaMemcpyDeviceToHost, st));
        FV_CUDA(cudaStreamSynchronize(st));
        if (residual)
            for (int q = 0; q < 4; ++q) residual[q] = r4[q];
        if (matvecs) *matvecs = mv;
        if (history)
            for (size_t i = 0; i < hh.size(); ++i) history[i] = hh[i];
        A->solved = true;
        if (lambda) adjh::download(A, A->lam, lambda);
        if (fsbar) {
            adjh::vjp_dev(A, A->lam, W.Jx);
            adjh::fsbar(A, fsbar);
        }
        FV_CUDA(cudaStreamSynchronize(st));
    });
}

}  // extern "C"
