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
//     updates its cells in place), or nu block-Jacobi sweeps;
//   - U += alpha dU, alpha <= 1 the largest step that changes no cell's
//     density or pressure by more than a set fraction (linear estimate).
// A step whose residual comes out more than ten times larger than the one
// before is undone and retried with the CFL number divided by four.
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

// Per block: the four squared residual sums; one fold per component.
__global__ void __launch_bounds__(kB) k_norm4(const St* __restrict__ R, int n, double* __restrict__ partials) {
    double t[4] = {0.0, 0.0, 0.0, 0.0};
    for (int c = blockIdx.x * kB + threadIdx.x; c < n; c += gridDim.x * kB) {
        const St r = ld_state(R, c);
        t[0] += r.r * r.r; t[1] += r.ru * r.ru; t[2] += r.rv * r.rv; t[3] += r.E * r.E;
    }
    for (int k = 0; k < 4; ++k) {
        const double s = block_sum(t[k]);
        if (threadIdx.x == 0) partials[(size_t)k * gridDim.x + blockIdx.x] = s;
    }
}

// Largest alpha <= 1 with no density or pressure falling by more than the
// fraction frac (linearised: dW = M dU); block minima, then one fold.
__global__ void __launch_bounds__(kB) k_alpha(const adjk::AdjArgs a, const St* __restrict__ du, double frac,
                                             double* __restrict__ partials) {
    double amin = 1.0;
    for (int c = blockIdx.x * kB + threadIdx.x; c < a.n_cells; c += gridDim.x * kB) {
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
        partials[blockIdx.x] = v;
    }
}

__global__ void __launch_bounds__(kB) k_min_fold(const double* __restrict__ partials, int nblk, double* __restrict__ out) {
    double v = DBL_MAX;
    for (int b = threadIdx.x; b < nblk; b += kB) v = fmin(v, partials[b]);
    v = warp_min(v);
    __shared__ double red[kB / 32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = red[0];
        for (int w = 1; w < kB / 32; ++w) m = fmin(m, red[w]);
        out[0] = m;
    }
}

// U += alpha dU
__global__ void k_update(St* __restrict__ U, const St* __restrict__ du, double alpha, int n) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    st_state(U, c, ld_state(U, c) + alpha * ld_state(du, c));
}

}  // namespace nk

namespace {

struct NewtonWork {
    int N = 0, m = 0;
    size_t n = 0;
    std::vector<void*> owned;
    double *V = nullptr, *Dinv = nullptr, *part = nullptr, *h = nullptr, *scal = nullptr;
    St *R = nullptr, *z = nullptr, *z2 = nullptr, *Mz = nullptr, *Jx = nullptr, *w = nullptr, *du = nullptr,
       *Ubak = nullptr, *tmp = nullptr;
    int kind = 1;                   // preconditioner: 0 block Jacobi, 1 multicolour symmetric Gauss-Seidel
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
void precondition(fv_adjoint_s* A, NewtonWork& W, const St* r, St* z, int sweeps, cudaStream_t s) {
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

void residual_norms(fv_adjoint_s* A, NewtonWork& W, double out[4], cudaStream_t s) {
    const int grid = std::min(nk::kGrid, nk::blocks(W.N));
    nk::k_norm4<<<grid, nk::kB, 0, s>>>(W.R, W.N, W.part);
    nk::k_mfold<<<4, nk::kB, 0, s>>>(W.part, grid, W.scal, 0, 1);
    check_launch();
    FV_CUDA(cudaMemcpyAsync(out, W.scal, 4 * sizeof(double), cudaMemcpyDeviceToHost, s));
    FV_CUDA(cudaStreamSynchronize(s));
}

// Right-preconditioned GMRES(m) from x = 0 on (V/dt - J) x = b; returns the
// matvec count and the final relative residual estimate.
int gmres(fv_adjoint_s* A, NewtonWork& W, const St* b, St* x, int m, double rtol, int sweeps, double* rel,
          cudaStream_t s) {
    const size_t n = W.n;
    const int vb = (int)((n + nk::kB - 1) / nk::kB);
    auto V = [&](int i) { return W.V + (size_t)i * n; };
    FV_CUDA(cudaMemcpyAsync(V(0), b, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    const double beta = norm2(W, V(0), W.scal, s);
    *rel = 1.0;
    if (!(beta > 0.0) || !std::isfinite(beta)) {
        FV_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, s));
        return 0;
    }
    nk::k_scale_inv<<<vb, nk::kB, 0, s>>>(V(0), V(0), W.scal, n);
    check_launch();
    std::vector<double> H((size_t)(m + 1) * m, 0.0), cs(m), sn(m), g(m + 1, 0.0), y(m), hc(m + 2);
    g[0] = beta;
    int k = 0;
    double* wv = reinterpret_cast<double*>(W.w);
    for (int j = 0; j < m; ++j) {
        precondition(A, W, reinterpret_cast<const St*>(V(j)), W.z, sweeps, s);
        adjh::jvp_dev(A, W.z, W.Jx);
        nk::k_ptc<<<nk::blocks(W.N), nk::kB, 0, s>>>(A->a.D, W.z, W.Jx, W.w, W.N);
        check_launch();
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
            if (!std::isfinite(hc[i])) fvgb::raise(FV_ERR_NONFINITE, "Newton-Krylov: non-finite Krylov vector");
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
        *rel = std::fabs(g[j + 1]) / beta;
        if (*rel <= rtol || !(hn > 0.0)) break;
    }
    for (int i = k - 1; i >= 0; --i) {
        double t = g[i];
        for (int l = i + 1; l < k; ++l) t -= H[(size_t)i * m + l] * y[l];
        y[i] = t / H[(size_t)i * m + i];
    }
    FV_CUDA(cudaMemcpyAsync(W.h, y.data(), sizeof(double) * k, cudaMemcpyHostToDevice, s));
    nk::k_combine<<<vb, nk::kB, 0, s>>>(reinterpret_cast<double*>(W.tmp), W.V, W.h, k, n);
    check_launch();
    precondition(A, W, W.tmp, x, sweeps, s);
    FV_CUDA(cudaStreamSynchronize(s));
    return k;
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
    o->krylov_dim = 40;
    o->krylov_rtol = 1e-2;
    o->precond_sweeps = 2;
    o->precond_kind = 1;
    o->max_rel_change = 0.2;
}

int fv_steady_newton(fv_solver_t solver, const fv_newton_t* opt, double* history, int32_t* iterations) {
    return fvgb::guarded([&] {
        if (!solver || !opt) fvgb::raise(FV_ERR_BAD_ARG, "null argument");
        const fv_newton_t o = *opt;
        if (o.max_newton < 0 || !(o.tol >= 0.0) || !(o.cfl0 > 0.0) || !(o.cfl_max >= o.cfl0) ||
            !(o.cfl_growth >= 1.0) || o.krylov_dim < 1 || o.krylov_dim > 200 || !(o.krylov_rtol > 0.0) ||
            o.precond_sweeps < 1 || o.precond_kind < 0 || o.precond_kind > 1 || !(o.max_rel_change > 0.0))
            fvgb::raise(FV_ERR_BAD_ARG, "fv_steady_newton: bad options");
        fvgb::Solver& s = solver->s;
        if (s.batch) fvgb::raise(FV_ERR_UNSUPPORTED, "fv_steady_newton: single (not batched) Euler solvers");
        fv_adjoint_t Ah = nullptr;
        {
            const int rc = fv_adjoint_create(solver, o.limiter_mode, &Ah);
            if (rc != FV_OK) fvgb::raise(rc, std::string("fv_steady_newton: ") + fvgb::last_error());
        }
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
        const int agrid = std::min(nk::kGrid, nk::blocks(s.N));
        W.kind = o.precond_kind;
        if (W.kind == 1) colour_cells(s, W, st);
        FV_CUDA(cudaStreamSynchronize(st));
        double prev = -1.0, cfl = o.cfl0;
        int it = 0, rejects = 0;
        double last_alpha = 0.0, last_rel = 0.0, last_cfl = 0.0;
        int last_mv = 0;
        bool retry = false;  // the state was just restored: keep the reduced CFL number
        for (;;) {
            FV_CUDA(cudaMemcpyAsync(A->U, s.U, sizeof(St) * (size_t)s.N, cudaMemcpyDeviceToDevice, st));
            adjh::linearise(A.get());
            adjh::residual_dev(A.get(), W.R);
            double nr[4];
            residual_norms(A.get(), W, nr, st);
            if (it == 0 && (!std::isfinite(nr[0]) || !std::isfinite(nr[3])))
                fvgb::raise(FV_ERR_NONFINITE, "fv_steady_newton: non-finite residual at the start");
            if (prev > 0.0 && !retry) {
                const double ratio = nr[0] / prev;
                if (!(ratio <= 10.0) || !std::isfinite(nr[3])) {
                    if (rejects < 10) {
                        // undo the step, retry at a quarter of the pseudo time step
                        FV_CUDA(cudaMemcpyAsync(s.U, W.Ubak, sizeof(St) * (size_t)s.N, cudaMemcpyDeviceToDevice, st));
                        cfl = std::max(o.cfl0 * 1e-3, 0.25 * last_cfl);
                        ++rejects;
                        retry = true;
                        continue;
                    }
                } else if (ratio < 1.0) {
                    cfl = std::min(o.cfl_max, last_cfl * o.cfl_growth);
                } else if (ratio < 2.0) {
                    cfl = last_cfl;
                } else {
                    cfl = std::max(o.cfl0 * 1e-3, 0.5 * last_cfl);
                }
            }
            if (!retry) rejects = 0;
            retry = false;
            if (history) {
                double* row = history + 8 * (size_t)it;
                for (int q = 0; q < 4; ++q) row[q] = nr[q];
                row[4] = last_cfl;
                row[5] = last_mv;
                row[6] = last_rel;
                row[7] = last_alpha;
            }
            prev = nr[0];
            if (nr[0] < o.tol || it >= o.max_newton) break;
            adjh::lin_dt(A.get(), cfl);
            nk::k_pc_diag<<<nk::blocks(s.N), nk::kB, 0, st>>>(A->a, W.Dinv);
            check_launch();
            double rel = 0.0;
            const int mv = gmres(A.get(), W, W.R, W.du, o.krylov_dim, o.krylov_rtol, o.precond_sweeps, &rel, st);
            nk::k_alpha<<<agrid, nk::kB, 0, st>>>(A->a, W.du, o.max_rel_change, W.part);
            nk::k_min_fold<<<1, nk::kB, 0, st>>>(W.part, agrid, W.scal);
            check_launch();
            double alpha = 0.0;
            FV_CUDA(cudaMemcpyAsync(&alpha, W.scal, sizeof(double), cudaMemcpyDeviceToHost, st));
            FV_CUDA(cudaStreamSynchronize(st));
            FV_CUDA(cudaMemcpyAsync(W.Ubak, s.U, sizeof(St) * (size_t)s.N, cudaMemcpyDeviceToDevice, st));
            nk::k_update<<<nk::blocks(s.N), nk::kB, 0, st>>>(s.U, W.du, alpha, s.N);
            check_launch();
            last_alpha = alpha;
            last_rel = rel;
            last_mv = mv;
            last_cfl = cfl;
            ++it;
        }
        if (iterations) *iterations = it;
        s.refresh_primitives();
        FV_CUDA(cudaStreamSynchronize(st));
    });
}

}  // extern "C"
