// Discrete adjoint of the Euler residual (first and second order, FP64).
//
// No reference counterpart: the reference has no adjoint.  The residual
// being differentiated is the one the solver's own kernels evaluate
// (euler_o2.cuh: k_grad / k_face / k_update, i.e. EulerFVMSolver::step's
// face and cell passes, src/EulerFVMSolver.cpp:61-111, extended to MUSCL):
//
//   W_c   = prim(U_c)
//   Gu_c  = sum_e a_e nb_e - s_c W_c        nb_e = W_j, or (W_c + ghost(W_c)) / 2
//   G_c   = psi_c (.) Gu_c                  psi frozen at the linearisation state
//   w_f^s = W_s + G_s . r_f^s               (W_s where the positivity test fell back)
//   F_f   = |f| flux(w_f^L, w_f^R or ghost(w_f^L, fs))
//   R_c   = sum_f -/+ F_f                   owner subtracts, neighbour adds
//
// Linearisation (once per state): per face, the flux Jacobians with
// respect to both reconstructed states (boundary: with respect to the
// interior state through the ghost state, and to the primitive
// freestream) are formed by forward-mode dual numbers running the same
// templated flux and ghost-state code as the residual kernels; per
// boundary face also the Jacobians of the gradient's boundary value.
// Then the tangent (forward, JVP) and cotangent (backward, VJP) maps are
// sparse products with these matrices, written as face passes followed by
// cell gathers in the residual's own CSR order: every kernel writes only
// its own face or cell, there are no atomics, and repeated runs are bit
// identical.  The scatter of a cell's gradient cotangent to its
// neighbours is turned into a gather through the "twin" of each CSR entry
// (the entry of the neighbour's row that points back through the same
// face).
//
// The adjoint equation (dR/dU)^T lambda = dJ/dU is solved by SSP-RK3 in
// pseudo-time on d lambda / d tau = D ((dR/dU)^T lambda - dJ/dU), D the
// primal's local dt / V: the linear part D (dR/dU)^T has the spectrum of
// the linearised primal iteration, so it is stable at the primal's CFL
// number and converges at the primal's asymptotic rate.
#define FV_KNS adjk
#include "euler_o2.cuh"

#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "capi_internal.h"
#include "adjoint_internal.h"

namespace adjk {

// ---------------------------------------------------------------------------
// Forward-mode dual numbers (value + N partials)
// ---------------------------------------------------------------------------
template <int N>
struct Dual {
    double v;
    double d[N];
    __device__ Dual() {}
    __device__ Dual(double x) : v(x) {
#pragma unroll
        for (int k = 0; k < N; ++k) d[k] = 0.0;
    }
};
using D4 = Dual<4>;

template <int N> __device__ __forceinline__ Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
    Dual<N> r;
    r.v = a.v + b.v;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] + b.d[k];
    return r;
}
template <int N> __device__ __forceinline__ Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
    Dual<N> r;
    r.v = a.v - b.v;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] - b.d[k];
    return r;
}
template <int N> __device__ __forceinline__ Dual<N> operator-(const Dual<N>& a) {
    Dual<N> r;
    r.v = -a.v;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = -a.d[k];
    return r;
}
template <int N> __device__ __forceinline__ Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
    Dual<N> r;
    r.v = a.v * b.v;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
    return r;
}
template <int N> __device__ __forceinline__ Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
    Dual<N> r;
    r.v = a.v / b.v;
    const double ib = 1.0 / b.v;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
    return r;
}
template <int N> __device__ __forceinline__ bool operator<(const Dual<N>& a, const Dual<N>& b) { return a.v < b.v; }
template <int N> __device__ __forceinline__ bool operator<=(const Dual<N>& a, const Dual<N>& b) { return a.v <= b.v; }
template <int N> __device__ __forceinline__ bool operator>(const Dual<N>& a, const Dual<N>& b) { return a.v > b.v; }
template <int N> __device__ __forceinline__ bool operator>=(const Dual<N>& a, const Dual<N>& b) { return a.v >= b.v; }
template <int N> __device__ __forceinline__ Dual<N> fabs(const Dual<N>& a) { return a.v < 0.0 ? -a : a; }
template <int N> __device__ __forceinline__ Dual<N> fmin(const Dual<N>& a, const Dual<N>& b) { return b.v < a.v ? b : a; }
template <int N> __device__ __forceinline__ Dual<N> fmax(const Dual<N>& a, const Dual<N>& b) { return b.v > a.v ? b : a; }
using ::fabs;
using ::fmax;
using ::fmin;

template <> __device__ __forceinline__ D4 tsqrt<D4>(D4 x) {
    D4 r;
    r.v = sqrt(x.v);
    const double h = 0.5 / r.v;
#pragma unroll
    for (int k = 0; k < 4; ++k) r.d[k] = x.d[k] * h;
    return r;
}
template <> __device__ __forceinline__ D4 trsqrt<D4>(D4 x) {
    D4 r;
    r.v = 1.0 / sqrt(x.v);
    const double h = -0.5 * r.v / x.v;
#pragma unroll
    for (int k = 0; k < 4; ++k) r.d[k] = x.d[k] * h;
    return r;
}
// a^b; the exponent's partials enter through log(a) only when present.
template <> __device__ __forceinline__ D4 tpow<D4>(D4 a, D4 b) {
    D4 r;
    r.v = pow(a.v, b.v);
    bool bd = false;
#pragma unroll
    for (int k = 0; k < 4; ++k) bd |= b.d[k] != 0.0;
    const double la = bd ? log(a.v) : 0.0;
    const double q = b.v * pow(a.v, b.v - 1.0);
#pragma unroll
    for (int k = 0; k < 4; ++k) r.d[k] = q * a.d[k] + (bd ? r.v * la * b.d[k] : 0.0);
    return r;
}

// ---------------------------------------------------------------------------


__device__ __forceinline__ V4<double> ldW(const St* W, int i) {
    const St s = ld_state(W, i);
    return {s.r, s.ru, s.rv, s.E};
}
__device__ __forceinline__ double vget(const V4<double>& w, int k) { return (&w.r)[k]; }
// Conserved freestream of boundary face f's farfield: the patch's, or (batched
// solvers) the owner cell's instance's.
__device__ __forceinline__ const double* fs_of(const AdjArgs& a, int patch, int f) {
    return a.inst_fs ? a.inst_fs + 4 * a.cell_inst[a.fl[f]] : a.bc.st[patch];
}
template <int N> __device__ __forceinline__ Dual<N> dget(const V4<Dual<N>>& w, int k) { return (&w.r)[k]; }

template <typename T>
__device__ __forceinline__ V4<T> flux_of(int flux, const V4<T>& L, const V4<T>& R, T nx, T ny, T g, T igm1) {
    return flux == FLUX_HLLC ? hllc_p<T>(L, R, nx, ny, g, igm1) : rusanov_p<T>(L, R, nx, ny, g, igm1);
}

__device__ __forceinline__ V4<D4> seed(const V4<double>& w) {
    V4<D4> r = {D4(w.r), D4(w.u), D4(w.v), D4(w.p)};
    r.r.d[0] = 1.0; r.u.d[1] = 1.0; r.v.d[2] = 1.0; r.p.d[3] = 1.0;
    return r;
}
__device__ __forceinline__ V4<D4> cst(const V4<double>& w) { return {D4(w.r), D4(w.u), D4(w.v), D4(w.p)}; }

__device__ __forceinline__ void store_jac(double* J, const V4<D4>& F, double ar) {
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int k = 0; k < 4; ++k) J[4 * i + k] = ar * dget(F, i).d[k];
}

// Reconstructed face states at the linearisation state and the positivity
// decisions (bit 0 owner side fell back, bit 1 neighbour side), as k_face.
__device__ __forceinline__ unsigned char recon_face(const AdjArgs& a, int f, int L, int R, V4<double>& wl,
                                                    V4<double>& wr) {
    wl = ldW(a.W, L);
    wr = {0, 0, 0, 0};
    unsigned char flags = 0;
    if (a.order == 2) {
        const double4_32a rr = a.frf[f];
        V4<double> o;
        double* ov = &o.r;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const double2 q = a.Gu[4 * L + k];
            const double p = a.psi[4 * L + k];
            ov[k] = vget(wl, k) + ((p * q.x) * rr.x + (p * q.y) * rr.y);
        }
        if (o.r > 0.0 && o.p > 0.0) wl = o;
        else flags |= 1;
        if (R >= 0) {
            wr = ldW(a.W, R);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const double2 q = a.Gu[4 * R + k];
                const double p = a.psi[4 * R + k];
                ov[k] = vget(wr, k) + ((p * q.x) * rr.z + (p * q.y) * rr.w);
            }
            if (o.r > 0.0 && o.p > 0.0) wr = o;
            else flags |= 2;
        }
    } else if (R >= 0) {
        wr = ldW(a.W, R);
    }
    return flags;
}

// Per face: reconstruction (with its positivity decisions), flux value and
// the flux Jacobians.
__global__ void k_lin_face(const AdjArgs a) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= a.n_faces) return;
    const int L = a.fl[f], R = a.fr[f];
    const double4_32a geo = a.fgeom[f];
    const double nx = geo.x, ny = geo.y, ar = geo.z;
    const double g = a.gamma;
    V4<double> wl, wr;
    const unsigned char flags = recon_face(a, f, L, R, wl, wr);
    const V4<double> wlc = ldW(a.W, L);
    a.fb[f] = flags;
    const D4 gD(g), iD(a.igm1), nxD(nx), nyD(ny);
    double* JL = a.JL + 16 * (size_t)f;
    double* JR = a.JR + 16 * (size_t)f;
    V4<D4> F1;
    if (R >= 0) {
        F1 = flux_of<D4>(a.flux, seed(wl), cst(wr), nxD, nyD, gD, iD);
        store_jac(JL, F1, ar);
        const V4<D4> F2 = flux_of<D4>(a.flux, cst(wl), seed(wr), nxD, nyD, gD, iD);
        store_jac(JR, F2, ar);
    } else {
        const int patch = a.fpatch[f];
        const int t = a.bc.type[patch];
        V4<double> fsp = {0, 0, 0, 0};
        if (t == BC_FARFIELD || t == BC_CHAR) fsp = fs_prim<double>(fs_of(a, patch, f), g);
        const D4 wu(t == BC_NOSLIP ? a.bc.wall_u[patch] : 0.0), wv(t == BC_NOSLIP ? a.bc.wall_v[patch] : 0.0);
        const V4<D4> wlD = seed(wl);
        F1 = flux_of<D4>(a.flux, wlD, ghost_core<D4>(t, wlD, nxD, nyD, gD, cst(fsp), wu, wv), nxD, nyD, gD, iD);
        store_jac(JL, F1, ar);
        const V4<D4> F2 = flux_of<D4>(a.flux, cst(wl), ghost_core<D4>(t, cst(wl), nxD, nyD, gD, seed(fsp), wu, wv),
                                      nxD, nyD, gD, iD);
        store_jac(JR, F2, ar);
        // the gradient's boundary value (W_c + ghost(W_c)) / 2 at the cell-centred state
        double* Gb = a.Gb + 32 * (size_t)(f - a.n_int_faces);
        const V4<D4> gw = ghost_core<D4>(t, seed(wlc), nxD, nyD, gD, cst(fsp), wu, wv);
        const V4<D4> gf = ghost_core<D4>(t, cst(wlc), nxD, nyD, gD, seed(fsp), wu, wv);
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                Gb[4 * i + k] = 0.5 * ((i == k ? 1.0 : 0.0) + dget(gw, i).d[k]);
                Gb[16 + 4 * i + k] = 0.5 * dget(gf, i).d[k];
            }
    }
    st_state(a.F, f, st_make(ar * F1.r.v, ar * F1.u.v, ar * F1.v.v, ar * F1.p.v));
}

// Per cell and variable: the limiter's active branch and its partials,
// recomputed with k_grad's formulas (neighbour extremes including the cell
// itself; face extrapolations D2 = Gu . (x_f - x_c); psi = min(1,
// phi(dmax, max D2 > 0), phi(-dmin, max -D2 over D2 < 0))).
__global__ void k_lin_lim(const AdjArgs a) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.n_cells) return;
    const V4<double> wc = ldW(a.W, c);
    const double g = a.gamma;
    const int e0 = a.cf_off[c], e1 = a.cf_off[c + 1];
    for (int k = 0; k < 4; ++k) {
        const double w0 = vget(wc, k);
        double vmax = w0, vmin = w0;
        int emax = -1, emin = -1;
        double ypos = 0.0, yneg = 0.0;
        int epos = -1, eneg = -1;
        const double2 gu = a.Gu[4 * c + k];
        for (int e = e0; e < e1; ++e) {
            const int nb = a.cnb[e];
            double v;
            if (nb >= 0) {
                v = vget(ldW(a.W, nb), k);
            } else {
                const int f = -1 - nb;
                const double4_32a geo = a.fgeom[f];
                const int patch = a.fpatch[f];
                const int t = a.bc.type[patch];
                V4<double> fsp = {0, 0, 0, 0};
                if (t == BC_FARFIELD || t == BC_CHAR) fsp = fs_prim<double>(fs_of(a, patch, f), g);
                const double wu = t == BC_NOSLIP ? a.bc.wall_u[patch] : 0.0;
                const double wv = t == BC_NOSLIP ? a.bc.wall_v[patch] : 0.0;
                const V4<double> gh = ghost_core<double>(t, wc, geo.x, geo.y, g, fsp, wu, wv);
                v = 0.5 * (w0 + vget(gh, k));
            }
            if (v > vmax) { vmax = v; emax = e; }
            if (v < vmin) { vmin = v; emin = e; }
            const double2 r = a.erf[e];
            const double d2 = gu.x * r.x + gu.y * r.y;
            if (d2 > ypos) { ypos = d2; epos = e; }
            if (-d2 > yneg) { yneg = -d2; eneg = e; }
        }
        const double eps2 = a.limiter == 2 ? a.eps2[c] : 0.0;
        double nmin = 1.0, dmn = 1.0;
        int side = 0;
        double pd1 = 0.0, py = 0.0, pe = 0.0;
        for (int sd = 0; sd < 2; ++sd) {
            const double y = sd == 0 ? ypos : yneg;
            if (!(y > 0.0)) continue;
            const double d1 = sd == 0 ? vmax - w0 : w0 - vmin;
            double num, den, nd1, ny, dd1, dy;
            if (a.limiter == 1) {
                num = d1; den = y; nd1 = 1.0; ny = 0.0; dd1 = 0.0; dy = 1.0;
            } else {
                const double p = d1 * y, q = d1 * d1 + eps2;
                num = q + 2.0 * p;
                den = (y + y) * y + (q + p);
                nd1 = 2.0 * d1 + 2.0 * y; ny = 2.0 * d1;
                dd1 = 2.0 * d1 + y; dy = 4.0 * y + d1;
            }
            if (num * dmn < nmin * den) {
                nmin = num; dmn = den;
                side = sd == 0 ? 1 : -1;
                pd1 = (nd1 * den - num * dd1) / (den * den);
                py = (ny * den - num * dy) / (den * den);
                // eps^2 enters num and den with unit weight
                pe = a.limiter == 1 ? 0.0 : (den - num) / (den * den);
            }
        }
        const int i = 4 * c + k;
        a.lside[i] = (signed char)side;
        a.led[i] = side == 1 ? emax : (side == -1 ? emin : -1);
        a.ler[i] = side == 1 ? epos : (side == -1 ? eneg : -1);
        a.lpd[i] = make_double2(pd1, py);
        a.lpe[i] = pe;
    }
}

// Per cell: D = cfl / sum_f lambda_f |f| (the primal's local time step over
// the volume), from the cell-centred states.
__global__ void k_lin_dt(const AdjArgs a) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.n_cells) return;
    double lam = 0.0;
    const double g = a.gamma;
    for (int e = a.cf_off[c]; e < a.cf_off[c + 1]; ++e) {
        const int f = a.cf[e] >> 1;
        const double4_32a geo = a.fgeom[f];
        const int L = a.fl[f], R = a.fr[f];
        const V4<double> wl = ldW(a.W, L);
        double Smax = fabs(wl.u * geo.x + wl.v * geo.y) + sqrt(g * wl.p / wl.r);
        if (R >= 0) {
            const V4<double> wr = ldW(a.W, R);
            Smax = rmax(Smax, fabs(wr.u * geo.x + wr.v * geo.y) + sqrt(g * wr.p / wr.r));
        }
        lam += Smax * geo.z;
    }
    a.D[c] = a.cfl / lam;
}

// dW/dU at primitive state w (row i = dW_i / dU).
__device__ __forceinline__ void prim_jac(const V4<double>& w, double g, double J[16]) {
    const double ir = 1.0 / w.r, gm1 = g - 1.0;
    J[0] = 1.0; J[1] = 0.0; J[2] = 0.0; J[3] = 0.0;
    J[4] = -w.u * ir; J[5] = ir; J[6] = 0.0; J[7] = 0.0;
    J[8] = -w.v * ir; J[9] = 0.0; J[10] = ir; J[11] = 0.0;
    J[12] = 0.5 * gm1 * (w.u * w.u + w.v * w.v); J[13] = -gm1 * w.u; J[14] = -gm1 * w.v; J[15] = gm1;
}

// ---------------------------------------------------------------------------
// Residual at the linearisation state: R_c = sum -/+ F_f.
__global__ void k_res_cell(const AdjArgs a, St* __restrict__ R) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.n_cells) return;
    St r = st_make(0.0, 0.0, 0.0, 0.0);
    for (int e = a.cf_off[c]; e < a.cf_off[c + 1]; ++e) {
        const int ent = a.cf[e];
        r += flip_if(ld_state(a.F, ent >> 1), ent);
    }
    st_state(R, c, r);
}

// ---------------------------------------------------------------------------
// Tangent map dR = (dR/dU) dU + (dR/dfs) dfs
__global__ void k_fwd_cell1(const AdjArgs a, const St* __restrict__ dU) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.n_cells) return;
    double J[16];
    prim_jac(ldW(a.W, c), a.gamma, J);
    const St u = ld_state(dU, c);
    const double x[4] = {u.r, u.ru, u.rv, u.E};
    double y[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) y[i] = J[4 * i] * x[0] + J[4 * i + 1] * x[1] + J[4 * i + 2] * x[2] + J[4 * i + 3] * x[3];
    st_state(a.dW, c, st_make(y[0], y[1], y[2], y[3]));
}

__global__ void k_fwd_cell2(const AdjArgs a) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.n_cells) return;
    const St wc = ld_state(a.dW, c);
    const double dwc[4] = {wc.r, wc.ru, wc.rv, wc.E};
    const double2 s = a.lsq_sum[c];
    double gx[4], gy[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) { gx[k] = -s.x * dwc[k]; gy[k] = -s.y * dwc[k]; }
    for (int e = a.cf_off[c]; e < a.cf_off[c + 1]; ++e) {
        const int nb = a.cnb[e];
        const double2 w = a.lsq[e];
        double v[4];
        if (nb >= 0) {
            const St q = ld_state(a.dW, nb);
            v[0] = q.r; v[1] = q.ru; v[2] = q.rv; v[3] = q.E;
        } else {
            const int f = -1 - nb;
            const double* Gb = a.Gb + 32 * (size_t)(f - a.n_int_faces);
            const double* df = a.dfs + 4 * a.fpatch[f];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                double t = 0.0;
#pragma unroll
                for (int k = 0; k < 4; ++k) t += Gb[4 * i + k] * dwc[k] + Gb[16 + 4 * i + k] * df[k];
                v[i] = t;
            }
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) { gx[k] += w.x * v[k]; gy[k] += w.y * v[k]; }
    }
    double dpsi[4] = {0.0, 0.0, 0.0, 0.0};
    if (a.full) {
        for (int k = 0; k < 4; ++k) {
            const int i = 4 * c + k;
            const int side = a.lside[i];
            if (!side) continue;
            const double2 pd = a.lpd[i];
            const double2 r = a.erf[a.ler[i]];
            const double dy = side * (gx[k] * r.x + gy[k] * r.y);
            double dd1 = 0.0;
            const int ed = a.led[i];
            if (ed >= 0) {
                const int nb = a.cnb[ed];
                double dn;
                if (nb >= 0) {
                    const St q = ld_state(a.dW, nb);
                    dn = (&q.r)[k];
                } else {
                    const int f = -1 - nb;
                    const double* Gb = a.Gb + 32 * (size_t)(f - a.n_int_faces);
                    const double* df = a.dfs + 4 * a.fpatch[f];
                    dn = 0.0;
                    for (int j = 0; j < 4; ++j) dn += Gb[4 * k + j] * dwc[j] + Gb[16 + 4 * k + j] * df[j];
                }
                dd1 = side * (dn - dwc[k]);
            }
            dpsi[k] = pd.x * dd1 + pd.y * dy;
        }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const double p = a.psi[4 * c + k];
        const double2 gu = a.Gu[4 * c + k];
        a.dG[4 * c + k] = make_double2(p * gx[k] + dpsi[k] * gu.x, p * gy[k] + dpsi[k] * gu.y);
    }
}

__global__ void k_fwd_face(const AdjArgs a) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= a.n_faces) return;
    const int L = a.fl[f], R = a.fr[f];
    const unsigned char fl = a.fb[f];
    double dl[4], dr[4];
    {
        const St q = ld_state(a.dW, L);
        dl[0] = q.r; dl[1] = q.ru; dl[2] = q.rv; dl[3] = q.E;
    }
    double4_32a rr = {0, 0, 0, 0};
    if (a.order == 2) rr = a.frf[f];
    if (a.order == 2 && !(fl & 1))
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const double2 q = a.dG[4 * L + k];
            dl[k] += q.x * rr.x + q.y * rr.y;
        }
    if (R >= 0) {
        const St q = ld_state(a.dW, R);
        dr[0] = q.r; dr[1] = q.ru; dr[2] = q.rv; dr[3] = q.E;
        if (a.order == 2 && !(fl & 2))
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const double2 g = a.dG[4 * R + k];
                dr[k] += g.x * rr.z + g.y * rr.w;
            }
    } else {
        const double* df = a.dfs + 4 * a.fpatch[f];
#pragma unroll
        for (int k = 0; k < 4; ++k) dr[k] = df[k];
    }
    const double* JL = a.JL + 16 * (size_t)f;
    const double* JR = a.JR + 16 * (size_t)f;
    double y[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        double t = 0.0;
#pragma unroll
        for (int k = 0; k < 4; ++k) t += JL[4 * i + k] * dl[k] + JR[4 * i + k] * dr[k];
        y[i] = t;
    }
    st_state(a.dF, f, st_make(y[0], y[1], y[2], y[3]));
}

__global__ void k_fwd_cell3(const AdjArgs a, St* __restrict__ dR) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.n_cells) return;
    St r = st_make(0.0, 0.0, 0.0, 0.0);
    for (int e = a.cf_off[c]; e < a.cf_off[c + 1]; ++e) {
        const int ent = a.cf[e];
        r += flip_if(ld_state(a.dF, ent >> 1), ent);
    }
    st_state(dR, c, r);
}

// ---------------------------------------------------------------------------
// Cotangent map: Ubar = (dR/dU)^T lam, fsbar = (dR/dfs)^T lam.
__global__ void k_bwd_face(const AdjArgs a, const St* __restrict__ lam) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= a.n_faces) return;
    const int L = a.fl[f], R = a.fr[f];
    // R_L -= F_f, R_R += F_f
    const St ll = ld_state(lam, L);
    double fbar[4] = {-ll.r, -ll.ru, -ll.rv, -ll.E};
    if (R >= 0) {
        const St lr = ld_state(lam, R);
        fbar[0] += lr.r; fbar[1] += lr.ru; fbar[2] += lr.rv; fbar[3] += lr.E;
    }
    const double* JL = a.JL + 16 * (size_t)f;
    const double* JR = a.JR + 16 * (size_t)f;
    double* wb = a.wbar + 8 * (size_t)f;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        double tl = 0.0, tr = 0.0;
#pragma unroll
        for (int i = 0; i < 4; ++i) { tl += JL[4 * i + k] * fbar[i]; tr += JR[4 * i + k] * fbar[i]; }
        wb[k] = tl;
        if (R >= 0) wb[4 + k] = tr;
        else a.fsb[4 * (size_t)(f - a.n_int_faces) + k] = tr;
    }
}

// Gather of the face-state cotangents: W-bar and the gradient cotangent.
// order 1: finishes Ubar here (MODE 0: write Ubar; 1..3: RK stage 0..2).
__device__ __forceinline__ void finish_cell(const AdjArgs& a, int c, const double wbar[4], int mode,
                                            St* __restrict__ out, St* __restrict__ lam, St* __restrict__ lam0,
                                            const St* __restrict__ rhs, double* __restrict__ r2) {
    double J[16];
    prim_jac(ldW(a.W, c), a.gamma, J);
    double u[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) u[k] = J[k] * wbar[0] + J[4 + k] * wbar[1] + J[8 + k] * wbar[2] + J[12 + k] * wbar[3];
    if (mode == 0) {
        st_state(out, c, st_make(u[0], u[1], u[2], u[3]));
        return;
    }
    // pseudo-time residual r = (dR/dU)^T lam - dJ/dU
    const St g = ld_state(rhs, c);
    const double r[4] = {u[0] - g.r, u[1] - g.ru, u[2] - g.rv, u[3] - g.E};
    const double d = a.D[c];
    const St l = ld_state(lam, c);
    St e = st_make(l.r + d * r[0], l.ru + d * r[1], l.rv + d * r[2], l.E + d * r[3]);
    St n;
    if (mode == 1) {
        st_state(lam0, c, l);
        n = e;
#pragma unroll
        for (int k = 0; k < 4; ++k) r2[k] = r[k] * r[k];
    } else if (mode == 2) {
        n = 0.75 * ld_state(lam0, c) + 0.25 * e;
    } else {
        n = (1.0 / 3.0) * ld_state(lam0, c) + (2.0 / 3.0) * e;
    }
    st_state(lam, c, n);
}

__device__ __forceinline__ void block_partials(double r2[4], double* partials) {
    __shared__ double red[8][4];
#pragma unroll
    for (int k = 0; k < 4; ++k) r2[k] = warp_sum(r2[k]);
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 4; ++k) red[threadIdx.x >> 5][k] = r2[k];
    __syncthreads();
    if (threadIdx.x == 0)
        for (int k = 0; k < 4; ++k) {
            double v = 0.0;
            for (int w = 0; w < 8; ++w) v += red[w][k];
            partials[4 * blockIdx.x + k] = v;
        }
}

__global__ void __launch_bounds__(256) k_bwd_cell1(const AdjArgs a, int mode, St* out, St* lam, St* lam0,
                                                   const St* rhs, double* partials) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    double r2[4] = {0.0, 0.0, 0.0, 0.0};
    if (c < a.n_cells) {
        double wb[4] = {0.0, 0.0, 0.0, 0.0}, gx[4] = {0.0, 0.0, 0.0, 0.0}, gy[4] = {0.0, 0.0, 0.0, 0.0};
        for (int e = a.cf_off[c]; e < a.cf_off[c + 1]; ++e) {
            const int ent = a.cf[e];
            const int f = ent >> 1;
            const bool owner = ent & 1;
            const double* w = a.wbar + 8 * (size_t)f + (owner ? 0 : 4);
#pragma unroll
            for (int k = 0; k < 4; ++k) wb[k] += w[k];
            if (a.order == 2 && !(a.fb[f] & (owner ? 1 : 2))) {
                const double4_32a rr = a.frf[f];
                const double rx = owner ? rr.x : rr.z, ry = owner ? rr.y : rr.w;
#pragma unroll
                for (int k = 0; k < 4; ++k) { gx[k] += w[k] * rx; gy[k] += w[k] * ry; }
            }
        }
        if (a.order == 2) {
            double gux[4], guy[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const double p = a.psi[4 * c + k];
                gux[k] = p * gx[k];
                guy[k] = p * gy[k];
            }
            if (a.full) {
                // psi-bar = Gbar . Gu; then through psi = phi(d1, y):
                // y = side * Gu . r_er, d1 = side * (nb_ed - W_c)
                for (int k = 0; k < 4; ++k) {
                    const int i = 4 * c + k;
                    const int side = a.lside[i];
                    a.ldb[i] = 0.0;
                    if (!side) continue;
                    const double2 gu = a.Gu[i];
                    const double psib = gx[k] * gu.x + gy[k] * gu.y;
                    const double2 pd = a.lpd[i];
                    const double yb = psib * pd.y, d1b = psib * pd.x;
                    const double2 r = a.erf[a.ler[i]];
                    gux[k] += side * yb * r.x;
                    guy[k] += side * yb * r.y;
                    const int ed = a.led[i];
                    if (ed < 0) continue;  // the cell's own value: d1 = 0 identically
                    wb[k] -= side * d1b;
                    const int nb = a.cnb[ed];
                    if (nb >= 0) {
                        a.ldb[i] = side * d1b;  // gathered by the neighbour
                    } else {
                        // boundary value (W_c + ghost(W_c)) / 2, row k of its Jacobians
                        const int f = -1 - nb;
                        const double* Gb = a.Gb + 32 * (size_t)(f - a.n_int_faces);
                        double* fs = a.fsb + 4 * (size_t)(f - a.n_int_faces);
                        for (int j = 0; j < 4; ++j) {
                            wb[j] += side * d1b * Gb[4 * k + j];
                            fs[j] += side * d1b * Gb[16 + 4 * k + j];
                        }
                    }
                }
            }
            St q = st_make(wb[0], wb[1], wb[2], wb[3]);
            st_state(a.Wbar, c, q);
#pragma unroll
            for (int k = 0; k < 4; ++k) a.Gub[4 * c + k] = make_double2(gux[k], guy[k]);
        } else {
            finish_cell(a, c, wb, mode, out, lam, lam0, rhs, r2);
        }
    }
    if (a.order == 1 && mode == 1) block_partials(r2, partials);
}

// Gradient cotangent to W-bar (gather through twin entries), then Ubar.
__global__ void __launch_bounds__(256) k_bwd_cell2(const AdjArgs a, int mode, St* out, St* lam, St* lam0,
                                                   const St* rhs, double* partials) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    double r2[4] = {0.0, 0.0, 0.0, 0.0};
    if (c < a.n_cells) {
        const St w0 = ld_state(a.Wbar, c);
        double wb[4] = {w0.r, w0.ru, w0.rv, w0.E};
        double2 gc[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) gc[k] = a.Gub[4 * c + k];
        const double2 s = a.lsq_sum[c];
#pragma unroll
        for (int k = 0; k < 4; ++k) wb[k] -= s.x * gc[k].x + s.y * gc[k].y;
        for (int e = a.cf_off[c]; e < a.cf_off[c + 1]; ++e) {
            const int nb = a.cnb[e];
            if (nb >= 0) {
                const int tw = a.twin[e];
                const double2 w = a.lsq[tw];
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const double2 q = a.Gub[4 * nb + k];
                    wb[k] += w.x * q.x + w.y * q.y;
                    if (a.full && a.led[4 * nb + k] == tw) wb[k] += a.ldb[4 * nb + k];
                }
            } else {
                const int f = -1 - nb;
                const double2 w = a.lsq[e];
                double v[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) v[k] = w.x * gc[k].x + w.y * gc[k].y;
                const double* Gb = a.Gb + 32 * (size_t)(f - a.n_int_faces);
                double* fs = a.fsb + 4 * (size_t)(f - a.n_int_faces);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    double tw = 0.0, tf = 0.0;
#pragma unroll
                    for (int i = 0; i < 4; ++i) { tw += Gb[4 * i + k] * v[i]; tf += Gb[16 + 4 * i + k] * v[i]; }
                    wb[k] += tw;
                    fs[k] += tf;
                }
            }
        }
        finish_cell(a, c, wb, mode, out, lam, lam0, rhs, r2);
    }
    if (mode == 1) block_partials(r2, partials);
}

// Norm of the stage-0 pseudo-time residual: block partials folded in block
// order by one block (deterministic); appended to the history.
__global__ void __launch_bounds__(256) k_adj_norms(const double* partials, int nblk, double* hist, int* counter,
                                                   int cap) {
    __shared__ double red[256][4];
    double t[4] = {0.0, 0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < nblk; b += 256)
        for (int k = 0; k < 4; ++k) t[k] += partials[4 * b + k];
    for (int k = 0; k < 4; ++k) red[threadIdx.x][k] = t[k];
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int k = 0; k < 4; ++k) red[threadIdx.x][k] += red[threadIdx.x + w][k];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const int it = *counter;
        if (it < cap)
            for (int k = 0; k < 4; ++k) hist[4 * it + k] = sqrt(red[0][k]);
        *counter = it + 1;
    }
}

// ---------------------------------------------------------------------------
// Geometry cotangents of lam^T R (shape sensitivities), after a backward
// pass at lam has filled wbar and Gub.  Per face: the unit normal, the
// length and the reconstruction offsets (x_f - x_L, x_f - x_R).
__global__ void k_geo_face(const AdjArgs a, const St* __restrict__ lam, double* __restrict__ out) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= a.n_faces) return;
    const int L = a.fl[f], R = a.fr[f];
    const double4_32a geo = a.fgeom[f];
    const double ar = geo.z, g = a.gamma;
    const St ll = ld_state(lam, L);
    double fbar[4] = {-ll.r, -ll.ru, -ll.rv, -ll.E};
    if (R >= 0) {
        const St lr = ld_state(lam, R);
        fbar[0] += lr.r; fbar[1] += lr.ru; fbar[2] += lr.rv; fbar[3] += lr.E;
    }
    V4<double> wl, wr;
    const unsigned char flags = recon_face(a, f, L, R, wl, wr);
    // d flux / d (nx, ny) by dual numbers (partials 0 and 1)
    D4 nxD(geo.x), nyD(geo.y);
    nxD.d[0] = 1.0;
    nyD.d[1] = 1.0;
    const D4 gD(g), iD(a.igm1);
    V4<D4> Fl;
    if (R >= 0) {
        Fl = flux_of<D4>(a.flux, cst(wl), cst(wr), nxD, nyD, gD, iD);
    } else {
        const int patch = a.fpatch[f];
        const int t = a.bc.type[patch];
        V4<double> fsp = {0, 0, 0, 0};
        if (t == BC_FARFIELD || t == BC_CHAR) fsp = fs_prim<double>(fs_of(a, patch, f), g);
        const D4 wu(t == BC_NOSLIP ? a.bc.wall_u[patch] : 0.0), wv(t == BC_NOSLIP ? a.bc.wall_v[patch] : 0.0);
        Fl = flux_of<D4>(a.flux, cst(wl), ghost_core<D4>(t, cst(wl), nxD, nyD, gD, cst(fsp), wu, wv), nxD, nyD, gD,
                         iD);
    }
    double nbx = 0.0, nby = 0.0, abar = 0.0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const D4 q = dget(Fl, i);
        nbx += fbar[i] * q.d[0];
        nby += fbar[i] * q.d[1];
        abar += fbar[i] * q.v;
    }
    double* o = out + 8 * (size_t)f;
    o[0] = ar * nbx;
    o[1] = ar * nby;
    o[2] = abar;
    double rl[2] = {0.0, 0.0}, rrr[2] = {0.0, 0.0};
    if (a.order == 2) {
        const double* wb = a.wbar + 8 * (size_t)f;
        if (!(flags & 1))
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const double2 q = a.Gu[4 * L + k];
                const double p = a.psi[4 * L + k];
                rl[0] += wb[k] * p * q.x;
                rl[1] += wb[k] * p * q.y;
            }
        if (R >= 0 && !(flags & 2))
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const double2 q = a.Gu[4 * R + k];
                const double p = a.psi[4 * R + k];
                rrr[0] += wb[4 + k] * p * q.x;
                rrr[1] += wb[4 + k] * p * q.y;
            }
    }
    o[3] = rl[0]; o[4] = rl[1]; o[5] = rrr[0]; o[6] = rrr[1]; o[7] = 0.0;
}

// Per cell: cotangents of the LSQ weights of each entry (abar, 2 per
// entry) and of their sums (sbar, 2 per cell); per boundary face the
// normal cotangent through the gradient's boundary value (nbg).
__global__ void k_geo_cell(const AdjArgs a, double* __restrict__ abar, double* __restrict__ sbar,
                           double* __restrict__ nbg) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.n_cells) return;
    const V4<double> wc = ldW(a.W, c);
    double2 gu[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) gu[k] = a.Gub[4 * c + k];
    double sx = 0.0, sy = 0.0;
#pragma unroll
    for (int k = 0; k < 4; ++k) { sx -= gu[k].x * vget(wc, k); sy -= gu[k].y * vget(wc, k); }
    sbar[2 * c] = sx;
    sbar[2 * c + 1] = sy;
    const double g = a.gamma;
    for (int e = a.cf_off[c]; e < a.cf_off[c + 1]; ++e) {
        const int nb = a.cnb[e];
        V4<double> v;
        if (nb >= 0) {
            v = ldW(a.W, nb);
        } else {
            const int f = -1 - nb;
            const double4_32a geo = a.fgeom[f];
            const int patch = a.fpatch[f];
            const int t = a.bc.type[patch];
            V4<double> fsp = {0, 0, 0, 0};
            if (t == BC_FARFIELD || t == BC_CHAR) fsp = fs_prim<double>(fs_of(a, patch, f), g);
            const D4 wu(t == BC_NOSLIP ? a.bc.wall_u[patch] : 0.0), wv(t == BC_NOSLIP ? a.bc.wall_v[patch] : 0.0);
            D4 nxD(geo.x), nyD(geo.y);
            nxD.d[0] = 1.0;
            nyD.d[1] = 1.0;
            const V4<D4> gh = ghost_core<D4>(t, cst(wc), nxD, nyD, D4(g), cst(fsp), wu, wv);
            v = {0.5 * (wc.r + gh.r.v), 0.5 * (wc.u + gh.u.v), 0.5 * (wc.v + gh.v.v), 0.5 * (wc.p + gh.p.v)};
            // cotangent of the boundary value: lsq weight of this entry times Gub
            const double2 w = a.lsq[e];
            double bx = 0.0, by = 0.0;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const double ci = w.x * gu[i].x + w.y * gu[i].y;
                bx += 0.5 * ci * dget(gh, i).d[0];
                by += 0.5 * ci * dget(gh, i).d[1];
            }
            nbg[2 * (size_t)(f - a.n_int_faces)] = bx;
            nbg[2 * (size_t)(f - a.n_int_faces) + 1] = by;
        }
        double ax = 0.0, ay = 0.0;
#pragma unroll
        for (int k = 0; k < 4; ++k) { ax += gu[k].x * vget(v, k); ay += gu[k].y * vget(v, k); }
        abar[2 * (size_t)e] = ax;
        abar[2 * (size_t)e + 1] = ay;
    }
}

// Full-limiter linearisation: geometry cotangents of the limiter values.
// psi depends on the nodes through the active face extrapolation
// y = side Gu . (x_f - x_c) (erb, per entry: added to the entry's offset),
// through eps^2 = (K sqrt(V))^3 (epb, per cell: the eps^2 cotangent) and,
// when the extreme neighbour value is a boundary value
// (W_c + ghost(W_c, n)) / 2, through the face normal (added to nbg).
// Runs after a backward pass at the same lam (wbar, fb in place) and after
// k_geo_cell (which writes nbg).
__global__ void k_geo_lim(const AdjArgs a, double* __restrict__ erb, double* __restrict__ epb,
                          double* __restrict__ nbg) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.n_cells) return;
    double gx[4] = {0.0, 0.0, 0.0, 0.0}, gy[4] = {0.0, 0.0, 0.0, 0.0};
    for (int e = a.cf_off[c]; e < a.cf_off[c + 1]; ++e) {
        const int ent = a.cf[e];
        const int f = ent >> 1;
        const bool owner = ent & 1;
        if (a.fb[f] & (owner ? 1 : 2)) continue;
        const double* w = a.wbar + 8 * (size_t)f + (owner ? 0 : 4);
        const double4_32a rr = a.frf[f];
        const double rx = owner ? rr.x : rr.z, ry = owner ? rr.y : rr.w;
#pragma unroll
        for (int k = 0; k < 4; ++k) { gx[k] += w[k] * rx; gy[k] += w[k] * ry; }
    }
    const V4<double> wc = ldW(a.W, c);
    const double g = a.gamma;
    double eb = 0.0;
    for (int k = 0; k < 4; ++k) {
        const int i = 4 * c + k;
        const int side = a.lside[i];
        if (!side) continue;
        const double2 gu = a.Gu[i];
        const double psib = gx[k] * gu.x + gy[k] * gu.y;
        const double2 pd = a.lpd[i];
        const double yb = psib * pd.y, d1b = psib * pd.x;
        const int er = a.ler[i];
        erb[2 * (size_t)er] += side * yb * gu.x;
        erb[2 * (size_t)er + 1] += side * yb * gu.y;
        eb += psib * a.lpe[i];
        const int ed = a.led[i];
        if (ed < 0) continue;
        const int nb = a.cnb[ed];
        if (nb >= 0) continue;
        const int f = -1 - nb;
        const double4_32a geo = a.fgeom[f];
        const int patch = a.fpatch[f];
        const int t = a.bc.type[patch];
        V4<double> fsp = {0, 0, 0, 0};
        if (t == BC_FARFIELD || t == BC_CHAR) fsp = fs_prim<double>(fs_of(a, patch, f), g);
        const D4 wu(t == BC_NOSLIP ? a.bc.wall_u[patch] : 0.0), wv(t == BC_NOSLIP ? a.bc.wall_v[patch] : 0.0);
        D4 nxD(geo.x), nyD(geo.y);
        nxD.d[0] = 1.0;
        nyD.d[1] = 1.0;
        const V4<D4> gh = ghost_core<D4>(t, cst(wc), nxD, nyD, D4(g), cst(fsp), wu, wv);
        // d1 = side (v - W_c), v = (W_c + ghost) / 2
        const size_t j = 2 * (size_t)(f - a.n_int_faces);
        nbg[j] += side * d1b * 0.5 * dget(gh, k).d[0];
        nbg[j + 1] += side * d1b * 0.5 * dget(gh, k).d[1];
    }
    epb[c] = eb;
}

__global__ void k_perm_gather(const St* __restrict__ in_ref, St* __restrict__ out_dev, const int* __restrict__ perm,
                              int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out_dev[i] = in_ref[perm[i]];
}
__global__ void k_perm_scatter(const St* __restrict__ in_dev, St* __restrict__ out_ref, const int* __restrict__ perm,
                               int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out_ref[perm[i]] = in_dev[i];
}


// ---------------------------------------------------------------------------
// Krylov vector kernels (GMRES on the fixed point of the pseudo-time
// iteration).  Vectors are flat double arrays (n = 4 N); a dot product is
// block partials over a fixed grid folded in block order by one block, so
// every reduction is deterministic.
constexpr int kKB = 256;
constexpr int kKGrid = 1024;

__device__ __forceinline__ double block_sum(double t) {
    __shared__ double red[kKB / 32];
    t = warp_sum(t);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
    __syncthreads();
    double v = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < kKB / 32; ++w) v += red[w];
    return v;
}

__global__ void __launch_bounds__(kKB) k_dot(const double* __restrict__ x, const double* __restrict__ y, size_t n,
                                             double* __restrict__ partials) {
    double t = 0.0;
    for (size_t i = blockIdx.x * (size_t)kKB + threadIdx.x; i < n; i += (size_t)gridDim.x * kKB) t += x[i] * y[i];
    const double v = block_sum(t);
    if (threadIdx.x == 0) partials[blockIdx.x] = v;
}

// out[0] = sum of the partials (its square root when sq)
__global__ void __launch_bounds__(kKB) k_fold(const double* __restrict__ partials, int nblk, double* __restrict__ out,
                                              int sq) {
    double t = 0.0;
    for (int b = threadIdx.x; b < nblk; b += kKB) t += partials[b];
    const double v = block_sum(t);
    if (threadIdx.x == 0) out[0] = sq ? sqrt(v) : v;
}

// y -= alpha[0] x
__global__ void k_axmy_dev(double* __restrict__ y, const double* __restrict__ x, const double* __restrict__ alpha,
                           size_t n) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) y[i] -= alpha[0] * x[i];
}

// out = x / nrm[0]
__global__ void k_div_dev(double* __restrict__ out, const double* __restrict__ x, const double* __restrict__ nrm,
                          size_t n) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = x[i] / nrm[0];
}

// w = v - p + c  ((I - M) v for the affine map p = M v + c)
__global__ void k_fp_apply(double* __restrict__ w, const double* __restrict__ v, const double* __restrict__ p,
                           const double* __restrict__ c, size_t n) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) w[i] = (v[i] - p[i]) + c[i];
}

// w = p - x
__global__ void k_sub(double* __restrict__ w, const double* __restrict__ p, const double* __restrict__ x, size_t n) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) w[i] = p[i] - x[i];
}

// y += a x
__global__ void k_axpy(double* __restrict__ y, const double* __restrict__ x, double a, size_t n) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) y[i] += a * x[i];
}

}  // namespace adjk

// ===========================================================================
// Host object and C ABI
// ===========================================================================
using adjk::AdjArgs;
using fvgb::St;

namespace fvgb {
const HostMesh& host_mesh_of(const fv_mesh_s* m);
}



namespace {

constexpr int kB = 256;
inline int blocks(int n) { return (n + kB - 1) / kB; }

void check_launch() { FV_CUDA(cudaGetLastError()); }

// device-order buffer <- host array in reference order
void upload_ref(fv_adjoint_s* A, const double* host, St* dev) {
    fvgb::Solver& s = A->solver->s;
    FV_CUDA(cudaMemcpyAsync(A->stage_ref, host, sizeof(St) * (size_t)A->N, cudaMemcpyHostToDevice, s.stream));
    adjk::k_perm_gather<<<blocks(A->N), kB, 0, s.stream>>>(A->stage_ref, dev, s.d_perm, A->N);
    check_launch();
}

void download_ref(fv_adjoint_s* A, const St* dev, double* host) {
    fvgb::Solver& s = A->solver->s;
    adjk::k_perm_scatter<<<blocks(A->N), kB, 0, s.stream>>>(dev, A->stage_ref, s.d_perm, A->N);
    check_launch();
    FV_CUDA(cudaMemcpyAsync(host, A->stage_ref, sizeof(St) * (size_t)A->N, cudaMemcpyDeviceToHost, s.stream));
    FV_CUDA(cudaStreamSynchronize(s.stream));
}

// fsbar per patch, summed over boundary faces in face order
void reduce_fsbar(fv_adjoint_s* A, double* out) {
    fvgb::Solver& s = A->solver->s;
    std::vector<double> fb(4 * (size_t)A->Fb);
    std::vector<int> patch(A->Fb);
    if (A->Fb) {
        FV_CUDA(cudaMemcpyAsync(fb.data(), A->a.fsb, sizeof(double) * fb.size(), cudaMemcpyDeviceToHost, s.stream));
        FV_CUDA(cudaMemcpyAsync(patch.data(), A->a.fpatch + A->a.n_int_faces, sizeof(int) * A->Fb,
                                cudaMemcpyDeviceToHost, s.stream));
    }
    FV_CUDA(cudaStreamSynchronize(s.stream));
    for (int i = 0; i < 4 * A->P; ++i) out[i] = 0.0;
    for (int i = 0; i < A->Fb; ++i)
        for (int k = 0; k < 4; ++k) out[4 * patch[i] + k] += fb[4 * (size_t)i + k];
}

void linearise(fv_adjoint_s* A) {
    fvgb::Solver& s = A->solver->s;
    AdjArgs& a = A->a;
    fvgb::StepCtl ctl;
    s.read_ctl(ctl);
    a.cfl = ctl.cfl;  // the pseudo-time CFL number is the primal's
    if (a.order == 2) {
        fvgb::O2Args o = s.o2_args();
        o.U = A->U;
        o.W = A->W;
        o.G = A->G;
        o.cs = A->cs;
        o.lim_gu = A->Gu;
        o.lim_psi = A->psi;
        o.active = nullptr;
        o.d2 = nullptr;  // limited gradients into G (the linearisation reads them)
        fvgb::o2::launch_prim_f64(o, s.stream);
        check_launch();
        fvgb::o2::launch_part_f64(o, s.cfg, 0, 0, s.stream);
        check_launch();
    } else {
        fvgb::O2Args o{};
        o.m = s.dm;
        o.U = A->U;
        o.W = A->W;
        o.cs = A->cs;
        o.gamma = s.gamma;
        fvgb::o2::launch_prim_f64(o, s.stream);
        check_launch();
    }
    adjk::k_lin_face<<<blocks(A->F), kB, 0, s.stream>>>(a);
    check_launch();
    if (a.full) {
        adjk::k_lin_lim<<<blocks(A->N), kB, 0, s.stream>>>(a);
        check_launch();
    }
    adjk::k_lin_dt<<<blocks(A->N), kB, 0, s.stream>>>(a);
    check_launch();
    A->linearised = true;
}

void backward(fv_adjoint_s* A, const St* lam, int mode, St* out) {
    fvgb::Solver& s = A->solver->s;
    AdjArgs& a = A->a;
    if (A->Fb) FV_CUDA(cudaMemsetAsync(a.fsb, 0, sizeof(double) * 4 * (size_t)A->Fb, s.stream));
    adjk::k_bwd_face<<<blocks(A->F), kB, 0, s.stream>>>(a, lam);
    check_launch();
    adjk::k_bwd_cell1<<<blocks(A->N), kB, 0, s.stream>>>(a, mode, out, A->lam, A->lam0, A->rhs, A->partials);
    check_launch();
    if (a.order == 2) {
        adjk::k_bwd_cell2<<<blocks(A->N), kB, 0, s.stream>>>(a, mode, out, A->lam, A->lam0, A->rhs, A->partials);
        check_launch();
    }
    if (mode == 1) {
        adjk::k_adj_norms<<<1, 256, 0, s.stream>>>(A->partials, blocks(A->N), A->hist, A->counter, A->hist_cap);
        check_launch();
    }
}

// lam^T dR/dX over the mesh nodes (reference node numbering), lam a
// residual cotangent in device order.  The device computes the cotangents
// of the geometric quantities R depends on (face normals, lengths and
// midpoints, reconstruction offsets, least-squares weights, and with the
// full-limiter linearisation the limiter's offsets, eps^2 and boundary
// extremes); this host code runs the reverse pass of the geometry itself.
void residual_geometry_vjp(fv_adjoint_s* A, const fvgb::HostMesh& h, const St* lam, std::vector<double>& xb,
                           std::vector<double>& yb) {
    fvgb::Solver& s = A->solver->s;
    const int N = A->N, F = A->F, Fb = A->Fb;
    const size_t E = (size_t)(2 * F - Fb);
    AdjArgs& a = A->a;
    const bool lim = a.order == 2 && a.full;
    // cotangents on the device
    backward(A, lam, 0, A->Rdev);
    if (!A->geo_face) {
        A->geo_face = A->alloc<double>(8 * (size_t)F);
        A->geo_ab = A->alloc<double>(2 * E);
        A->geo_sb = A->alloc<double>(2 * (size_t)N);
        A->geo_nbg = A->alloc<double>(2 * (size_t)std::max(Fb, 1));
        A->geo_er = A->alloc<double>(2 * E);
        A->geo_ep = A->alloc<double>((size_t)N);
    }
    double *d_face = A->geo_face, *d_ab = A->geo_ab, *d_sb = A->geo_sb, *d_nbg = A->geo_nbg;
    FV_CUDA(cudaMemsetAsync(d_nbg, 0, sizeof(double) * 2 * (size_t)std::max(Fb, 1), s.stream));
    FV_CUDA(cudaMemsetAsync(d_ab, 0, sizeof(double) * 2 * E, s.stream));
    FV_CUDA(cudaMemsetAsync(d_sb, 0, sizeof(double) * 2 * (size_t)N, s.stream));
    adjk::k_geo_face<<<blocks(F), kB, 0, s.stream>>>(a, lam, d_face);
    check_launch();
    if (a.order == 2) {
        adjk::k_geo_cell<<<blocks(N), kB, 0, s.stream>>>(a, d_ab, d_sb, d_nbg);
        check_launch();
    }
    if (lim) {
        FV_CUDA(cudaMemsetAsync(A->geo_er, 0, sizeof(double) * 2 * E, s.stream));
        adjk::k_geo_lim<<<blocks(N), kB, 0, s.stream>>>(a, A->geo_er, A->geo_ep, d_nbg);
        check_launch();
    }
    std::vector<double> face(8 * (size_t)F), ab(2 * E), sb(2 * (size_t)N), nbg(2 * (size_t)std::max(Fb, 1));
    FV_CUDA(cudaMemcpyAsync(face.data(), d_face, sizeof(double) * face.size(), cudaMemcpyDeviceToHost, s.stream));
    FV_CUDA(cudaMemcpyAsync(ab.data(), d_ab, sizeof(double) * ab.size(), cudaMemcpyDeviceToHost, s.stream));
    FV_CUDA(cudaMemcpyAsync(sb.data(), d_sb, sizeof(double) * sb.size(), cudaMemcpyDeviceToHost, s.stream));
    FV_CUDA(cudaMemcpyAsync(nbg.data(), d_nbg, sizeof(double) * nbg.size(), cudaMemcpyDeviceToHost, s.stream));
    std::vector<double> er(lim ? 2 * E : 0), ep(lim ? (size_t)N : 0);
    if (lim) {
        FV_CUDA(cudaMemcpyAsync(er.data(), A->geo_er, sizeof(double) * er.size(), cudaMemcpyDeviceToHost, s.stream));
        FV_CUDA(cudaMemcpyAsync(ep.data(), A->geo_ep, sizeof(double) * ep.size(), cudaMemcpyDeviceToHost, s.stream));
    }
    FV_CUDA(cudaStreamSynchronize(s.stream));
    // cotangents of the geometric quantities, reference numbering
    std::vector<double> nxb(F, 0.0), nyb(F, 0.0), arb(F, 0.0), fxb(F, 0.0), fyb(F, 0.0), cxb(N, 0.0),
        cyb(N, 0.0);
    for (int i = 0; i < F; ++i) {
        const int f = h.fperm[i];
        const double* o = face.data() + 8 * (size_t)i;
        nxb[f] += o[0];
        nyb[f] += o[1];
        arb[f] += o[2];
        if (i >= h.n_int_faces) {
            nxb[f] += nbg[2 * (size_t)(i - h.n_int_faces)];
            nyb[f] += nbg[2 * (size_t)(i - h.n_int_faces) + 1];
        }
        if (a.order == 2) {
            // r_L = x_f - x_L, r_R = x_f - x_R
            fxb[f] += o[3]; fyb[f] += o[4];
            cxb[h.fl[f]] -= o[3]; cyb[h.fl[f]] -= o[4];
            if (h.fr[f] >= 0) {
                fxb[f] += o[5]; fyb[f] += o[6];
                cxb[h.fr[f]] -= o[5]; cyb[h.fr[f]] -= o[6];
            }
        }
    }
    if (a.order == 2) {
        // least-squares weights a_e = B w_e d_e, B = M^-1, M = sum w d d^T,
        // w = 1/|d|^2, d = x_nb - x_c (x_nb: neighbour centroid or the
        // boundary face midpoint); their sums s_c pass sbar to every a_e
        for (int i = 0; i < N; ++i) {
            const int c = h.perm[i];
            const double xc = h.cx[c], yc = h.cy[c];
            const int e0 = h.d_cf_off[i], e1 = h.d_cf_off[i + 1];
            double m00 = 0.0, m01 = 0.0, m11 = 0.0;
            for (int e = e0; e < e1; ++e) {
                const int f = h.fperm[h.d_cf[e] >> 1];
                double px, py;
                if (h.fr[f] < 0) { px = h.fxm[f]; py = h.fym[f]; }
                else { const int nb = h.fl[f] == c ? h.fr[f] : h.fl[f]; px = h.cx[nb]; py = h.cy[nb]; }
                const double dx = px - xc, dy = py - yc, w = 1.0 / (dx * dx + dy * dy);
                m00 += w * dx * dx; m01 += w * dx * dy; m11 += w * dy * dy;
            }
            const double det = m00 * m11 - m01 * m01;
            const double b00 = m11 / det, b01 = -m01 / det, b11 = m00 / det;
            double B00 = 0.0, B01 = 0.0, B10 = 0.0, B11 = 0.0;  // Bbar
            for (int e = e0; e < e1; ++e) {
                const int f = h.fperm[h.d_cf[e] >> 1];
                double px, py;
                if (h.fr[f] < 0) { px = h.fxm[f]; py = h.fym[f]; }
                else { const int nb = h.fl[f] == c ? h.fr[f] : h.fl[f]; px = h.cx[nb]; py = h.cy[nb]; }
                const double dx = px - xc, dy = py - yc, w = 1.0 / (dx * dx + dy * dy);
                const double ax = ab[2 * (size_t)e] + sb[2 * (size_t)i], ay = ab[2 * (size_t)e + 1] + sb[2 * (size_t)i + 1];
                B00 += ax * w * dx; B01 += ax * w * dy; B10 += ay * w * dx; B11 += ay * w * dy;
            }
            // Mbar = -B^T Bbar B^T (B symmetric)
            const double t00 = b00 * B00 + b01 * B10, t01 = b00 * B01 + b01 * B11;
            const double t10 = b01 * B00 + b11 * B10, t11 = b01 * B01 + b11 * B11;
            const double M00 = -(t00 * b00 + t01 * b01), M01 = -(t00 * b01 + t01 * b11);
            const double M10 = -(t10 * b00 + t11 * b01), M11 = -(t10 * b01 + t11 * b11);
            for (int e = e0; e < e1; ++e) {
                const int f = h.fperm[h.d_cf[e] >> 1];
                const bool bnd = h.fr[f] < 0;
                int nb = -1;
                double px, py;
                if (bnd) { px = h.fxm[f]; py = h.fym[f]; }
                else { nb = h.fl[f] == c ? h.fr[f] : h.fl[f]; px = h.cx[nb]; py = h.cy[nb]; }
                const double dx = px - xc, dy = py - yc, w = 1.0 / (dx * dx + dy * dy);
                const double ax = ab[2 * (size_t)e] + sb[2 * (size_t)i], ay = ab[2 * (size_t)e + 1] + sb[2 * (size_t)i + 1];
                // (w d)bar = B a_bar
                const double vx = b00 * ax + b01 * ay, vy = b01 * ax + b11 * ay;
                // M = sum w d d^T: dbar += w (Mbar + Mbar^T) d, wbar += d^T Mbar d
                double ddx = w * ((M00 + M00) * dx + (M01 + M10) * dy) + w * vx;
                double ddy = w * ((M10 + M01) * dx + (M11 + M11) * dy) + w * vy;
                const double wb = dx * (M00 * dx + M01 * dy) + dy * (M10 * dx + M11 * dy) + dx * vx + dy * vy;
                ddx += wb * (-2.0 * w * w * dx);
                ddy += wb * (-2.0 * w * w * dy);
                if (bnd) { fxb[f] += ddx; fyb[f] += ddy; }
                else { cxb[nb] += ddx; cyb[nb] += ddy; }
                cxb[c] -= ddx;
                cyb[c] -= ddy;
            }
        }
    }
    // limiter: extrapolation offsets x_f - x_c of the active entries, eps^2
    std::vector<double> epsb(lim ? N : 0, 0.0);
    if (lim) {
        for (int i = 0; i < N; ++i) {
            const int c = h.perm[i];
            for (int e = h.d_cf_off[i]; e < h.d_cf_off[i + 1]; ++e) {
                const double bx = er[2 * (size_t)e], by = er[2 * (size_t)e + 1];
                if (bx == 0.0 && by == 0.0) continue;
                const int f = h.fperm[h.d_cf[e] >> 1];
                fxb[f] += bx; fyb[f] += by;
                cxb[c] -= bx; cyb[c] -= by;
            }
            epsb[c] = ep[i];
        }
    }
    const double K3 = s.opt.venkat_k * s.opt.venkat_k * s.opt.venkat_k;
    // node cotangents of lam^T R
    const int nn = h.n_nodes;
    xb.assign(nn, 0.0);
    yb.assign(nn, 0.0);
    for (int c = 0; c < N; ++c) {
        const double eb = lim ? epsb[c] : 0.0;
        if (cxb[c] == 0.0 && cyb[c] == 0.0 && eb == 0.0) continue;
        const int64_t lo = h.cnode_off[c], hi = h.cnode_off[c + 1];
        const int k = (int)(hi - lo);
        const int32_t* ids = h.cnodes.data() + lo;
        double area = 0.0, Sx = 0.0, Sy = 0.0;
        for (int j = 0; j < k; ++j) {
            const int p0 = ids[j], p1 = ids[(j + 1) % k];
            const double cr = h.nx_[p0] * h.ny_[p1] - h.nx_[p1] * h.ny_[p0];
            area += cr;
            Sx += (h.nx_[p0] + h.nx_[p1]) * cr;
            Sy += (h.ny_[p0] + h.ny_[p1]) * cr;
        }
        area *= 0.5;
        // C = S / (6 area)
        const double Sbx = cxb[c] / (6.0 * area), Sby = cyb[c] / (6.0 * area);
        double Ab = -(cxb[c] * Sx + cyb[c] * Sy) / (6.0 * area * area);
        // eps^2 = K^3 V^1.5 with V = |area|
        if (eb != 0.0) Ab += eb * 1.5 * K3 * std::sqrt(std::fabs(area)) * (area < 0.0 ? -1.0 : 1.0);
        for (int j = 0; j < k; ++j) {
            const int p0 = ids[j], p1 = ids[(j + 1) % k];
            const double x0 = h.nx_[p0], y0 = h.ny_[p0], x1 = h.nx_[p1], y1 = h.ny_[p1];
            const double cr = x0 * y1 - x1 * y0;
            xb[p0] += Sbx * cr; xb[p1] += Sbx * cr;
            yb[p0] += Sby * cr; yb[p1] += Sby * cr;
            const double crb = Sbx * (x0 + x1) + Sby * (y0 + y1) + 0.5 * Ab;
            xb[p0] += crb * y1; yb[p1] += crb * x0;
            xb[p1] -= crb * y0; yb[p0] -= crb * x1;
        }
    }
    for (int f = 0; f < F; ++f) {
        const int n1 = h.fn1[f], n2 = h.fn2[f];
        const double dx = h.nx_[n2] - h.nx_[n1], dy = h.ny_[n2] - h.ny_[n1];
        const double ln = std::sqrt(dx * dx + dy * dy);
        // n = (dy, -dx) / ln, length ln, midpoint (p1 + p2) / 2
        const double lb = arb[f] - (nxb[f] * dy - nyb[f] * dx) / (ln * ln);
        const double dyb = nxb[f] / ln + lb * dy / ln;
        const double dxb = -nyb[f] / ln + lb * dx / ln;
        xb[n2] += dxb; xb[n1] -= dxb;
        yb[n2] += dyb; yb[n1] -= dyb;
        xb[n1] += 0.5 * fxb[f]; xb[n2] += 0.5 * fxb[f];
        yb[n1] += 0.5 * fyb[f]; yb[n2] += 0.5 * fyb[f];
    }
}

// One SSP-RK3 pseudo-time iteration of the adjoint, in place on A->lam:
// lam <- P(lam) = M lam + c, affine with c = P(0).
void rk_step(fv_adjoint_s* A) {
    for (int st = 1; st <= 3; ++st) backward(A, A->lam, st, nullptr);
}

// sqrt(<x, y>) or <x, y> into the device scalar *out
void kdot(fv_adjoint_s* A, const double* x, const double* y, double* out, bool sq) {
    fvgb::Solver& s = A->solver->s;
    const size_t n = 4 * (size_t)A->N;
    const int grid = (int)std::min<size_t>(adjk::kKGrid, (n + adjk::kKB - 1) / adjk::kKB);
    adjk::k_dot<<<grid, adjk::kKB, 0, s.stream>>>(x, y, n, A->kpart);
    adjk::k_fold<<<1, adjk::kKB, 0, s.stream>>>(A->kpart, grid, out, sq ? 1 : 0);
    check_launch();
}

}  // namespace

namespace adjh {
void linearise(fv_adjoint_s* A) { ::linearise(A); }
void lin_dt(fv_adjoint_s* A, double cfl) {
    fvgb::Solver& s = A->solver->s;
    A->a.cfl = cfl;
    adjk::k_lin_dt<<<blocks(A->N), kB, 0, s.stream>>>(A->a);
    check_launch();
}
void residual_dev(fv_adjoint_s* A, St* R) {
    fvgb::Solver& s = A->solver->s;
    adjk::k_res_cell<<<blocks(A->N), kB, 0, s.stream>>>(A->a, R);
    check_launch();
}
void jvp_dev(fv_adjoint_s* A, const St* dU, St* dR) {
    fvgb::Solver& s = A->solver->s;
    FV_CUDA(cudaMemsetAsync(A->dfs_dev, 0, sizeof(double) * 4 * fvgb::kMaxPatches, s.stream));
    adjk::k_fwd_cell1<<<blocks(A->N), kB, 0, s.stream>>>(A->a, dU);
    check_launch();
    if (A->a.order == 2) {
        adjk::k_fwd_cell2<<<blocks(A->N), kB, 0, s.stream>>>(A->a);
        check_launch();
    }
    adjk::k_fwd_face<<<blocks(A->F), kB, 0, s.stream>>>(A->a);
    check_launch();
    adjk::k_fwd_cell3<<<blocks(A->N), kB, 0, s.stream>>>(A->a, dR);
    check_launch();
}
void vjp_dev(fv_adjoint_s* A, const St* lam, St* out) { backward(A, lam, 0, out); }
void upload(fv_adjoint_s* A, const double* host_ref, St* dev) { upload_ref(A, host_ref, dev); }
void download(fv_adjoint_s* A, const St* dev, double* host_ref) { download_ref(A, dev, host_ref); }
void fsbar(fv_adjoint_s* A, double* out) { reduce_fsbar(A, out); }
}  // namespace adjh

void adjh::create(fv_solver_t solver, int limiter_mode, bool allow_batch, fv_adjoint_t* out) {
    {
        if (!solver || !out) fvgb::raise(FV_ERR_BAD_ARG, "null argument");
        if (limiter_mode != FV_ADJ_FROZEN_LIMITER && limiter_mode != FV_ADJ_FULL_LIMITER)
            fvgb::raise(FV_ERR_BAD_ARG, "limiter_mode: FV_ADJ_FROZEN_LIMITER or FV_ADJ_FULL_LIMITER");
        fvgb::Solver& s = solver->s;
        if (s.viscous || (s.batch && !allow_batch))
            fvgb::raise(FV_ERR_UNSUPPORTED, "adjoint: Euler solvers only (not NS, not batched)");
        if (s.opt.precision != FV_PREC_FP64) fvgb::raise(FV_ERR_UNSUPPORTED, "adjoint: FP64 solvers only");
        if (s.opt.flux != FV_FLUX_RUSANOV && s.opt.flux != FV_FLUX_HLLC)
            fvgb::raise(FV_ERR_UNSUPPORTED, "adjoint: Rusanov or HLLC flux");
        const int order = s.opt.order;
        if (order == 2 && (!s.general || s.opt.gradient != FV_GRAD_LSQ))
            fvgb::raise(FV_ERR_UNSUPPORTED, "adjoint: second order needs least-squares gradients");
        auto A = std::make_unique<fv_adjoint_s>();
        A->solver = solver;
        A->N = s.N;
        A->F = s.F;
        A->Fb = s.F - s.dm.n_int_faces;
        A->P = s.bc.n;
        AdjArgs& a = A->a;
        a.n_cells = s.N;
        a.n_faces = s.F;
        a.n_int_faces = s.dm.n_int_faces;
        a.order = order;
        a.flux = s.opt.flux;
        a.fl = s.dm.fl;
        a.fr = s.dm.fr;
        a.fpatch = s.dm.fpatch;
        a.fgeom = s.dm.fgeom;
        a.cf_off = s.dm.cf_off;
        a.cf = s.dm.cf;
        a.bc = s.bc;
        a.gamma = s.gamma;
        a.igm1 = 1.0 / (s.gamma - 1.0);
        const size_t N = s.N, F = s.F, Fb = A->Fb;
        A->U = A->alloc<St>(N);
        A->W = A->alloc<St>(N);
        A->cs = A->alloc<double>(N);
        A->stage_ref = A->alloc<St>(N);
        A->stage_dev = A->alloc<St>(N);
        A->lam = A->alloc<St>(N);
        A->lam0 = A->alloc<St>(N);
        A->rhs = A->alloc<St>(N);
        A->Rdev = A->alloc<St>(N);
        A->Gu = A->alloc<double2>(4 * N);
        A->G = A->alloc<double2>(4 * N);
        A->psi = A->alloc<double>(4 * N);
        A->partials = A->alloc<double>(4 * (size_t)blocks(s.N));
        A->counter = A->alloc<int>(1);
        A->dfs_dev = A->alloc<double>(4 * fvgb::kMaxPatches);
        a.W = A->W;
        a.Gu = A->Gu;
        a.psi = A->psi;
        a.JL = A->alloc<double>(16 * F);
        a.JR = A->alloc<double>(16 * F);
        a.Gb = A->alloc<double>(32 * Fb);
        a.fb = A->alloc<unsigned char>(F);
        a.F = A->alloc<St>(F);
        a.D = A->alloc<double>(N);
        a.wbar = A->alloc<double>(8 * F);
        a.Wbar = A->alloc<St>(N);
        a.Gub = A->alloc<double2>(4 * N);
        a.fsb = A->alloc<double>(4 * Fb);
        a.dW = A->alloc<St>(N);
        a.dG = A->alloc<double2>(4 * N);
        a.dF = A->alloc<St>(F);
        a.dfs = A->dfs_dev;
        if (order == 2) {
            a.cnb = s.cnb;
            a.lsq = static_cast<const double2*>(s.lsq);
            a.lsq_sum = static_cast<const double2*>(s.lsq_sum);
            a.frf = static_cast<const double4_32a*>(s.frf);
            a.limiter = s.opt.limiter;
            a.full = limiter_mode == FV_ADJ_FULL_LIMITER && s.opt.limiter != FV_LIM_NONE;
            if (a.full) {
                a.erf = static_cast<const double2*>(s.erf);
                a.eps2 = static_cast<const double*>(s.eps2);
                a.lside = A->alloc<signed char>(4 * N);
                a.led = A->alloc<int>(4 * N);
                a.ler = A->alloc<int>(4 * N);
                a.lpd = A->alloc<double2>(4 * N);
                a.lpe = A->alloc<double>(4 * N);
                a.ldb = A->alloc<double>(4 * N);
            }
            // twin entries: the entry of the neighbour's row through the same face
            const size_t E = (size_t)(2 * s.F - A->Fb);
            std::vector<int> off(N + 1), cf(E), cnb(E), twin(E, -1);
            FV_CUDA(cudaMemcpy(off.data(), s.dm.cf_off, sizeof(int) * (N + 1), cudaMemcpyDeviceToHost));
            FV_CUDA(cudaMemcpy(cf.data(), s.dm.cf, sizeof(int) * E, cudaMemcpyDeviceToHost));
            FV_CUDA(cudaMemcpy(cnb.data(), s.cnb, sizeof(int) * E, cudaMemcpyDeviceToHost));
            for (size_t c = 0; c < N; ++c)
                for (int e = off[c]; e < off[c + 1]; ++e) {
                    const int f = cf[e] >> 1, nb = cnb[e];
                    if (nb < 0) {
                        if (-1 - nb != f) fvgb::raise(FV_ERR_BAD_MESH, "adjoint: CSR and neighbour lists disagree");
                        continue;
                    }
                    for (int e2 = off[nb]; e2 < off[nb + 1]; ++e2)
                        if ((cf[e2] >> 1) == f) { twin[e] = e2; break; }
                    if (twin[e] < 0) fvgb::raise(FV_ERR_BAD_MESH, "adjoint: face without a twin entry");
                }
            int* d_twin = A->alloc<int>(E);
            fvgb::h2d_sync(d_twin, twin.data(), sizeof(int) * E, s.stream);
            a.twin = d_twin;
        }
        if (s.batch) {
            a.cell_inst = s.cell_inst;
            a.inst_fs = s.inst_fs;
        }
        *out = A.release();
    }
}

extern "C" {

int fv_adjoint_create(fv_solver_t solver, int32_t limiter_mode, fv_adjoint_t* out) {
    return fvgb::guarded([&] { adjh::create(solver, limiter_mode, false, out); });
}

int fv_adjoint_destroy(fv_adjoint_t adj) {
    return fvgb::guarded([&] { delete adj; });
}

int fv_residual_forward(fv_adjoint_t A, const double* U, double* R) {
    return fvgb::guarded([&] {
        if (!A) fvgb::raise(FV_ERR_BAD_ARG, "null adjoint");
        fvgb::Solver& s = A->solver->s;
        FV_CUDA(cudaStreamSynchronize(s.stream));
        if (U) upload_ref(A, U, A->U);
        else FV_CUDA(cudaMemcpyAsync(A->U, s.U, sizeof(St) * (size_t)A->N, cudaMemcpyDeviceToDevice, s.stream));
        linearise(A);
        A->solved = false;
        if (R) {
            adjk::k_res_cell<<<blocks(A->N), kB, 0, s.stream>>>(A->a, A->Rdev);
            check_launch();
            download_ref(A, A->Rdev, R);
        }
        FV_CUDA(cudaStreamSynchronize(s.stream));
    });
}

int fv_residual_jvp(fv_adjoint_t A, const double* dU, const double* dfs, double* dR) {
    return fvgb::guarded([&] {
        if (!A || !dU || !dR) fvgb::raise(FV_ERR_BAD_ARG, "null argument");
        if (!A->linearised) fvgb::raise(FV_ERR_BAD_ARG, "call fv_residual_forward first");
        fvgb::Solver& s = A->solver->s;
        std::vector<double> d(4 * fvgb::kMaxPatches, 0.0);
        if (dfs)
            for (int i = 0; i < 4 * A->P; ++i) d[i] = dfs[i];
        FV_CUDA(cudaMemcpyAsync(A->dfs_dev, d.data(), sizeof(double) * d.size(), cudaMemcpyHostToDevice, s.stream));
        upload_ref(A, dU, A->stage_dev);
        adjk::k_fwd_cell1<<<blocks(A->N), kB, 0, s.stream>>>(A->a, A->stage_dev);
        check_launch();
        if (A->a.order == 2) {
            adjk::k_fwd_cell2<<<blocks(A->N), kB, 0, s.stream>>>(A->a);
            check_launch();
        }
        adjk::k_fwd_face<<<blocks(A->F), kB, 0, s.stream>>>(A->a);
        check_launch();
        adjk::k_fwd_cell3<<<blocks(A->N), kB, 0, s.stream>>>(A->a, A->Rdev);
        check_launch();
        download_ref(A, A->Rdev, dR);
    });
}

int fv_residual_backward(fv_adjoint_t A, const double* Rbar, double* Ubar, double* fsbar) {
    return fvgb::guarded([&] {
        if (!A || !Rbar || !Ubar) fvgb::raise(FV_ERR_BAD_ARG, "null argument");
        if (!A->linearised) fvgb::raise(FV_ERR_BAD_ARG, "call fv_residual_forward first");
        upload_ref(A, Rbar, A->stage_dev);
        backward(A, A->stage_dev, 0, A->Rdev);
        download_ref(A, A->Rdev, Ubar);
        if (fsbar) reduce_fsbar(A, fsbar);
    });
}

int fv_adjoint_solve(fv_adjoint_t A, const double* dJdU, int32_t max_iter, double tol, double* lambda,
                     double* fsbar, double* history, int32_t* iterations) {
    return fvgb::guarded([&] {
        if (!A || !dJdU || max_iter < 0) fvgb::raise(FV_ERR_BAD_ARG, "bad argument");
        if (!A->linearised) fvgb::raise(FV_ERR_BAD_ARG, "call fv_residual_forward first");
        fvgb::Solver& s = A->solver->s;
        if (A->hist_cap < max_iter) {
            if (A->hist) cudaFree(A->hist);
            A->hist = nullptr;
            FV_CUDA(cudaMalloc(&A->hist, sizeof(double) * 4 * (size_t)std::max(max_iter, 1)));
            A->hist_cap = max_iter;
        }
        upload_ref(A, dJdU, A->rhs);
        FV_CUDA(cudaMemsetAsync(A->lam, 0, sizeof(St) * (size_t)A->N, s.stream));
        FV_CUDA(cudaMemsetAsync(A->counter, 0, sizeof(int), s.stream));
        // SSP-RK3 in pseudo-time; the stage-0 residual norm is checked every chunk
        const int chunk = 50;
        int done = 0;
        std::vector<double> last(4);
        while (done < max_iter) {
            const int n = std::min(chunk, max_iter - done);
            for (int i = 0; i < n; ++i)
                for (int st = 1; st <= 3; ++st) backward(A, A->lam, st, nullptr);
            done += n;
            FV_CUDA(cudaMemcpyAsync(last.data(), A->hist + 4 * (size_t)(done - 1), sizeof(double) * 4,
                                    cudaMemcpyDeviceToHost, s.stream));
            FV_CUDA(cudaStreamSynchronize(s.stream));
            if (!std::isfinite(last[0])) fvgb::raise(FV_ERR_NONFINITE, "adjoint iteration diverged");
            if (tol > 0 && last[0] < tol && last[1] < tol && last[2] < tol && last[3] < tol) break;
        }
        if (iterations) *iterations = done;
        if (history && done)
            FV_CUDA(cudaMemcpy(history, A->hist, sizeof(double) * 4 * (size_t)done, cudaMemcpyDeviceToHost));
        A->solved = true;
        if (lambda) download_ref(A, A->lam, lambda);
        if (fsbar) {
            // lam^T dR/dfs at the converged lam
            backward(A, A->lam, 0, A->Rdev);
            reduce_fsbar(A, fsbar);
        }
        FV_CUDA(cudaStreamSynchronize(s.stream));
    });
}

// Restarted GMRES on the fixed point of the pseudo-time iteration:
// lam = P(lam) = M lam + c  <=>  (I - M) lam = c, each application of
// (I - M) one SSP-RK3 pseudo-time iteration.  The fixed point is the
// adjoint solution whatever the spectral radius of M: GMRES converges
// where the iteration itself diverges (a primal whose explicit iteration
// limit-cycles at the converged state, or a frozen-limiter linearisation
// with growing modes).  Arnoldi with modified Gram-Schmidt; the Hessenberg
// columns come to the host once per matvec for the Givens rotations.
int fv_adjoint_solve_gmres(fv_adjoint_t A, const double* dJdU, int32_t restart, int32_t max_matvec, double rtol,
                           double* lambda, double* fsbar, double* history, int32_t* matvecs, double residual[4]) {
    return fvgb::guarded([&] {
        if (!A || !dJdU || restart < 1 || max_matvec < 1 || !(rtol > 0.0)) fvgb::raise(FV_ERR_BAD_ARG, "bad argument");
        if (!A->linearised) fvgb::raise(FV_ERR_BAD_ARG, "call fv_residual_forward first");
        fvgb::Solver& s = A->solver->s;
        const size_t n = 4 * (size_t)A->N;
        const int m = restart;
        if (A->k_restart < m) {
            // a larger basis replaces the smaller one (the old buffers stay owned until destroy)
            A->kV = A->alloc<double>((size_t)(m + 1) * n);
            A->kh = A->alloc<double>((size_t)m + 2);
            A->k_restart = m;
        }
        if (!A->kc) {
            A->kc = A->alloc<double>(n);
            A->kw = A->alloc<double>(n);
            A->kx = A->alloc<double>(n);
            A->kpart = A->alloc<double>(adjk::kKGrid);
        }
        const int vb = (int)((n + 255) / 256);
        double* lam = reinterpret_cast<double*>(A->lam);
        auto V = [&](int i) { return A->kV + (size_t)i * n; };
        upload_ref(A, dJdU, A->rhs);
        // c = P(0)
        FV_CUDA(cudaMemsetAsync(A->lam, 0, sizeof(St) * (size_t)A->N, s.stream));
        FV_CUDA(cudaMemsetAsync(A->counter, 0, sizeof(int), s.stream));
        rk_step(A);
        FV_CUDA(cudaMemcpyAsync(A->kc, lam, sizeof(double) * n, cudaMemcpyDeviceToDevice, s.stream));
        FV_CUDA(cudaMemsetAsync(A->kx, 0, sizeof(double) * n, s.stream));
        double beta0 = 0.0;
        kdot(A, A->kc, A->kc, A->kh, true);
        FV_CUDA(cudaMemcpyAsync(&beta0, A->kh, sizeof(double), cudaMemcpyDeviceToHost, s.stream));
        FV_CUDA(cudaStreamSynchronize(s.stream));
        if (!std::isfinite(beta0)) fvgb::raise(FV_ERR_NONFINITE, "adjoint GMRES: non-finite right-hand side");
        int mv = 1;  // c = P(0) took one pseudo-time iteration
        std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), y(m), hcol(m + 2);
        std::vector<double> hh((size_t)max_matvec, -1.0);  // relative residual after each matvec
        hh[0] = 1.0;
        bool done = beta0 == 0.0;
        while (!done && mv < max_matvec) {
            // r = c - (I - M) x = P(x) - x
            FV_CUDA(cudaMemcpyAsync(lam, A->kx, sizeof(double) * n, cudaMemcpyDeviceToDevice, s.stream));
            rk_step(A);
            ++mv;
            adjk::k_sub<<<vb, 256, 0, s.stream>>>(V(0), lam, A->kx, n);
            kdot(A, V(0), V(0), A->kh, true);
            double beta = 0.0;
            FV_CUDA(cudaMemcpyAsync(&beta, A->kh, sizeof(double), cudaMemcpyDeviceToHost, s.stream));
            FV_CUDA(cudaStreamSynchronize(s.stream));
            if (!std::isfinite(beta)) fvgb::raise(FV_ERR_NONFINITE, "adjoint GMRES diverged");
            hh[mv - 1] = beta / beta0;
            if (beta <= rtol * beta0) break;
            adjk::k_div_dev<<<vb, 256, 0, s.stream>>>(V(0), V(0), A->kh, n);
            check_launch();
            std::fill(g.begin(), g.end(), 0.0);
            g[0] = beta;
            int k = 0;
            for (int j = 0; j < m && mv < max_matvec; ++j) {
                // w = (I - M) V_j = V_j - P(V_j) + c
                FV_CUDA(cudaMemcpyAsync(lam, V(j), sizeof(double) * n, cudaMemcpyDeviceToDevice, s.stream));
                rk_step(A);
                ++mv;
                adjk::k_fp_apply<<<vb, 256, 0, s.stream>>>(A->kw, V(j), lam, A->kc, n);
                for (int i = 0; i <= j; ++i) {
                    kdot(A, A->kw, V(i), A->kh + i, false);
                    adjk::k_axmy_dev<<<vb, 256, 0, s.stream>>>(A->kw, V(i), A->kh + i, n);
                }
                kdot(A, A->kw, A->kw, A->kh + j + 1, true);
                FV_CUDA(cudaMemcpyAsync(hcol.data(), A->kh, sizeof(double) * (j + 2), cudaMemcpyDeviceToHost,
                                        s.stream));
                FV_CUDA(cudaStreamSynchronize(s.stream));
                for (int i = 0; i <= j + 1; ++i)
                    if (!std::isfinite(hcol[i])) fvgb::raise(FV_ERR_NONFINITE, "adjoint GMRES diverged");
                const double hnext = hcol[j + 1];
                if (hnext > 0.0) {
                    adjk::k_div_dev<<<vb, 256, 0, s.stream>>>(V(j + 1), A->kw, A->kh + j + 1, n);
                    check_launch();
                }
                // Givens rotations of column j
                for (int i = 0; i < j; ++i) {
                    const double t = cs[i] * hcol[i] + sn[i] * hcol[i + 1];
                    hcol[i + 1] = -sn[i] * hcol[i] + cs[i] * hcol[i + 1];
                    hcol[i] = t;
                }
                const double den = std::hypot(hcol[j], hcol[j + 1]);
                cs[j] = den > 0.0 ? hcol[j] / den : 1.0;
                sn[j] = den > 0.0 ? hcol[j + 1] / den : 0.0;
                hcol[j] = den;
                g[j + 1] = -sn[j] * g[j];
                g[j] = cs[j] * g[j];
                for (int i = 0; i <= j; ++i) H[(size_t)i * m + j] = hcol[i];
                k = j + 1;
                const double res = std::fabs(g[j + 1]);
                hh[mv - 1] = res / beta0;
                if (res <= rtol * beta0 || !(hnext > 0.0)) {
                    done = true;
                    break;
                }
            }
            // x += V y, H y = g (upper triangular, k x k)
            for (int i = k - 1; i >= 0; --i) {
                double t = g[i];
                for (int l = i + 1; l < k; ++l) t -= H[(size_t)i * m + l] * y[l];
                y[i] = t / H[(size_t)i * m + i];
            }
            for (int i = 0; i < k; ++i) {
                adjk::k_axpy<<<vb, 256, 0, s.stream>>>(A->kx, V(i), y[i], n);
                check_launch();
            }
        }
        if (matvecs) *matvecs = mv;
        if (history)
            for (int i = 0; i < mv && i < max_matvec; ++i) history[i] = hh[i] >= 0.0 ? hh[i] : (i ? history[i - 1] : 1.0);
        // lam = x; the adjoint residual norms (dR/dU)^T lam - dJdU of one stage-0 evaluation
        if (A->hist_cap < 1) {
            if (A->hist) cudaFree(A->hist);
            A->hist = nullptr;
            FV_CUDA(cudaMalloc(&A->hist, sizeof(double) * 4));
            A->hist_cap = 1;
        }
        FV_CUDA(cudaMemcpyAsync(lam, A->kx, sizeof(double) * n, cudaMemcpyDeviceToDevice, s.stream));
        FV_CUDA(cudaMemsetAsync(A->counter, 0, sizeof(int), s.stream));
        backward(A, A->lam, 1, nullptr);
        double r4[4];
        FV_CUDA(cudaMemcpyAsync(r4, A->hist, sizeof(double) * 4, cudaMemcpyDeviceToHost, s.stream));
        FV_CUDA(cudaMemcpyAsync(lam, A->kx, sizeof(double) * n, cudaMemcpyDeviceToDevice, s.stream));
        FV_CUDA(cudaStreamSynchronize(s.stream));
        if (residual)
            for (int q = 0; q < 4; ++q) residual[q] = r4[q];
        A->solved = true;
        if (lambda) download_ref(A, A->lam, lambda);
        if (fsbar) {
            backward(A, A->lam, 0, A->Rdev);
            reduce_fsbar(A, fsbar);
        }
        FV_CUDA(cudaStreamSynchronize(s.stream));
    });
}

// Shape gradient: dJ/dX over the mesh nodes, X in the caller's node
// numbering, with J a wall-force coefficient and lam the adjoint of the
// last fv_adjoint_solve (which must have been solved for the same J).
// dJ/dX = dJ/dX|explicit - lam^T dR/dX, where R depends on the nodes
// through the face normals, lengths and midpoints, the cell centroids
// (shoelace, src/MeshReader.cpp:56-76), the least-squares weights built
// from them and (full-limiter linearisation only) the limiter values.
int fv_adjoint_shape_gradient(fv_adjoint_t A, fv_mesh_t mesh, int32_t objective, const double ref[7],
                              double* dJdX) {
    return fvgb::guarded([&] {
        if (!A || !mesh || !ref || !dJdX) fvgb::raise(FV_ERR_BAD_ARG, "null argument");
        if (!A->solved) fvgb::raise(FV_ERR_BAD_ARG, "call fv_adjoint_solve first");
        if (objective < 0 || objective > 2) fvgb::raise(FV_ERR_BAD_ARG, "objective: 0 drag, 1 lift, 2 moment");
        const fvgb::HostMesh& h = fvgb::host_mesh_of(mesh);
        fvgb::Solver& s = A->solver->s;
        if (h.n_cells != A->N || h.n_faces != A->F) fvgb::raise(FV_ERR_BAD_ARG, "mesh does not match the solver");
        if (h.cnode_off.empty())
            fvgb::raise(FV_ERR_UNSUPPORTED, "shape gradient: the mesh must be built from cell polygons");
        std::vector<double> xb, yb;
        residual_geometry_vjp(A, h, A->lam, xb, yb);
        const int N = A->N, nn = h.n_nodes;
        // explicit part: J = sum_wall p_c (k . n) |f| / qL at the adjoint's state
        std::vector<double> U(4 * (size_t)N);
        download_ref(A, A->U, U.data());
        const double vmag = std::hypot(ref[1], ref[2]);
        const double ddx = ref[1] / vmag, ddy = ref[2] / vmag;
        const double qL = 0.5 * ref[0] * vmag * vmag * ref[4];
        const double g = s.gamma;
        std::vector<double> ex(nn, 0.0), ey(nn, 0.0);
        for (const fvgb::WallFace& w : s.wall_faces) {
            int f = -1;
            // the wall face in reference numbering
            f = h.fperm[w.dev_face];
            const double* u = U.data() + 4 * (size_t)w.cell;
            const double uu = u[1] / u[0], vv = u[2] / u[0];
            const double p = (g - 1.0) * (u[3] - 0.5 * u[0] * (uu * uu + vv * vv));
            const int n1 = h.fn1[f], n2 = h.fn2[f];
            const double dx = h.nx_[n2] - h.nx_[n1], dy = h.ny_[n2] - h.ny_[n1];
            double bdx, bdy, bxm = 0.0, bym = 0.0;
            if (objective == 0) { bdy = p * ddx / qL; bdx = -p * ddy / qL; }
            else if (objective == 1) { bdy = p * (-ddy) / qL; bdx = -p * ddx / qL; }
            else {
                const double L = ref[4];
                const double rx = 0.5 * (h.nx_[n1] + h.nx_[n2]) - ref[5], ry = 0.5 * (h.ny_[n1] + h.ny_[n2]) - ref[6];
                // J = -p (rx dx + ry dy) / (qL L)
                bdx = -p * rx / (qL * L);
                bdy = -p * ry / (qL * L);
                bxm = -p * dx / (qL * L);
                bym = -p * dy / (qL * L);
            }
            ex[n2] += bdx; ex[n1] -= bdx;
            ey[n2] += bdy; ey[n1] -= bdy;
            ex[n1] += 0.5 * bxm; ex[n2] += 0.5 * bxm;
            ey[n1] += 0.5 * bym; ey[n2] += 0.5 * bym;
        }
        for (int i = 0; i < nn; ++i) {
            dJdX[2 * (size_t)i] = ex[i] - xb[i];
            dJdX[2 * (size_t)i + 1] = ey[i] - yb[i];
        }
    });
}

// (dR/dX)^T Rbar over the mesh nodes at the linearisation state.
int fv_residual_shape_vjp(fv_adjoint_t A, fv_mesh_t mesh, const double* Rbar, double* Xbar) {
    return fvgb::guarded([&] {
        if (!A || !mesh || !Rbar || !Xbar) fvgb::raise(FV_ERR_BAD_ARG, "null argument");
        if (!A->linearised) fvgb::raise(FV_ERR_BAD_ARG, "call fv_residual_forward first");
        const fvgb::HostMesh& h = fvgb::host_mesh_of(mesh);
        if (h.n_cells != A->N || h.n_faces != A->F) fvgb::raise(FV_ERR_BAD_ARG, "mesh does not match the solver");
        if (h.cnode_off.empty())
            fvgb::raise(FV_ERR_UNSUPPORTED, "shape cotangent: the mesh must be built from cell polygons");
        upload_ref(A, Rbar, A->stage_dev);
        std::vector<double> xb, yb;
        residual_geometry_vjp(A, h, A->stage_dev, xb, yb);
        for (int i = 0; i < h.n_nodes; ++i) {
            Xbar[2 * (size_t)i] = xb[i];
            Xbar[2 * (size_t)i + 1] = yb[i];
        }
    });
}

// dJ/dU of a wall-force coefficient (pressure part, owner-cell pressure as
// in compute_wall_forces, src/WallTraction.cpp:163-217) at the solver's
// current state, in reference cell order; returns J.
int fv_force_gradient(fv_solver_t solver, int32_t objective, const double ref[7], double* value, double* dJdU) {
    return fvgb::guarded([&] {
        if (!solver || !ref) fvgb::raise(FV_ERR_BAD_ARG, "null argument");
        if (objective < 0 || objective > 2) fvgb::raise(FV_ERR_BAD_ARG, "objective: 0 drag, 1 lift, 2 moment");
        fvgb::Solver& s = solver->s;
        if (s.viscous) fvgb::raise(FV_ERR_UNSUPPORTED, "force gradient: Euler solvers only");
        std::vector<double> f(4 * (size_t)s.N);
        s.download_field(f.data());
        const double vmag = std::hypot(ref[1], ref[2]);
        const double dx = ref[1] / vmag, dy = ref[2] / vmag, lx = -dy, ly = dx;
        const double qL = 0.5 * ref[0] * vmag * vmag * ref[4];
        const double g = s.gamma;
        if (dJdU) std::memset(dJdU, 0, sizeof(double) * 4 * (size_t)s.N);
        double J = 0.0;
        for (const fvgb::WallFace& w : s.wall_faces) {
            const double* u = f.data() + 4 * (size_t)w.cell;
            const double uu = u[1] / u[0], vv = u[2] / u[0];
            const double p = (g - 1.0) * (u[3] - 0.5 * u[0] * (uu * uu + vv * vv));
            double kx, ky;
            if (objective == 0) { kx = dx; ky = dy; }
            else if (objective == 1) { kx = lx; ky = ly; }
            else {
                // moment about (ref[5], ref[6]) of the force A p n, over qL * L
                const double rx = w.xm - ref[5], ry = w.ym - ref[6];
                kx = -ry / ref[4];
                ky = rx / ref[4];
            }
            const double c = w.area * (w.nx * kx + w.ny * ky) / qL;
            J += c * p;
            if (dJdU) {
                double* d = dJdU + 4 * (size_t)w.cell;
                d[0] += c * (g - 1.0) * 0.5 * (uu * uu + vv * vv);
                d[1] += c * (g - 1.0) * (-uu);
                d[2] += c * (g - 1.0) * (-vv);
                d[3] += c * (g - 1.0);
            }
        }
        if (value) *value = J;
    });
}

}  // extern "C"
