// Spalart-Allmaras RANS explicit step: RANSTurbulenceSASolver::step /
// compute_dt / build_boundary_fields / build_boundary_nut / ghost_state
// (src/RANSTurbulenceSASolver.cpp), the SA-noft2 source terms of
// compute_sa_source_terms (src/SpalartAllmaras.cpp), the wall distance of
// compute_wall_distance (src/WallDistance.cpp:26-44) and the wall traction
// with the effective viscosity (src/WallTraction.cpp:95-142).
//
//   k_sa_wall_distance  min over no-slip wall segments of the clamped
//                       point-segment distance from the cell centroid
//   k_sa_prim           u, v, T, nu-tilde; nu = mu / rho, nu_t = nut fv1
//   k_sa_grad           gradients of u, v, T and nu-tilde with the boundary
//                       values of build_boundary_fields / build_boundary_nut
//   k_sa_face           viscous CFL candidate with nu + nu_t, inviscid flux,
//                       first-order upwind nu-tilde advection, viscous flux
//                       with mu + rho nu_t and cp (mu/Pr + rho nu_t/Pr_t),
//                       nu-tilde diffusion (nu + nu_t) / sigma
//   k_sa_cell           gather of both fluxes, volume x (production -
//                       destruction + cross diffusion), five norms, update
// Built twice: without FMA contraction, in the reference's evaluation order
// (this file), and with contraction (rans_fast.cu defines FV_NS_FAST and
// includes it; kernel namespace ransk_fast, launchers suffixed _fast).
#ifdef FV_NS_FAST
#define FV_KNS ransk_fast
#define FV_NS_FN(name) name##_fast
#else
#define FV_KNS ransk
#define FV_NS_FN(name) name
#endif
#include "euler_o1.cuh"
#include "gradients.cuh"
#include "rans.h"

namespace FV_KNS {

using fvgb::RansArgs;

// sa_fv1 / sa_eddy_viscosity (src/SpalartAllmaras.cpp)
__device__ __forceinline__ double sa_fv1(double nut, double nu, const double* c) {
    if (nut <= 0.0) return 0.0;
    double chi = nut / nu;
    double chi3 = chi * chi * chi;
    return chi3 / (chi3 + c[6] * c[6] * c[6]);
}
__device__ __forceinline__ double sa_nut(double nut, double nu, const double* c) { return nut * sa_fv1(nut, nu, c); }

// constants c[]: cb1, cb2, sigma, kappa, cw2, cw3, cv1, cv2, cv3; cw3_6 = cw3^6.
// The model's integer powers r^6, g^6 are formed by three multiplies and
// its sixth root as cbrt(sqrt(.)): within a few ulp of pow(), at a small
// fraction of its FP64-pipe cost.
__device__ __forceinline__ double sa_source(double nut, double nu, double omega, double d, double gx, double gy,
                                            const double* c, double cw3_6) {
    const double cb1 = c[0], cb2 = c[1], sigma = c[2], kappa = c[3], cw2 = c[4], cv2 = c[7], cv3 = c[8];
    double chi = (nut > 0.0) ? nut / nu : 0.0;
    double fv1 = sa_fv1(nut, nu, c);
    double fv2 = 1.0 - chi / (1.0 + chi * fv1);
    double d2 = d * d;
    double s_bar = (nut / (kappa * kappa * d2)) * fv2;
    double s_tilde;
    if (s_bar >= -cv2 * omega) s_tilde = omega + s_bar;
    else s_tilde = omega + omega * (cv2 * cv2 * omega + cv3 * s_bar) / ((cv3 - 2.0 * cv2) * omega - s_bar);
    const double production = cb1 * s_tilde * nut;
    double destruction = 0.0;
    if (nut > 0.0) {
        double s_tilde_safe = rmax(s_tilde, 1e-10);
        double r = rmin(nut / (s_tilde_safe * kappa * kappa * d2), 10.0);
        const double r2 = r * r;
        double g = r + cw2 * (r2 * r2 * r2 - r);
        const double g2 = g * g;
        double fw = g * cbrt(sqrt((1.0 + cw3_6) / (g2 * g2 * g2 + cw3_6)));
        double nut_over_d = nut / d;
        const double cw1 = cb1 / (kappa * kappa) + (1.0 + cb2) / sigma;
        destruction = cw1 * fw * nut_over_d * nut_over_d;
    }
    const double cross = (cb2 / sigma) * (gx * gx + gy * gy);
    return production - destruction + cross;
}

__global__ void k_sa_wall_distance(const RansArgs a, const double4_32a* __restrict__ seg, int n_seg) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.ns.g.n_cells) return;
    const double2 p = a.cxy[c];
    double best = INFINITY;
    for (int i = 0; i < n_seg; ++i) {
        const double4_32a s = seg[i];
        double dx = s.z - s.x, dy = s.w - s.y;
        double len_sq = dx * dx + dy * dy;
        double t = (len_sq > 0.0) ? ((p.x - s.x) * dx + (p.y - s.y) * dy) / len_sq : 0.0;
        t = (t < 0.0) ? 0.0 : ((1.0 < t) ? 1.0 : t);
        double ex = p.x - (s.x + t * dx);
        double ey = p.y - (s.y + t * dy);
        double d2 = ex * ex + ey * ey;
        best = rmin(best, d2);
    }
    a.walld[c] = sqrt(best);
}

__global__ void __launch_bounds__(fvgb::kCellBlock) k_sa_prim(const RansArgs a) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.ns.g.n_cells) return;
    const St s = ld_state(a.ns.U, c);
    double4_32a w;
    w.x = s.ru / s.r;
    w.y = s.rv / s.r;
    w.z = pressure(s, a.ns.gamma) / (s.r * a.ns.gas_constant);
    w.w = a.nut[c];
    a.ns.prim[c] = w;
    const double nu = a.ns.mu / s.r;
    a.nu[c] = make_double2(nu, sa_nut(w.w, nu, a.sa));
}

// build_boundary_fields / build_boundary_nut for one boundary face owned by
// cell cl, variable k (0 u, 1 v, 2 T, 3 nu-tilde).
__device__ __forceinline__ double boundary_field(const RansArgs& a, int face, int cl, int k) {
    const int p = a.ns.fpatch[face];
    const int t = a.ns.bc.type[p];
    const double4_32a w = a.ns.prim[cl];
    if (k == 3) {
        if (t == BC_NOSLIP) return 0.0;
        if (t == BC_FARFIELD) return a.farfield_nut[p];
        return w.w;
    }
    if (t == BC_NOSLIP) {
        if (k == 0) return a.ns.bc.wall_u[p];
        if (k == 1) return a.ns.bc.wall_v[p];
        return a.ns.bc.isothermal[p] ? a.ns.bc.wall_T[p] : w.z;
    }
    return k == 0 ? w.x : (k == 1 ? w.y : w.z);
}

__global__ void __launch_bounds__(fvgb::kCellBlock) k_sa_grad(const RansArgs a) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.ns.g.n_cells) return;
    double gx[4], gy[4];
    fvgb::cell_gradient<4>(
        a.ns.g, c,
        [&](int i, int k) {
            const double4_32a w = a.ns.prim[i];
            return k == 0 ? w.x : (k == 1 ? w.y : (k == 2 ? w.z : w.w));
        },
        [&](int f, int k) { return boundary_field(a, f, c, k); }, gx, gy);
#pragma unroll
    for (int k = 0; k < 4; ++k) a.grad[4 * c + k] = make_double2(gx[k], gy[k]);
}

template <int FLUX>
__global__ void __launch_bounds__(fvgb::kFaceBlock) k_sa_face(const RansArgs a) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    double cand = DBL_MAX;
    if (f < a.ns.g.n_faces) {
        const fvgb::NSArgs& n = a.ns;
        const int cl = n.fl[f], cr = n.g.fr[f];
        const bool bnd = cr < 0;
        const double4_32a geo = n.fgeom[f];
        const double nx = geo.x, ny = geo.y, area = geo.z;
        const double* fg = n.g.fgrad + 8 * (size_t)f;
        const St UL = ld_state(n.U, cl);
        const St UR = bnd ? ghost_state(n.bc, n.fpatch[f], UL, nx, ny, n.gamma) : ld_state(n.U, cr);
        const double2 nuL = a.nu[cl];
        const double4_32a wl = n.prim[cl];
        // interior neighbour's primitives and (nu, nu_t); the cell pass
        // formed them from the same U by the same operations (u = ru / r,
        // nu = mu / r, nu_t = sa_nut(nut, nu)), so reading them is exact
        const double4_32a wr = bnd ? wl : n.prim[cr];
        const double2 nuR = bnd ? nuL : a.nu[cr];

        // compute_dt (src/RANSTurbulenceSASolver.cpp, nu + nu_t diffusion limit)
        {
            double VnL = wl.x * nx + wl.y * ny;
            double Smax = fabs(VnL) + sound_speed(UL, n.gamma);
            double nu_t_max = nuL.y;
            // mu / min(rho_L, rho_R) = max(mu / rho_L, mu / rho_R) (rounding is monotone)
            double nu_max = nuL.x;
            if (!bnd) {
                double VnR = wr.x * nx + wr.y * ny;
                Smax = rmax(Smax, fabs(VnR) + sound_speed(UR, n.gamma));
                nu_max = rmax(nu_max, nuR.x);
                nu_t_max = rmax(nu_t_max, nuR.y);
            }
            const double length = fg[5];
            const double nu_lam = (n.mu > 0.0) ? nu_max : 0.0;
            const double nu_eff = nu_lam + nu_t_max;
            const double Smax_total = Smax + 2.0 * nu_eff / length;
            cand = n.ctl->cfl * length / Smax_total;
        }

        const St inv = num_flux<FLUX>(UL, UR, nx, ny, n.gamma, n.exact_tol, n.exact_max_iter);
        const double nut_L = wl.w;
        const double nut_R = bnd ? boundary_field(a, f, cl, 3) : wr.w;
        // advection with the face-averaged velocity of the inviscid state pair
        const double u_R_ghost = bnd ? UR.ru / UR.r : wr.x, v_R_ghost = bnd ? UR.rv / UR.r : wr.y;
        const double Vn = 0.5 * ((wl.x + u_R_ghost) * nx + (wl.y + v_R_ghost) * ny);
        const double nut_upwind = (Vn >= 0.0) ? nut_L : nut_R;
        const double nut_adv = Vn * nut_upwind * area;

        St visc = st_make(0.0, 0.0, 0.0, 0.0);
        double nut_diff = 0.0;
        const int p = bnd ? n.fpatch[f] : 0;
        const bool has_visc = !bnd || n.bc.type[p] == BC_NOSLIP;
        if (has_visc) {
            double pR[3];
            double2 gR[4];
            if (bnd) {
                for (int k = 0; k < 3; ++k) pR[k] = boundary_field(a, f, cl, k);
                for (int k = 0; k < 4; ++k) gR[k] = make_double2(0.0, 0.0);
            } else {
                pR[0] = wr.x; pR[1] = wr.y; pR[2] = wr.z;
                for (int k = 0; k < 4; ++k) gR[k] = a.grad[4 * cr + k];
            }
            const double pL[3] = {wl.x, wl.y, wl.z};
            fvgb::FaceGrad fgv[3];
            for (int k = 0; k < 3; ++k) {
                const double2 gL = a.grad[4 * cl + k];
                fgv[k] = fvgb::face_gradient(fg, bnd, pL[k], pR[k], gL.x, gL.y, gR[k].x, gR[k].y);
            }
            const double nu_lam_R = nuR.x;
            const double nu_t_R = bnd ? sa_nut(nut_R, nu_lam_R, a.sa) : nuR.y;
            const double rho_R = bnd ? UL.r : UR.r;
            const double turb = 0.5 * (UL.r * nuL.y + rho_R * nu_t_R);
            const double mu_eff = n.mu + turb;
            const double k_eff = a.k_lam + a.cp * turb / a.prandtl_t;
            const double u_face = bnd ? pR[0] : 0.5 * (wl.x + pR[0]);
            const double v_face = bnd ? pR[1] : 0.5 * (wl.y + pR[1]);
            const double div_v = fgv[0].gx + fgv[1].gy;
            const double tau_xx = mu_eff * (2.0 * fgv[0].gx - (2.0 / 3.0) * div_v);
            const double tau_yy = mu_eff * (2.0 * fgv[1].gy - (2.0 / 3.0) * div_v);
            const double tau_xy = mu_eff * (fgv[0].gy + fgv[1].gx);
            double qx = -k_eff * fgv[2].gx;
            double qy = -k_eff * fgv[2].gy;
            if (bnd && !n.bc.isothermal[p]) {
                qx = 0.0;
                qy = 0.0;
            }
            visc.ru = tau_xx * nx + tau_xy * ny;
            visc.rv = tau_xy * nx + tau_yy * ny;
            visc.E = (u_face * tau_xx + v_face * tau_xy - qx) * nx + (u_face * tau_xy + v_face * tau_yy - qy) * ny;

            const double nu_lam_face = 0.5 * (nuL.x + nu_lam_R);
            const double nu_t_face = 0.5 * (nuL.y + nu_t_R);
            const double2 gnL = a.grad[4 * cl + 3];
            const fvgb::FaceGrad fn = fvgb::face_gradient(fg, bnd, nut_L, nut_R, gnL.x, gnL.y, gR[3].x, gR[3].y);
            const double diffusivity = (nu_lam_face + nu_t_face) / a.sa[2];
            nut_diff = -diffusivity * fn.dphidn * area;
        }
        st_state(n.ff, f, area * (inv - visc));
        a.nut_ff[f] = nut_adv + nut_diff;
    }
    __shared__ double smin[fvgb::kFaceBlock / 32];
    cand = warp_min(cand);
    if ((threadIdx.x & 31) == 0) smin[threadIdx.x >> 5] = cand;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = smin[0];
        for (int w = 1; w < fvgb::kFaceBlock / 32; ++w) v = fmin(v, smin[w]);
        atomicMin(&a.ns.ctl->dt_bits, (unsigned long long)__double_as_longlong(v));
    }
}

// Cell pass: gathers, SA sources, five norms (deterministic last-block
// fold, as the Euler cell pass), U and nu-tilde updates with the global dt.
__global__ void __launch_bounds__(fvgb::kCellBlock) k_sa_cell(const RansArgs a) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    double s[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    fvgb::StepCtl* ctl = a.ns.ctl;
    if (c < a.ns.g.n_cells) {
        St R = st_make(0.0, 0.0, 0.0, 0.0);
        double Rn = 0.0;
        for (int e = a.cf_off[c]; e < a.cf_off[c + 1]; ++e) {
            const int ent = a.cf[e];
            const int f = ent >> 1;
            R += flip_if(ld_state(a.ns.ff, f), ent);
            if (ent & 1) Rn -= a.nut_ff[f];
            else Rn += a.nut_ff[f];
        }
        const double2 gu = a.grad[4 * c], gv = a.grad[4 * c + 1], gn = a.grad[4 * c + 3];
        const double omega = fabs(gv.x - gu.y);
        const double vol = a.vol[c];
        Rn += vol * sa_source(a.nut[c], a.nu[c].x, omega, a.walld[c], gn.x, gn.y, a.sa, a.cw3_6);
        s[0] = R.r * R.r; s[1] = R.ru * R.ru; s[2] = R.rv * R.rv; s[3] = R.E * R.E; s[4] = Rn * Rn;
        const double dt = __longlong_as_double((long long)ctl->dt_bits);
        const double k = dt / vol;
        const St u = ld_state(a.ns.U, c);
        st_state(a.ns.U, c, u + k * R);
        a.nut[c] = a.nut[c] + k * Rn;
    }
    __shared__ double red[fvgb::kCellBlock / 32][5];
    __shared__ bool last;
    const int w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < 5; ++q) s[q] = warp_sum(s[q]);
    if ((threadIdx.x & 31) == 0)
        for (int q = 0; q < 5; ++q) red[w][q] = s[q];
    __syncthreads();
    if (threadIdx.x < 5) {
        double v = 0.0;
        for (int i = 0; i < fvgb::kCellBlock / 32; ++i) v += red[i][threadIdx.x];
        a.partials[blockIdx.x * 5 + threadIdx.x] = v;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = (atomicAdd(&ctl->done_blocks, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!last) return;
    __threadfence();
    double t[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
        const volatile double* p = a.partials + 5 * b;
        for (int q = 0; q < 5; ++q) t[q] += p[q];
    }
#pragma unroll
    for (int q = 0; q < 5; ++q) t[q] = warp_sum(t[q]);
    __syncthreads();
    if ((threadIdx.x & 31) == 0)
        for (int q = 0; q < 5; ++q) red[w][q] = t[q];
    __syncthreads();
    if (threadIdx.x == 0) {
        double nrm[5];
        int bad = 0;
        for (int q = 0; q < 5; ++q) {
            double v = 0.0;
            for (int i = 0; i < fvgb::kCellBlock / 32; ++i) v += red[i][q];
            nrm[q] = sqrt(v);
            if (!isfinite(nrm[q])) bad = 1;
        }
        for (int q = 0; q < 4; ++q) ctl->norms[q] = nrm[q];
        const int row = ctl->step % a.hist_cap;
        for (int q = 0; q < 4; ++q) a.hist[row * 4 + q] = nrm[q];
        a.nut_hist[row] = nrm[4];
        a.nut_norm[0] = nrm[4];
        if (bad) ctl->nonfinite = 1;
        ctl->step += 1;
        ctl->done_blocks = 0u;
        ctl->dt_bits = (unsigned long long)__double_as_longlong(DBL_MAX);
    }
}

// compute_wall_traction with mu_eff = mu + rho nu_t of the owner cell:
// out = (tau_wall, p of the owner cell).
__global__ void k_sa_wall(const RansArgs a, const int* __restrict__ faces, int n, double2* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int f = faces[i];
    const int cl = a.ns.fl[f];
    const double* fg = a.ns.g.fgrad + 8 * (size_t)f;
    const double4_32a wl = a.ns.prim[cl];
    const double2 gu0 = a.grad[4 * cl], gv0 = a.grad[4 * cl + 1];
    const fvgb::FaceGrad fu = fvgb::face_gradient(fg, true, wl.x, boundary_field(a, f, cl, 0), gu0.x, gu0.y, 0.0, 0.0);
    const fvgb::FaceGrad fv = fvgb::face_gradient(fg, true, wl.y, boundary_field(a, f, cl, 1), gv0.x, gv0.y, 0.0, 0.0);
    const St s = ld_state(a.ns.U, cl);
    const double mu = a.ns.mu + s.r * a.nu[cl].y;
    const double div_v = fu.gx + fv.gy;
    const double tau_xx = mu * (2.0 * fu.gx - (2.0 / 3.0) * div_v);
    const double tau_yy = mu * (2.0 * fv.gy - (2.0 / 3.0) * div_v);
    const double tau_xy = mu * (fu.gy + fv.gx);
    const double nx = fg[6], ny = fg[7];
    const double traction_x = tau_xx * nx + tau_xy * ny;
    const double traction_y = tau_xy * nx + tau_yy * ny;
    const double tx = -ny, ty = nx;
    out[i] = make_double2(-(traction_x * tx + traction_y * ty), pressure(s, a.ns.gamma));
}

}  // namespace FV_KNS

namespace fvgb {

#ifndef FV_NS_FAST  // the wall distance is built once, in the strict unit
void rans_wall_distance(const RansArgs& a, const double4_32a* seg, int n_seg, cudaStream_t s) {
    const int cb = (a.ns.g.n_cells + kCellBlock - 1) / kCellBlock;
    FV_KNS::k_sa_wall_distance<<<cb, kCellBlock, 0, s>>>(a, seg, n_seg);
}
#endif

void FV_NS_FN(rans_launch_step)(const RansArgs& a, cudaStream_t s) {
    const int cb = (a.ns.g.n_cells + kCellBlock - 1) / kCellBlock;
    const int fb = (a.ns.g.n_faces + kFaceBlock - 1) / kFaceBlock;
    FV_KNS::k_sa_prim<<<cb, kCellBlock, 0, s>>>(a);
    FV_KNS::k_sa_grad<<<cb, kCellBlock, 0, s>>>(a);
    switch (a.ns.flux) {
        case 1: FV_KNS::k_sa_face<1><<<fb, kFaceBlock, 0, s>>>(a); break;
        case 2: FV_KNS::k_sa_face<2><<<fb, kFaceBlock, 0, s>>>(a); break;
        default: FV_KNS::k_sa_face<0><<<fb, kFaceBlock, 0, s>>>(a); break;
    }
    FV_KNS::k_sa_cell<<<cb, kCellBlock, 0, s>>>(a);
}

void FV_NS_FN(rans_launch_wall)(const RansArgs& a, const int* faces, int n, double2* out, cudaStream_t s) {
    const int cb = (a.ns.g.n_cells + kCellBlock - 1) / kCellBlock;
    FV_KNS::k_sa_prim<<<cb, kCellBlock, 0, s>>>(a);
    FV_KNS::k_sa_grad<<<cb, kCellBlock, 0, s>>>(a);
    if (n > 0) FV_KNS::k_sa_wall<<<(n + 127) / 128, 128, 0, s>>>(a, faces, n, out);
}

}  // namespace fvgb
