// Navier-Stokes explicit step: NavierStokesFVMSolver::step / compute_dt /
// build_boundary_fields / ghost_state (src/NavierStokesFVMSolver.cpp:55-284)
// and the wall traction of compute_wall_traction (src/WallTraction.cpp:95-142).
//
//   k_ns_prim   u, v, T per cell (:99-104)
//   k_ns_grad   gradients of u, v, T with the boundary fields of
//               build_boundary_fields (no-slip: wall velocity and wall or
//               cell temperature; open boundaries: the cell values)
//   k_ns_face   viscous CFL candidate (face-normal distance, Smax + 2 nu/len,
//               block min + atomicMin), inviscid flux with the no-slip ghost,
//               Jasak-corrected face gradients, Newtonian stress and Fourier
//               heat flux; face_flux = length * (inviscid - viscous)
//   cell pass   the Euler cell pass (gather, norms, U += dt/V R)
// Built twice: without FMA contraction, in the reference's evaluation order
// (this file), and with contraction (ns_fast.cu defines FV_NS_FAST and
// includes it; kernel namespace nsk_fast, launchers suffixed _fast).
#ifdef FV_NS_FAST
#define FV_KNS nsk_fast
#define FV_NS_FN(name) name##_fast
#else
#define FV_KNS nsk
#define FV_NS_FN(name) name
#endif
#include "euler_o1.cuh"
#include "gradients.cuh"
#include "ns.h"

namespace FV_KNS {

using fvgb::NSArgs;

__global__ void __launch_bounds__(fvgb::kCellBlock) k_ns_prim(const NSArgs a) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.g.n_cells) return;
    const St s = ld_state(a.U, c);
    double4_32a w;
    w.x = s.ru / s.r;
    w.y = s.rv / s.r;
    w.z = pressure(s, a.gamma) / (s.r * a.gas_constant);
    w.w = 0.0;
    a.prim[c] = w;
}

// build_boundary_fields (src/NavierStokesFVMSolver.cpp:55-84) for one
// boundary face owned by cell cl, variable k (0 u, 1 v, 2 T).
__device__ __forceinline__ double boundary_field(const NSArgs& a, int face, int cl, int k) {
    const int p = a.fpatch[face];
    if (a.bc.type[p] == BC_NOSLIP) {
        if (k == 0) return a.bc.wall_u[p];
        if (k == 1) return a.bc.wall_v[p];
        return a.bc.isothermal[p] ? a.bc.wall_T[p] : a.prim[cl].z;
    }
    const double4_32a w = a.prim[cl];
    return k == 0 ? w.x : (k == 1 ? w.y : w.z);
}

__global__ void __launch_bounds__(fvgb::kCellBlock) k_ns_grad(const NSArgs a) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.g.n_cells) return;
    double gx[3], gy[3];
    fvgb::cell_gradient<3>(
        a.g, c,
        [&](int i, int k) {
            const double4_32a w = a.prim[i];
            return k == 0 ? w.x : (k == 1 ? w.y : w.z);
        },
        [&](int f, int k) { return boundary_field(a, f, c, k); }, gx, gy);
    a.grad[3 * c] = make_double2(gx[0], gy[0]);
    a.grad[3 * c + 1] = make_double2(gx[1], gy[1]);
    a.grad[3 * c + 2] = make_double2(gx[2], gy[2]);
}

template <int FLUX>
__global__ void __launch_bounds__(fvgb::kFaceBlock) k_ns_face(const NSArgs a) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    double cand = DBL_MAX;
    if (f < a.g.n_faces) {
        const int cl = a.fl[f], cr = a.g.fr[f];
        const bool bnd = cr < 0;
        const double4_32a geo = a.fgeom[f];
        const double nx = geo.x, ny = geo.y, area = geo.z;
        const double* fg = a.g.fgrad + 8 * (size_t)f;
        const St UL = ld_state(a.U, cl);
        const St UR = bnd ? ghost_state(a.bc, a.fpatch[f], UL, nx, ny, a.gamma) : ld_state(a.U, cr);

        // compute_dt (src/NavierStokesFVMSolver.cpp:226-262)
        {
            double uL = UL.ru / UL.r;
            double vL = UL.rv / UL.r;
            double VnL = uL * nx + vL * ny;
            double Smax = fabs(VnL) + sound_speed(UL, a.gamma);
            double rho_min = UL.r;
            if (!bnd) {
                double uR = UR.ru / UR.r;
                double vR = UR.rv / UR.r;
                double VnR = uR * nx + vR * ny;
                Smax = rmax(Smax, fabs(VnR) + sound_speed(UR, a.gamma));
                rho_min = rmin(rho_min, UR.r);
            }
            const double length = fg[5];
            const double nu = (a.mu > 0.0) ? a.mu / rho_min : 0.0;
            const double Smax_total = Smax + 2.0 * nu / length;
            cand = a.ctl->cfl * length / Smax_total;
        }

        const St inv = num_flux<FLUX>(UL, UR, nx, ny, a.gamma, a.exact_tol, a.exact_max_iter);
        St visc = st_make(0.0, 0.0, 0.0, 0.0);
        const int p = bnd ? a.fpatch[f] : 0;
        const bool has_visc = !bnd || a.bc.type[p] == BC_NOSLIP;
        if (has_visc) {
            const double4_32a wl = a.prim[cl];
            double pR[3];
            double2 gR[3];
            if (bnd) {
                for (int k = 0; k < 3; ++k) { pR[k] = boundary_field(a, f, cl, k); gR[k] = make_double2(0.0, 0.0); }
            } else {
                const double4_32a wr = a.prim[cr];
                pR[0] = wr.x; pR[1] = wr.y; pR[2] = wr.z;
                for (int k = 0; k < 3; ++k) gR[k] = a.grad[3 * cr + k];
            }
            const double pL[3] = {wl.x, wl.y, wl.z};
            fvgb::FaceGrad fgv[3];
            for (int k = 0; k < 3; ++k) {
                const double2 gL = a.grad[3 * cl + k];
                fgv[k] = fvgb::face_gradient(fg, bnd, pL[k], pR[k], gL.x, gL.y, gR[k].x, gR[k].y);
            }
            const double u_face = bnd ? pR[0] : 0.5 * (wl.x + pR[0]);
            const double v_face = bnd ? pR[1] : 0.5 * (wl.y + pR[1]);
            const double mu = a.mu;
            const double div_v = fgv[0].gx + fgv[1].gy;
            const double tau_xx = mu * (2.0 * fgv[0].gx - (2.0 / 3.0) * div_v);
            const double tau_yy = mu * (2.0 * fgv[1].gy - (2.0 / 3.0) * div_v);
            const double tau_xy = mu * (fgv[0].gy + fgv[1].gx);
            double qx = -a.kcond * fgv[2].gx;
            double qy = -a.kcond * fgv[2].gy;
            if (bnd && !a.bc.isothermal[p]) {
                qx = 0.0;
                qy = 0.0;
            }
            visc.ru = tau_xx * nx + tau_xy * ny;
            visc.rv = tau_xy * nx + tau_yy * ny;
            visc.E = (u_face * tau_xx + v_face * tau_xy - qx) * nx + (u_face * tau_xy + v_face * tau_yy - qy) * ny;
        }
        st_state(a.ff, f, area * (inv - visc));
    }
    __shared__ double smin[fvgb::kFaceBlock / 32];
    cand = warp_min(cand);
    if ((threadIdx.x & 31) == 0) smin[threadIdx.x >> 5] = cand;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = smin[0];
        for (int w = 1; w < fvgb::kFaceBlock / 32; ++w) v = fmin(v, smin[w]);
        atomicMin(&a.ctl->dt_bits, (unsigned long long)__double_as_longlong(v));
    }
}

// compute_wall_traction for one wall face (src/WallTraction.cpp:110-139):
// out = (tau_wall, p of the owner cell).
__global__ void k_ns_wall(const NSArgs a, const int* __restrict__ faces, int n, double2* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int f = faces[i];
    const int cl = a.fl[f];
    const double* fg = a.g.fgrad + 8 * (size_t)f;
    const double4_32a wl = a.prim[cl];
    const double2 gu0 = a.grad[3 * cl], gv0 = a.grad[3 * cl + 1];
    const fvgb::FaceGrad fu = fvgb::face_gradient(fg, true, wl.x, boundary_field(a, f, cl, 0), gu0.x, gu0.y, 0.0, 0.0);
    const fvgb::FaceGrad fv = fvgb::face_gradient(fg, true, wl.y, boundary_field(a, f, cl, 1), gv0.x, gv0.y, 0.0, 0.0);
    const double mu = a.mu;
    const double div_v = fu.gx + fv.gy;
    const double tau_xx = mu * (2.0 * fu.gx - (2.0 / 3.0) * div_v);
    const double tau_yy = mu * (2.0 * fv.gy - (2.0 / 3.0) * div_v);
    const double tau_xy = mu * (fu.gy + fv.gx);
    const double nx = fg[6], ny = fg[7];
    const double traction_x = tau_xx * nx + tau_xy * ny;
    const double traction_y = tau_xy * nx + tau_yy * ny;
    const double tx = -ny, ty = nx;
    const St s = ld_state(a.U, cl);
    out[i] = make_double2(-(traction_x * tx + traction_y * ty), pressure(s, a.gamma));
}

}  // namespace FV_KNS

namespace fvgb {

void FV_NS_FN(ns_launch_step)(const NSArgs& a, const O1Args& cell, cudaStream_t s) {
    const int cb = (a.g.n_cells + kCellBlock - 1) / kCellBlock;
    const int fb = (a.g.n_faces + kFaceBlock - 1) / kFaceBlock;
    FV_KNS::k_ns_prim<<<cb, kCellBlock, 0, s>>>(a);
    FV_KNS::k_ns_grad<<<cb, kCellBlock, 0, s>>>(a);
    switch (a.flux) {
        case 1: FV_KNS::k_ns_face<1><<<fb, kFaceBlock, 0, s>>>(a); break;
        case 2: FV_KNS::k_ns_face<2><<<fb, kFaceBlock, 0, s>>>(a); break;
        default: FV_KNS::k_ns_face<0><<<fb, kFaceBlock, 0, s>>>(a); break;
    }
    FV_KNS::k_cell_o1<false><<<cb, kCellBlock, 0, s>>>(cell);
}

void FV_NS_FN(ns_launch_wall)(const NSArgs& a, const int* faces, int n, double2* out, cudaStream_t s) {
    const int cb = (a.g.n_cells + kCellBlock - 1) / kCellBlock;
    FV_KNS::k_ns_prim<<<cb, kCellBlock, 0, s>>>(a);
    FV_KNS::k_ns_grad<<<cb, kCellBlock, 0, s>>>(a);
    if (n > 0) FV_KNS::k_ns_wall<<<(n + 127) / 128, 128, 0, s>>>(a, faces, n, out);
}

}  // namespace fvgb
