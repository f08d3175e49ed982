// Cell gradients and corrected face gradients on the device:
// GradientCalculator::compute (src/GradientReconstruction.cpp:83-150),
// face_gradient (:153-183), corrected_face_gradient_vector (:193-199) and
// face_normal_distance (:186-190).  Geometry comes precomputed by
// build_grad_geom with the reference's own expressions; the arithmetic here
// keeps the reference's evaluation order, so a translation unit built
// without FMA contraction reproduces the reference's values bit for bit.
#pragma once

#include "types.h"

namespace fvgb {

struct GradDev {
    int n_cells, n_faces, scheme;  // scheme 0 LSQ, 1 Green-Gauss
    const int* cf_off;
    const int* nb;                 // per entry: neighbour or -1-face
    const double2* lsq_w;          // per entry: w*dx, w*dy
    const double* lsq_inv;         // per cell: inv00, inv01, inv11
    const double4_32a* gg;         // per entry: outward nx, ny, length, owner weight
    const double* vol;
    const double* fgrad;           // per face: dist, cos_theta, kx, ky, w_L, nd, nx, ny
    const int* fr;
};

// Gradients of NV cell fields.  phi(c, k): cell value; bphi(face, k): value
// at a boundary face's midpoint.
template <int NV, class Phi, class BPhi>
__device__ __forceinline__ void cell_gradient(const GradDev& g, int c, const Phi& phi, const BPhi& bphi,
                                              double gx[NV], double gy[NV]) {
    const int e0 = g.cf_off[c], e1 = g.cf_off[c + 1];
    if (g.scheme == 0) {
        double bx[NV], by[NV], pc[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) { bx[k] = 0.0; by[k] = 0.0; pc[k] = phi(c, k); }
        for (int e = e0; e < e1; ++e) {
            const int nb = g.nb[e];
            const double2 w = g.lsq_w[e];
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                const double pn = nb >= 0 ? phi(nb, k) : bphi(-1 - nb, k);
                const double dphi = pn - pc[k];
                bx[k] += w.x * dphi;
                by[k] += w.y * dphi;
            }
        }
        const double i0 = g.lsq_inv[3 * c], i1 = g.lsq_inv[3 * c + 1], i2 = g.lsq_inv[3 * c + 2];
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            gx[k] = i0 * bx[k] + i1 * by[k];
            gy[k] = i1 * bx[k] + i2 * by[k];
        }
    } else {
        double sx[NV], sy[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) { sx[k] = 0.0; sy[k] = 0.0; }
        for (int e = e0; e < e1; ++e) {
            const int nb = g.nb[e];
            const double4_32a q = g.gg[e];
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                double pf;
                if (nb < 0) pf = bphi(-1 - nb, k);
                else pf = q.w * phi(c, k) + (1.0 - q.w) * phi(nb, k);
                sx[k] += pf * q.x * q.z;
                sy[k] += pf * q.y * q.z;
            }
        }
        const double v = g.vol[c];
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            gx[k] = sx[k] / v;
            gy[k] = sy[k] / v;
        }
    }
}

struct FaceGrad {
    double dphidn, gx, gy;  // corrected normal derivative, corrected full gradient
};

// face_gradient + corrected_face_gradient_vector for one face.  phiL/phiR:
// owner / neighbour value (phiR = the boundary value on a boundary face);
// gL/gR: cell gradients (gR unused on a boundary face).
__device__ __forceinline__ FaceGrad face_gradient(const double* fg, bool boundary, double phiL, double phiR,
                                                  double gLx, double gLy, double gRx, double gRy) {
    const double direct = (phiR - phiL) / (fg[0] * fg[1]);
    double gfx, gfy;
    if (boundary) {
        gfx = gLx;
        gfy = gLy;
    } else {
        const double wL = fg[4];
        gfx = wL * gLx + (1.0 - wL) * gRx;
        gfy = wL * gLy + (1.0 - wL) * gRy;
    }
    FaceGrad r;
    r.dphidn = direct + gfx * fg[2] + gfy * fg[3];
    const double nx = fg[6], ny = fg[7];
    const double avg = gfx * nx + gfy * ny;
    const double delta = r.dphidn - avg;
    r.gx = gfx + delta * nx;
    r.gy = gfy + delta * ny;
    return r;
}

}  // namespace fvgb
