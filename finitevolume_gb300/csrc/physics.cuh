// Euler physics and numerical fluxes, device side.
//
// Every expression keeps the reference's evaluation order so that a build
// without FMA contraction (nvcc --fmad=false: the "strict" kernels) is
// IEEE op-for-op identical to the reference compiled without -ffast-math
// (sqrt and division are correctly rounded on both sides).  The default
// build contracts mul+add into FMA and differs in the last bits only.
//
// Reference: include/EulerState.h:15-101, include/RusanovFlux.h:33-43,
// include/HllcFlux.h:35-76, include/ExactRiemannFlux.h:23-234,
// src/EulerFVMSolver.cpp:174-193 (ghost states).
#pragma once

#include <cfloat>
#include <cstdint>

#include "types.h"

namespace FV_KNS {

using fvgb::St;
using fvgb::BCTable;
using fvgb::kMaxPatches;

__device__ __forceinline__ St st_make(double a, double b, double c, double d) { St s; s.r = a; s.ru = b; s.rv = c; s.E = d; return s; }
__device__ __forceinline__ St operator+(const St& a, const St& b) { return st_make(a.r + b.r, a.ru + b.ru, a.rv + b.rv, a.E + b.E); }
__device__ __forceinline__ St operator-(const St& a, const St& b) { return st_make(a.r - b.r, a.ru - b.ru, a.rv - b.rv, a.E - b.E); }
__device__ __forceinline__ St operator*(double s, const St& a) { return st_make(s * a.r, s * a.ru, s * a.rv, s * a.E); }
__device__ __forceinline__ St& operator+=(St& a, const St& b) { a.r += b.r; a.ru += b.ru; a.rv += b.rv; a.E += b.E; return a; }

// std::max / std::min semantics ((a < b) ? b : a and (b < a) ? b : a), so
// signed zeros and NaNs propagate exactly as in the reference.
__device__ __forceinline__ double rmax(double a, double b) { return (a < b) ? b : a; }
__device__ __forceinline__ float rmax(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ double rmin(double a, double b) { return (b < a) ? b : a; }

__device__ __forceinline__ St ld_state(const St* __restrict__ U, int i) {
    const double2* p = reinterpret_cast<const double2*>(U + i);
    double2 a = __ldg(p), b = __ldg(p + 1);
    return st_make(a.x, a.y, b.x, b.y);
}
__device__ __forceinline__ void st_state(St* U, int i, const St& s) {
    double2* p = reinterpret_cast<double2*>(U + i);
    p[0] = make_double2(s.r, s.ru);
    p[1] = make_double2(s.rv, s.E);
}

// -F when neg is set, by flipping sign bits on the integer pipe.  IEEE
// defines a - b as a + (-b), so R += signed(F) is bit-identical to the
// reference's "owner subtracts, neighbour adds" (src/EulerFVMSolver.cpp:92-96)
// while issuing one FP64 add per component instead of a predicated
// add/subtract pair.
__device__ __forceinline__ St flip_if(const St& F, int neg) {
    const unsigned long long m = (unsigned long long)(neg & 1) << 63;
    return st_make(__longlong_as_double(__double_as_longlong(F.r) ^ m),
                   __longlong_as_double(__double_as_longlong(F.ru) ^ m),
                   __longlong_as_double(__double_as_longlong(F.rv) ^ m),
                   __longlong_as_double(__double_as_longlong(F.E) ^ m));
}

// EulerState.h:45-52
__device__ __forceinline__ St from_primitive(double rho, double u, double v, double p, double g) {
    St s;
    s.r = rho;
    s.ru = rho * u;
    s.rv = rho * v;
    s.E = p / (g - 1.0) + 0.5 * rho * (u * u + v * v);
    return s;
}
// EulerState.h:58-62
__device__ __forceinline__ double pressure(const St& s, double g) {
    double u = s.ru / s.r;
    double v = s.rv / s.r;
    return (g - 1.0) * (s.E - 0.5 * s.r * (u * u + v * v));
}
// EulerState.h:80-82
__device__ __forceinline__ double sound_speed(const St& s, double g) { return sqrt(g * pressure(s, g) / s.r); }
// EulerState.h:89-101
__device__ __forceinline__ St phys_flux(const St& s, double nx, double ny, double g) {
    double u = s.ru / s.r;
    double v = s.rv / s.r;
    double Vn = u * nx + v * ny;
    double p = pressure(s, g);
    St f;
    f.r = s.r * Vn;
    f.ru = s.ru * Vn + p * nx;
    f.rv = s.rv * Vn + p * ny;
    f.E = (s.E + p) * Vn;
    return f;
}

// RusanovFlux.h:33-43
__device__ __forceinline__ St rusanov(const St& L, const St& R, double nx, double ny, double g) {
    double VnL = (L.ru * nx + L.rv * ny) / L.r;
    double VnR = (R.ru * nx + R.rv * ny) / R.r;
    double Smax = rmax(fabs(VnL) + sound_speed(L, g), fabs(VnR) + sound_speed(R, g));
    St FL = phys_flux(L, nx, ny, g);
    St FR = phys_flux(R, nx, ny, g);
    return 0.5 * (FL + FR) - 0.5 * Smax * (R - L);
}

// HllcFlux.h:35-76 (Davis wave speeds, Toro eq. 10.37-10.39)
__device__ __forceinline__ St hllc(const St& UL, const St& UR, double nx, double ny, double g) {
    double tx = -ny, ty = nx;
    double rL = UL.r, rR = UR.r;
    double uL = UL.ru / rL, vL = UL.rv / rL;
    double uR = UR.ru / rR, vR = UR.rv / rR;
    double VnL = uL * nx + vL * ny, VnR = uR * nx + vR * ny;
    double VtL = uL * tx + vL * ty, VtR = uR * tx + vR * ty;
    double pL = pressure(UL, g), pR = pressure(UR, g);
    double cL = sound_speed(UL, g), cR = sound_speed(UR, g);
    double SL = rmin(VnL - cL, VnR - cR);
    double SR = rmax(VnL + cL, VnR + cR);
    if (SL >= 0.0) return phys_flux(UL, nx, ny, g);
    if (SR <= 0.0) return phys_flux(UR, nx, ny, g);
    double Ss = (pR - pL + rL * VnL * (SL - VnL) - rR * VnR * (SR - VnR)) / (rL * (SL - VnL) - rR * (SR - VnR));
    bool left = (Ss >= 0.0);
    double SK = left ? SL : SR;
    double rK = left ? rL : rR;
    double VnK = left ? VnL : VnR;
    double VtK = left ? VtL : VtR;
    double pK = left ? pL : pR;
    const St& UK = left ? UL : UR;
    double factor = rK * (SK - VnK) / (SK - Ss);
    double mn = factor * Ss;
    double mt = factor * VtK;
    double Es = factor * (UK.E / rK + (Ss - VnK) * (Ss + pK / (rK * (SK - VnK))));
    St Us;
    Us.r = factor;
    Us.ru = mn * nx - mt * ny;
    Us.rv = mn * ny + mt * nx;
    Us.E = Es;
    return phys_flux(UK, nx, ny, g) + SK * (Us - UK);
}

// ---------------------------------------------------------------------------
// Exact Riemann solver (Toro, "Riemann Solvers and Numerical Methods for
// Fluid Dynamics", ch. 4), with the reference's choices: two-shock guess
// seeded by PVRS and floored at 1e-6, Newton with the 1e-10 positivity
// floor and the 2|dp|/(p_new+p) stopping test, vacuum branch, sampling at
// x/t = 0.  ExactRiemannFlux.h:28-234.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double er_f(double p, double rK, double pK, double cK, double g) {
    if (p > pK) {
        double A = 2.0 / ((g + 1.0) * rK);
        double B = (g - 1.0) / (g + 1.0) * pK;
        return (p - pK) * sqrt(A / (p + B));
    }
    return (2.0 * cK / (g - 1.0)) * (pow(p / pK, (g - 1.0) / (2.0 * g)) - 1.0);
}
__device__ __forceinline__ double er_df(double p, double rK, double pK, double cK, double g) {
    if (p > pK) {
        double A = 2.0 / ((g + 1.0) * rK);
        double B = (g - 1.0) / (g + 1.0) * pK;
        return sqrt(A / (p + B)) * (1.0 - 0.5 * (p - pK) / (p + B));
    }
    return (1.0 / (rK * cK)) * pow(p / pK, -(g + 1.0) / (2.0 * g));
}
__device__ __forceinline__ void er_fan_left(double rL, double uL, double pL, double cL, double g, double S,
                                            double& ro, double& uo, double& po) {
    double cf = (2.0 / (g + 1.0)) * (cL + 0.5 * (g - 1.0) * (uL - S));
    uo = (2.0 / (g + 1.0)) * (cL + 0.5 * (g - 1.0) * uL + S);
    ro = rL * pow(cf / cL, 2.0 / (g - 1.0));
    po = pL * pow(cf / cL, 2.0 * g / (g - 1.0));
}
__device__ __forceinline__ void er_fan_right(double rR, double uR, double pR, double cR, double g, double S,
                                             double& ro, double& uo, double& po) {
    double cf = (2.0 / (g + 1.0)) * (cR - 0.5 * (g - 1.0) * (uR - S));
    uo = (2.0 / (g + 1.0)) * (-cR + 0.5 * (g - 1.0) * uR + S);
    ro = rR * pow(cf / cR, 2.0 / (g - 1.0));
    po = pR * pow(cf / cR, 2.0 * g / (g - 1.0));
}

__device__ __forceinline__ St exact_riemann(const St& UL, const St& UR, double nx, double ny, double g, double tol,
                                            int max_iter) {
    double tx = -ny, ty = nx;
    double rL = UL.r, rR = UR.r;
    double uxL = UL.ru / rL, uyL = UL.rv / rL;
    double uxR = UR.ru / rR, uyR = UR.rv / rR;
    double uL = uxL * nx + uyL * ny, vL = uxL * tx + uyL * ty;
    double uR = uxR * nx + uyR * ny, vR = uxR * tx + uyR * ty;
    double pL = pressure(UL, g), pR = pressure(UR, g);
    double cL = sound_speed(UL, g), cR = sound_speed(UR, g);
    double rs, us, ps, vs;
    if (2.0 * (cL + cR) / (g - 1.0) <= uR - uL) {
        double SLv = uL + 2.0 * cL / (g - 1.0);
        double SRv = uR - 2.0 * cR / (g - 1.0);
        if (0.0 <= uL - cL) { rs = rL; us = uL; ps = pL; vs = vL; }
        else if (0.0 <= SLv) { er_fan_left(rL, uL, pL, cL, g, 0.0, rs, us, ps); vs = vL; }
        else if (0.0 < SRv) { return st_make(0.0, 0.0, 0.0, 0.0); }
        else if (0.0 <= uR + cR) { er_fan_right(rR, uR, pR, cR, g, 0.0, rs, us, ps); vs = vR; }
        else { rs = rR; us = uR; ps = pR; vs = vR; }
    } else {
        // Two-shock guess from the PVRS estimate (Toro eq. 4.46-4.47).
        double ppv = rmax(1e-6, 0.5 * (pL + pR) - 0.125 * (uR - uL) * (rL + rR) * (cL + cR));
        double AL = 2.0 / ((g + 1.0) * rL), BL = (g - 1.0) / (g + 1.0) * pL;
        double AR = 2.0 / ((g + 1.0) * rR), BR = (g - 1.0) / (g + 1.0) * pR;
        double gL = sqrt(AL / (ppv + BL));
        double gR = sqrt(AR / (ppv + BR));
        double p = rmax(1e-6, (gL * pL + gR * pR - (uR - uL)) / (gL + gR));
        for (int it = 0; it < max_iter; ++it) {
            double f = er_f(p, rL, pL, cL, g) + er_f(p, rR, pR, cR, g) + (uR - uL);
            double fd = er_df(p, rL, pL, cL, g) + er_df(p, rR, pR, cR, g);
            double pn = p - f / fd;
            if (pn < 1e-10) pn = 1e-10;
            double change = 2.0 * fabs(pn - p) / (pn + p);
            p = pn;
            if (change < tol) break;
        }
        double pst = p;
        double ust = 0.5 * (uL + uR) + 0.5 * (er_f(pst, rR, pR, cR, g) - er_f(pst, rL, pL, cL, g));
        if (0.0 <= ust) {
            if (pst > pL) {
                double SLs = uL - cL * sqrt((g + 1.0) / (2.0 * g) * (pst / pL) + (g - 1.0) / (2.0 * g));
                if (0.0 <= SLs) { rs = rL; us = uL; ps = pL; }
                else {
                    double ratio = pst / pL;
                    rs = rL * (ratio + (g - 1.0) / (g + 1.0)) / ((g - 1.0) / (g + 1.0) * ratio + 1.0);
                    us = ust; ps = pst;
                }
            } else {
                double csL = cL * pow(pst / pL, (g - 1.0) / (2.0 * g));
                double SHL = uL - cL, STL = ust - csL;
                if (0.0 <= SHL) { rs = rL; us = uL; ps = pL; }
                else if (0.0 >= STL) { rs = rL * pow(pst / pL, 1.0 / g); us = ust; ps = pst; }
                else er_fan_left(rL, uL, pL, cL, g, 0.0, rs, us, ps);
            }
            vs = vL;
        } else {
            if (pst > pR) {
                double SRs = uR + cR * sqrt((g + 1.0) / (2.0 * g) * (pst / pR) + (g - 1.0) / (2.0 * g));
                if (0.0 >= SRs) { rs = rR; us = uR; ps = pR; }
                else {
                    double ratio = pst / pR;
                    rs = rR * (ratio + (g - 1.0) / (g + 1.0)) / ((g - 1.0) / (g + 1.0) * ratio + 1.0);
                    us = ust; ps = pst;
                }
            } else {
                double csR = cR * pow(pst / pR, (g - 1.0) / (2.0 * g));
                double SHR = uR + cR, STR = ust + csR;
                if (0.0 >= SHR) { rs = rR; us = uR; ps = pR; }
                else if (0.0 <= STR) { rs = rR * pow(pst / pR, 1.0 / g); us = ust; ps = pst; }
                else er_fan_right(rR, uR, pR, cR, g, 0.0, rs, us, ps);
            }
            vs = vR;
        }
    }
    double uxs = us * nx - vs * ny;
    double uys = us * ny + vs * nx;
    return phys_flux(from_primitive(rs, uxs, uys, ps, g), nx, ny, g);
}

// ---------------------------------------------------------------------------
// Boundary conditions
// ---------------------------------------------------------------------------
enum { BC_WALL = 0, BC_FARFIELD = 1, BC_OUTFLOW = 2, BC_CHAR = 3, BC_NOSLIP = 4 };

// Characteristic (locally one-dimensional Riemann-invariant) farfield.
// New functionality with no reference counterpart: the reference's farfield
// returns the fixed state (src/EulerFVMSolver.cpp:178-180).  With outward
// unit normal n, R+ = Vn_i + 2c_i/(g-1) is carried out of the domain and
// R- = Vn_inf - 2c_inf/(g-1) into it; the boundary normal velocity and
// sound speed follow from both; entropy and tangential velocity come from
// the upwind side.  Supersonic inflow/outflow take the freestream/interior
// state whole.
__device__ __forceinline__ St char_farfield(const St& Ui, const double* sinf, double nx, double ny, double g) {
#ifndef FV_STRICT_ORDER
    // The same boundary state with one power instead of three: with the
    // upwind side's entropy s = p / rho^g and c^2 = g p / rho there,
    // (cb^2 / (g s))^(1/(g-1)) = rho * |cb / c|^(2/(g-1)).  Agrees with the
    // three-power form to a few ulps; the strict build keeps that form.
    {
        const double ri = Ui.r, iri = 1.0 / ri, ui = Ui.ru * iri, vi = Ui.rv * iri;
        const double pi_ = (g - 1.0) * (Ui.E - 0.5 * ri * (ui * ui + vi * vi));
        const double ci = sqrt(g * pi_ * iri);
        const double rf = sinf[0], irf = 1.0 / rf, uf = sinf[1] * irf, vf = sinf[2] * irf;
        const double pf = (g - 1.0) * (sinf[3] - 0.5 * rf * (uf * uf + vf * vf));
        const double cf = sqrt(g * pf * irf);
        const double vni = ui * nx + vi * ny, vnf = uf * nx + vf * ny;
        if (vnf <= -cf) return st_make(sinf[0], sinf[1], sinf[2], sinf[3]);  // supersonic inflow
        if (vni >= ci) return Ui;                                             // supersonic outflow
        const double k = 2.0 / (g - 1.0);
        const double Rp = vni + k * ci, Rm = vnf - k * cf;
        const double vnb = 0.5 * (Rp + Rm);
        const double cb = 0.25 * (g - 1.0) * (Rp - Rm);
        double rb, ut, vt;
        if (vnb > 0.0) { rb = ri * pow(fabs(cb) / ci, k); ut = ui - vni * nx; vt = vi - vni * ny; }
        else { rb = rf * pow(fabs(cb) / cf, k); ut = uf - vnf * nx; vt = vf - vnf * ny; }
        const double pb = rb * cb * cb / g;
        return from_primitive(rb, ut + vnb * nx, vt + vnb * ny, pb, g);
    }
#endif
    double ri = Ui.r, ui = Ui.ru / ri, vi = Ui.rv / ri;
    double pi_ = pressure(Ui, g);
    double ci = sqrt(g * pi_ / ri);
    double rf = sinf[0], uf = sinf[1] / rf, vf = sinf[2] / rf;
    double pf = (g - 1.0) * (sinf[3] - 0.5 * rf * (uf * uf + vf * vf));
    double cf = sqrt(g * pf / rf);
    double vni = ui * nx + vi * ny, vnf = uf * nx + vf * ny;
    if (vnf <= -cf) return st_make(sinf[0], sinf[1], sinf[2], sinf[3]);  // supersonic inflow
    if (vni >= ci) return Ui;                                             // supersonic outflow
    double k = 2.0 / (g - 1.0);
    double Rp = vni + k * ci;
    double Rm = vnf - k * cf;
    double vnb = 0.5 * (Rp + Rm);
    double cb = 0.25 * (g - 1.0) * (Rp - Rm);
    double s, ut, vt;
    if (vnb > 0.0) { s = pi_ / pow(ri, g); ut = ui - vni * nx; vt = vi - vni * ny; }
    else { s = pf / pow(rf, g); ut = uf - vnf * nx; vt = vf - vnf * ny; }
    double rb = pow(cb * cb / (g * s), 1.0 / (g - 1.0));
    double pb = rb * cb * cb / g;
    return from_primitive(rb, ut + vnb * nx, vt + vnb * ny, pb, g);
}

// EulerFVMSolver::ghost_state (src/EulerFVMSolver.cpp:174-193) and the
// no-slip ghost of NavierStokesFVMSolver::ghost_state
// (src/NavierStokesFVMSolver.cpp:265-284).
__device__ __forceinline__ St ghost_state(const BCTable& bc, int patch, const St& UL, double nx, double ny, double g) {
    int t = bc.type[patch];
    if (t == BC_FARFIELD) return st_make(bc.st[patch][0], bc.st[patch][1], bc.st[patch][2], bc.st[patch][3]);
    if (t == BC_OUTFLOW) return UL;
    if (t == BC_CHAR) return char_farfield(UL, bc.st[patch], nx, ny, g);
    double uL = UL.ru / UL.r;
    double vL = UL.rv / UL.r;
    if (t == BC_NOSLIP) {
        double pL = pressure(UL, g);
        return from_primitive(UL.r, 2.0 * bc.wall_u[patch] - uL, 2.0 * bc.wall_v[patch] - vL, pL, g);
    }
    double Vn = uL * nx + vL * ny;
    double ug = uL - 2.0 * Vn * nx;
    double vg = vL - 2.0 * Vn * ny;
    double pL = pressure(UL, g);
    return from_primitive(UL.r, ug, vg, pL, g);
}

enum { FLUX_RUSANOV = 0, FLUX_HLLC = 1, FLUX_EXACT = 2 };

template <int FLUX>
__device__ __forceinline__ St num_flux(const St& L, const St& R, double nx, double ny, double g, double tol, int maxit) {
    if constexpr (FLUX == FLUX_HLLC) return hllc(L, R, nx, ny, g);
    else if constexpr (FLUX == FLUX_EXACT) return exact_riemann(L, R, nx, ny, g, tol, maxit);
    else return rusanov(L, R, nx, ny, g);
}

}  // namespace FV_KNS
