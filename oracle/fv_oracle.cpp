// ORACLE -- test infrastructure only.
//
// CPU restatement of FiniteVolume's explicit residual-and-update loop, used
// (a) by the tests as the checker of the CUDA library and (b) by bench.py as
// the timed CPU baseline ("port").  Nothing in the product links or calls
// this file.  It keeps the reference's data structures and cost profile on
// purpose -- AoS faces, a std::vector of faces per cell, OpenMP face pass +
// cell pass, a fresh face-flux vector every step -- and its floating-point
// expressions in the reference's evaluation order; built with
// -ffp-contract=off it is bit-identical to the reference compiled without
// -ffast-math (pinned by tests/test_oracle.py against outputs of the
// reference itself, tests/golden/).
//
// Reference files restated here:
//   mesh build       src/MeshReader.cpp:32-76 (shoelace), :317-456 (faces)
//   geometry         include/UnstructuredMesh.h:89-105
//   state / physics  include/EulerState.h:45-101
//   fluxes           include/RusanovFlux.h:33-43, include/HllcFlux.h:35-76,
//                    include/ExactRiemannFlux.h:23-234
//   Euler step       src/EulerFVMSolver.cpp:58-112, compute_dt :133-162,
//                    ghost_state :174-193, IC :24-37
//   diffusion step   src/UnstructuredFVMSolver.cpp:44-129
//   gradients        src/GradientReconstruction.cpp:45-200
//   wall forces      src/WallTraction.cpp:163-217 (pressure part)
//   RANS-SA step     src/RANSTurbulenceSASolver.cpp:118-336, 415-431,
//                    src/SpalartAllmaras.cpp, src/WallDistance.cpp:11-44
// Extensions (no reference code; this file is their CPU FP64 definition):
//   local time stepping, characteristic farfield, MUSCL reconstruction of
//   primitive variables with Barth-Jespersen / Venkatakrishnan limiting,
//   SSP-RK3.  With all extensions off the path is the reference's.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <unordered_map>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

struct Node { double x, y; };
struct Face {
    int node1, node2, cell_left, cell_right, patch_id;
    double nx, ny, area, x_mid, y_mid;
};
struct Cell {
    double volume, x_centroid, y_centroid;
    std::vector<int> faces;
};
struct Mesh {
    std::vector<Node> nodes;
    std::vector<Face> faces;
    std::vector<Cell> cells;
    int n_patches = 0;
};

struct State { double rho = 0, rho_u = 0, rho_v = 0, E = 0; };
inline State operator+(const State& a, const State& b) { return {a.rho + b.rho, a.rho_u + b.rho_u, a.rho_v + b.rho_v, a.E + b.E}; }
inline State operator-(const State& a, const State& b) { return {a.rho - b.rho, a.rho_u - b.rho_u, a.rho_v - b.rho_v, a.E - b.E}; }
inline State operator*(double s, const State& a) { return {s * a.rho, s * a.rho_u, s * a.rho_v, s * a.E}; }
inline State& operator+=(State& a, const State& b) { a.rho += b.rho; a.rho_u += b.rho_u; a.rho_v += b.rho_v; a.E += b.E; return a; }

// ---------------------------------------------------------------- mesh ---
// Faces from each cell's edges in order; first visitor owns (cell_left).
bool build_mesh(Mesh& m, int n_nodes, const double* xy, int n_cells, const int64_t* off, const int* cn, int n_be,
                const int* be, const int* bp, int n_patches) {
    m.nodes.resize(n_nodes);
    for (int i = 0; i < n_nodes; ++i) m.nodes[i] = {xy[2 * i], xy[2 * i + 1]};
    m.cells.assign(n_cells, Cell{});
    m.faces.clear();
    m.n_patches = n_patches;
    std::unordered_map<uint64_t, int> e2f;
    e2f.reserve((size_t)off[n_cells]);
    auto key = [](int a, int b) { return ((uint64_t)(uint32_t)std::min(a, b) << 32) | (uint32_t)std::max(a, b); };
    for (int c = 0; c < n_cells; ++c) {
        int n = (int)(off[c + 1] - off[c]);
        const int* ids = cn + off[c];
        for (int e = 0; e < n; ++e) {
            int a = ids[e], b = ids[(e + 1) % n];
            auto it = e2f.find(key(a, b));
            if (it == e2f.end()) {
                Face f{};
                f.node1 = a; f.node2 = b; f.cell_left = c; f.cell_right = -1; f.patch_id = -1;
                int fi = (int)m.faces.size();
                m.faces.push_back(f);
                m.cells[c].faces.push_back(fi);
                e2f[key(a, b)] = fi;
            } else {
                m.faces[it->second].cell_right = c;
                m.cells[c].faces.push_back(it->second);
            }
        }
        double area = 0.0;
        for (int i = 0; i < n; ++i) {
            const Node& p0 = m.nodes[ids[i]];
            const Node& p1 = m.nodes[ids[(i + 1) % n]];
            area += p0.x * p1.y - p1.x * p0.y;
        }
        area = 0.5 * area;
        double cx = 0.0, cy = 0.0;
        for (int i = 0; i < n; ++i) {
            const Node& p0 = m.nodes[ids[i]];
            const Node& p1 = m.nodes[ids[(i + 1) % n]];
            double cross = p0.x * p1.y - p1.x * p0.y;
            cx += (p0.x + p1.x) * cross;
            cy += (p0.y + p1.y) * cross;
        }
        cx /= (6.0 * area);
        cy /= (6.0 * area);
        m.cells[c].volume = std::fabs(area);
        m.cells[c].x_centroid = cx;
        m.cells[c].y_centroid = cy;
    }
    for (int i = 0; i < n_be; ++i) {
        auto it = e2f.find(key(be[2 * i], be[2 * i + 1]));
        if (it != e2f.end()) m.faces[it->second].patch_id = bp[i];
    }
    for (const Face& f : m.faces)
        if (f.cell_right == -1 && f.patch_id == -1) return false;
    for (Face& f : m.faces) {
        const Node& n1 = m.nodes[f.node1];
        const Node& n2 = m.nodes[f.node2];
        f.x_mid = 0.5 * (n1.x + n2.x);
        f.y_mid = 0.5 * (n1.y + n2.y);
        double dx = n2.x - n1.x, dy = n2.y - n1.y;
        f.area = std::sqrt(dx * dx + dy * dy);
        f.nx = dy / f.area;
        f.ny = -dx / f.area;
    }
    return true;
}

// ------------------------------------------------------------- physics ---
inline State from_primitive(double rho, double u, double v, double p, double g) {
    State s;
    s.rho = rho; s.rho_u = rho * u; s.rho_v = rho * v;
    s.E = p / (g - 1.0) + 0.5 * rho * (u * u + v * v);
    return s;
}
inline double pressure(const State& s, double g) {
    double u = s.rho_u / s.rho, v = s.rho_v / s.rho;
    return (g - 1.0) * (s.E - 0.5 * s.rho * (u * u + v * v));
}
inline double sound_speed(const State& s, double g) { return std::sqrt(g * pressure(s, g) / s.rho); }
inline State phys_flux(const State& s, double nx, double ny, double g) {
    double u = s.rho_u / s.rho, v = s.rho_v / s.rho;
    double Vn = u * nx + v * ny;
    double p = pressure(s, g);
    State f;
    f.rho = s.rho * Vn;
    f.rho_u = s.rho_u * Vn + p * nx;
    f.rho_v = s.rho_v * Vn + p * ny;
    f.E = (s.E + p) * Vn;
    return f;
}
State rusanov(const State& L, const State& R, double nx, double ny, double g) {
    double VnL = (L.rho_u * nx + L.rho_v * ny) / L.rho;
    double VnR = (R.rho_u * nx + R.rho_v * ny) / R.rho;
    double Smax = std::max(std::fabs(VnL) + sound_speed(L, g), std::fabs(VnR) + sound_speed(R, g));
    State FL = phys_flux(L, nx, ny, g), FR = phys_flux(R, nx, ny, g);
    return 0.5 * (FL + FR) - 0.5 * Smax * (R - L);
}
State hllc(const State& UL, const State& UR, double nx, double ny, double g) {
    double tx = -ny, ty = nx;
    double rL = UL.rho, rR = UR.rho;
    double uL = UL.rho_u / rL, vL = UL.rho_v / rL, uR = UR.rho_u / rR, vR = UR.rho_v / rR;
    double VnL = uL * nx + vL * ny, VnR = uR * nx + vR * ny;
    double VtL = uL * tx + vL * ty, VtR = uR * tx + vR * ty;
    double pL = pressure(UL, g), pR = pressure(UR, g);
    double cL = sound_speed(UL, g), cR = sound_speed(UR, g);
    double SL = std::min(VnL - cL, VnR - cR), SR = std::max(VnL + cL, VnR + cR);
    if (SL >= 0.0) return phys_flux(UL, nx, ny, g);
    if (SR <= 0.0) return phys_flux(UR, nx, ny, g);
    double Ss = (pR - pL + rL * VnL * (SL - VnL) - rR * VnR * (SR - VnR)) / (rL * (SL - VnL) - rR * (SR - VnR));
    bool left = Ss >= 0.0;
    double SK = left ? SL : SR, rK = left ? rL : rR, VnK = left ? VnL : VnR, VtK = left ? VtL : VtR;
    double pK = left ? pL : pR;
    const State& UK = left ? UL : UR;
    double fac = rK * (SK - VnK) / (SK - Ss);
    double mn = fac * Ss, mt = fac * VtK;
    double Es = fac * (UK.E / rK + (Ss - VnK) * (Ss + pK / (rK * (SK - VnK))));
    State Us;
    Us.rho = fac; Us.rho_u = mn * nx - mt * ny; Us.rho_v = mn * ny + mt * nx; Us.E = Es;
    return phys_flux(UK, nx, ny, g) + SK * (Us - UK);
}

// Exact Riemann solver (Toro ch. 4) with the reference's guess, Newton and
// sampling choices (include/ExactRiemannFlux.h:28-234).
namespace er {
double f(double p, double rK, double pK, double cK, double g) {
    if (p > pK) {
        double A = 2.0 / ((g + 1.0) * rK), B = (g - 1.0) / (g + 1.0) * pK;
        return (p - pK) * std::sqrt(A / (p + B));
    }
    return (2.0 * cK / (g - 1.0)) * (std::pow(p / pK, (g - 1.0) / (2.0 * g)) - 1.0);
}
double df(double p, double rK, double pK, double cK, double g) {
    if (p > pK) {
        double A = 2.0 / ((g + 1.0) * rK), B = (g - 1.0) / (g + 1.0) * pK;
        return std::sqrt(A / (p + B)) * (1.0 - 0.5 * (p - pK) / (p + B));
    }
    return (1.0 / (rK * cK)) * std::pow(p / pK, -(g + 1.0) / (2.0 * g));
}
void fan_l(double rL, double uL, double pL, double cL, double g, double S, double& ro, double& uo, double& po) {
    double cf = (2.0 / (g + 1.0)) * (cL + 0.5 * (g - 1.0) * (uL - S));
    uo = (2.0 / (g + 1.0)) * (cL + 0.5 * (g - 1.0) * uL + S);
    ro = rL * std::pow(cf / cL, 2.0 / (g - 1.0));
    po = pL * std::pow(cf / cL, 2.0 * g / (g - 1.0));
}
void fan_r(double rR, double uR, double pR, double cR, double g, double S, double& ro, double& uo, double& po) {
    double cf = (2.0 / (g + 1.0)) * (cR - 0.5 * (g - 1.0) * (uR - S));
    uo = (2.0 / (g + 1.0)) * (-cR + 0.5 * (g - 1.0) * uR + S);
    ro = rR * std::pow(cf / cR, 2.0 / (g - 1.0));
    po = pR * std::pow(cf / cR, 2.0 * g / (g - 1.0));
}
}  // namespace er

State exact(const State& UL, const State& UR, double nx, double ny, double g, double tol, int maxit) {
    double tx = -ny, ty = nx;
    double rL = UL.rho, rR = UR.rho;
    double uxL = UL.rho_u / rL, uyL = UL.rho_v / rL, uxR = UR.rho_u / rR, uyR = UR.rho_v / rR;
    double uL = uxL * nx + uyL * ny, vL = uxL * tx + uyL * ty;
    double uR = uxR * nx + uyR * ny, vR = uxR * tx + uyR * ty;
    double pL = pressure(UL, g), pR = pressure(UR, g);
    double cL = sound_speed(UL, g), cR = sound_speed(UR, g);
    double rs, us, ps, vs;
    if (2.0 * (cL + cR) / (g - 1.0) <= uR - uL) {
        double SLv = uL + 2.0 * cL / (g - 1.0), SRv = uR - 2.0 * cR / (g - 1.0);
        if (0.0 <= uL - cL) { rs = rL; us = uL; ps = pL; vs = vL; }
        else if (0.0 <= SLv) { er::fan_l(rL, uL, pL, cL, g, 0.0, rs, us, ps); vs = vL; }
        else if (0.0 < SRv) return State{0.0, 0.0, 0.0, 0.0};
        else if (0.0 <= uR + cR) { er::fan_r(rR, uR, pR, cR, g, 0.0, rs, us, ps); vs = vR; }
        else { rs = rR; us = uR; ps = pR; vs = vR; }
    } else {
        double ppv = std::max(1e-6, 0.5 * (pL + pR) - 0.125 * (uR - uL) * (rL + rR) * (cL + cR));
        double AL = 2.0 / ((g + 1.0) * rL), BL = (g - 1.0) / (g + 1.0) * pL;
        double AR = 2.0 / ((g + 1.0) * rR), BR = (g - 1.0) / (g + 1.0) * pR;
        double gL = std::sqrt(AL / (ppv + BL)), gR = std::sqrt(AR / (ppv + BR));
        double p = std::max(1e-6, (gL * pL + gR * pR - (uR - uL)) / (gL + gR));
        for (int it = 0; it < maxit; ++it) {
            double fv = er::f(p, rL, pL, cL, g) + er::f(p, rR, pR, cR, g) + (uR - uL);
            double fd = er::df(p, rL, pL, cL, g) + er::df(p, rR, pR, cR, g);
            double pn = p - fv / fd;
            if (pn < 1e-10) pn = 1e-10;
            double ch = 2.0 * std::fabs(pn - p) / (pn + p);
            p = pn;
            if (ch < tol) break;
        }
        double ust = 0.5 * (uL + uR) + 0.5 * (er::f(p, rR, pR, cR, g) - er::f(p, rL, pL, cL, g));
        if (0.0 <= ust) {
            if (p > pL) {
                double SLs = uL - cL * std::sqrt((g + 1.0) / (2.0 * g) * (p / pL) + (g - 1.0) / (2.0 * g));
                if (0.0 <= SLs) { rs = rL; us = uL; ps = pL; }
                else {
                    double ratio = p / pL;
                    rs = rL * (ratio + (g - 1.0) / (g + 1.0)) / ((g - 1.0) / (g + 1.0) * ratio + 1.0);
                    us = ust; ps = p;
                }
            } else {
                double csL = cL * std::pow(p / pL, (g - 1.0) / (2.0 * g));
                if (0.0 <= uL - cL) { rs = rL; us = uL; ps = pL; }
                else if (0.0 >= ust - csL) { rs = rL * std::pow(p / pL, 1.0 / g); us = ust; ps = p; }
                else er::fan_l(rL, uL, pL, cL, g, 0.0, rs, us, ps);
            }
            vs = vL;
        } else {
            if (p > pR) {
                double SRs = uR + cR * std::sqrt((g + 1.0) / (2.0 * g) * (p / pR) + (g - 1.0) / (2.0 * g));
                if (0.0 >= SRs) { rs = rR; us = uR; ps = pR; }
                else {
                    double ratio = p / pR;
                    rs = rR * (ratio + (g - 1.0) / (g + 1.0)) / ((g - 1.0) / (g + 1.0) * ratio + 1.0);
                    us = ust; ps = p;
                }
            } else {
                double csR = cR * std::pow(p / pR, (g - 1.0) / (2.0 * g));
                if (0.0 >= uR + cR) { rs = rR; us = uR; ps = pR; }
                else if (0.0 <= ust + csR) { rs = rR * std::pow(p / pR, 1.0 / g); us = ust; ps = p; }
                else er::fan_r(rR, uR, pR, cR, g, 0.0, rs, us, ps);
            }
            vs = vR;
        }
    }
    double uxs = us * nx - vs * ny, uys = us * ny + vs * nx;
    return phys_flux(from_primitive(rs, uxs, uys, ps, g), nx, ny, g);
}

enum { BC_WALL = 0, BC_FARFIELD = 1, BC_OUTFLOW = 2, BC_CHAR = 3, BC_NOSLIP = 4 };
struct BC {
    int type = BC_WALL;
    State state;
    double wall_u = 0, wall_v = 0;
};

// Characteristic farfield: locally 1D Riemann invariants along the outward
// normal; entropy and tangential velocity from the upwind side.
State char_farfield(const State& Ui, const State& Sf, double nx, double ny, double g) {
    double ri = Ui.rho, ui = Ui.rho_u / ri, vi = Ui.rho_v / ri;
    double pi_ = pressure(Ui, g);
    double ci = std::sqrt(g * pi_ / ri);
    double rf = Sf.rho, uf = Sf.rho_u / rf, vf = Sf.rho_v / rf;
    double pf = (g - 1.0) * (Sf.E - 0.5 * rf * (uf * uf + vf * vf));
    double cf = std::sqrt(g * pf / rf);
    double vni = ui * nx + vi * ny, vnf = uf * nx + vf * ny;
    if (vnf <= -cf) return Sf;
    if (vni >= ci) return Ui;
    double k = 2.0 / (g - 1.0);
    double Rp = vni + k * ci, Rm = vnf - k * cf;
    double vnb = 0.5 * (Rp + Rm);
    double cb = 0.25 * (g - 1.0) * (Rp - Rm);
    double s, ut, vt;
    if (vnb > 0.0) { s = pi_ / std::pow(ri, g); ut = ui - vni * nx; vt = vi - vni * ny; }
    else { s = pf / std::pow(rf, g); ut = uf - vnf * nx; vt = vf - vnf * ny; }
    double rb = std::pow(cb * cb / (g * s), 1.0 / (g - 1.0));
    double pb = rb * cb * cb / g;
    return from_primitive(rb, ut + vnb * nx, vt + vnb * ny, pb, g);
}

State ghost(const BC& bc, const Face& f, const State& UL, double g) {
    if (bc.type == BC_FARFIELD) return bc.state;
    if (bc.type == BC_OUTFLOW) return UL;
    if (bc.type == BC_CHAR) return char_farfield(UL, bc.state, f.nx, f.ny, g);
    double uL = UL.rho_u / UL.rho, vL = UL.rho_v / UL.rho;
    if (bc.type == BC_NOSLIP) return from_primitive(UL.rho, 2.0 * bc.wall_u - uL, 2.0 * bc.wall_v - vL, pressure(UL, g), g);
    double Vn = uL * f.nx + vL * f.ny;
    double ug = uL - 2.0 * Vn * f.nx, vg = vL - 2.0 * Vn * f.ny;
    double pL = pressure(UL, g);
    return from_primitive(UL.rho, ug, vg, pL, g);
}

// ------------------------------------------------- 2nd-order extension ---
struct Prim { double r, u, v, p; };
inline Prim to_prim(const State& s, double g) {
    double u = s.rho_u / s.rho, v = s.rho_v / s.rho;
    return {s.rho, u, v, (g - 1.0) * (s.E - 0.5 * s.rho * (u * u + v * v))};
}
inline State to_cons(const Prim& w, double g) { return from_primitive(w.r, w.u, w.v, w.p, g); }

struct Grad4 { double gx[4], gy[4]; };

// ------------------------------------------------------------- solver ---
struct Euler {
    Mesh mesh;
    std::vector<State> U, U0;
    std::vector<BC> bcs;
    double gamma = 1.4, cfl = 0.5, tol = 1e-6;
    int maxit = 20, flux = 0, order = 1, rk = 1, local_dt = 0, gradient = 0, limiter = 2;
    double venkat_k = 5.0;
    double last[4] = {0, 0, 0, 0};
    // 2nd-order geometry: LSQ inverse matrices over face neighbours
    std::vector<double> lsq;      // 3 per cell
    std::vector<double> dtc;      // local dt per cell

    State numflux(const State& L, const State& R, double nx, double ny) const {
        if (flux == 1) return hllc(L, R, nx, ny, gamma);
        if (flux == 2) return exact(L, R, nx, ny, gamma, tol, maxit);
        return rusanov(L, R, nx, ny, gamma);
    }

    // EulerFVMSolver::compute_dt per-face candidate.
    double face_dt(const Face& f, const std::vector<State>& V) const {
        const State& UL = V[f.cell_left];
        double uL = UL.rho_u / UL.rho, vL = UL.rho_v / UL.rho;
        double VnL = uL * f.nx + vL * f.ny;
        double Smax = std::fabs(VnL) + sound_speed(UL, gamma);
        double length;
        if (f.cell_right != -1) {
            const State& UR = V[f.cell_right];
            double uR = UR.rho_u / UR.rho, vR = UR.rho_v / UR.rho;
            double VnR = uR * f.nx + vR * f.ny;
            Smax = std::max(Smax, std::fabs(VnR) + sound_speed(UR, gamma));
            length = std::min(mesh.cells[f.cell_left].volume, mesh.cells[f.cell_right].volume) / f.area;
        } else {
            length = mesh.cells[f.cell_left].volume / f.area;
        }
        return cfl * length / Smax;
    }

    double compute_dt() const {
        double dt = std::numeric_limits<double>::max();
#pragma omp parallel for reduction(min : dt)
        for (long i = 0; i < (long)mesh.faces.size(); ++i) dt = std::min(dt, face_dt(mesh.faces[i], U));
        return dt;
    }

    // Face spectral radius times length: max(|Vn|+c) over the face's cells
    // (the wave-speed estimate of compute_dt) times the face length.
    double face_lambda_area(const Face& f, const std::vector<State>& V) const {
        const State& UL = V[f.cell_left];
        double uL = UL.rho_u / UL.rho, vL = UL.rho_v / UL.rho;
        double Smax = std::fabs(uL * f.nx + vL * f.ny) + sound_speed(UL, gamma);
        if (f.cell_right != -1) {
            const State& UR = V[f.cell_right];
            double uR = UR.rho_u / UR.rho, vR = UR.rho_v / UR.rho;
            Smax = std::max(Smax, std::fabs(uR * f.nx + vR * f.ny) + sound_speed(UR, gamma));
        }
        return Smax * f.area;
    }

    // Local time stepping (new): dt_i = CFL * V_i / sum_f lambda_f A_f, the
    // usual local-CFL definition for steady explicit solvers.
    void compute_local_dt() {
        std::vector<double> la(mesh.faces.size());
#pragma omp parallel for
        for (long i = 0; i < (long)mesh.faces.size(); ++i) la[i] = face_lambda_area(mesh.faces[i], U);
        dtc.resize(mesh.cells.size());
#pragma omp parallel for
        for (long c = 0; c < (long)mesh.cells.size(); ++c) {
            double s = 0.0;
            for (int f : mesh.cells[c].faces) s += la[f];
            dtc[c] = cfl * mesh.cells[c].volume / s;
        }
    }

    // -- 2nd order: LSQ matrices (GradientCalculator ctor,
    //    src/GradientReconstruction.cpp:45-80) over face neighbours, with
    //    boundary-face midpoints standing in for the missing neighbour.
    void setup_lsq() {
        lsq.resize(3 * mesh.cells.size());
        for (size_t c = 0; c < mesh.cells.size(); ++c) {
            const Cell& cell = mesh.cells[c];
            double m00 = 0, m01 = 0, m11 = 0;
            for (int fi : cell.faces) {
                const Face& f = mesh.faces[fi];
                double px, py;
                if (f.cell_right == -1) { px = f.x_mid; py = f.y_mid; }
                else {
                    int nb = f.cell_left == (int)c ? f.cell_right : f.cell_left;
                    px = mesh.cells[nb].x_centroid; py = mesh.cells[nb].y_centroid;
                }
                double dx = px - cell.x_centroid, dy = py - cell.y_centroid;
                double w = 1.0 / (dx * dx + dy * dy);
                m00 += w * dx * dx; m01 += w * dx * dy; m11 += w * dy * dy;
            }
            double det = m00 * m11 - m01 * m01;
            lsq[3 * c] = m11 / det; lsq[3 * c + 1] = -m01 / det; lsq[3 * c + 2] = m00 / det;
        }
    }

    // Boundary value of the primitive variables at a boundary face: the
    // average of the interior state and its ghost state.
    Prim boundary_prim(const Face& f, const State& Ui) const {
        State Ug = ghost(bcs[f.patch_id], f, Ui, gamma);
        Prim a = to_prim(Ui, gamma), b = to_prim(Ug, gamma);
        return {0.5 * (a.r + b.r), 0.5 * (a.u + b.u), 0.5 * (a.v + b.v), 0.5 * (a.p + b.p)};
    }

    // Limited gradients of (rho, u, v, p) per cell.
    void gradients(const std::vector<State>& V, std::vector<Prim>& W, std::vector<Grad4>& G) const {
        size_t N = mesh.cells.size();
        W.resize(N);
        G.resize(N);
#pragma omp parallel for
        for (long c = 0; c < (long)N; ++c) W[c] = to_prim(V[c], gamma);
#pragma omp parallel for
        for (long c = 0; c < (long)N; ++c) {
            const Cell& cell = mesh.cells[c];
            const double* wi = &W[c].r;
            double bx[4] = {0, 0, 0, 0}, by[4] = {0, 0, 0, 0};
            double dmax[4] = {0, 0, 0, 0}, dmin[4] = {0, 0, 0, 0};
            for (int fi : cell.faces) {
                const Face& f = mesh.faces[fi];
                Prim wn;
                double px, py;
                if (f.cell_right == -1) { wn = boundary_prim(f, V[c]); px = f.x_mid; py = f.y_mid; }
                else {
                    int nb = f.cell_left == (int)c ? f.cell_right : f.cell_left;
                    wn = W[nb]; px = mesh.cells[nb].x_centroid; py = mesh.cells[nb].y_centroid;
                }
                const double* wj = &wn.r;
                double dx = px - cell.x_centroid, dy = py - cell.y_centroid;
                for (int k = 0; k < 4; ++k) {
                    double d = wj[k] - wi[k];
                    dmax[k] = std::max(dmax[k], d);
                    dmin[k] = std::min(dmin[k], d);
                    if (gradient == 0) {
                        double w = 1.0 / (dx * dx + dy * dy);
                        bx[k] += w * dx * d;
                        by[k] += w * dy * d;
                    } else {
                        // Green-Gauss, inverse-distance face value
                        // (src/GradientReconstruction.cpp:89-118).
                        double phi_f;
                        if (f.cell_right == -1) phi_f = wj[k];
                        else {
                            double d_c = std::hypot(cell.x_centroid - f.x_mid, cell.y_centroid - f.y_mid);
                            double d_o = std::hypot(px - f.x_mid, py - f.y_mid);
                            double w_c = d_o / (d_c + d_o);
                            phi_f = w_c * wi[k] + (1.0 - w_c) * wj[k];
                        }
                        double sgn = f.cell_left == (int)c ? 1.0 : -1.0;
                        bx[k] += phi_f * (sgn * f.nx) * f.area;
                        by[k] += phi_f * (sgn * f.ny) * f.area;
                    }
                }
            }
            Grad4& g = G[c];
            for (int k = 0; k < 4; ++k) {
                if (gradient == 0) {
                    g.gx[k] = lsq[3 * c] * bx[k] + lsq[3 * c + 1] * by[k];
                    g.gy[k] = lsq[3 * c + 1] * bx[k] + lsq[3 * c + 2] * by[k];
                } else {
                    g.gx[k] = bx[k] / cell.volume;
                    g.gy[k] = by[k] / cell.volume;
                }
            }
            if (limiter == 0) continue;
            double eps2 = 0.0;
            if (limiter == 2) {
                double h = std::sqrt(cell.volume);
                double kh = venkat_k * h;
                eps2 = kh * kh * kh;
            }
            for (int k = 0; k < 4; ++k) {
                double psi = 1.0;
                for (int fi : cell.faces) {
                    const Face& f = mesh.faces[fi];
                    double d2 = g.gx[k] * (f.x_mid - cell.x_centroid) + g.gy[k] * (f.y_mid - cell.y_centroid);
                    double p = 1.0;
                    if (d2 > 0.0 || d2 < 0.0) {
                        double d1 = d2 > 0.0 ? dmax[k] : dmin[k];
                        if (limiter == 1) p = std::min(1.0, d1 / d2);
                        else {
                            double num = d1 * d1 + eps2 + 2.0 * d2 * d1;
                            double den = d1 * d1 + 2.0 * d2 * d2 + d1 * d2 + eps2;
                            p = num / den;
                        }
                    }
                    psi = std::min(psi, p);
                }
                g.gx[k] *= psi;
                g.gy[k] *= psi;
            }
        }
    }

    // Residual R(V) (net flux in) into R; returns nothing else.
    void residual(const std::vector<State>& V, std::vector<State>& R) const {
        size_t F = mesh.faces.size(), N = mesh.cells.size();
        std::vector<State> ff(F);
        std::vector<Prim> W;
        std::vector<Grad4> G;
        if (order == 2) gradients(V, W, G);
#pragma omp parallel for
        for (long i = 0; i < (long)F; ++i) {
            const Face& f = mesh.faces[i];
            int L = f.cell_left, Rr = f.cell_right;
            State UL, UR;
            if (order == 1) {
                UL = V[L];
                UR = (Rr != -1) ? V[Rr] : ghost(bcs[f.patch_id], f, UL, gamma);
            } else {
                Prim wl = recon(W[L], G[L], mesh.cells[L], f);
                UL = to_cons(wl, gamma);
                if (Rr != -1) UR = to_cons(recon(W[Rr], G[Rr], mesh.cells[Rr], f), gamma);
                else UR = ghost(bcs[f.patch_id], f, UL, gamma);
            }
            ff[i] = f.area * numflux(UL, UR, f.nx, f.ny);
        }
        R.resize(N);
#pragma omp parallel for
        for (long c = 0; c < (long)N; ++c) {
            State r;
            for (int fi : mesh.cells[c].faces) {
                if (mesh.faces[fi].cell_left == (int)c) r = r - ff[fi];
                else r += ff[fi];
            }
            R[c] = r;
        }
    }

    // Reconstructed primitive state at a face midpoint; falls back to the
    // cell value when the linear extrapolation loses positivity.
    Prim recon(const Prim& w, const Grad4& g, const Cell& c, const Face& f) const {
        double dx = f.x_mid - c.x_centroid, dy = f.y_mid - c.y_centroid;
        Prim o;
        o.r = w.r + (g.gx[0] * dx + g.gy[0] * dy);
        o.u = w.u + (g.gx[1] * dx + g.gy[1] * dy);
        o.v = w.v + (g.gx[2] * dx + g.gy[2] * dy);
        o.p = w.p + (g.gx[3] * dx + g.gy[3] * dy);
        if (!(o.r > 0.0) || !(o.p > 0.0)) return w;
        return o;
    }

    void norms_of(const std::vector<State>& R) {
        double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
#pragma omp parallel for reduction(+ : s0, s1, s2, s3)
        for (long c = 0; c < (long)R.size(); ++c) {
            s0 += R[c].rho * R[c].rho; s1 += R[c].rho_u * R[c].rho_u;
            s2 += R[c].rho_v * R[c].rho_v; s3 += R[c].E * R[c].E;
        }
        last[0] = std::sqrt(s0); last[1] = std::sqrt(s1); last[2] = std::sqrt(s2); last[3] = std::sqrt(s3);
    }

    // Reference-mode step: exactly EulerFVMSolver::step (two OpenMP passes,
    // fused residual/norm/update cell pass, fresh face-flux vector).
    void step_reference() {
        double dt = compute_dt();
        std::vector<State> face_flux(mesh.faces.size());
#pragma omp parallel for
        for (long i = 0; i < (long)mesh.faces.size(); ++i) {
            const Face& f = mesh.faces[i];
            const State& UL = U[f.cell_left];
            State UR = (f.cell_right != -1) ? U[f.cell_right] : ghost(bcs[f.patch_id], f, UL, gamma);
            face_flux[i] = f.area * numflux(UL, UR, f.nx, f.ny);
        }
        double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
#pragma omp parallel for reduction(+ : s0, s1, s2, s3)
        for (long c = 0; c < (long)mesh.cells.size(); ++c) {
            State r;
            for (int fi : mesh.cells[c].faces) {
                if (mesh.faces[fi].cell_left == (int)c) r = r - face_flux[fi];
                else r += face_flux[fi];
            }
            s0 += r.rho * r.rho; s1 += r.rho_u * r.rho_u; s2 += r.rho_v * r.rho_v; s3 += r.E * r.E;
            U[c] += (dt / mesh.cells[c].volume) * r;
        }
        last[0] = std::sqrt(s0); last[1] = std::sqrt(s1); last[2] = std::sqrt(s2); last[3] = std::sqrt(s3);
    }

    void step() {
        if (order == 1 && rk == 1 && !local_dt) { step_reference(); return; }
        size_t N = mesh.cells.size();
        double dtg = 0.0;
        if (local_dt) compute_local_dt();
        else dtg = compute_dt();
        auto dt_of = [&](long c) { return local_dt ? dtc[c] : dtg; };
        std::vector<State> R;
        if (rk == 1) {
            residual(U, R);
            norms_of(R);
#pragma omp parallel for
            for (long c = 0; c < (long)N; ++c) U[c] += (dt_of(c) / mesh.cells[c].volume) * R[c];
            return;
        }
        // SSP-RK3 (Shu-Osher): U1 = U0 + dt L(U0); U2 = 3/4 U0 + 1/4 (U1 + dt L(U1));
        // U3 = 1/3 U0 + 2/3 (U2 + dt L(U2)); the reported norms are stage 1's.
        U0 = U;
        std::vector<State> Us = U;
        for (int s = 0; s < 3; ++s) {
            residual(Us, R);
            if (s == 0) norms_of(R);
#pragma omp parallel for
            for (long c = 0; c < (long)N; ++c) {
                State e = Us[c] + (dt_of(c) / mesh.cells[c].volume) * R[c];
                if (s == 0) Us[c] = e;
                else if (s == 1) Us[c] = 0.75 * U0[c] + 0.25 * e;
                else Us[c] = (1.0 / 3.0) * U0[c] + (2.0 / 3.0) * e;
            }
        }
        U = Us;
    }
};

// ---------------------------------------------------------- diffusion ---
struct Diffusion {
    Mesh mesh;
    std::vector<double> phi;
    std::vector<int> ptype;   // 0 Dirichlet, 1 Neumann
    std::vector<double> pval;
    double alpha = 1.0, dt = 1e-4, last = 0.0;

    void step() {
        std::vector<double> ff(mesh.faces.size());
#pragma omp parallel for
        for (long i = 0; i < (long)mesh.faces.size(); ++i) {
            const Face& f = mesh.faces[i];
            double pL = phi[f.cell_left];
            if (f.cell_right != -1) {
                double pR = phi[f.cell_right];
                double dx = mesh.cells[f.cell_right].x_centroid - mesh.cells[f.cell_left].x_centroid;
                double dy = mesh.cells[f.cell_right].y_centroid - mesh.cells[f.cell_left].y_centroid;
                double d = std::sqrt(dx * dx + dy * dy);
                double gn = (pR - pL) / d;
                ff[i] = -alpha * gn * f.area;
            } else if (ptype[f.patch_id] == 1) {
                ff[i] = pval[f.patch_id] * f.area;
            } else {
                double dx = f.x_mid - mesh.cells[f.cell_left].x_centroid;
                double dy = f.y_mid - mesh.cells[f.cell_left].y_centroid;
                double d = std::sqrt(dx * dx + dy * dy);
                double gn = (pval[f.patch_id] - pL) / d;
                ff[i] = -alpha * gn * f.area;
            }
        }
        double s = 0.0;
#pragma omp parallel for reduction(+ : s)
        for (long c = 0; c < (long)mesh.cells.size(); ++c) {
            double r = 0.0;
            for (int fi : mesh.cells[c].faces) {
                if (mesh.faces[fi].cell_left == (int)c) r -= ff[fi];
                else r += ff[fi];
            }
            s += r * r;
            phi[c] += (dt / mesh.cells[c].volume) * r;
        }
        last = std::sqrt(s);
    }
};

// ------------------------------------------------------ RANS-SA step ---
// RANSTurbulenceSASolver (src/RANSTurbulenceSASolver.cpp:118-282, compute_dt
// :296-336, ghost_state :415-431, boundary fields :70-110), its gradients
// (src/GradientReconstruction.cpp:45-200: GradientCalculator, face_gradient,
// corrected_face_gradient_vector, face_normal_distance), the SA-noft2
// source terms (src/SpalartAllmaras.cpp, constants include/SpalartAllmaras.h:
// 13-23) and the wall distance (src/WallDistance.cpp:11-44), in the
// reference's evaluation order.  Patch kinds: BC_NOSLIP, BC_FARFIELD,
// BC_OUTFLOW (NSBoundaryType); NoSlipWall patches carry wall_u, wall_v and,
// when isothermal, wall_T.
struct G2 { double x = 0.0, y = 0.0; };
struct FaceGrad { double dn; G2 gf; };

struct SAConst {
    double cb1 = 0.1355, cb2 = 0.622, sigma = 2.0 / 3.0, kappa = 0.41, cw2 = 0.3, cw3 = 2.0, cv1 = 7.1,
           cv2 = 0.7, cv3 = 0.9;
};
inline double sa_cw1(const SAConst& c) { return c.cb1 / (c.kappa * c.kappa) + (1.0 + c.cb2) / c.sigma; }
inline double sa_fv1(double nut, double nu, const SAConst& c) {
    if (nut <= 0.0) return 0.0;
    double chi = nut / nu;
    double chi3 = chi * chi * chi;
    return chi3 / (chi3 + c.cv1 * c.cv1 * c.cv1);
}
inline double sa_nut(double nut, double nu, const SAConst& c) { return nut * sa_fv1(nut, nu, c); }
// production - destruction + cross-diffusion (SpalartAllmaras.cpp).
inline double sa_source(double nut, double nu, double omega, double d, const G2& gn, const SAConst& c) {
    double chi = (nut > 0.0) ? nut / nu : 0.0;
    double fv1 = sa_fv1(nut, nu, c);
    double fv2 = 1.0 - chi / (1.0 + chi * fv1);
    double d2 = d * d;
    double s_bar = (nut / (c.kappa * c.kappa * d2)) * fv2;
    double s_tilde;
    if (s_bar >= -c.cv2 * omega) s_tilde = omega + s_bar;
    else s_tilde = omega + omega * (c.cv2 * c.cv2 * omega + c.cv3 * s_bar) / ((c.cv3 - 2.0 * c.cv2) * omega - s_bar);
    double production = c.cb1 * s_tilde * nut;
    double destruction = 0.0;
    if (nut > 0.0) {
        double s_safe = std::max(s_tilde, 1e-10);
        double r = std::min(nut / (s_safe * c.kappa * c.kappa * d2), 10.0);
        double g = r + c.cw2 * (std::pow(r, 6.0) - r);
        double fw = g * std::pow((1.0 + std::pow(c.cw3, 6.0)) / (std::pow(g, 6.0) + std::pow(c.cw3, 6.0)), 1.0 / 6.0);
        double nd = nut / d;
        destruction = sa_cw1(c) * fw * nd * nd;
    }
    double cross = (c.cb2 / c.sigma) * (gn.x * gn.x + gn.y * gn.y);
    return production - destruction + cross;
}

struct RansBC {
    int type = BC_NOSLIP;
    State state;
    double wall_u = 0.0, wall_v = 0.0, wall_T = 0.0, nut = 0.0;
    int isothermal = 0;
};

struct Rans {
    Mesh mesh;
    std::vector<State> U;
    std::vector<double> nut, walld, lsq;
    std::vector<RansBC> bcs;
    double gamma = 1.4, R = 287.0, mu = 0.0, Pr = 0.72, Prt = 0.9, cfl = 0.5, tol = 1e-6;
    int flux = 0, gradient = 0, maxit = 20;
    SAConst sa;
    double last[5] = {0, 0, 0, 0, 0};

    // GradientCalculator ctor (least squares over face neighbours, boundary
    // midpoints standing in for the missing neighbour).
    void setup() {
        lsq.assign(3 * mesh.cells.size(), 0.0);
        if (gradient == 0)
            for (size_t c = 0; c < mesh.cells.size(); ++c) {
                const Cell& cell = mesh.cells[c];
                double m00 = 0.0, m01 = 0.0, m11 = 0.0;
                for (int fi : cell.faces) {
                    const Face& f = mesh.faces[fi];
                    double px, py;
                    if (f.cell_right == -1) { px = f.x_mid; py = f.y_mid; }
                    else {
                        int nb = (f.cell_left == (int)c) ? f.cell_right : f.cell_left;
                        px = mesh.cells[nb].x_centroid; py = mesh.cells[nb].y_centroid;
                    }
                    double dx = px - cell.x_centroid, dy = py - cell.y_centroid;
                    double w = 1.0 / (dx * dx + dy * dy);
                    m00 += w * dx * dx; m01 += w * dx * dy; m11 += w * dy * dy;
                }
                double det = m00 * m11 - m01 * m01;
                lsq[3 * c] = m11 / det; lsq[3 * c + 1] = -m01 / det; lsq[3 * c + 2] = m00 / det;
            }
        // compute_wall_distance over the no-slip boundary faces
        std::vector<int> wf;
        for (size_t i = 0; i < mesh.faces.size(); ++i)
            if (mesh.faces[i].cell_right == -1 && bcs[mesh.faces[i].patch_id].type == BC_NOSLIP) wf.push_back((int)i);
        walld.assign(mesh.cells.size(), std::numeric_limits<double>::infinity());
        if (wf.empty()) return;
#pragma omp parallel for
        for (long c = 0; c < (long)mesh.cells.size(); ++c) {
            const Cell& cell = mesh.cells[c];
            double m = std::numeric_limits<double>::infinity();
            for (int fi : wf) {
                const Face& f = mesh.faces[fi];
                const Node& a = mesh.nodes[f.node1];
                const Node& b = mesh.nodes[f.node2];
                double dx = b.x - a.x, dy = b.y - a.y;
                double ls = dx * dx + dy * dy;
                double t = (ls > 0.0) ? ((cell.x_centroid - a.x) * dx + (cell.y_centroid - a.y) * dy) / ls : 0.0;
                t = std::clamp(t, 0.0, 1.0);
                double ex = cell.x_centroid - (a.x + t * dx), ey = cell.y_centroid - (a.y + t * dy);
                m = std::min(m, ex * ex + ey * ey);
            }
            walld[c] = std::sqrt(m);
        }
    }

    // GradientCalculator::compute for one scalar with boundary-face values.
    void grad(const std::vector<double>& phi, const std::vector<double>& bphi, std::vector<G2>& g) const {
        g.assign(mesh.cells.size(), G2{});
        if (gradient == 1) {
#pragma omp parallel for
            for (long c = 0; c < (long)mesh.cells.size(); ++c) {
                const Cell& cell = mesh.cells[c];
                double sx = 0.0, sy = 0.0;
                for (int fi : cell.faces) {
                    const Face& f = mesh.faces[fi];
                    double pf;
                    if (f.cell_right == -1) pf = bphi[fi];
                    else {
                        int o = (f.cell_left == (int)c) ? f.cell_right : f.cell_left;
                        double dc = std::hypot(cell.x_centroid - f.x_mid, cell.y_centroid - f.y_mid);
                        double dn = std::hypot(mesh.cells[o].x_centroid - f.x_mid, mesh.cells[o].y_centroid - f.y_mid);
                        double wc = dn / (dc + dn);
                        pf = wc * phi[c] + (1.0 - wc) * phi[o];
                    }
                    double nx = f.cell_left == (int)c ? f.nx : -f.nx, ny = f.cell_left == (int)c ? f.ny : -f.ny;
                    sx += pf * nx * f.area;
                    sy += pf * ny * f.area;
                }
                g[c].x = sx / cell.volume;
                g[c].y = sy / cell.volume;
            }
            return;
        }
#pragma omp parallel for
        for (long c = 0; c < (long)mesh.cells.size(); ++c) {
            const Cell& cell = mesh.cells[c];
            double bx = 0.0, by = 0.0;
            for (int fi : cell.faces) {
                const Face& f = mesh.faces[fi];
                double px, py, pn;
                if (f.cell_right == -1) { px = f.x_mid; py = f.y_mid; pn = bphi[fi]; }
                else {
                    int nb = (f.cell_left == (int)c) ? f.cell_right : f.cell_left;
                    px = mesh.cells[nb].x_centroid; py = mesh.cells[nb].y_centroid; pn = phi[nb];
                }
                double dx = px - cell.x_centroid, dy = py - cell.y_centroid;
                double w = 1.0 / (dx * dx + dy * dy);
                double d = pn - phi[c];
                bx += w * dx * d;
                by += w * dy * d;
            }
            g[c].x = lsq[3 * c] * bx + lsq[3 * c + 1] * by;
            g[c].y = lsq[3 * c + 1] * bx + lsq[3 * c + 2] * by;
        }
    }

    // face_normal_geometry: distance, cos theta and unit direction from the
    // owner's centroid to the neighbour's centroid (boundary: the midpoint).
    void face_geom(const Face& f, double& dist, double& cth, double& hx, double& hy) const {
        const Cell& L = mesh.cells[f.cell_left];
        bool b = f.cell_right == -1;
        double xr = b ? f.x_mid : mesh.cells[f.cell_right].x_centroid;
        double yr = b ? f.y_mid : mesh.cells[f.cell_right].y_centroid;
        double dx = xr - L.x_centroid, dy = yr - L.y_centroid;
        dist = std::hypot(dx, dy);
        hx = dx / dist; hy = dy / dist;
        cth = f.nx * hx + f.ny * hy;
    }
    FaceGrad face_gradient(const Face& f, double pL, double pR, const G2& gL, const G2& gR, double pb) const {
        const Cell& L = mesh.cells[f.cell_left];
        bool b = f.cell_right == -1;
        double xr = b ? f.x_mid : mesh.cells[f.cell_right].x_centroid;
        double yr = b ? f.y_mid : mesh.cells[f.cell_right].y_centroid;
        double pRv = b ? pb : pR;
        double dist, cth, hx, hy;
        face_geom(f, dist, cth, hx, hy);
        double direct = (pRv - pL) / (dist * cth);
        double kx = f.nx - hx / cth, ky = f.ny - hy / cth;
        G2 gf;
        if (b) gf = gL;
        else {
            double dL = std::hypot(L.x_centroid - f.x_mid, L.y_centroid - f.y_mid);
            double dR = std::hypot(xr - f.x_mid, yr - f.y_mid);
            double wL = dR / (dL + dR);
            gf.x = wL * gL.x + (1.0 - wL) * gR.x;
            gf.y = wL * gL.y + (1.0 - wL) * gR.y;
        }
        return {direct + gf.x * kx + gf.y * ky, gf};
    }
    static G2 corrected(const FaceGrad& fg, double nx, double ny) {
        double avg = fg.gf.x * nx + fg.gf.y * ny;
        double d = fg.dn - avg;
        return {fg.gf.x + d * nx, fg.gf.y + d * ny};
    }
    double temperature(const State& s) const { return pressure(s, gamma) / (s.rho * R); }

    State ghost_ns(const Face& f, const State& UL) const {
        const RansBC& bc = bcs[f.patch_id];
        if (bc.type == BC_FARFIELD) return bc.state;
        if (bc.type == BC_OUTFLOW) return UL;
        double uL = UL.rho_u / UL.rho, vL = UL.rho_v / UL.rho;
        double pL = pressure(UL, gamma);
        return from_primitive(UL.rho, 2.0 * bc.wall_u - uL, 2.0 * bc.wall_v - vL, pL, gamma);
    }
    State numflux(const State& L, const State& Rs, double nx, double ny) const {
        if (flux == 1) return hllc(L, Rs, nx, ny, gamma);
        if (flux == 2) return exact(L, Rs, nx, ny, gamma, tol, maxit);
        return rusanov(L, Rs, nx, ny, gamma);
    }

    double compute_dt() const {
        double dt = std::numeric_limits<double>::max();
#pragma omp parallel for reduction(min : dt)
        for (long i = 0; i < (long)mesh.faces.size(); ++i) {
            const Face& f = mesh.faces[i];
            const State& UL = U[f.cell_left];
            double uL = UL.rho_u / UL.rho, vL = UL.rho_v / UL.rho;
            double VnL = uL * f.nx + vL * f.ny;
            double Smax = std::fabs(VnL) + sound_speed(UL, gamma);
            double rmin = UL.rho;
            double ntmax = sa_nut(nut[f.cell_left], mu / UL.rho, sa);
            if (f.cell_right != -1) {
                const State& UR = U[f.cell_right];
                double uR = UR.rho_u / UR.rho, vR = UR.rho_v / UR.rho;
                double VnR = uR * f.nx + vR * f.ny;
                Smax = std::max(Smax, std::fabs(VnR) + sound_speed(UR, gamma));
                rmin = std::min(rmin, UR.rho);
                ntmax = std::max(ntmax, sa_nut(nut[f.cell_right], mu / UR.rho, sa));
            }
            double dist, cth, hx, hy;
            face_geom(f, dist, cth, hx, hy);
            double length = dist * cth;
            double nl = (mu > 0.0) ? mu / rmin : 0.0;
            double ne = nl + ntmax;
            double St = Smax + 2.0 * ne / length;
            dt = std::min(dt, cfl * length / St);
        }
        return dt;
    }

    void step() {
        double dt = compute_dt();
        const size_t N = mesh.cells.size(), F = mesh.faces.size();
        std::vector<double> u(N), v(N), T(N), nl(N), nt(N);
        for (size_t c = 0; c < N; ++c) {
            u[c] = U[c].rho_u / U[c].rho;
            v[c] = U[c].rho_v / U[c].rho;
            T[c] = temperature(U[c]);
            nl[c] = mu / U[c].rho;
            nt[c] = sa_nut(nut[c], nl[c], sa);
        }
        std::vector<double> bu(F, 0.0), bv(F, 0.0), bT(F, 0.0), bn(F, 0.0);
        for (size_t i = 0; i < F; ++i) {
            const Face& f = mesh.faces[i];
            if (f.cell_right != -1) continue;
            int cl = f.cell_left;
            const RansBC& bc = bcs[f.patch_id];
            if (bc.type == BC_NOSLIP) {
                bu[i] = bc.wall_u; bv[i] = bc.wall_v; bT[i] = bc.isothermal ? bc.wall_T : T[cl];
                bn[i] = 0.0;
            } else {
                bu[i] = u[cl]; bv[i] = v[cl]; bT[i] = T[cl];
                bn[i] = bc.type == BC_FARFIELD ? bc.nut : nut[cl];
            }
        }
        std::vector<G2> gu, gv, gT, gn;
        grad(u, bu, gu);
        grad(v, bv, gv);
        grad(T, bT, gT);
        grad(nut, bn, gn);
        std::vector<double> src(N);
#pragma omp parallel for
        for (long c = 0; c < (long)N; ++c) {
            double omega = std::fabs(gv[c].x - gu[c].y);
            src[c] = sa_source(nut[c], nl[c], omega, walld[c], gn[c], sa);
        }
        double cp = gamma * R / (gamma - 1.0);
        std::vector<State> ff(F);
        std::vector<double> nf(F);
#pragma omp parallel for
        for (long i = 0; i < (long)F; ++i) {
            const Face& f = mesh.faces[i];
            int cl = f.cell_left, cr = f.cell_right;
            bool b = cr == -1;
            const State& UL = U[cl];
            State UR = b ? ghost_ns(f, UL) : U[cr];
            State inv = numflux(UL, UR, f.nx, f.ny);
            double uRg = UR.rho_u / UR.rho, vRg = UR.rho_v / UR.rho;
            double Vn = 0.5 * ((u[cl] + uRg) * f.nx + (v[cl] + vRg) * f.ny);
            double nR = b ? bn[i] : nut[cr];
            double nup = (Vn >= 0.0) ? nut[cl] : nR;
            double nadv = Vn * nup * f.area;
            State vis;
            double ndiff = 0.0;
            bool visc = !b || bcs[f.patch_id].type == BC_NOSLIP;
            if (visc) {
                double pu = b ? bu[i] : u[cr], pv = b ? bv[i] : v[cr], pT = b ? bT[i] : T[cr];
                G2 gru = b ? G2{} : gu[cr], grv = b ? G2{} : gv[cr], grT = b ? G2{} : gT[cr];
                FaceGrad fu = face_gradient(f, u[cl], pu, gu[cl], gru, bu[i]);
                FaceGrad fv = face_gradient(f, v[cl], pv, gv[cl], grv, bv[i]);
                FaceGrad fT = face_gradient(f, T[cl], pT, gT[cl], grT, bT[i]);
                G2 a = corrected(fu, f.nx, f.ny), bb = corrected(fv, f.nx, f.ny), cT = corrected(fT, f.nx, f.ny);
                double nlR = b ? nl[cl] : nl[cr];
                double ntR = b ? sa_nut(bn[i], nlR, sa) : nt[cr];
                double rR = b ? U[cl].rho : U[cr].rho;
                double tdv = 0.5 * (U[cl].rho * nt[cl] + rR * ntR);
                double mue = mu + tdv;
                double ke = cp * mu / Pr + cp * tdv / Prt;
                double uf = b ? bu[i] : 0.5 * (u[cl] + u[cr]);
                double vf = b ? bv[i] : 0.5 * (v[cl] + v[cr]);
                double dv = a.x + bb.y;
                double txx = mue * (2.0 * a.x - (2.0 / 3.0) * dv);
                double tyy = mue * (2.0 * bb.y - (2.0 / 3.0) * dv);
                double txy = mue * (a.y + bb.x);
                double qx = -ke * cT.x, qy = -ke * cT.y;
                if (b && !bcs[f.patch_id].isothermal) { qx = 0.0; qy = 0.0; }
                vis.rho_u = txx * f.nx + txy * f.ny;
                vis.rho_v = txy * f.nx + tyy * f.ny;
                vis.E = (uf * txx + vf * txy - qx) * f.nx + (uf * txy + vf * tyy - qy) * f.ny;
                double nlf = 0.5 * (nl[cl] + nlR);
                double ntf = 0.5 * (nt[cl] + ntR);
                G2 grn = b ? G2{} : gn[cr];
                FaceGrad fn = face_gradient(f, nut[cl], nR, gn[cl], grn, bn[i]);
                double dif = (nlf + ntf) / sa.sigma;
                ndiff = -dif * fn.dn * f.area;
            }
            ff[i] = f.area * (inv - vis);
            nf[i] = nadv + ndiff;
        }
        double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0, s4 = 0.0;
#pragma omp parallel for reduction(+ : s0, s1, s2, s3, s4)
        for (long c = 0; c < (long)N; ++c) {
            State r;
            double rn = 0.0;
            for (int fi : mesh.cells[c].faces) {
                const Face& f = mesh.faces[fi];
                if ((long)f.cell_left == c) { r = r - ff[fi]; rn -= nf[fi]; }
                else { r += ff[fi]; rn += nf[fi]; }
            }
            rn += mesh.cells[c].volume * src[c];
            s0 += r.rho * r.rho; s1 += r.rho_u * r.rho_u; s2 += r.rho_v * r.rho_v; s3 += r.E * r.E; s4 += rn * rn;
            U[c] += (dt / mesh.cells[c].volume) * r;
            nut[c] += (dt / mesh.cells[c].volume) * rn;
        }
        last[0] = std::sqrt(s0); last[1] = std::sqrt(s1); last[2] = std::sqrt(s2); last[3] = std::sqrt(s3);
        last[4] = std::sqrt(s4);
    }
};

}  // namespace orc

// =========================================================== C API ======
extern "C" {

void* orc_mesh_build(int n_nodes, const double* xy, int n_cells, const int64_t* off, const int* cn, int n_be,
                     const int* be, const int* bp, int n_patches) {
    auto* m = new orc::Mesh;
    if (!orc::build_mesh(*m, n_nodes, xy, n_cells, off, cn, n_be, be, bp, n_patches)) {
        delete m;
        return nullptr;
    }
    return m;
}
void orc_mesh_free(void* m) { delete static_cast<orc::Mesh*>(m); }
int orc_mesh_counts(void* mp, int64_t* out) {
    auto* m = static_cast<orc::Mesh*>(mp);
    out[0] = (int64_t)m->cells.size();
    out[1] = (int64_t)m->faces.size();
    return 0;
}

// bc_type[n_patches], bc_state[4*n_patches] (conserved); ic[14]: two_region,
// rho,u,v,p, rho_l,u_l,v_l,p_l, rho_r,u_r,v_r,p_r, x0; iopt[8]: flux, order,
// rk, local_dt, gradient, limiter, maxit, unused; dopt[4]: gamma, cfl, tol, K.
void* orc_euler_create(void* mp, const int* bc_type, const double* bc_state, const double* ic, const int* iopt,
                       const double* dopt) {
    auto* m = static_cast<orc::Mesh*>(mp);
    auto* e = new orc::Euler;
    e->mesh = *m;
    e->gamma = dopt[0]; e->cfl = dopt[1]; e->tol = dopt[2]; e->venkat_k = dopt[3];
    e->flux = iopt[0]; e->order = iopt[1]; e->rk = iopt[2]; e->local_dt = iopt[3];
    e->gradient = iopt[4]; e->limiter = iopt[5]; e->maxit = iopt[6];
    e->bcs.resize(m->n_patches);
    for (int p = 0; p < m->n_patches; ++p) {
        e->bcs[p].type = bc_type[p];
        e->bcs[p].state = {bc_state[4 * p], bc_state[4 * p + 1], bc_state[4 * p + 2], bc_state[4 * p + 3]};
    }
    size_t N = m->cells.size();
    e->U.resize(N);
    for (size_t i = 0; i < N; ++i) {
        if (ic[0] == 0.0) e->U[i] = orc::from_primitive(ic[1], ic[2], ic[3], ic[4], e->gamma);
        else if (m->cells[i].x_centroid < ic[13]) e->U[i] = orc::from_primitive(ic[5], ic[6], ic[7], ic[8], e->gamma);
        else e->U[i] = orc::from_primitive(ic[9], ic[10], ic[11], ic[12], e->gamma);
    }
    if (e->order == 2 && e->gradient == 0) e->setup_lsq();
    return e;
}
void orc_euler_free(void* e) { delete static_cast<orc::Euler*>(e); }
// One numerical flux (0 Rusanov, 1 HLLC, 2 exact Riemann; 3 the physical
// flux of UL) of conserved states UL, UR [4] through the unit normal
// (nx, ny): out [4].  For the flux known-answer tests.
void orc_flux(int flux, const double* UL, const double* UR, double nx, double ny, double g, double tol, int maxit,
              double* out) {
    const orc::State L{UL[0], UL[1], UL[2], UL[3]}, R{UR[0], UR[1], UR[2], UR[3]};
    orc::State F;
    if (flux == 0) F = orc::rusanov(L, R, nx, ny, g);
    else if (flux == 1) F = orc::hllc(L, R, nx, ny, g);
    else if (flux == 2) F = orc::exact(L, R, nx, ny, g, tol, maxit);
    else F = orc::phys_flux(L, nx, ny, g);
    out[0] = F.rho; out[1] = F.rho_u; out[2] = F.rho_v; out[3] = F.E;
}
void orc_euler_run(void* ep, int n, double* hist) {
    auto* e = static_cast<orc::Euler*>(ep);
    for (int s = 0; s < n; ++s) {
        e->step();
        if (hist) std::memcpy(hist + 4 * (size_t)s, e->last, sizeof(e->last));
    }
}
void orc_euler_field(void* ep, double* out) {
    auto* e = static_cast<orc::Euler*>(ep);
    std::memcpy(out, e->U.data(), e->U.size() * sizeof(orc::State));
}
void orc_euler_set_field(void* ep, const double* in) {
    auto* e = static_cast<orc::Euler*>(ep);
    std::memcpy(e->U.data(), in, e->U.size() * sizeof(orc::State));
}
// Limited gradients of (rho, u, v, p) for the current state: N x 8
// (gx[4], gy[4]); also the primitive state N x 4.
void orc_euler_gradients(void* ep, double* grad, double* prim) {
    auto* e = static_cast<orc::Euler*>(ep);
    std::vector<orc::Prim> W;
    std::vector<orc::Grad4> G;
    e->gradients(e->U, W, G);
    for (size_t c = 0; c < W.size(); ++c) {
        std::memcpy(grad + 8 * c, &G[c], 8 * sizeof(double));
        std::memcpy(prim + 4 * c, &W[c], 4 * sizeof(double));
    }
}
void orc_euler_set_cfl(void* ep, double cfl) { static_cast<orc::Euler*>(ep)->cfl = cfl; }
// Pressure-only wall forces (inviscid): same accumulation as compute_wall_forces.
void orc_euler_wall_forces(void* ep, const int* is_wall, const double* ref, double* out) {
    auto* e = static_cast<orc::Euler*>(ep);
    double vmag = std::hypot(ref[1], ref[2]);
    double dx = ref[1] / vmag, dy = ref[2] / vmag, lx = -dy, ly = dx;
    double qL = 0.5 * ref[0] * vmag * vmag * ref[4], qL2 = qL * ref[4];
    double fd = 0, pd = 0, td = 0, lift = 0, mom = 0, n = 0;
    for (const orc::Face& f : e->mesh.faces) {
        if (f.cell_right != -1 || !is_wall[f.patch_id]) continue;
        double p = orc::pressure(e->U[f.cell_left], e->gamma);
        double fx = 0.0, fy = 0.0, px = f.area * p * f.nx, py = f.area * p * f.ny;
        double rx = f.x_mid - ref[5], ry = f.y_mid - ref[6];
        double fdi = fx * dx + fy * dy, pdi = px * dx + py * dy;
        fd += fdi; pd += pdi; td += fdi + pdi;
        lift += (fx + px) * lx + (fy + py) * ly;
        mom += rx * (fy + py) - ry * (fx + px);
        n += 1;
    }
    double r[11] = {fd, pd, td, lift, mom, fd / qL, pd / qL, td / qL, lift / qL, mom / qL2, n};
    std::memcpy(out, r, sizeof(r));
}

void* orc_diff_create(void* mp, double alpha, double dt, double v0, double r0, const int* ptype, const double* pval) {
    auto* m = static_cast<orc::Mesh*>(mp);
    auto* d = new orc::Diffusion;
    d->mesh = *m;
    d->alpha = alpha; d->dt = dt;
    d->ptype.assign(ptype, ptype + m->n_patches);
    d->pval.assign(pval, pval + m->n_patches);
    d->phi.assign(m->cells.size(), 0.0);
    for (size_t i = 0; i < m->cells.size(); ++i)
        if (std::sqrt(m->cells[i].x_centroid * m->cells[i].x_centroid + m->cells[i].y_centroid * m->cells[i].y_centroid) < r0)
            d->phi[i] = v0;
    return d;
}
void orc_diff_free(void* d) { delete static_cast<orc::Diffusion*>(d); }
void orc_diff_run(void* dp, int n, double* hist) {
    auto* d = static_cast<orc::Diffusion*>(dp);
    for (int s = 0; s < n; ++s) {
        d->step();
        if (hist) hist[s] = d->last;
    }
}
void orc_diff_field(void* dp, double* out) {
    auto* d = static_cast<orc::Diffusion*>(dp);
    std::memcpy(out, d->phi.data(), d->phi.size() * sizeof(double));
}

// RANS-SA (RANSTurbulenceSASolver): per patch bc_type (BC_NOSLIP,
// BC_FARFIELD, BC_OUTFLOW), bc_state [4] (farfield, conserved), bc_wall [4]
// (wall_u, wall_v, wall_T, farfield nu-tilde), bc_iso (isothermal wall);
// ic[14] as orc_euler_create; iopt[3]: flux, gradient (0 LSQ, 1 GG), maxit;
// dopt[8]: gamma, R, mu, Pr, Pr_t, cfl, exact tol, initial nu-tilde.
void* orc_rans_create(void* mp, const int* bc_type, const double* bc_state, const double* bc_wall, const int* bc_iso,
                      const double* ic, const int* iopt, const double* dopt) {
    auto* m = static_cast<orc::Mesh*>(mp);
    auto* r = new orc::Rans;
    r->mesh = *m;
    r->gamma = dopt[0]; r->R = dopt[1]; r->mu = dopt[2]; r->Pr = dopt[3]; r->Prt = dopt[4]; r->cfl = dopt[5];
    r->tol = dopt[6];
    r->flux = iopt[0]; r->gradient = iopt[1]; r->maxit = iopt[2];
    r->bcs.resize(m->n_patches);
    for (int p = 0; p < m->n_patches; ++p) {
        orc::RansBC& b = r->bcs[p];
        b.type = bc_type[p];
        b.state = {bc_state[4 * p], bc_state[4 * p + 1], bc_state[4 * p + 2], bc_state[4 * p + 3]};
        b.wall_u = bc_wall[4 * p]; b.wall_v = bc_wall[4 * p + 1]; b.wall_T = bc_wall[4 * p + 2];
        b.nut = bc_wall[4 * p + 3];
        b.isothermal = bc_iso[p];
    }
    size_t N = m->cells.size();
    r->U.resize(N);
    r->nut.assign(N, dopt[7]);
    for (size_t i = 0; i < N; ++i) {
        if (ic[0] == 0.0) r->U[i] = orc::from_primitive(ic[1], ic[2], ic[3], ic[4], r->gamma);
        else if (m->cells[i].x_centroid < ic[13]) r->U[i] = orc::from_primitive(ic[5], ic[6], ic[7], ic[8], r->gamma);
        else r->U[i] = orc::from_primitive(ic[9], ic[10], ic[11], ic[12], r->gamma);
    }
    r->setup();
    return r;
}
void orc_rans_free(void* r) { delete static_cast<orc::Rans*>(r); }
// n steps; hist [5 n] (four mean-flow residual norms and nu-tilde's), may be NULL
void orc_rans_run(void* rp, int n, double* hist) {
    auto* r = static_cast<orc::Rans*>(rp);
    for (int s = 0; s < n; ++s) {
        r->step();
        if (hist) std::memcpy(hist + 5 * (size_t)s, r->last, sizeof(r->last));
    }
}
// field [4 N] conserved, nut [N], walld [N]; each may be NULL
void orc_rans_get(void* rp, double* field, double* nut, double* walld) {
    auto* r = static_cast<orc::Rans*>(rp);
    if (field) std::memcpy(field, r->U.data(), r->U.size() * sizeof(orc::State));
    if (nut) std::memcpy(nut, r->nut.data(), r->nut.size() * sizeof(double));
    if (walld) std::memcpy(walld, r->walld.data(), r->walld.size() * sizeof(double));
}

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#endif
}

}  // extern "C"
