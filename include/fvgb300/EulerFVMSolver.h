// Drop-in replacement for the reference's include/EulerFVMSolver.h.
//
// Same types, names and member signatures as the reference header
// (include/EulerFVMSolver.h:17-196), backed by the GB300 library through its
// C ABI (fv_gb300.h).  Put include/fvgb300 ahead of the reference's include
// directory, keep the reference's UnstructuredMesh.h and EulerState.h, link
// libfvgb300.so, and a driver written against the reference (run_euler,
// the verification modes) compiles and runs unchanged on the GPU.
//
// Differences a caller can observe: the solver is move-only (it owns a GPU
// solver handle); field() returns a host copy refreshed after each step
// (same lifetime contract: valid until the next step()/set_field()); errors
// of the ABI (no GPU, invalid mesh) throw std::runtime_error, while a
// diverged state is reported the reference's way, through residual().
#ifndef EULERFVMSOLVER_H_INCLUDED
#define EULERFVMSOLVER_H_INCLUDED

#include <cassert>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "EulerState.h"
#include "UnstructuredMesh.h"
#include "fv_gb300.h"

enum class EulerBoundaryType : int { Wall = 0, Farfield = 1, Outflow = 2 };

struct EulerBoundaryCondition {
    EulerBoundaryType type = EulerBoundaryType::Wall;
    EulerState farfield_state;
};

enum class EulerICMode { Freestream, TwoRegion };

enum class NumericalFluxScheme { Rusanov, HLLC, Exact };

struct EulerResidualNorms {
    double rho = 0.0, rho_u = 0.0, rho_v = 0.0, E = 0.0;
};

struct EulerInitialCondition {
    EulerICMode mode = EulerICMode::Freestream;
    double rho = 1.0, u = 0.0, v = 0.0, p = 1.0;
    double rho_l = 1.0, u_l = 0.0, v_l = 0.0, p_l = 1.0;
    double rho_r = 0.125, u_r = 0.0, v_r = 0.0, p_r = 0.1;
    double x0 = 0.0;
};

namespace fvgb300_shim {

inline void check(int status) {
    if (status != FV_OK) throw std::runtime_error(std::string("fvgb300: ") + fv_last_error());
}

// UnstructuredMesh (reference numbering) -> device mesh handle.
inline fv_mesh_t make_mesh(const UnstructuredMesh& m) {
    std::vector<double> xy(2 * m.nodes.size());
    for (size_t i = 0; i < m.nodes.size(); ++i) {
        xy[2 * i] = m.nodes[i].x;
        xy[2 * i + 1] = m.nodes[i].y;
    }
    std::vector<int32_t> fn(2 * m.faces.size()), fc(2 * m.faces.size()), fp(m.faces.size());
    for (size_t f = 0; f < m.faces.size(); ++f) {
        fn[2 * f] = m.faces[f].node1;
        fn[2 * f + 1] = m.faces[f].node2;
        fc[2 * f] = m.faces[f].cell_left;
        fc[2 * f + 1] = m.faces[f].cell_right;
        fp[f] = m.faces[f].patch_id;
    }
    std::vector<int32_t> off(1, 0), cf;
    std::vector<double> geom(3 * m.cells.size());
    for (size_t c = 0; c < m.cells.size(); ++c) {
        cf.insert(cf.end(), m.cells[c].faces.begin(), m.cells[c].faces.end());
        off.push_back((int32_t)cf.size());
        geom[3 * c] = m.cells[c].volume;
        geom[3 * c + 1] = m.cells[c].x_centroid;
        geom[3 * c + 2] = m.cells[c].y_centroid;
    }
    fv_mesh_t h = nullptr;
    check(fv_mesh_create_faces((int32_t)m.nodes.size(), xy.data(), (int32_t)m.faces.size(), fn.data(), fc.data(),
                               fp.data(), (int32_t)m.cells.size(), off.data(), cf.data(), geom.data(),
                               (int32_t)m.patches.size(), FV_REORDER_MORTON, &h));
    return h;
}

inline fv_ic_t make_ic(const EulerInitialCondition& ic) {
    fv_ic_t s{};
    s.two_region = ic.mode == EulerICMode::TwoRegion;
    s.rho = ic.rho; s.u = ic.u; s.v = ic.v; s.p = ic.p;
    s.rho_l = ic.rho_l; s.u_l = ic.u_l; s.v_l = ic.v_l; s.p_l = ic.p_l;
    s.rho_r = ic.rho_r; s.u_r = ic.u_r; s.v_r = ic.v_r; s.p_r = ic.p_r;
    s.x0 = ic.x0;
    return s;
}

// Shared state handling of the GPU-backed solver classes.
class SolverHandle {
public:
    SolverHandle() = default;
    SolverHandle(const SolverHandle&) = delete;
    SolverHandle& operator=(const SolverHandle&) = delete;
    SolverHandle(SolverHandle&& o) noexcept { *this = std::move(o); }
    SolverHandle& operator=(SolverHandle&& o) noexcept {
        std::swap(h_, o.h_);
        std::swap(n_, o.n_);
        U_.swap(o.U_);
        std::swap(fresh_, o.fresh_);
        return *this;
    }
    ~SolverHandle() {
        if (h_) fv_solver_destroy(h_);
    }

    void create(const UnstructuredMesh& mesh, const std::vector<fv_bc_t>& bcs, double gamma, double cfl,
                const EulerInitialCondition& ic, const fv_options_t& opt) {
        fv_mesh_t m = make_mesh(mesh);
        fv_ic_t c = make_ic(ic);
        int rc = fv_solver_create(m, bcs.data(), (int32_t)bcs.size(), gamma, cfl, &c, &opt, &h_);
        fv_mesh_destroy(m);
        check(rc);
        n_ = mesh.cells.size();
        U_.resize(n_);
    }
    // step() never reports divergence in the reference; a non-finite state
    // shows up in residual() (src/main.cpp:3496-3500).
    void steps(int n) {
        int rc = fv_step(h_, n, nullptr);
        if (rc != FV_OK && rc != FV_ERR_NONFINITE) check(rc);
        fresh_ = false;
    }
    const std::vector<EulerState>& field() const {
        if (!fresh_) {
            check(fv_get_field(h_, reinterpret_cast<double*>(U_.data())));
            fresh_ = true;
        }
        return U_;
    }
    const EulerResidualNorms& residual() const {
        double r[4];
        check(fv_get_residual(h_, r));
        res_ = {r[0], r[1], r[2], r[3]};
        return res_;
    }
    void set_field(const std::vector<EulerState>& U) {
        assert(U.size() == n_);
        check(fv_set_field(h_, reinterpret_cast<const double*>(U.data())));
        U_ = U;
        fresh_ = true;
    }
    void set_cfl(double cfl) { check(fv_set_cfl(h_, cfl)); }
    double gamma() const {
        double g = 0.0;
        check(fv_get_gamma(h_, &g));
        return g;
    }
    fv_solver_t handle() const { return h_; }

private:
    fv_solver_t h_ = nullptr;
    size_t n_ = 0;
    mutable std::vector<EulerState> U_;
    mutable bool fresh_ = false;
    mutable EulerResidualNorms res_;
};

static_assert(sizeof(EulerState) == 4 * sizeof(double), "EulerState must be four packed doubles");

}  // namespace fvgb300_shim

// EulerFVMSolver (include/EulerFVMSolver.h:83-196) on the GPU.
class EulerFVMSolver {
public:
    EulerFVMSolver(const UnstructuredMesh& input_mesh, const std::vector<EulerBoundaryCondition>& boundary_conditions,
                   double gamma, double cfl, const EulerInitialCondition& initial_condition,
                   NumericalFluxScheme flux_scheme, double exact_riemann_tol, int exact_riemann_max_iter) {
        std::vector<fv_bc_t> bcs(boundary_conditions.size());
        for (size_t i = 0; i < bcs.size(); ++i) {
            bcs[i] = fv_bc_t{};
            bcs[i].type = (int32_t)boundary_conditions[i].type;
            const EulerState& s = boundary_conditions[i].farfield_state;
            bcs[i].state[0] = s.rho;
            bcs[i].state[1] = s.rho_u;
            bcs[i].state[2] = s.rho_v;
            bcs[i].state[3] = s.E;
        }
        fv_options_t opt;
        fv_options_default(&opt);
        opt.flux = (int32_t)flux_scheme;
        opt.exact_tol = exact_riemann_tol;
        opt.exact_max_iter = exact_riemann_max_iter;
        s_.create(input_mesh, bcs, gamma, cfl, initial_condition, opt);
    }

    void step() { s_.steps(1); }
    void run(int total_steps) {
        s_.steps(total_steps);
        std::cout << "Simulation completed across " << total_steps << " steps.\n";
    }
    const std::vector<EulerState>& field() const { return s_.field(); }
    double gas_gamma() const { return s_.gamma(); }
    const EulerResidualNorms& residual() const { return s_.residual(); }
    void set_field(const std::vector<EulerState>& new_U) { s_.set_field(new_U); }
    void set_cfl(double new_cfl) { s_.set_cfl(new_cfl); }

    // Extension: the underlying ABI handle (second-order options, timing).
    fv_solver_t gpu_handle() const { return s_.handle(); }

private:
    fvgb300_shim::SolverHandle s_;
};

#endif  // EULERFVMSOLVER_H_INCLUDED
