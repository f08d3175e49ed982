// Drop-in replacement for the reference's include/NavierStokesFVMSolver.h
// (types and solver API, include/NavierStokesFVMSolver.h:19-218) backed by
// the GB300 library.  GradientScheme comes from the reference's own
// GradientReconstruction.h, which stays in the build unchanged.
//
// Not provided (diagnostics outside the residual-and-update loop):
// compute_resolution_diagnostics and the boundary-layer profile samplers.
// Wall forces are available through wall_forces() (compute_wall_traction +
// compute_wall_forces, domain total).
#ifndef NAVIERSTOKESFVMSOLVER_H_INCLUDED
#define NAVIERSTOKESFVMSOLVER_H_INCLUDED

#include <vector>

#include "EulerFVMSolver.h"
#include "GradientReconstruction.h"

enum class NSBoundaryType : int { NoSlipWall = 0, Farfield = 1, Outflow = 2 };

struct NSBoundaryCondition {
    NSBoundaryType type = NSBoundaryType::NoSlipWall;
    double wall_u = 0.0, wall_v = 0.0;
    bool is_isothermal_wall = false;
    double wall_temperature = 0.0;
    EulerState farfield_state;
};

// Domain total of compute_wall_forces (include/WallTraction.h:122-128).
struct GpuWallForces {
    double friction_drag = 0.0, pressure_drag = 0.0, total_drag = 0.0, lift = 0.0, moment = 0.0;
    double cd_friction = 0.0, cd_pressure = 0.0, cd_total = 0.0, cl = 0.0, cm = 0.0;
};

class NavierStokesFVMSolver {
public:
    NavierStokesFVMSolver(const UnstructuredMesh& input_mesh,
                          const std::vector<NSBoundaryCondition>& boundary_conditions, double gamma,
                          double gas_constant, double mu, double prandtl, double cfl,
                          const EulerInitialCondition& initial_condition, NumericalFluxScheme flux_scheme,
                          GradientScheme gradient_scheme, double exact_riemann_tol, int exact_riemann_max_iter) {
        std::vector<fv_bc_t> bcs(boundary_conditions.size());
        for (size_t i = 0; i < bcs.size(); ++i) {
            const NSBoundaryCondition& b = boundary_conditions[i];
            bcs[i] = fv_bc_t{};
            bcs[i].type = b.type == NSBoundaryType::NoSlipWall ? FV_BC_NOSLIP
                                                               : (b.type == NSBoundaryType::Farfield ? FV_BC_FARFIELD
                                                                                                    : FV_BC_OUTFLOW);
            bcs[i].isothermal = b.is_isothermal_wall ? 1 : 0;
            bcs[i].wall_u = b.wall_u;
            bcs[i].wall_v = b.wall_v;
            bcs[i].wall_T = b.wall_temperature;
            bcs[i].state[0] = b.farfield_state.rho;
            bcs[i].state[1] = b.farfield_state.rho_u;
            bcs[i].state[2] = b.farfield_state.rho_v;
            bcs[i].state[3] = b.farfield_state.E;
        }
        fv_options_t opt;
        fv_options_default(&opt);
        opt.viscous = 1;
        opt.gas_constant = gas_constant;
        opt.mu = mu;
        opt.prandtl = prandtl;
        opt.flux = (int32_t)flux_scheme;
        opt.gradient = gradient_scheme == GradientScheme::GreenGauss ? FV_GRAD_GG : FV_GRAD_LSQ;
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

    // Extension: wall forces over every no-slip face (reference quantities as
    // in WallReferenceQuantities, include/WallTraction.h:99-105).
    GpuWallForces wall_forces(double rho_ref, double u_ref, double v_ref, double p_ref, double length_ref,
                              double moment_x, double moment_y) const {
        const double ref[7] = {rho_ref, u_ref, v_ref, p_ref, length_ref, moment_x, moment_y};
        double o[11];
        fvgb300_shim::check(fv_wall_forces(s_.handle(), ref, o));
        return {o[0], o[1], o[2], o[3], o[4], o[5], o[6], o[7], o[8], o[9]};
    }
    fv_solver_t gpu_handle() const { return s_.handle(); }

private:
    fvgb300_shim::SolverHandle s_;
};

#endif  // NAVIERSTOKESFVMSOLVER_H_INCLUDED
