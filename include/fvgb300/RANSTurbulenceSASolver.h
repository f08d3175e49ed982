// Drop-in replacement for the reference's include/RANSTurbulenceSASolver.h
// (RANSBoundaryConditionSA and the RANSTurbulenceSASolver API) backed by the
// GB300 library (fv_solver_create with viscous = 2).
//
// Not provided (diagnostics outside the residual-and-update loop): the
// resolution report and the boundary-layer profile samplers.  Wall forces
// are available through wall_forces() (domain total, effective viscosity).
#ifndef RANSTURBULENCESASOLVER_H_INCLUDED
#define RANSTURBULENCESASOLVER_H_INCLUDED

#include <iostream>
#include <vector>

#include "EulerFVMSolver.h"
#include "NavierStokesFVMSolver.h"
#include "SpalartAllmaras.h"

struct RANSBoundaryConditionSA {
    NSBoundaryCondition ns;
    double farfield_nut = 0.0;
};

class RANSTurbulenceSASolver {
public:
    RANSTurbulenceSASolver(const UnstructuredMesh& input_mesh,
                           const std::vector<RANSBoundaryConditionSA>& boundary_conditions, double gamma,
                           double gas_constant, double mu, double prandtl, double prandtl_t, double cfl,
                           const EulerInitialCondition& initial_condition, double initial_nut,
                           NumericalFluxScheme flux_scheme, GradientScheme gradient_scheme, double exact_riemann_tol,
                           int exact_riemann_max_iter, const SAModelConstants& sa_constants = SAModelConstants{}) {
        std::vector<fv_bc_t> bcs(boundary_conditions.size());
        for (size_t i = 0; i < bcs.size(); ++i) {
            const NSBoundaryCondition& b = boundary_conditions[i].ns;
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
            bcs[i].nut = boundary_conditions[i].farfield_nut;
        }
        fv_options_t opt;
        fv_options_default(&opt);
        opt.viscous = 2;
        opt.gas_constant = gas_constant;
        opt.mu = mu;
        opt.prandtl = prandtl;
        opt.prandtl_t = prandtl_t;
        opt.initial_nut = initial_nut;
        const double sa[9] = {sa_constants.cb1, sa_constants.cb2, sa_constants.sigma, sa_constants.kappa,
                              sa_constants.cw2, sa_constants.cw3, sa_constants.cv1, sa_constants.cv2,
                              sa_constants.cv3};
        for (int i = 0; i < 9; ++i) opt.sa[i] = sa[i];
        opt.flux = (int32_t)flux_scheme;
        opt.gradient = gradient_scheme == GradientScheme::GreenGauss ? FV_GRAD_GG : FV_GRAD_LSQ;
        opt.exact_tol = exact_riemann_tol;
        opt.exact_max_iter = exact_riemann_max_iter;
        s_.create(input_mesh, bcs, gamma, cfl, initial_condition, opt);
        nut_.resize(input_mesh.cells.size());
    }

    void step() { s_.steps(1); }
    void run(int total_steps) {
        s_.steps(total_steps);
        std::cout << "Simulation completed across " << total_steps << " steps.\n";
    }
    const std::vector<EulerState>& field() const { return s_.field(); }
    const std::vector<double>& nut_field() const {
        fvgb300_shim::check(fv_get_nut(s_.handle(), nut_.data()));
        return nut_;
    }
    double gas_gamma() const { return s_.gamma(); }
    const EulerResidualNorms& residual() const { return s_.residual(); }
    double nut_residual() const {
        double r = 0.0;
        fvgb300_shim::check(fv_get_nut_residual(s_.handle(), &r));
        return r;
    }
    void set_field(const std::vector<EulerState>& new_U, const std::vector<double>& new_nut) {
        s_.set_field(new_U);
        fvgb300_shim::check(fv_set_nut(s_.handle(), new_nut.data()));
    }
    void set_field(const std::vector<EulerState>& new_U) { s_.set_field(new_U); }
    void set_cfl(double new_cfl) { s_.set_cfl(new_cfl); }

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
    mutable std::vector<double> nut_;
};

#endif  // RANSTURBULENCESASOLVER_H_INCLUDED
