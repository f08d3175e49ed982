// Compile-only check of the drop-in headers' class surface: every member
// the reference's solver classes expose to a driver, called with the
// reference's argument types (include/EulerFVMSolver.h:107-160,
// include/NavierStokesFVMSolver.h:118-218,
// include/RANSTurbulenceSASolver.h, include/UnstructuredFVMSolver.h:34-73).
// Never run; tests/test_shim.py compiles it with -fsyntax-only.
#include <vector>

#include "EulerFVMSolver.h"
#include "NavierStokesFVMSolver.h"
#include "RANSTurbulenceSASolver.h"
#include "UnstructuredFVMSolver.h"

double use_euler(const UnstructuredMesh& mesh, const std::vector<EulerBoundaryCondition>& bcs,
                 const EulerInitialCondition& ic) {
    EulerFVMSolver s(mesh, bcs, 1.4, 0.5, ic, NumericalFluxScheme::HLLC, 1e-6, 20);
    s.step();
    s.run(10);
    const std::vector<EulerState>& U = s.field();
    const EulerResidualNorms& r = s.residual();
    s.set_field(U);
    s.set_cfl(0.8);
    return s.gas_gamma() + r.rho + r.rho_u + r.rho_v + r.E;
}

double use_ns(const UnstructuredMesh& mesh, const std::vector<NSBoundaryCondition>& bcs,
              const EulerInitialCondition& ic) {
    NavierStokesFVMSolver s(mesh, bcs, 1.4, 287.0, 1.8e-5, 0.72, 0.5, ic, NumericalFluxScheme::Rusanov,
                            GradientScheme::GreenGauss, 1e-6, 20);
    s.step();
    s.run(10);
    s.set_field(s.field());
    s.set_cfl(0.4);
    return s.gas_gamma() + s.residual().rho;
}

double use_rans(const UnstructuredMesh& mesh, const std::vector<RANSBoundaryConditionSA>& bcs,
                const EulerInitialCondition& ic) {
    RANSTurbulenceSASolver s(mesh, bcs, 1.4, 287.0, 1.8e-5, 0.72, 0.9, 0.5, ic, 3.0 * 1.8e-5,
                             NumericalFluxScheme::HLLC, GradientScheme::LeastSquares, 1e-6, 20);
    s.step();
    s.run(10);
    s.set_field(s.field(), s.nut_field());
    s.set_field(s.field());
    return s.residual().rho + s.nut_field()[0];
}

double use_diffusion(const UnstructuredMesh& mesh) {
    UnstructuredFVMSolver s(mesh, 1.0, 1e-3, 1.0, 0.2);
    s.step();
    s.run(10);
    std::vector<double> phi = s.field();
    s.set_field(phi);
    return s.residual_norm();
}
