// Drop-in replacement for the reference's include/UnstructuredFVMSolver.h
// (include/UnstructuredFVMSolver.h:21-92) backed by the GB300 library.  As
// in the reference, each boundary patch's BoundaryType and value are read
// from mesh.patches at construction.
#ifndef UNSTRUCTUREDFVMSOLVER_H
#define UNSTRUCTUREDFVMSOLVER_H

#include <cassert>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "EulerFVMSolver.h"  // fvgb300_shim::make_mesh / check
#include "UnstructuredMesh.h"

class UnstructuredFVMSolver {
public:
    UnstructuredFVMSolver(const UnstructuredMesh& input_mesh, double alpha, double dt, double initial_value,
                          double initial_radius) {
        std::vector<int32_t> type(input_mesh.patches.size());
        std::vector<double> value(input_mesh.patches.size());
        for (size_t p = 0; p < input_mesh.patches.size(); ++p) {
            type[p] = input_mesh.patches[p].type == BoundaryType::Neumann ? 1 : 0;
            value[p] = input_mesh.patches[p].value;
        }
        fv_mesh_t m = fvgb300_shim::make_mesh(input_mesh);
        int rc = fv_diffusion_create(m, alpha, dt, initial_value, initial_radius, type.data(), value.data(), &h_);
        fv_mesh_destroy(m);
        fvgb300_shim::check(rc);
        phi_.resize(input_mesh.cells.size());
    }
    UnstructuredFVMSolver(const UnstructuredFVMSolver&) = delete;
    UnstructuredFVMSolver& operator=(const UnstructuredFVMSolver&) = delete;
    ~UnstructuredFVMSolver() {
        if (h_) fv_diffusion_destroy(h_);
    }

    void step() { advance(1); }
    void run(int total_steps) {
        advance(total_steps);
        std::cout << "Simulation completed across " << total_steps << " steps.\n";
    }
    const std::vector<double>& field() const {
        if (!fresh_) {
            fvgb300_shim::check(fv_diffusion_get_field(h_, phi_.data()));
            fresh_ = true;
        }
        return phi_;
    }
    double residual_norm() const {
        double r = 0.0;
        fvgb300_shim::check(fv_diffusion_residual(h_, &r));
        return r;
    }
    void set_field(const std::vector<double>& new_phi) {
        assert(new_phi.size() == phi_.size());
        fvgb300_shim::check(fv_diffusion_set_field(h_, new_phi.data()));
        phi_ = new_phi;
        fresh_ = true;
    }

private:
    void advance(int n) {
        while (n > 0) {
            const int k = n < 65536 ? n : 65536;
            const int rc = fv_diffusion_step(h_, k, nullptr);
            if (rc != FV_OK && rc != FV_ERR_NONFINITE) fvgb300_shim::check(rc);
            n -= k;
        }
        fresh_ = false;
    }
    fv_diffusion_t h_ = nullptr;
    mutable std::vector<double> phi_;
    mutable bool fresh_ = false;
};

#endif  // UNSTRUCTUREDFVMSOLVER_H
