// Navier-Stokes step arguments (see ns.cu).
#pragma once

#include "gradients.cuh"
#include "types.h"

namespace fvgb {

struct NSArgs {
    GradDev g;                 // gradient geometry (also n_cells, n_faces, fr)
    const int* fl;
    const int* fpatch;
    const double4_32a* fgeom;  // nx, ny, length, CFL length
    St* U;
    St* ff;
    double4_32a* prim;         // u, v, T, unused
    double2* grad;             // 3 per cell: grad u, grad v, grad T
    StepCtl* ctl;
    BCTable bc;
    double gamma, gas_constant, mu, kcond, exact_tol;
    int exact_max_iter, flux;
};

// Strict (no FMA contraction, reference evaluation order) and _fast
// (contracted) builds of the same kernels.
void ns_launch_step(const NSArgs& a, const O1Args& cell, cudaStream_t s);
void ns_launch_wall(const NSArgs& a, const int* faces, int n, double2* out, cudaStream_t s);
void ns_launch_step_fast(const NSArgs& a, const O1Args& cell, cudaStream_t s);
void ns_launch_wall_fast(const NSArgs& a, const int* faces, int n, double2* out, cudaStream_t s);

}  // namespace fvgb
