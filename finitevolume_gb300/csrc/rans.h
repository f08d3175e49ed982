// Spalart-Allmaras RANS step arguments (see rans.cu).
#pragma once

#include "ns.h"

namespace fvgb {

struct RansArgs {
    NSArgs ns;             // mean flow; ns.prim holds u, v, T, nu-tilde
    const int* cf_off;
    const int* cf;
    const double* vol;
    const double2* cxy;
    double* nut;           // [N] nu-tilde
    double* nut_ff;        // [F] nu-tilde face flux
    double2* nu;           // [N] molecular and eddy kinematic viscosity
    double2* grad;         // [4N] gradients of u, v, T, nu-tilde
    double* walld;         // [N] distance to the nearest no-slip wall
    double* partials;      // [5 * cell blocks]
    double* hist;          // [hist_cap * 4] mean-flow norms
    double* nut_hist;      // [hist_cap] nu-tilde norms
    double* nut_norm;      // [1] last nu-tilde norm
    int hist_cap;
    double farfield_nut[kMaxPatches];
    double sa[9];          // cb1, cb2, sigma, kappa, cw2, cw3, cv1, cv2, cv3
    double cw3_6;          // cw3^6, formed on the host by std::pow
    double cp, prandtl, prandtl_t;
    double k_lam;          // cp * mu / Pr, formed on the host in that order
};

void rans_wall_distance(const RansArgs& a, const double4_32a* seg, int n_seg, cudaStream_t s);
// Strict and _fast (FMA-contracted) builds, as for the NS kernels.
void rans_launch_step(const RansArgs& a, cudaStream_t s);
void rans_launch_wall(const RansArgs& a, const int* faces, int n, double2* out, cudaStream_t s);
void rans_launch_step_fast(const RansArgs& a, cudaStream_t s);
void rans_launch_wall_fast(const RansArgs& a, const int* faces, int n, double2* out, cudaStream_t s);

}  // namespace fvgb
