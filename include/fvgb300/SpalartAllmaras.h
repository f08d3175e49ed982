// Drop-in replacement for the reference's include/SpalartAllmaras.h: the
// SA-noft2 model constants and the per-cell model functions, for callers
// that use them outside the solver.  The solver itself evaluates the model
// on the GPU (finitevolume_gb300/csrc/rans.cu).
#ifndef SPALARTALLMARAS_H_INCLUDED
#define SPALARTALLMARAS_H_INCLUDED

#include <algorithm>
#include <cmath>

#include "GradientReconstruction.h"  // Gradient2

// include/SpalartAllmaras.h:13-23 (same members, same defaults)
struct SAModelConstants {
    double cb1 = 0.1355;
    double cb2 = 0.622;
    double sigma = 2.0 / 3.0;
    double kappa = 0.41;
    double cw2 = 0.3;
    double cw3 = 2.0;
    double cv1 = 7.1;
    double cv2 = 0.7;
    double cv3 = 0.9;
};

struct SASourceTerms {
    double production = 0.0;
    double destruction = 0.0;
    double cross_diffusion = 0.0;
};

// cw1 = cb1 / kappa^2 + (1 + cb2) / sigma
inline double sa_cw1(const SAModelConstants& c) { return c.cb1 / (c.kappa * c.kappa) + (1.0 + c.cb2) / c.sigma; }

// fv1 = chi^3 / (chi^3 + cv1^3), chi = nut / nu; 0 for nut <= 0
inline double sa_fv1(double nut, double nu, const SAModelConstants& c = SAModelConstants{}) {
    if (nut <= 0.0) return 0.0;
    const double chi = nut / nu;
    const double chi3 = chi * chi * chi;
    return chi3 / (chi3 + c.cv1 * c.cv1 * c.cv1);
}

inline double sa_eddy_viscosity(double nut, double nu, const SAModelConstants& c = SAModelConstants{}) {
    return nut * sa_fv1(nut, nu, c);
}

// Production cb1 S~ nut (S~ with the negative-S~ modification of Allmaras,
// Johnson and Spalart 2012), destruction cw1 fw (nut/d)^2 (r clipped at 10),
// cross diffusion (cb2/sigma) |grad nut|^2.
inline SASourceTerms compute_sa_source_terms(double nut, double nu, double omega, double wall_distance,
                                             const Gradient2& grad_nut, const SAModelConstants& c = SAModelConstants{}) {
    SASourceTerms t;
    const double chi = nut > 0.0 ? nut / nu : 0.0;
    const double fv1 = sa_fv1(nut, nu, c);
    const double fv2 = 1.0 - chi / (1.0 + chi * fv1);
    const double d2 = wall_distance * wall_distance;
    const double s_bar = (nut / (c.kappa * c.kappa * d2)) * fv2;
    const double s_tilde = s_bar >= -c.cv2 * omega
                               ? omega + s_bar
                               : omega + omega * (c.cv2 * c.cv2 * omega + c.cv3 * s_bar) /
                                             ((c.cv3 - 2.0 * c.cv2) * omega - s_bar);
    t.production = c.cb1 * s_tilde * nut;
    if (nut > 0.0) {
        const double r = std::min(nut / (std::max(s_tilde, 1e-10) * c.kappa * c.kappa * d2), 10.0);
        const double g = r + c.cw2 * (std::pow(r, 6.0) - r);
        const double fw = g * std::pow((1.0 + std::pow(c.cw3, 6.0)) / (std::pow(g, 6.0) + std::pow(c.cw3, 6.0)), 1.0 / 6.0);
        const double q = nut / wall_distance;
        t.destruction = sa_cw1(c) * fw * q * q;
    }
    t.cross_diffusion = (c.cb2 / c.sigma) * (grad_nut.dphidx * grad_nut.dphidx + grad_nut.dphidy * grad_nut.dphidy);
    return t;
}

#endif  // SPALARTALLMARAS_H_INCLUDED
