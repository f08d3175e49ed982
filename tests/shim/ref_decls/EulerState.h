// Stand-in for the reference's include/EulerState.h (the conserved-state
// struct, include/EulerState.h:15-20) where the reference is not installed.
#ifndef EULERSTATE_H_INCLUDED
#define EULERSTATE_H_INCLUDED
struct EulerState {
    double rho = 0.0;
    double rho_u = 0.0;
    double rho_v = 0.0;
    double E = 0.0;
};
#endif
