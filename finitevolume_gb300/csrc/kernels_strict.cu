// The same kernels compiled with --fmad=false: IEEE op-for-op identical to
// the reference built without -ffast-math (bit-identical fields for the
// Rusanov and HLLC fluxes).
#define FV_KNS strict
#define FV_STRICT_ORDER
#define FV_DEFINE_O1_LAUNCH
#include "euler_o1.cuh"
#include "euler_o1p.cuh"
