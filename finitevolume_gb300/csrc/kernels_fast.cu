// Kernels compiled with FMA contraction (the default production build).
#define FV_KNS fast
#define FV_DEFINE_O1_LAUNCH
#include "euler_o1.cuh"
#include "euler_o1p.cuh"
