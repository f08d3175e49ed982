// Kernels compiled with FMA contraction (the default production build).
#define FV_KNS fast
#include "euler_o1.cuh"
