// The NS kernels with FMA contraction (see ns.cu).
#define FV_NS_FAST
#include "ns.cu"
