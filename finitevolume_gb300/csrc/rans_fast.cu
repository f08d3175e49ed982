// The RANS-SA kernels with FMA contraction (see rans.cu).
#define FV_NS_FAST
#include "rans.cu"
