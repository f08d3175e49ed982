// Checks fvconv::rcp_nr3 (fpconv.cuh) against the IEEE round-to-nearest
// reciprocal __drcp_rn on pseudo-random doubles over every exponent (the
// out-of-range inputs take the division and must match exactly) plus the
// seed's worst cases (fractions just below a power of two) and special
// values.  Prints "rcp_checked N rcp_inexact K rcp_max_ulp U rcp_bad B";
// an input whose result is more than one ulp off, or any mismatch in the
// fallback range, counts as bad.
#include <cstdio>
#include <cstdint>

#include "fpconv.cuh"

__device__ unsigned long long g_count[3];  // inexact, bad, max ulp
__device__ unsigned long long g_first_bad;

__device__ __forceinline__ uint64_t mix(uint64_t x) {
    x ^= x >> 33; x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return x;
}

__global__ void check_rcp(uint64_t count, uint64_t seed) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count; i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t b = mix(i * 0x9e3779b97f4a7c15ull + seed);
        const uint32_t kind = (uint32_t)(i & 7u);
        if (kind >= 2) {
            // the solver's range: exponents of 2^-40 .. 2^40
            const uint64_t e = 983u + (mix(b) % 81u);
            b = (b & 0x800fffffffffffffull) | (e << 52);
            if (kind == 7) b |= 0x000fffffe0000000ull;  // fraction just below 2: largest truncation
        }
        const double x = __longlong_as_double((long long)b);
        const double mine = fvconv::rcp_nr3(x), ref = __drcp_rn(x);
        const long long d = __double_as_longlong(mine) - __double_as_longlong(ref);
        const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
        const bool fallback = e - 898u > 250u;
        bool bad;
        if (mine != mine || ref != ref) bad = !(mine != mine && ref != ref);
        else bad = (fallback && d != 0) || d > 1 || d < -1;
        if (d != 0) {
            atomicAdd(&g_count[0], 1ull);
            atomicMax(&g_count[2], (unsigned long long)(d < 0 ? -d : d));
        }
        if (bad && atomicAdd(&g_count[1], 1ull) == 0) g_first_bad = b;
    }
}

int main() {
    unsigned long long zero[3] = {0, 0, 0};
    cudaMemcpyToSymbol(g_count, zero, sizeof(zero));
    const uint64_t n = 1ull << 30;
    check_rcp<<<152 * 8, 256>>>(n, 777);
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        printf("cuda_error %s\n", cudaGetErrorString(e));
        return 2;
    }
    unsigned long long c[3], first = 0;
    cudaMemcpyFromSymbol(c, g_count, sizeof(c));
    cudaMemcpyFromSymbol(&first, g_first_bad, sizeof(first));
    printf("rcp_checked %llu rcp_inexact %llu rcp_max_ulp %llu rcp_bad %llu\n", (unsigned long long)n, c[0], c[2], c[1]);
    if (c[1]) printf("first_bad 0x%llx\n", first);
    return c[1] ? 1 : 0;
}
