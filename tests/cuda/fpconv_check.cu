// Checks the integer-pipe float<->double conversions of fpconv.cuh against
// the hardware conversions, bit for bit (NaN: NaN-ness only):
//   f2d: every one of the 2^32 float bit patterns;
//   d2f: 2^31 pseudo-random double bit patterns (all exponents), plus
//        patterns concentrated on the float normal / subnormal / overflow
//        boundaries and exact rounding ties.
// Prints "f2d_mismatch N d2f_mismatch M" and the first mismatching inputs.
#include <cstdio>
#include <cstdint>

#include "fpconv.cuh"

__device__ unsigned long long g_bad[2];
__device__ unsigned long long g_first[2][4];

__device__ __forceinline__ uint64_t mix(uint64_t x) {
    x ^= x >> 33; x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return x;
}

__device__ void record(int k, unsigned long long in) {
    const unsigned long long n = atomicAdd(&g_bad[k], 1ull);
    if (n < 4) g_first[k][n] = in;
}

__global__ void check_f2d(uint64_t start, uint64_t count) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t b = (uint32_t)(start + i);
        const float x = __uint_as_float(b);
        const double mine = fvconv::f2d(x), hw = (double)x;
        const bool ok = (mine != mine && hw != hw) || __double_as_longlong(mine) == __double_as_longlong(hw);
        if (!ok) record(0, b);
    }
}

__global__ void check_d2f(uint64_t count, uint64_t seed) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count; i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t b = mix(i * 0x9e3779b97f4a7c15ull + seed);
        const uint32_t kind = (uint32_t)(i & 7u);
        if (kind >= 4) {
            // exponent near the float boundaries: normal min (897), subnormal
            // range (871..896), max (1150/1151)
            const uint64_t r = mix(b);
            const uint32_t lo_e[4] = {865u, 890u, 1140u, 1015u};
            const uint64_t e = lo_e[kind - 4] + (r % 16u);
            b = (b & 0x800fffffffffffffull) | (e << 52);
            if ((r >> 20) & 1u) b = (b & ~0x1fffffffull) | 0x10000000ull;  // exact tie in the normal range
            if ((r >> 21) & 1u) b |= 0x1fffffffull;                        // just below a carry
        }
        const double x = __longlong_as_double((long long)b);
        const float mine = fvconv::d2f(x), hw = __double2float_rn(x);
        const bool ok = (mine != mine && hw != hw) || __float_as_uint(mine) == __float_as_uint(hw);
        if (!ok) record(1, b);
    }
}

int main() {
    unsigned long long zero[2] = {0, 0};
    cudaMemcpyToSymbol(g_bad, zero, sizeof(zero));
    // all 2^32 floats in four launches
    for (int q = 0; q < 4; ++q) check_f2d<<<152 * 8, 256>>>((uint64_t)q << 30, 1ull << 30);
    check_d2f<<<152 * 8, 256>>>(1ull << 31, 12345);
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        printf("cuda_error %s\n", cudaGetErrorString(e));
        return 2;
    }
    unsigned long long bad[2], first[2][4];
    cudaMemcpyFromSymbol(bad, g_bad, sizeof(bad));
    cudaMemcpyFromSymbol(first, g_first, sizeof(first));
    printf("f2d_mismatch %llu d2f_mismatch %llu\n", bad[0], bad[1]);
    for (int k = 0; k < 2; ++k)
        for (unsigned long long j = 0; j < bad[k] && j < 4; ++j) printf("first_%s 0x%llx\n", k ? "d2f" : "f2d", first[k][j]);
    return bad[0] || bad[1] ? 1 : 0;
}
