// First-order (piecewise-constant) explicit step: the reference's two-pass
// kernel (src/EulerFVMSolver.cpp:58-112, compute_dt :133-162) as two
// device passes.
//
//   face pass  one thread per face: ghost state, numerical flux times face
//              length, and the face's CFL time step (compute_dt's per-face
//              candidate; fused here because both read the same two states).
//              Global dt: warp/block min, one atomicMin per block on the bit
//              pattern of the (positive) double.  Local dt: stored per face.
//   cell pass  one thread per cell: signed gather of its faces' fluxes in
//              the reference's per-cell face order (owner subtracts,
//              neighbour adds), squared-residual sums, U += dt/vol * R.
//              Norm partials are reduced per block in a fixed tree order and
//              the last block to finish folds them in block order, so the
//              norms are bitwise reproducible run to run (no float atomics).
//
// Included by kernels_fast.cu and kernels_strict.cu with FV_KNS defined.
#pragma once

#include "physics.cuh"

namespace FV_KNS {

using fvgb::DevMesh;
using fvgb::O1Args;
using fvgb::StepCtl;

__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
// Warp sums of four values at once, transposed: the first exchange leaves
// each lane two partial sums (values 0,1 or 2,3, by lane bit 4), the second
// one (by lane bit 3), and three ordinary butterfly steps finish it.  Lane
// l returns the sum of value (l >> 3) & 3: 6 FP64 additions per lane
// instead of 20 for four separate warp_sum calls (the selects run on the
// integer pipe).  Deterministic; the addition order differs from warp_sum.
__device__ __forceinline__ double warp_sum4(double v0, double v1, double v2, double v3) {
    const int lane = threadIdx.x & 31;
    const bool b4 = lane & 16, b3 = lane & 8;
    const double k0 = b4 ? v2 : v0, k1 = b4 ? v3 : v1;
    const double a = k0 + __shfl_xor_sync(0xffffffffu, b4 ? v0 : v2, 16);
    const double b = k1 + __shfl_xor_sync(0xffffffffu, b4 ? v1 : v3, 16);
    double v = (b3 ? b : a) + __shfl_xor_sync(0xffffffffu, b3 ? a : b, 8);
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Per-face wave-speed estimate max(|Vn|+c) of EulerFVMSolver::compute_dt
// (src/EulerFVMSolver.cpp:140-150).
__device__ __forceinline__ double face_smax(const St& UL, const St& UR, bool interior, double nx, double ny,
                                            double g) {
    double uL = UL.ru / UL.r;
    double vL = UL.rv / UL.r;
    double VnL = uL * nx + vL * ny;
    double Smax = fabs(VnL) + sound_speed(UL, g);
    if (interior) {
        double uR = UR.ru / UR.r;
        double vR = UR.rv / UR.r;
        double VnR = uR * nx + vR * ny;
        Smax = rmax(Smax, fabs(VnR) + sound_speed(UR, g));
    }
    return Smax;
}

template <int FLUX, bool LOCAL>
__global__ void __launch_bounds__(fvgb::kFaceBlock) k_face_o1(const O1Args a) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    const double g = a.gamma;
    double cand = DBL_MAX;
    if (f < a.m.n_faces) {
        const int L = a.m.fl[f], R = a.m.fr[f];
        const double4_32a geo = a.m.fgeom[f];
        const St UL = ld_state(a.U, L);
        const St UR = (R >= 0) ? ld_state(a.U, R) : ghost_state(a.bc, a.m.fpatch[f], UL, geo.x, geo.y, g);
        const St F = num_flux<FLUX>(UL, UR, geo.x, geo.y, g, a.exact_tol, a.exact_max_iter);
        st_state(a.ff, f, geo.z * F);
        const double Smax = face_smax(UL, UR, R >= 0, geo.x, geo.y, g);
        // Global: the face's CFL step cfl * length / Smax (compute_dt).
        // Local: the face's lambda * A for dt_i = cfl V_i / sum_f lambda_f A_f.
        if (LOCAL) a.dtf[f] = Smax * geo.z;
        else cand = a.ctl->cfl * geo.w / Smax;
    }
    if (!LOCAL) {
        __shared__ double smin[fvgb::kFaceBlock / 32];
        cand = warp_min(cand);
        if ((threadIdx.x & 31) == 0) smin[threadIdx.x >> 5] = cand;
        __syncthreads();
        if (threadIdx.x == 0) {
            double v = smin[0];
            for (int w = 1; w < fvgb::kFaceBlock / 32; ++w) v = fmin(v, smin[w]);
            atomicMin(&a.ctl->dt_bits, (unsigned long long)__double_as_longlong(v));
        }
    }
}

// Fold one block's four squared-residual sums into partials[blockIdx];
// the last block to arrive folds all partials (fixed order) into the
// norms, records the history row, and re-arms the control block.
__device__ __forceinline__ void finish_norms(double s0, double s1, double s2, double s3, StepCtl* ctl,
                                             double* partials, double* hist, int hist_cap) {
    // up to 512 threads per block (launch shapes are tunable)
    __shared__ double red[16][4];
    __shared__ bool last;
    const int nw = blockDim.x >> 5;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const double ws = warp_sum4(s0, s1, s2, s3);
    if ((lane & 7) == 0) red[w][lane >> 3] = ws;
    __syncthreads();
    if (threadIdx.x < 4) {
        double v = 0.0;
        for (int i = 0; i < nw; ++i) v += red[i][threadIdx.x];
        partials[blockIdx.x * 4 + threadIdx.x] = v;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = (atomicAdd(&ctl->done_blocks, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!last) return;
    __threadfence();
    double t[4] = {0.0, 0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
        const volatile double* p = partials + 4 * b;
        t[0] += p[0]; t[1] += p[1]; t[2] += p[2]; t[3] += p[3];
    }
    const double ts = warp_sum4(t[0], t[1], t[2], t[3]);
    __syncthreads();
    if ((lane & 7) == 0) red[w][lane >> 3] = ts;
    __syncthreads();
    if (threadIdx.x == 0) {
        double n[4];
        int bad = 0;
        for (int k = 0; k < 4; ++k) {
            double v = 0.0;
            for (int i = 0; i < nw; ++i) v += red[i][k];
            n[k] = sqrt(v);
            if (!isfinite(n[k])) bad = 1;
            ctl->norms[k] = n[k];
        }
        const int row = ctl->step % hist_cap;
        for (int k = 0; k < 4; ++k) hist[row * 4 + k] = n[k];
        if (bad) ctl->nonfinite = 1;
        ctl->step += 1;
        ctl->done_blocks = 0u;
        ctl->dt_bits = (unsigned long long)__double_as_longlong(DBL_MAX);
    }
}

template <bool LOCAL>
__global__ void __launch_bounds__(fvgb::kCellBlock) k_cell_o1(const O1Args a) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    if (c < a.m.n_cells) {
        double dt = LOCAL ? 0.0 : __longlong_as_double((long long)a.ctl->dt_bits);
        St R = st_make(0.0, 0.0, 0.0, 0.0);
        const int e0 = a.m.cf_off[c], e1 = a.m.cf_off[c + 1];
        for (int e = e0; e < e1; ++e) {
            const int ent = a.m.cf[e];
            const int f = ent >> 1;
            R += flip_if(ld_state(a.ff, f), ent);
            if (LOCAL) dt += a.dtf[f];
        }
        if (LOCAL) dt = a.ctl->cfl * a.m.vol[c] / dt;
        s0 = R.r * R.r; s1 = R.ru * R.ru; s2 = R.rv * R.rv; s3 = R.E * R.E;
        const St u = ld_state(a.U, c);
        st_state(a.U, c, u + (dt / a.m.vol[c]) * R);
    }
    finish_norms(s0, s1, s2, s3, a.ctl, a.partials, a.hist, a.hist_cap);
}

template <int FLUX>
static void launch_flux(const O1Args& a, int part, cudaStream_t s) {
    const int fb = (a.m.n_faces + fvgb::kFaceBlock - 1) / fvgb::kFaceBlock;
    const int cb = (a.m.n_cells + fvgb::kCellBlock - 1) / fvgb::kCellBlock;
    if (part == 0) {
        if (a.local_dt) k_face_o1<FLUX, true><<<fb, fvgb::kFaceBlock, 0, s>>>(a);
        else k_face_o1<FLUX, false><<<fb, fvgb::kFaceBlock, 0, s>>>(a);
    } else {
        if (a.local_dt) k_cell_o1<true><<<cb, fvgb::kCellBlock, 0, s>>>(a);
        else k_cell_o1<false><<<cb, fvgb::kCellBlock, 0, s>>>(a);
    }
}

}  // namespace FV_KNS

#ifdef FV_DEFINE_O1_LAUNCH
namespace fvgb {
namespace FV_KNS {
void launch_o1_part(const O1Args& a, int part, cudaStream_t s) {
    switch (a.flux) {
        case 1: ::FV_KNS::launch_flux<1>(a, part, s); break;
        case 2: ::FV_KNS::launch_flux<2>(a, part, s); break;
        default: ::FV_KNS::launch_flux<0>(a, part, s); break;
    }
}
}  // namespace FV_KNS
}  // namespace fvgb
#endif  // FV_DEFINE_O1_LAUNCH
