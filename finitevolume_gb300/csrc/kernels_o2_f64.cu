// Second-order kernels instantiated for double flux/gradient arithmetic.
#define FV_KNS fast
#include "euler_o2.cuh"

namespace {
using R = double;
using namespace ::fast;
using fvgb::O2Args;
using fvgb::O2Config;

template <int GRAD, int LIM>
void grad(const O2Args& a, int bs, cudaStream_t s) {
    const int cb = (a.m.n_cells + bs - 1) / bs;
    k_grad<R, GRAD, LIM><<<cb, bs, 0, s>>>(a);
}

template <int FLUX, int ORDER>
void face(const O2Args& a, int dt, int bs, cudaStream_t s) {
    const int fb = (a.m.n_faces + bs - 1) / bs;
    if (dt == 1) k_face<R, FLUX, ORDER, 1><<<fb, bs, 0, s>>>(a);
    else if (dt == 2) k_face<R, FLUX, ORDER, 2><<<fb, bs, 0, s>>>(a);
    else k_face<R, FLUX, ORDER, 0><<<fb, bs, 0, s>>>(a);
}

template <int ST, int NST>
void update(const O2Args& a, int local, int bs, cudaStream_t s) {
    const int cb = (a.m.n_cells + bs - 1) / bs;
    if (local) k_update<R, ST, NST, 2><<<cb, bs, 0, s>>>(a);
    else k_update<R, ST, NST, 1><<<cb, bs, 0, s>>>(a);
}
}  // namespace

namespace fvgb {
namespace o2 {

void launch_batch_norms(const O2Args& a, int n_inst, const int* inst_off, double* inst_norms, int* inst_iter,
                        int* active, double tol, cudaStream_t s) {
    ::fast::k_batch_norms<<<n_inst, 256, 0, s>>>(a, inst_off, inst_norms, inst_iter, active, tol);
}

void launch_prim_f64(const O2Args& a, cudaStream_t s) {
    const int cb = (a.m.n_cells + kCellBlock - 1) / kCellBlock;
    ::fast::k_prim<R><<<cb, kCellBlock, 0, s>>>(a);
}

void launch_residual_f64(const O2Args& a, cudaStream_t s) {
    const int cb = (a.m.n_cells + kCellBlock - 1) / kCellBlock;
    ::fast::k_residual<R><<<cb, kCellBlock, 0, s>>>(a);
}

void launch_part_f64(const O2Args& a, const O2Config& c, int stage, int part, cudaStream_t s) {
    if (part == 0) {
        if (c.order != 2) return;
        switch (c.gradient * 3 + c.limiter) {
            case 0: grad<0, 0>(a, c.blk_grad, s); break;
            case 1: grad<0, 1>(a, c.blk_grad, s); break;
            case 2: grad<0, 2>(a, c.blk_grad, s); break;
            case 3: grad<1, 0>(a, c.blk_grad, s); break;
            case 4: grad<1, 1>(a, c.blk_grad, s); break;
            default: grad<1, 2>(a, c.blk_grad, s); break;
        }
    } else if (part == 1) {
        const int dt = stage == 0 ? (c.local_dt ? 2 : 1) : 0;
        switch (c.flux * 2 + (c.order == 2 ? 1 : 0)) {
            case 0: face<0, 1>(a, dt, c.blk_face, s); break;
            case 1: face<0, 2>(a, dt, c.blk_face, s); break;
            case 2: face<1, 1>(a, dt, c.blk_face, s); break;
            case 3: face<1, 2>(a, dt, c.blk_face, s); break;
            case 4: face<2, 1>(a, dt, c.blk_face, s); break;
            default: face<2, 2>(a, dt, c.blk_face, s); break;
        }
    } else {
        if (c.stages == 1) update<0, 1>(a, c.local_dt, c.blk_cell, s);
        else if (stage == 0) update<0, 3>(a, c.local_dt, c.blk_cell, s);
        else if (stage == 1) update<1, 3>(a, c.local_dt, c.blk_cell, s);
        else update<2, 3>(a, c.local_dt, c.blk_cell, s);
    }
}

}  // namespace o2
}  // namespace fvgb
