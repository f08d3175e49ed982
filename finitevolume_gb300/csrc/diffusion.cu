// Scalar diffusion solver: UnstructuredFVMSolver (include/UnstructuredFVMSolver.h:21-92,
// src/UnstructuredFVMSolver.cpp:44-129) on the device.
//
//   face pass  flux = -alpha (phi_R - phi_L) / d_LR * length on internal
//              faces; Neumann: value * length; Dirichlet: the one-sided
//              difference to the face midpoint (boundary_flux, :113-129).
//              The centroid distances are mesh geometry, computed once on
//              the host with the reference's formula.
//   cell pass  signed gather in the reference's per-cell face order, the
//              squared-residual sum and phi += dt / V * r.
// Expressions keep the reference's evaluation order; built without FMA
// contraction (strict) the field is bit-identical to the reference.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "../../include/fv_gb300.h"
#include "errors.h"
#include "mesh_host.h"
#include "types.h"

namespace fvgb {
namespace {

struct DiffArgs {
    int n_cells, n_faces;
    const int* fl;
    const int* fr;
    const int* fpatch;
    const double* farea;
    const double* fdist;   // internal: centroid-centroid; boundary: centroid-midpoint
    const int* cf_off;
    const int* cf;
    const double* vol;
    double* phi;
    double* ff;
    double* partials;
    double* hist;
    int hist_cap;
    StepCtl* ctl;
    double alpha, dt;
    int ptype[kMaxPatches];
    double pval[kMaxPatches];
};

__device__ __forceinline__ double flip1(double x, int neg) {
    return __longlong_as_double(__double_as_longlong(x) ^ ((unsigned long long)(neg & 1) << 63));
}

__global__ void __launch_bounds__(kFaceBlock) k_diff_face(const DiffArgs a) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= a.n_faces) return;
    const double phiL = a.phi[a.fl[f]];
    const int R = a.fr[f];
    double flux;
    if (R >= 0) {
        const double gn = (a.phi[R] - phiL) / a.fdist[f];
        flux = -a.alpha * gn * a.farea[f];
    } else {
        const int p = a.fpatch[f];
        if (a.ptype[p] == 1) {
            flux = a.pval[p] * a.farea[f];
        } else {
            const double gn = (a.pval[p] - phiL) / a.fdist[f];
            flux = -a.alpha * gn * a.farea[f];
        }
    }
    a.ff[f] = flux;
}

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(kCellBlock) k_diff_cell(const DiffArgs a) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    double s = 0.0;
    if (c < a.n_cells) {
        double r = 0.0;
        for (int e = a.cf_off[c]; e < a.cf_off[c + 1]; ++e) {
            const int ent = a.cf[e];
            r += flip1(a.ff[ent >> 1], ent);
        }
        s = r * r;
        a.phi[c] += (a.dt / a.vol[c]) * r;
    }
    __shared__ double red[kCellBlock / 32];
    __shared__ bool last;
    s = wsum(s);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = 0.0;
        for (int i = 0; i < kCellBlock / 32; ++i) v += red[i];
        a.partials[blockIdx.x] = v;
        __threadfence();
        last = (atomicAdd(&a.ctl->done_blocks, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    __threadfence();
    double t = 0.0;
    for (int b = 0; b < (int)gridDim.x; ++b) t += ((volatile double*)a.partials)[b];
    const double n = sqrt(t);
    a.ctl->norms[0] = n;
    a.hist[a.ctl->step % a.hist_cap] = n;
    if (!isfinite(n)) a.ctl->nonfinite = 1;
    a.ctl->step += 1;
    a.ctl->done_blocks = 0u;
}

__global__ void k_diff_scatter(const double* __restrict__ phi, double* __restrict__ out, const int* __restrict__ perm,
                               int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[perm[i]] = phi[i];
}
__global__ void k_diff_gather(const double* __restrict__ in, double* __restrict__ phi, const int* __restrict__ perm,
                              int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) phi[i] = in[perm[i]];
}

}  // namespace

struct DiffSolver {
    DiffArgs a{};
    int N = 0, F = 0, nblk = 0;
    int* d_perm = nullptr;
    double* staging = nullptr;
    cudaStream_t stream = nullptr;
    std::vector<void*> owned;
    std::vector<cudaGraphExec_t> graph;  // one 16-step graph

    template <typename T>
    T* up(const std::vector<T>& v) {
        void* p = nullptr;
        FV_CUDA(cudaMalloc(&p, std::max<size_t>(v.size(), 1) * sizeof(T)));
        owned.push_back(p);
        if (!v.empty()) h2d_sync(p, v.data(), v.size() * sizeof(T));
        return static_cast<T*>(p);
    }
    template <typename T>
    T* alloc(size_t n) {
        void* p = nullptr;
        FV_CUDA(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)));
        owned.push_back(p);
        return static_cast<T*>(p);
    }
    ~DiffSolver() {
        for (auto g : graph) cudaGraphExecDestroy(g);
        for (void* p : owned) cudaFree(p);
        if (stream) cudaStreamDestroy(stream);
    }

    void launch() {
        k_diff_face<<<(F + kFaceBlock - 1) / kFaceBlock, kFaceBlock, 0, stream>>>(a);
        k_diff_cell<<<nblk, kCellBlock, 0, stream>>>(a);
    }
};

}  // namespace fvgb

struct fv_diffusion_s {
    fvgb::DiffSolver s;
};
struct fv_mesh_s;
namespace fvgb {
const HostMesh& host_mesh_of(const fv_mesh_s* m);
}

using fvgb::raise;

template <typename Fn>
static int dguard(Fn&& fn) {
    try {
        fn();
        return FV_OK;
    } catch (const fvgb::Error& e) {
        fvgb::set_last_error(e.msg);
        return e.code;
    } catch (const std::exception& e) {
        fvgb::set_last_error(e.what());
        return FV_ERR_BAD_ARG;
    }
}

extern "C" {

int fv_diffusion_create(fv_mesh_t mesh, double alpha, double dt, double initial_value, double initial_radius,
                        const int32_t* patch_type, const double* patch_value, fv_diffusion_t* out) {
    return dguard([&] {
        if (!mesh || !out) raise(FV_ERR_BAD_ARG, "null argument");
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) raise(FV_ERR_CUDA, "no CUDA device available");
        const fvgb::HostMesh& h = fvgb::host_mesh_of(mesh);
        if (h.n_patches > fvgb::kMaxPatches) raise(FV_ERR_UNSUPPORTED, "more than 32 boundary patches");
        if (h.n_patches > 0 && (!patch_type || !patch_value)) raise(FV_ERR_BAD_ARG, "null patch arrays");
        auto d = std::make_unique<fv_diffusion_s>();
        fvgb::DiffSolver& s = d->s;
        s.N = h.n_cells;
        s.F = h.n_faces;
        s.nblk = (s.N + fvgb::kCellBlock - 1) / fvgb::kCellBlock;
        FV_CUDA(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking));
        // Face distances with the reference's own formula
        // (src/UnstructuredFVMSolver.cpp:58-62, :122-125), device face order.
        std::vector<double> area(s.F), dist(s.F);
        for (int i = 0; i < s.F; ++i) {
            int f = h.fperm[i];
            area[i] = h.farea[f];
            double dx, dy;
            if (h.fr[f] >= 0) {
                dx = h.cx[h.fr[f]] - h.cx[h.fl[f]];
                dy = h.cy[h.fr[f]] - h.cy[h.fl[f]];
            } else {
                dx = h.fxm[f] - h.cx[h.fl[f]];
                dy = h.fym[f] - h.cy[h.fl[f]];
            }
            dist[i] = std::sqrt(dx * dx + dy * dy);
        }
        fvgb::DiffArgs& a = s.a;
        a.n_cells = s.N;
        a.n_faces = s.F;
        a.fl = s.up(h.d_fl);
        a.fr = s.up(h.d_fr);
        a.fpatch = s.up(h.d_fpatch);
        a.farea = s.up(area);
        a.fdist = s.up(dist);
        a.cf_off = s.up(h.d_cf_off);
        a.cf = s.up(h.d_cf);
        a.vol = s.up(h.d_vol);
        a.phi = s.alloc<double>(s.N);
        a.ff = s.alloc<double>(s.F);
        a.partials = s.alloc<double>(s.nblk);
        a.hist_cap = 1 << 16;
        a.hist = s.alloc<double>(a.hist_cap);
        a.ctl = s.alloc<fvgb::StepCtl>(1);
        FV_CUDA(cudaMemsetAsync(a.ctl, 0, sizeof(fvgb::StepCtl), s.stream));
        a.alpha = alpha;
        a.dt = dt;
        for (int p = 0; p < h.n_patches; ++p) {
            if (patch_type[p] != 0 && patch_type[p] != 1) raise(FV_ERR_BAD_ARG, "patch type must be 0 or 1");
            a.ptype[p] = patch_type[p];
            a.pval[p] = patch_value[p];
        }
        s.d_perm = s.up(h.perm);
        s.staging = s.alloc<double>(s.N);
        // Initial condition: phi = initial_value inside the disc about the
        // origin (src/UnstructuredFVMSolver.cpp:6-19).
        std::vector<double> phi0(s.N, 0.0);
        for (int c = 0; c < s.N; ++c)
            if (std::sqrt(h.cx[c] * h.cx[c] + h.cy[c] * h.cy[c]) < initial_radius) phi0[c] = initial_value;
        fvgb::h2d_sync(s.staging, phi0.data(), sizeof(double) * s.N, s.stream);
        fvgb::k_diff_gather<<<(s.N + 255) / 256, 256, 0, s.stream>>>(s.staging, a.phi, s.d_perm, s.N);
        FV_CUDA(cudaStreamSynchronize(s.stream));
        *out = d.release();
    });
}

int fv_diffusion_destroy(fv_diffusion_t d) {
    delete d;
    return FV_OK;
}

int fv_diffusion_step(fv_diffusion_t d, int32_t n, double* history) {
    return dguard([&] {
        if (!d || n < 0 || n > (1 << 16)) raise(FV_ERR_BAD_ARG, "bad argument (n must be 0..65536)");
        fvgb::DiffSolver& s = d->s;
        if (s.graph.empty()) {
            cudaGraph_t g;
            FV_CUDA(cudaStreamBeginCapture(s.stream, cudaStreamCaptureModeThreadLocal));
            for (int i = 0; i < 16; ++i) s.launch();
            FV_CUDA(cudaStreamEndCapture(s.stream, &g));
            cudaGraphExec_t ge;
            FV_CUDA(cudaGraphInstantiate(&ge, g, 0));
            cudaGraphDestroy(g);
            s.graph.push_back(ge);
        }
        for (int i = 0; i < n / 16; ++i) FV_CUDA(cudaGraphLaunch(s.graph[0], s.stream));
        for (int i = 0; i < n % 16; ++i) s.launch();
        FV_CUDA(cudaGetLastError());
        fvgb::StepCtl c;
        FV_CUDA(cudaMemcpyAsync(&c, s.a.ctl, sizeof(c), cudaMemcpyDeviceToHost, s.stream));
        FV_CUDA(cudaStreamSynchronize(s.stream));
        if (history && n > 0) {
            std::vector<double> all(s.a.hist_cap);
            FV_CUDA(cudaMemcpy(all.data(), s.a.hist, sizeof(double) * all.size(), cudaMemcpyDeviceToHost));
            for (int i = 0; i < n; ++i) history[i] = all[(c.step - n + i) % s.a.hist_cap];
        }
        if (c.nonfinite) raise(FV_ERR_NONFINITE, "non-finite residual norm");
    });
}

int fv_diffusion_get_field(fv_diffusion_t d, double* phi) {
    return dguard([&] {
        if (!d || !phi) raise(FV_ERR_BAD_ARG, "null argument");
        fvgb::DiffSolver& s = d->s;
        fvgb::k_diff_scatter<<<(s.N + 255) / 256, 256, 0, s.stream>>>(s.a.phi, s.staging, s.d_perm, s.N);
        FV_CUDA(cudaMemcpyAsync(phi, s.staging, sizeof(double) * s.N, cudaMemcpyDeviceToHost, s.stream));
        FV_CUDA(cudaStreamSynchronize(s.stream));
    });
}

int fv_diffusion_set_field(fv_diffusion_t d, const double* phi) {
    return dguard([&] {
        if (!d || !phi) raise(FV_ERR_BAD_ARG, "null argument");
        fvgb::DiffSolver& s = d->s;
        FV_CUDA(cudaMemcpyAsync(s.staging, phi, sizeof(double) * s.N, cudaMemcpyHostToDevice, s.stream));
        fvgb::k_diff_gather<<<(s.N + 255) / 256, 256, 0, s.stream>>>(s.staging, s.a.phi, s.d_perm, s.N);
        static const double z = 0.0;
        FV_CUDA(cudaMemcpyAsync(reinterpret_cast<char*>(s.a.ctl) + offsetof(fvgb::StepCtl, norms), &z, sizeof(z),
                                cudaMemcpyHostToDevice, s.stream));
        FV_CUDA(cudaStreamSynchronize(s.stream));
    });
}

int fv_diffusion_residual(fv_diffusion_t d, double* norm) {
    return dguard([&] {
        if (!d || !norm) raise(FV_ERR_BAD_ARG, "null argument");
        fvgb::StepCtl c;
        FV_CUDA(cudaMemcpyAsync(&c, d->s.a.ctl, sizeof(c), cudaMemcpyDeviceToHost, d->s.stream));
        FV_CUDA(cudaStreamSynchronize(d->s.stream));
        *norm = c.norms[0];
    });
}

}  // extern "C"
