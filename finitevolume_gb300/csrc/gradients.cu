// GradientCalculator / face_gradient interface (include/GradientReconstruction.h:46-162)
// on the device.  Built without FMA contraction: values are bit-identical
// to the reference's.
#include <memory>
#include <vector>

#include "../../include/fv_gb300.h"
#include "errors.h"
#include "gradients.cuh"
#include "mesh_host.h"

struct fv_mesh_s;
namespace fvgb {
const HostMesh& host_mesh_of(const fv_mesh_s* m);

namespace {

__global__ void k_api_grad(const GradDev g, const double* __restrict__ phi, const double* __restrict__ bphi,
                           double2* __restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.n_cells) return;
    double gx[1], gy[1];
    cell_gradient<1>(g, c, [&](int i, int) { return phi[i]; }, [&](int f, int) { return bphi[f]; }, gx, gy);
    out[c] = make_double2(gx[0], gy[0]);
}

__global__ void k_api_facegrad(const GradDev g, const int* __restrict__ fl, const double* __restrict__ phi,
                               const double* __restrict__ bphi, const double2* __restrict__ grad,
                               double4_32a* __restrict__ out) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= g.n_faces) return;
    const int L = fl[f], R = g.fr[f];
    const bool b = R < 0;
    const double* fg = g.fgrad + 8 * (size_t)f;
    const double2 gL = grad[L];
    const double2 gR = b ? make_double2(0.0, 0.0) : grad[R];
    const FaceGrad r = face_gradient(fg, b, phi[L], b ? bphi[f] : phi[R], gL.x, gL.y, gR.x, gR.y);
    double4_32a o;
    o.x = r.dphidn;
    o.y = r.gx;
    o.z = r.gy;
    o.w = fg[5];
    out[f] = o;
}

__global__ void k_perm_gather(const double* __restrict__ in, double* __restrict__ out, const int* __restrict__ perm,
                              int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = in[perm[i]];
}
template <typename V>
__global__ void k_perm_scatter(const V* __restrict__ in, V* __restrict__ out, const int* __restrict__ perm, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[perm[i]] = in[i];
}

}  // namespace

struct GradApi {
    GradDev g{};
    int N = 0, F = 0;
    const int* fl = nullptr;
    int* perm = nullptr;
    int* fperm = nullptr;
    double *phi_ref = nullptr, *phi = nullptr, *bphi_ref = nullptr, *bphi = nullptr;
    double2 *grad = nullptr, *grad_ref = nullptr;
    double4_32a *fout = nullptr, *fout_ref = nullptr;
    std::vector<void*> owned;
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
    ~GradApi() {
        for (void* p : owned) cudaFree(p);
    }
};

}  // namespace fvgb

struct fv_gradient_s {
    fvgb::GradApi a;
};

template <typename Fn>
static int gguard(Fn&& fn) {
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

int fv_gradient_create(fv_mesh_t mesh, int32_t scheme, fv_gradient_t* out) {
    return gguard([&] {
        if (!mesh || !out) fvgb::raise(FV_ERR_BAD_ARG, "null argument");
        if (scheme != FV_GRAD_LSQ && scheme != FV_GRAD_GG) fvgb::raise(FV_ERR_BAD_ARG, "unknown gradient scheme");
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) fvgb::raise(FV_ERR_CUDA, "no CUDA device available");
        const fvgb::HostMesh& h = fvgb::host_mesh_of(mesh);
        fvgb::HostGradGeom hg;
        fvgb::build_grad_geom(h, hg);
        auto r = std::make_unique<fv_gradient_s>();
        fvgb::GradApi& a = r->a;
        a.N = h.n_cells;
        a.F = h.n_faces;
        fvgb::GradDev& g = a.g;
        g.n_cells = a.N;
        g.n_faces = a.F;
        g.scheme = scheme;
        g.cf_off = a.up(h.d_cf_off);
        g.nb = a.up(hg.nb);
        g.lsq_w = reinterpret_cast<const double2*>(a.up(hg.lsq_w));
        g.lsq_inv = a.up(hg.lsq_inv);
        g.gg = reinterpret_cast<const double4_32a*>(a.up(hg.gg));
        g.vol = a.up(h.d_vol);
        g.fgrad = a.up(hg.fgrad);
        g.fr = a.up(h.d_fr);
        a.fl = a.up(h.d_fl);
        a.perm = a.up(h.perm);
        a.fperm = a.up(h.fperm);
        a.phi_ref = a.alloc<double>(a.N);
        a.phi = a.alloc<double>(a.N);
        a.bphi_ref = a.alloc<double>(a.F);
        a.bphi = a.alloc<double>(a.F);
        a.grad = a.alloc<double2>(a.N);
        a.grad_ref = a.alloc<double2>(a.N);
        a.fout = a.alloc<double4_32a>(a.F);
        a.fout_ref = a.alloc<double4_32a>(a.F);
        *out = r.release();
    });
}

int fv_gradient_destroy(fv_gradient_t g) {
    delete g;
    return FV_OK;
}

int fv_gradient_compute(fv_gradient_t h, const double* phi, const double* boundary_phi, double* grad,
                        double* face_out) {
    return gguard([&] {
        if (!h || !phi || !boundary_phi || !grad) fvgb::raise(FV_ERR_BAD_ARG, "null argument");
        fvgb::GradApi& a = h->a;
        const int N = a.N, F = a.F;
        fvgb::h2d_sync(a.phi_ref, phi, sizeof(double) * N);
        fvgb::h2d_sync(a.bphi_ref, boundary_phi, sizeof(double) * F);
        fvgb::k_perm_gather<<<(N + 255) / 256, 256>>>(a.phi_ref, a.phi, a.perm, N);
        fvgb::k_perm_gather<<<(F + 255) / 256, 256>>>(a.bphi_ref, a.bphi, a.fperm, F);
        fvgb::k_api_grad<<<(N + 255) / 256, 256>>>(a.g, a.phi, a.bphi, a.grad);
        fvgb::k_perm_scatter<double2><<<(N + 255) / 256, 256>>>(a.grad, a.grad_ref, a.perm, N);
        if (face_out) {
            fvgb::k_api_facegrad<<<(F + 255) / 256, 256>>>(a.g, a.fl, a.phi, a.bphi, a.grad, a.fout);
            fvgb::k_perm_scatter<double4_32a><<<(F + 255) / 256, 256>>>(a.fout, a.fout_ref, a.fperm, F);
        }
        FV_CUDA(cudaGetLastError());
        FV_CUDA(cudaMemcpy(grad, a.grad_ref, sizeof(double2) * N, cudaMemcpyDeviceToHost));
        if (face_out) FV_CUDA(cudaMemcpy(face_out, a.fout_ref, sizeof(double4_32a) * F, cudaMemcpyDeviceToHost));
    });
}

}  // extern "C"
