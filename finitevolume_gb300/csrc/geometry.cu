// Mesh geometry recomputed on the device after the nodes move:
// UnstructuredMesh::compute_geometry (include/UnstructuredMesh.h:89-105:
// face midpoint, length, unit normal), the shoelace area and centroid of
// compute_cell_geometry (src/MeshReader.cpp:56-76), the CFL length of
// compute_dt (src/EulerFVMSolver.cpp:151-156), and the second-order
// reconstruction geometry (least-squares weights folded with the inverse
// normal matrix, their sums, Green-Gauss coefficients, face offsets and the
// Venkatakrishnan eps^2) in the solver's device numbering.  The expressions
// and their evaluation order are the host builder's (mesh_host.cpp), and
// this unit is built without FMA contraction, so a moved mesh gets the same
// geometry bits as a solver built from it on the host (the Green-Gauss
// interpolation weights go through hypot, whose last bit can differ).
#include <cmath>
#include <cstring>
#include <vector>

#include "capi_internal.h"

namespace fvgb {
const HostMesh& host_mesh_of(const fv_mesh_s* m);
}

namespace geo {

struct GeoArgs {
    int n_cells, n_faces, n_int_faces;
    const double2* xy;         // [n_nodes] caller's node numbering
    const int2* fnodes;        // [F] device face -> (node1, node2)
    const long long* coff;     // [N+1] device cell -> polygon CSR
    const int* cnodes;
    const int* fl;
    const int* fr;
    const int* cf_off;
    const int* cf;
    // outputs (device order)
    double4_32a* fgeom;
    double2* fmid;
    double* vol;
    double2* cxy;
    // second order (null unless the solver has them); flux precision
    int fp32;
    void* lsq;
    void* lsq_sum;
    void* gg;
    void* erf;
    void* frf;
    void* eps2;
    float4* fgeom32;
    double venkat_k;
};

__global__ void k_face_geom(const GeoArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n_faces) return;
    const int2 nn = a.fnodes[i];
    const double2 p1 = a.xy[nn.x], p2 = a.xy[nn.y];
    double4_32a g;
    double2 m;
    m.x = 0.5 * (p1.x + p2.x);
    m.y = 0.5 * (p1.y + p2.y);
    const double dx = p2.x - p1.x, dy = p2.y - p1.y;
    const double len = sqrt(dx * dx + dy * dy);
    g.x = dy / len;
    g.y = -dx / len;
    g.z = len;
    g.w = 0.0;
    a.fgeom[i] = g;
    a.fmid[i] = m;
}

__global__ void k_cell_geom(const GeoArgs a) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.n_cells) return;
    const long long lo = a.coff[c], hi = a.coff[c + 1];
    const int k = (int)(hi - lo);
    double area = 0.0;
    for (int i = 0; i < k; ++i) {
        const double2 p0 = a.xy[a.cnodes[lo + i]], p1 = a.xy[a.cnodes[lo + (i + 1) % k]];
        area += p0.x * p1.y - p1.x * p0.y;
    }
    area = 0.5 * area;
    double sx = 0.0, sy = 0.0;
    for (int i = 0; i < k; ++i) {
        const double2 p0 = a.xy[a.cnodes[lo + i]], p1 = a.xy[a.cnodes[lo + (i + 1) % k]];
        const double cross = p0.x * p1.y - p1.x * p0.y;
        sx += (p0.x + p1.x) * cross;
        sy += (p0.y + p1.y) * cross;
    }
    sx /= (6.0 * area);
    sy /= (6.0 * area);
    a.vol[c] = fabs(area);
    a.cxy[c] = make_double2(sx, sy);
}

// CFL length min(V_L, V_R) / |f| (boundary: V_L / |f|)
__global__ void k_face_len(const GeoArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n_faces) return;
    const int L = a.fl[i], R = a.fr[i];
    double4_32a g = a.fgeom[i];
    if (R >= 0) {
        const double vl = a.vol[L], vr = a.vol[R];
        g.w = ((vr < vl) ? vr : vl) / g.z;
    } else {
        g.w = a.vol[L] / g.z;
    }
    a.fgeom[i] = g;
    if (a.fgeom32) a.fgeom32[i] = make_float4((float)g.x, (float)g.y, (float)g.z, (float)g.w);
}

template <typename T> __device__ __forceinline__ void put2(void* p, size_t i, double x, double y) {
    static_cast<T*>(p)[2 * i] = (T)x;
    static_cast<T*>(p)[2 * i + 1] = (T)y;
}

// Second-order geometry of one cell (build_o2_geometry in mesh_host.cpp).
template <typename T>
__global__ void k_o2_geom(const GeoArgs a) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.n_cells) return;
    const double2 pc = a.cxy[c];
    const double xc = pc.x, yc = pc.y;
    const int e0 = a.cf_off[c], e1 = a.cf_off[c + 1];
    double m00 = 0.0, m01 = 0.0, m11 = 0.0;
    for (int e = e0; e < e1; ++e) {
        const int f = a.cf[e] >> 1;
        double px, py;
        if (a.fr[f] < 0) { px = a.fmid[f].x; py = a.fmid[f].y; }
        else {
            const int nb = a.fl[f] == c ? a.fr[f] : a.fl[f];
            px = a.cxy[nb].x; py = a.cxy[nb].y;
        }
        const double dx = px - xc, dy = py - yc;
        const double w = 1.0 / (dx * dx + dy * dy);
        m00 += w * dx * dx; m01 += w * dx * dy; m11 += w * dy * dy;
    }
    const double det = m00 * m11 - m01 * m01;
    const double i00 = m11 / det, i01 = -m01 / det, i11 = m00 / det;
    const double vol = a.vol[c];
    double sx = 0.0, sy = 0.0;
    for (int e = e0; e < e1; ++e) {
        const int ent = a.cf[e];
        const int f = ent >> 1;
        const bool owner = ent & 1;
        const bool bnd = a.fr[f] < 0;
        double px, py;
        if (bnd) { px = a.fmid[f].x; py = a.fmid[f].y; }
        else {
            const int nb = owner ? a.fr[f] : a.fl[f];
            px = a.cxy[nb].x; py = a.cxy[nb].y;
        }
        const double dx = px - xc, dy = py - yc;
        const double w = 1.0 / (dx * dx + dy * dy);
        const double lx = i00 * (w * dx) + i01 * (w * dy);
        const double ly = i01 * (w * dx) + i11 * (w * dy);
        if (a.lsq) put2<T>(a.lsq, e, lx, ly);
        sx += lx;
        sy += ly;
        if (a.gg) {
            const double4_32a g = a.fgeom[f];
            const double sgn = owner ? 1.0 : -1.0;
            double wgt = 0.0;
            if (!bnd) {
                const double d_c = hypot(xc - a.fmid[f].x, yc - a.fmid[f].y);
                const double d_o = hypot(px - a.fmid[f].x, py - a.fmid[f].y);
                wgt = d_o / (d_c + d_o);
            }
            T* q = static_cast<T*>(a.gg) + 4 * (size_t)e;
            q[0] = (T)(sgn * g.x * g.z / vol);
            q[1] = (T)(sgn * g.y * g.z / vol);
            q[2] = (T)wgt;
            q[3] = (T)0.0;
        }
        put2<T>(a.erf, e, a.fmid[f].x - xc, a.fmid[f].y - yc);
    }
    if (a.lsq_sum) put2<T>(a.lsq_sum, c, sx, sy);
    // eps^2 = (K sqrt(V))^3, formed in FP64 then (FP32 mode) cubed in float
    const double kh = a.venkat_k * sqrt(vol);
    if (a.fp32) {
        const float khf = (float)kh;
        static_cast<float*>(a.eps2)[c] = khf * khf * khf;
    } else {
        static_cast<double*>(a.eps2)[c] = kh * kh * kh;
    }
}

template <typename T>
__global__ void k_o2_face_offsets(const GeoArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n_faces) return;
    const double2 m = a.fmid[i], l = a.cxy[a.fl[i]];
    T* q = static_cast<T*>(a.frf) + 4 * (size_t)i;
    q[0] = (T)(m.x - l.x);
    q[1] = (T)(m.y - l.y);
    if (a.fr[i] >= 0) {
        const double2 r = a.cxy[a.fr[i]];
        q[2] = (T)(m.x - r.x);
        q[3] = (T)(m.y - r.y);
    } else {
        q[2] = (T)0.0;
        q[3] = (T)0.0;
    }
}

}  // namespace geo

namespace {
struct GeoCache {
    void* xy = nullptr;
    void* fnodes = nullptr;
    void* coff = nullptr;
    void* cnodes = nullptr;
    size_t n_nodes = 0;
};
}  // namespace

extern "C" int fv_solver_update_nodes(fv_solver_t solver, fv_mesh_t mesh, const double* xy) {
    return fvgb::guarded([&] {
        if (!solver || !mesh || !xy) fvgb::raise(FV_ERR_BAD_ARG, "null argument");
        fvgb::Solver& s = solver->s;
        const fvgb::HostMesh& h = fvgb::host_mesh_of(mesh);
        if (h.n_cells != s.N || h.n_faces != s.F) fvgb::raise(FV_ERR_BAD_ARG, "mesh does not match the solver");
        if (h.cnode_off.empty())
            fvgb::raise(FV_ERR_UNSUPPORTED, "node update: the mesh must be built from cell polygons");
        if (s.viscous || s.batch)
            fvgb::raise(FV_ERR_UNSUPPORTED, "node update: Euler solvers (the viscous gradient geometry stays fixed)");
        if (s.general && s.opt.order == 2 && s.opt.gradient != FV_GRAD_LSQ && s.opt.gradient != FV_GRAD_GG)
            fvgb::raise(FV_ERR_UNSUPPORTED, "node update: unknown gradient scheme");
        for (int i = 0; i < h.n_nodes; ++i)
            if (!std::isfinite(xy[2 * i]) || !std::isfinite(xy[2 * i + 1]))
                fvgb::raise(FV_ERR_BAD_MESH, "node update: non-finite coordinate");
        // topology in device order (uploaded once per call; small next to the geometry)
        std::vector<int2> fn(s.F);
        for (int i = 0; i < s.F; ++i) {
            const int f = h.fperm[i];
            fn[i] = make_int2(h.fn1[f], h.fn2[f]);
        }
        std::vector<long long> coff(s.N + 1);
        std::vector<int> cn;
        cn.reserve(h.cnodes.size());
        coff[0] = 0;
        for (int i = 0; i < s.N; ++i) {
            const int c = h.perm[i];
            for (long long k = h.cnode_off[c]; k < h.cnode_off[c + 1]; ++k) cn.push_back(h.cnodes[k]);
            coff[i + 1] = (long long)cn.size();
        }
        std::vector<void*> tmp;
        auto up = [&](const void* src, size_t bytes) {
            void* d = nullptr;
            FV_CUDA(cudaMalloc(&d, bytes ? bytes : 1));
            tmp.push_back(d);
            if (bytes) fvgb::h2d_sync(d, src, bytes, s.stream);
            return d;
        };
        struct Free {
            std::vector<void*>& v;
            ~Free() { for (void* p : v) cudaFree(p); }
        } guard{tmp};
        geo::GeoArgs a{};
        a.n_cells = s.N;
        a.n_faces = s.F;
        a.n_int_faces = s.dm.n_int_faces;
        a.xy = static_cast<const double2*>(up(xy, sizeof(double) * 2 * (size_t)h.n_nodes));
        a.fnodes = static_cast<const int2*>(up(fn.data(), sizeof(int2) * fn.size()));
        a.coff = static_cast<const long long*>(up(coff.data(), sizeof(long long) * coff.size()));
        a.cnodes = static_cast<const int*>(up(cn.data(), sizeof(int) * cn.size()));
        a.fl = s.dm.fl;
        a.fr = s.dm.fr;
        a.cf_off = s.dm.cf_off;
        a.cf = s.dm.cf;
        a.fgeom = const_cast<double4_32a*>(s.dm.fgeom);
        a.fmid = const_cast<double2*>(s.dm.fmid);
        a.vol = const_cast<double*>(s.dm.vol);
        a.cxy = const_cast<double2*>(s.dm.cxy);
        a.fp32 = s.general && s.cfg.fp32;
        a.fgeom32 = const_cast<float4*>(s.fgeom32);
        a.venkat_k = s.opt.venkat_k;
        const int B = 256;
        FV_CUDA(cudaStreamSynchronize(s.stream));
        geo::k_face_geom<<<(s.F + B - 1) / B, B, 0, s.stream>>>(a);
        geo::k_cell_geom<<<(s.N + B - 1) / B, B, 0, s.stream>>>(a);
        geo::k_face_len<<<(s.F + B - 1) / B, B, 0, s.stream>>>(a);
        FV_CUDA(cudaGetLastError());
        if (s.general && s.opt.order == 2) {
            a.lsq = const_cast<void*>(s.lsq);
            a.lsq_sum = const_cast<void*>(s.lsq_sum);
            a.gg = const_cast<void*>(s.gg);
            a.erf = const_cast<void*>(s.erf);
            a.frf = const_cast<void*>(s.frf);
            a.eps2 = const_cast<void*>(s.eps2);
            if (a.fp32) {
                geo::k_o2_geom<float><<<(s.N + B - 1) / B, B, 0, s.stream>>>(a);
                geo::k_o2_face_offsets<float><<<(s.F + B - 1) / B, B, 0, s.stream>>>(a);
            } else {
                geo::k_o2_geom<double><<<(s.N + B - 1) / B, B, 0, s.stream>>>(a);
                geo::k_o2_face_offsets<double><<<(s.F + B - 1) / B, B, 0, s.stream>>>(a);
            }
            FV_CUDA(cudaGetLastError());
        }
        FV_CUDA(cudaStreamSynchronize(s.stream));
        // host copies of the wall faces (force integration)
        for (fvgb::WallFace& w : s.wall_faces) {
            const int f = h.fperm[w.dev_face];
            const double x1 = xy[2 * h.fn1[f]], y1 = xy[2 * h.fn1[f] + 1];
            const double x2 = xy[2 * h.fn2[f]], y2 = xy[2 * h.fn2[f] + 1];
            w.xm = 0.5 * (x1 + x2);
            w.ym = 0.5 * (y1 + y2);
            const double dx = x2 - x1, dy = y2 - y1;
            const double len = std::sqrt(dx * dx + dy * dy);
            w.area = len;
            w.nx = dy / len;
            w.ny = -dx / len;
        }
        // graphs replay pointers only; the arrays were rewritten in place
    });
}
