// Solver object and the C ABI (include/fv_gb300.h).
//
// One solver = one mesh uploaded in device order + the conserved state and
// its work arrays, all resident in HBM for the solver's lifetime.  Steps are
// replayed from captured CUDA graphs (one graph per chunk length), so a
// 3000-step run is ~100 graph launches; everything a graph reads that the
// host may change (CFL number, step counter) lives in device memory.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/fv_gb300.h"
#include "errors.h"
#include "mesh_host.h"
#include "solver.h"
#include "types.h"
#include "capi_internal.h"

using fvgb::HostMesh;

struct fv_mesh_s {
    HostMesh h;
};

namespace fvgb {
const HostMesh& host_mesh_of(const fv_mesh_s* m) { return m->h; }
}  // namespace fvgb

namespace fvgb {

template <typename T>
static T* dalloc(size_t n, std::vector<void*>& owned) {
    void* p = nullptr;
    FV_CUDA(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)));
    owned.push_back(p);
    return static_cast<T*>(p);
}

static std::vector<float> to_float(const std::vector<double>& v) {
    std::vector<float> o(v.size());
    for (size_t i = 0; i < v.size(); ++i) o[i] = (float)v[i];
    return o;
}

template <typename T>
static T* dupload(const std::vector<T>& v, std::vector<void*>& owned) {
    T* p = dalloc<T>(v.size(), owned);
    if (!v.empty()) h2d_sync(p, v.data(), v.size() * sizeof(T));
    return p;
}

Solver::~Solver() {
    for (cudaEvent_t e : events) cudaEventDestroy(e);
    for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
    for (void* p : owned) cudaFree(p);
    if (hist) cudaFree(hist);
    if (nut_hist) cudaFree(nut_hist);
    if (own_stream && stream) cudaStreamDestroy(stream);
}

void Solver::init(const HostMesh& hm, const fv_bc_t* bcs, int n_bcs, double g, double cfl0, const fv_ic_t& ic,
                  const fv_options_t& o, const double* batch_freestream) {
    batch = batch_freestream != nullptr;
    if (batch) {
        if (hm.group_off.size() < 2) raise(FV_ERR_BAD_ARG, "batched solver needs a batch mesh (fv_mesh_create_batch)");
        if (o.viscous || o.dt_mode != FV_DT_LOCAL)
            raise(FV_ERR_UNSUPPORTED, "batched solves are inviscid steady solves with local time stepping");
        group_off = hm.group_off;
        n_inst = (int)group_off.size() - 1;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) raise(FV_ERR_CUDA, "no CUDA device available");
    if (n_bcs < hm.n_patches) raise(FV_ERR_BAD_ARG, "fewer boundary conditions than mesh patches");
    if (hm.n_patches > kMaxPatches) raise(FV_ERR_UNSUPPORTED, "more than 32 boundary patches");
    if (!(g > 1.0)) raise(FV_ERR_BAD_ARG, "gamma must be > 1");
    opt = o;
    if (opt.flux < 0 || opt.flux > 2) raise(FV_ERR_BAD_ARG, "unknown flux scheme");
    if (opt.order != 1 && opt.order != 2) raise(FV_ERR_BAD_ARG, "order must be 1 or 2");
    if (opt.rk_stages != 1 && opt.rk_stages != 3) raise(FV_ERR_BAD_ARG, "rk_stages must be 1 or 3");
    if (opt.precision != FV_PREC_FP64 && opt.precision != FV_PREC_FP32_FLUX) raise(FV_ERR_BAD_ARG, "unknown precision");
    if (opt.gradient < 0 || opt.gradient > 1 || opt.limiter < 0 || opt.limiter > 2)
        raise(FV_ERR_BAD_ARG, "unknown gradient scheme or limiter");
    if (opt.dt_mode != FV_DT_GLOBAL && opt.dt_mode != FV_DT_LOCAL) raise(FV_ERR_BAD_ARG, "unknown dt mode");
    if (opt.viscous && (opt.order != 1 || opt.rk_stages != 1 || opt.precision != FV_PREC_FP64 ||
                        opt.dt_mode != FV_DT_GLOBAL))
        raise(FV_ERR_UNSUPPORTED, "the Navier-Stokes path is the reference's scheme: order 1, forward Euler, "
                                  "global dt, FP64");
    if (opt.viscous && !(opt.gas_constant > 0.0 && opt.prandtl > 0.0 && opt.mu >= 0.0))
        raise(FV_ERR_BAD_ARG, "viscous solver needs gas_constant > 0, prandtl > 0, mu >= 0");
    if (opt.viscous < 0 || opt.viscous > 2) raise(FV_ERR_BAD_ARG, "viscous: 0 Euler, 1 Navier-Stokes, 2 RANS-SA");
    if (opt.viscous == 2 && !(opt.mu > 0.0 && opt.prandtl_t > 0.0 && opt.initial_nut >= 0.0))
        raise(FV_ERR_BAD_ARG, "RANS-SA needs mu > 0, prandtl_t > 0, initial_nut >= 0");
    viscous = opt.viscous != 0;
    rans = opt.viscous == 2;
    general = batch || (!viscous && !(opt.order == 1 && opt.rk_stages == 1 && opt.precision == FV_PREC_FP64));
    if (general && opt.strict) raise(FV_ERR_UNSUPPORTED, "strict mode covers the reference's first-order scheme only");
    if (general && opt.precision == FV_PREC_FP32_FLUX && opt.flux == FV_FLUX_EXACT)
        raise(FV_ERR_UNSUPPORTED, "the exact Riemann flux runs in FP64 only");
    cfg.fp32 = opt.precision == FV_PREC_FP32_FLUX;
    cfg.flux = opt.flux;
    cfg.order = opt.order;
    cfg.gradient = opt.gradient;
    cfg.limiter = opt.limiter;
    cfg.stages = opt.rk_stages;
    cfg.local_dt = opt.dt_mode == FV_DT_LOCAL;
    cfg.blk_grad = cfg.blk_face = cfg.blk_cell = 256;
    gamma = g;
    N = hm.n_cells;
    F = hm.n_faces;
    perm = hm.perm;
    wall_faces.clear();
    std::memset(&bc, 0, sizeof(bc));
    bc.n = hm.n_patches;
    for (int p = 0; p < hm.n_patches; ++p) {
        const fv_bc_t& b = bcs[p];
        if (b.type < FV_BC_WALL || b.type > FV_BC_NOSLIP) raise(FV_ERR_BAD_ARG, "unknown boundary type");
        bc.type[p] = b.type;
        for (int k = 0; k < 4; ++k) bc.st[p][k] = b.state[k];
        bc.wall_u[p] = b.wall_u;
        bc.wall_v[p] = b.wall_v;
        bc.isothermal[p] = b.isothermal;
        bc.wall_T[p] = b.wall_T;
    }
    // Host copies needed after construction: wall faces in reference face
    // order (the order compute_wall_forces accumulates them in).
    for (int f = 0; f < F; ++f) {
        if (hm.fr[f] >= 0) continue;
        int p = hm.fpatch[f];
        if (bc.type[p] == FV_BC_WALL || bc.type[p] == FV_BC_NOSLIP) {
            wall_faces.push_back({hm.fl[f], hm.fnx[f], hm.fny[f], hm.farea[f], hm.fxm[f], hm.fym[f], hm.ifperm[f]});
            if (batch)
                wall_inst.push_back((int)(std::upper_bound(group_off.begin(), group_off.end(), hm.fl[f]) -
                                          group_off.begin()) - 1);
        }
    }

    FV_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    own_stream = true;

    DevMesh& m = dm;
    m.n_cells = N;
    m.n_faces = F;
    m.n_int_faces = hm.n_int_faces;
    m.fl = dupload(hm.d_fl, owned);
    m.fr = dupload(hm.d_fr, owned);
    m.fpatch = dupload(hm.d_fpatch, owned);
    m.fgeom = reinterpret_cast<const double4_32a*>(dupload(hm.d_fgeom, owned));
    m.fmid = reinterpret_cast<const double2*>(dupload(hm.d_fmid, owned));
    m.cf_off = dupload(hm.d_cf_off, owned);
    m.cf = dupload(hm.d_cf, owned);
    m.vol = dupload(hm.d_vol, owned);
    m.cxy = reinterpret_cast<const double2*>(dupload(hm.d_cxy, owned));

    U = dalloc<St>(N, owned);
    staging = dalloc<St>(N, owned);
    d_perm = dupload(hm.perm, owned);
    if (!(general && cfg.fp32)) ff = dalloc<St>(F, owned);
    dtf = dalloc<double>(F, owned);
    n_cell_blocks = (N + kCellBlock - 1) / kCellBlock;
    // sized for the smallest tunable cell block
    partials = dalloc<double>(4 * (size_t)((N + kMinBlock - 1) / kMinBlock), owned);
    ctl = dalloc<StepCtl>(1, owned);
    StepCtl c0;
    std::memset(&c0, 0, sizeof(c0));
    c0.cfl = cfl0;
    double dmax = DBL_MAX;
    std::memcpy(&c0.dt_bits, &dmax, sizeof(dmax));
    h2d_sync(ctl, &c0, sizeof(c0));
    ensure_history(64);

    if (!general && !viscous) {
        // Persistent first-order path: co-resident grid sized to the larger
        // of the face tiles and the 256-cell tiles, rounded up to a whole
        // number of blocks per SM (the face phase splits the faces evenly
        // over the blocks), capped at what fits.
        int dev = 0, coop = 0, sms = 0;
        FV_CUDA(cudaGetDevice(&dev));
        FV_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
        FV_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        const int per_sm = opt.strict ? strict::o1p_max_blocks_per_sm(opt.flux, opt.dt_mode == FV_DT_LOCAL)
                                      : fast::o1p_max_blocks_per_sm(opt.flux, opt.dt_mode == FV_DT_LOCAL);
        int want = std::max((F + kCellBlock - 1) / kCellBlock, (N + kCellBlock - 1) / kCellBlock);
        if (sms > 0 && want > sms) want = (want + sms - 1) / sms * sms;
        p_grid = std::min(want, per_sm * sms);
        persistent_ok = coop != 0 && p_grid > 0;
        if (persistent_ok) {
            Pc = dalloc<double4_32a>(N, owned);
            pctl = dalloc<PersistCtl>(1, owned);
            PersistCtl p0;
            std::memset(&p0, 0, sizeof(p0));
            p0.limit = kDefaultWaitCycles;
            h2d_sync(pctl, &p0, sizeof(p0), stream);
            persistent = true;
            if (opt.dt_mode == FV_DT_LOCAL) build_dataflow(hm, sms);
        }
    }

    if (general) {
        HostMesh h2 = hm;  // the per-entry geometry is derived on a copy
        h2.build_o2_geometry();
        const size_t wsz = cfg.fp32 ? 16 : 32;
        U0 = dalloc<St>(N, owned);
        W = dalloc<char>(wsz * (size_t)N, owned);
        G = dalloc<char>(2 * wsz * (size_t)N, owned);
        if (cfg.fp32) ff = reinterpret_cast<St*>(dalloc<char>(16 * (size_t)F, owned));
        cs = dalloc<char>(wsz / 4 * (size_t)N, owned);
        dtv = dalloc<double>(N, owned);
        cnb = dupload(h2.d_cnb, owned);
        // Venkatakrishnan eps^2 = (K h)^3 per cell, formed as the kernels
        // formed it before (K h in FP64, rounded to the flux precision,
        // cubed in that precision).
        std::vector<double> e64(N);
        std::vector<float> e32(N);
        for (int c = 0; c < N; ++c) {
            const double kh = opt.venkat_k * h2.d_h[c];
            const float khf = (float)kh;
            e64[c] = kh * kh * kh;
            e32[c] = khf * khf * khf;
        }
        // The per-entry / per-face reconstruction geometry is stored in the
        // flux precision: FP32-flux mode then converts nothing per use.
        auto up = [&](const std::vector<double>& v) -> const void* {
            return cfg.fp32 ? static_cast<const void*>(dupload(to_float(v), owned))
                            : static_cast<const void*>(dupload(v, owned));
        };
        if (cfg.gradient == 0) {
            lsq = up(h2.d_lsq);
            lsq_sum = up(h2.d_lsq_sum);
        }
        else gg = up(h2.d_gg);
        erf = up(h2.d_erf);
        frf = up(h2.d_frf);
        eps2 = cfg.fp32 ? static_cast<const void*>(dupload(e32, owned)) : static_cast<const void*>(dupload(e64, owned));
        if (cfg.fp32) fgeom32 = reinterpret_cast<const float4*>(dupload(to_float(hm.d_fgeom), owned));
        if (!cfg.fp32 && cfg.order == 2 && cfg.limiter != 0) {
            const size_t E = h2.d_cf.size();
            std::vector<int2> fev(F, make_int2(-1, -1));
            for (size_t e = 0; e < E; ++e) {
                const int ent = h2.d_cf[e];
                if (ent & 1) fev[ent >> 1].x = (int)e;
                else fev[ent >> 1].y = (int)e;
            }
            d2 = dalloc<St>(E, owned);
            psi4 = dalloc<St>(N, owned);
            fe = dupload(fev, owned);
        }
    }

    if (batch) {
        // Instances are contiguous and in order in device numbering, with
        // the same cell ranges as in reference numbering.
        std::vector<int> ci(N);
        for (int i = 0; i < n_inst; ++i)
            for (int c = group_off[i]; c < group_off[i + 1]; ++c) ci[c] = i;
        cell_inst = dupload(ci, owned);
        inst_off = dupload(std::vector<int>(group_off.begin(), group_off.end()), owned);
        active = dupload(std::vector<int>(n_inst, 1), owned);
        inst_iter = dupload(std::vector<int>(n_inst, 0), owned);
        inst_fs_host.assign(batch_freestream, batch_freestream + 4 * (size_t)n_inst);
        inst_fs = dupload(inst_fs_host, owned);
        inst_norms = dupload(std::vector<double>(4 * (size_t)n_inst, 0.0), owned);
        r2 = dalloc<double4_32a>(N, owned);
    }

    if (viscous) {
        HostGradGeom hg;
        build_grad_geom(hm, hg);
        // The viscous time step divides by the face-normal distance between
        // the two centroids (face_normal_distance, src/GradientReconstruction
        // .cpp:186-190); it is positive on any mesh whose cells do not
        // overlap.  The reference takes the minimum over faces unguarded,
        // so one non-positive distance makes its dt non-positive; it is
        // refused here instead of being silently skipped by the device min.
        for (int i = 0; i < F; ++i)
            if (!(hg.fgrad[8 * (size_t)i + 5] > 0.0))
                raise(FV_ERR_BAD_MESH, "face " + std::to_string(hm.fperm[i]) +
                                           ": neighbouring centroids on one side (overlapping cells)");
        NSArgs& a = ns;
        a.g.n_cells = N;
        a.g.n_faces = F;
        a.g.scheme = opt.gradient;
        a.g.cf_off = m.cf_off;
        a.g.nb = dupload(hg.nb, owned);
        a.g.lsq_w = reinterpret_cast<const double2*>(dupload(hg.lsq_w, owned));
        a.g.lsq_inv = dupload(hg.lsq_inv, owned);
        a.g.gg = reinterpret_cast<const double4_32a*>(dupload(hg.gg, owned));
        a.g.vol = m.vol;
        a.g.fgrad = dupload(hg.fgrad, owned);
        a.g.fr = m.fr;
        a.fl = m.fl;
        a.fpatch = m.fpatch;
        a.fgeom = m.fgeom;
        a.U = U;
        a.ff = ff;
        a.prim = dalloc<double4_32a>(N, owned);
        a.grad = dalloc<double2>(3 * (size_t)N, owned);
        a.ctl = ctl;
        a.bc = bc;
        a.gamma = gamma;
        a.gas_constant = opt.gas_constant;
        a.mu = opt.mu;
        const double cp = gamma * opt.gas_constant / (gamma - 1.0);  // src/NavierStokesFVMSolver.cpp:113-114
        a.kcond = opt.mu * cp / opt.prandtl;
        a.exact_tol = opt.exact_tol;
        a.exact_max_iter = opt.exact_max_iter;
        a.flux = opt.flux;
        std::vector<int> wf;
        for (const WallFace& w : wall_faces) wf.push_back(w.dev_face);
        ns_wall_faces = dupload(wf, owned);
        ns_wall_out = dalloc<double2>(wf.size(), owned);
    }

    if (rans) {
        // RANSTurbulenceSASolver ctor: uniform initial nu-tilde, the wall
        // distance from the no-slip faces (compute_wall_distance), model
        // constants and effective-conductivity factors.
        RansArgs& r = rs;
        r.cf_off = m.cf_off;
        r.cf = m.cf;
        r.vol = m.vol;
        r.cxy = m.cxy;
        r.nut = dupload(std::vector<double>(N, opt.initial_nut), owned);
        r.nut_ff = dalloc<double>(F, owned);
        r.nu = dalloc<double2>(N, owned);
        r.grad = dalloc<double2>(4 * (size_t)N, owned);
        r.walld = dalloc<double>(N, owned);
        r.partials = dalloc<double>(5 * (size_t)n_cell_blocks, owned);
        r.nut_norm = dupload(std::vector<double>(1, 0.0), owned);
        for (int p = 0; p < kMaxPatches; ++p) r.farfield_nut[p] = p < hm.n_patches ? bcs[p].nut : 0.0;
        for (int i = 0; i < 9; ++i) r.sa[i] = opt.sa[i];
        r.cw3_6 = std::pow(opt.sa[5], 6.0);
        r.cp = gamma * opt.gas_constant / (gamma - 1.0);
        r.prandtl = opt.prandtl;
        r.prandtl_t = opt.prandtl_t;
        r.k_lam = r.cp * opt.mu / opt.prandtl;
        std::vector<double4_32a> seg;
        for (int f = 0; f < F; ++f) {
            if (hm.fr[f] >= 0 || bc.type[hm.fpatch[f]] != FV_BC_NOSLIP) continue;
            double4_32a q;
            q.x = hm.nx_[hm.fn1[f]]; q.y = hm.ny_[hm.fn1[f]];
            q.z = hm.nx_[hm.fn2[f]]; q.w = hm.ny_[hm.fn2[f]];
            seg.push_back(q);
        }
        if (seg.empty()) {
            // no wall: infinite distance, as compute_wall_distance
            h2d_sync(r.walld, std::vector<double>(N, INFINITY).data(), sizeof(double) * N);
        } else {
            double4_32a* d_seg = dupload(seg, owned);
            RansArgs tmp = rans_args();
            rans_wall_distance(tmp, d_seg, (int)seg.size(), stream);
            FV_CUDA(cudaGetLastError());
            FV_CUDA(cudaStreamSynchronize(stream));
        }
    }

    // Initial condition, reference numbering then device order
    // (src/EulerFVMSolver.cpp:24-37).
    std::vector<St> u0(N);
    for (int c = 0; c < N; ++c) {
        double r, u, v, p;
        if (!ic.two_region) { r = ic.rho; u = ic.u; v = ic.v; p = ic.p; }
        else if (hm.cx[c] < ic.x0) { r = ic.rho_l; u = ic.u_l; v = ic.v_l; p = ic.p_l; }
        else { r = ic.rho_r; u = ic.u_r; v = ic.v_r; p = ic.p_r; }
        St s;
        s.r = r;
        s.ru = r * u;
        s.rv = r * v;
        s.E = p / (g - 1.0) + 0.5 * r * (u * u + v * v);
        u0[c] = s;
    }
    if (batch)  // each instance starts from its own freestream
        for (int i = 0; i < n_inst; ++i)
            for (int c = group_off[i]; c < group_off[i + 1]; ++c) {
                const double* q = batch_freestream + 4 * (size_t)i;
                u0[c].r = q[0]; u0[c].ru = q[1]; u0[c].rv = q[2]; u0[c].E = q[3];
            }
    upload_field(u0.data());
}

void Solver::ensure_history(int n) {
    if (hist && hist_cap >= n) return;
    const int cap = std::max(64, n);
    // Rows already recorded move to their slots in the larger ring (row =
    // step % capacity), so a later history() still returns them.
    int step = 0;
    if (hist) {
        FV_CUDA(cudaMemcpyAsync(&step, reinterpret_cast<const char*>(ctl) + offsetof(StepCtl, step), sizeof(int),
                                cudaMemcpyDeviceToHost, stream));
        FV_CUDA(cudaStreamSynchronize(stream));
    }
    auto regrow = [&](double*& ring, int width) {
        std::vector<double> next((size_t)width * cap, 0.0);
        if (ring) {
            std::vector<double> prev((size_t)width * hist_cap);
            FV_CUDA(cudaMemcpyAsync(prev.data(), ring, prev.size() * sizeof(double), cudaMemcpyDeviceToHost, stream));
            FV_CUDA(cudaStreamSynchronize(stream));
            for (int s = std::max(0, step - hist_cap); s < step; ++s)
                std::memcpy(&next[(size_t)width * (s % cap)], &prev[(size_t)width * (s % hist_cap)],
                            sizeof(double) * width);
        }
        double* h = nullptr;
        FV_CUDA(cudaMalloc(&h, sizeof(double) * next.size()));
        h2d_sync(h, next.data(), sizeof(double) * next.size(), stream);
        if (ring) cudaFree(ring);
        ring = h;
    };
    regrow(hist, 4);
    if (rans) regrow(nut_hist, 1);
    hist_cap = cap;
    for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
    graphs.clear();
}

RansArgs Solver::rans_args() const {
    RansArgs r = rs;
    r.ns = ns;
    r.hist = hist;
    r.hist_cap = hist_cap;
    r.nut_hist = nut_hist;
    return r;
}

O1Args Solver::o1_args() const {
    O1Args a;
    a.m = dm;
    a.U = U;
    a.ff = ff;
    a.dtf = dtf;
    a.ctl = ctl;
    a.partials = partials;
    a.hist = hist;
    a.hist_cap = hist_cap;
    a.bc = bc;
    a.gamma = gamma;
    a.exact_tol = opt.exact_tol;
    a.exact_max_iter = opt.exact_max_iter;
    a.flux = opt.flux;
    a.local_dt = opt.dt_mode == FV_DT_LOCAL;
    return a;
}

O2Args Solver::o2_args() const {
    O2Args a;
    a.m = dm;
    a.cnb = cnb;
    a.lsq = lsq;
    a.lsq_sum = lsq_sum;
    a.gg = gg;
    a.erf = erf;
    a.frf = frf;
    a.eps2 = eps2;
    a.fgeom32 = fgeom32;
    a.U = U;
    a.U0 = U0;
    a.W = W;
    a.G = G;
    a.ff = ff;
    a.cs = cs;
    a.dtf = dtf;
    a.dtv = dtv;
    a.ctl = ctl;
    a.partials = partials;
    a.hist = hist;
    a.hist_cap = hist_cap;
    a.bc = bc;
    a.gamma = gamma;
    a.venkat_k = opt.venkat_k;
    a.igm1 = 1.0 / (gamma - 1.0);
    a.gamma32 = (float)gamma;
    a.igm1_32 = (float)a.igm1;
    a.exact_tol = opt.exact_tol;
    a.exact_max_iter = opt.exact_max_iter;
    a.cell_inst = cell_inst;
    a.active = active;
    a.inst_fs = inst_fs;
    a.r2 = r2;
    a.lim_gu = nullptr;
    a.lim_psi = nullptr;
    a.psi_buf = psi_buf;
    a.psi_mode = psi_mode;
    a.d2 = d2;
    a.psi4 = psi4;
    a.fe = fe;
    a.forcing = forcing;
    a.resid = nullptr;
    return a;
}

void Solver::refresh_primitives() {
    if (!general) return;
    O2Args a = o2_args();
    if (cfg.fp32) o2::launch_prim_f32(a, stream);
    else o2::launch_prim_f64(a, stream);
    FV_CUDA(cudaGetLastError());
}

// Launches one step's kernels in order; kernel class of each launch is
// appended to *classes when given (0 gradients, 1 face fluxes, 2 update).
void Solver::launch_step(std::vector<int>* classes, std::vector<cudaEvent_t>* events, size_t* ev_pos) {
    auto mark = [&](int cls) {
        if (classes) classes->push_back(cls);
        if (events) FV_CUDA(cudaEventRecord((*events)[++*ev_pos], stream));
    };
    if (rans) {
        if (opt.strict) rans_launch_step(rans_args(), stream);
        else rans_launch_step_fast(rans_args(), stream);
        mark(1);
        return;
    }
    if (viscous) {
        // NS step: prim + gradients + face fluxes + cell pass, timed as one.
        if (opt.strict) ns_launch_step(ns, o1_args(), stream);
        else ns_launch_step_fast(ns, o1_args(), stream);
        mark(1);
        return;
    }
    if (!general) {
        O1Args a = o1_args();
        for (int part = 0; part < 2; ++part) {
            if (opt.strict) strict::launch_o1_part(a, part, stream);
            else fast::launch_o1_part(a, part, stream);
            mark(part + 1);
        }
        return;
    }
    O2Args a = o2_args();
    for (int st = 0; st < cfg.stages; ++st) {
        for (int part = (cfg.order == 2 ? 0 : 1); part < 3; ++part) {
            if (cfg.fp32) o2::launch_part_f32(a, cfg, st, part, stream);
            else o2::launch_part_f64(a, cfg, st, part, stream);
            mark(part);
        }
    }
    if (batch) {
        o2::launch_batch_norms(a, n_inst, inst_off, inst_norms, inst_iter, active, tol, stream);
        mark(2);
    }
}

bool dataflow_plan(const HostMesh& hm, const int* patch_type, int sms, DataflowPlan& p) {
    // One block per SM (fewer on a mesh of fewer 32-cell warps), each
    // owning a share of whole cell warps and the faces whose left cell it
    // owns; the dependency lists are the blocks it shares faces with.  A
    // mesh whose cell order leaves a block more neighbours than kDfMaxDeps
    // has no plan (the barrier form runs).
    const int N = hm.n_cells, F = hm.n_faces;
    if (sms < 1 || N < 1) return false;
    const int Wn = (N + 31) / 32;
    const int nb = std::min(sms, Wn);
    // Cell warps split into equal shares of weight: a warp with a cell on a
    // characteristic farfield face weighs 1.7, the others 1.  That face's
    // ghost state is the longest dependent chain of the face phase, so the
    // few blocks that hold those faces get fewer cells.
    std::vector<double> wsum(Wn + 1, 0.0);
    {
        std::vector<char> far(Wn, 0);
        for (int f = 0; f < F; ++f)
            if (hm.d_fr[f] < 0 && patch_type[hm.d_fpatch[f]] == FV_BC_CHAR_FARFIELD) far[hm.d_fl[f] / 32] = 1;
        for (int w = 0; w < Wn; ++w) wsum[w + 1] = wsum[w] + (far[w] ? 1.7 : 1.0);
    }
    p.nb = nb;
    p.cell_off.assign(nb + 1, 0);
    std::vector<int> owner(N);
    for (int b = 0; b <= nb; ++b) {
        const int w = b == nb ? Wn
                              : (int)(std::lower_bound(wsum.begin(), wsum.end(), wsum[Wn] * b / nb) - wsum.begin());
        p.cell_off[b] = (int)std::min<long long>(32LL * std::min(w, Wn), N);
    }
    for (int b = 0; b < nb; ++b)
        for (int c = p.cell_off[b]; c < p.cell_off[b + 1]; ++c) owner[c] = b;
    // A block's boundary faces come first: their ghost states are the
    // longest dependent chains of the face phase, and the lowest warps of a
    // block get issue priority.
    p.face_off.assign(nb + 1, 0);
    p.faces.assign(F, 0);
    for (int f = 0; f < F; ++f) ++p.face_off[owner[hm.d_fl[f]] + 1];
    for (int b = 0; b < nb; ++b) p.face_off[b + 1] += p.face_off[b];
    {
        std::vector<int> pos(p.face_off.begin(), p.face_off.end() - 1);
        for (int pass = 0; pass < 2; ++pass)
            for (int f = 0; f < F; ++f)
                if ((hm.d_fr[f] < 0) == (pass == 0)) p.faces[pos[owner[hm.d_fl[f]]]++] = f;
    }
    std::vector<std::vector<int>> dface(nb), dcell(nb);
    for (int f = 0; f < F; ++f) {
        if (hm.d_fr[f] < 0) continue;
        const int a = owner[hm.d_fl[f]], r = owner[hm.d_fr[f]];
        if (a == r) continue;
        dface[a].push_back(r);  // a's face phase reads r's cells
        dcell[r].push_back(a);  // r's cell phase reads a's faces
    }
    p.dep_face.clear();
    p.dep_cell.clear();
    p.dep_face_off.assign(nb + 1, 0);
    p.dep_cell_off.assign(nb + 1, 0);
    bool ok = true;
    for (int b = 0; b < nb; ++b) {
        for (auto* v : {&dface[b], &dcell[b]}) {
            std::sort(v->begin(), v->end());
            v->erase(std::unique(v->begin(), v->end()), v->end());
            if ((int)v->size() > kDfMaxDeps) ok = false;
        }
        p.dep_face.insert(p.dep_face.end(), dface[b].begin(), dface[b].end());
        p.dep_cell.insert(p.dep_cell.end(), dcell[b].begin(), dcell[b].end());
        p.dep_face_off[b + 1] = (int)p.dep_face.size();
        p.dep_cell_off[b + 1] = (int)p.dep_cell.size();
    }
    return ok;
}

void Solver::build_dataflow(const HostMesh& hm, int sms) {
    const int per_sm = opt.strict ? strict::o1df_max_blocks_per_sm(opt.flux) : fast::o1df_max_blocks_per_sm(opt.flux);
    if (per_sm < 1) return;
    DataflowPlan p;
    if (!dataflow_plan(hm, bc.type, sms, p)) return;
    const int nb = p.nb, Wn = (N + 31) / 32;
    std::vector<int> df = p.dep_face, dc = p.dep_cell;
    if (df.empty()) df.push_back(0);
    if (dc.empty()) dc.push_back(0);
    dfp.faces = dupload(p.faces, owned);
    dfp.face_off = dupload(p.face_off, owned);
    dfp.cell_off = dupload(p.cell_off, owned);
    dfp.dep_face = dupload(df, owned);
    dfp.dep_face_off = dupload(p.dep_face_off, owned);
    dfp.dep_cell = dupload(dc, owned);
    dfp.dep_cell_off = dupload(p.dep_cell_off, owned);
    // the per-warp partials of every step of a launch: up to kPersistChunk
    // steps, fewer on a large mesh (kDfPartialBytes)
    const size_t per_step = (size_t)Wn * 4 * sizeof(double);
    dfp.max_steps = (int)std::max<size_t>(8, std::min<size_t>(kPersistChunk, kDfPartialBytes / per_step));
    dfp.prog = dalloc<unsigned int>((size_t)nb * kDfProgStride, owned);
    dfp.wpart = dalloc<double>((size_t)dfp.max_steps * Wn * 4, owned);
    dfp.n_warps = Wn;
    df_grid = nb;
    dataflow_ok = true;
}

int Solver::persistent_form() const {
    if (!persistent) return 0;
    return dataflow_ok && !barrier_form ? 2 : 1;
}

void Solver::launch_steps(int k, std::vector<int>* classes, std::vector<cudaEvent_t>* events, size_t* ev_pos) {
    if (!persistent) {
        for (int i = 0; i < k; ++i) launch_step(classes, events, ev_pos);
        return;
    }
    // One launch per chunk (the dataflow form keeps every step's norm
    // partials of a launch), each re-arming the barrier's arrival counter.
    // The error flag is cleared once per fv_step (reset_wait_error), so
    // that a wait that ran out in an early launch is still reported.
    const O1Args a = o1_args();
    const bool df = persistent_form() == 2;
    for (int done = 0; done < k;) {
        const int n = df ? std::min(k - done, dfp.max_steps) : k;
        FV_CUDA(cudaMemsetAsync(pctl, 0, sizeof(int), stream));
        cudaError_t rc;
        if (df)
            rc = opt.strict ? strict::launch_o1_dataflow(a, Pc, pctl, dfp, n, df_grid, stream)
                            : fast::launch_o1_dataflow(a, Pc, pctl, dfp, n, df_grid, stream);
        else
            rc = opt.strict ? strict::launch_o1_persistent(a, Pc, pctl, n, p_grid, stream)
                            : fast::launch_o1_persistent(a, Pc, pctl, n, p_grid, stream);
        FV_CUDA(rc);
        done += n;
    }
    if (classes) classes->push_back(1);
    if (events) FV_CUDA(cudaEventRecord((*events)[++*ev_pos], stream));
}

void Solver::set_persistent(int mode) {
    if (mode < 0 || mode > 2) raise(FV_ERR_BAD_ARG, "persistent mode must be 0, 1 or 2");
    const bool on = mode != 0;
    if (on && !persistent_ok)
        raise(FV_ERR_UNSUPPORTED, "the persistent kernel covers the first-order forward-Euler FP64 Euler path on a "
                                  "device with cooperative launch");
    FV_CUDA(cudaStreamSynchronize(stream));
    persistent = on;
    barrier_form = mode == 2;
    for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
    graphs.clear();
}

void Solver::set_wait_limit(long long cycles, int phantom) {
    if (!persistent_ok) raise(FV_ERR_UNSUPPORTED, "no persistent kernel on this solver");
    if (cycles <= 0 || phantom < 0) raise(FV_ERR_BAD_ARG, "wait limit must be > 0 cycles, phantom arrivals >= 0");
    FV_CUDA(cudaStreamSynchronize(stream));
    h2d_sync(reinterpret_cast<char*>(pctl) + offsetof(PersistCtl, phantom), &phantom, sizeof(int), stream);
    h2d_sync(reinterpret_cast<char*>(pctl) + offsetof(PersistCtl, limit), &cycles, sizeof(long long), stream);
}

void Solver::reset_wait_error() {
    if (persistent_ok)
        FV_CUDA(cudaMemsetAsync(reinterpret_cast<char*>(pctl) + offsetof(PersistCtl, err), 0, sizeof(int), stream));
}

void Solver::check_persistent() {
    if (!persistent_ok) return;
    int err = 0;
    FV_CUDA(cudaMemcpyAsync(&err, reinterpret_cast<const char*>(pctl) + offsetof(PersistCtl, err), sizeof(int),
                            cudaMemcpyDeviceToHost, stream));
    FV_CUDA(cudaStreamSynchronize(stream));
    if (err)
        raise(FV_ERR_TIMEOUT,
              "a wait of the persistent kernel (grid barrier or neighbour progress) gave up (the state is unspecified)");
}

void Solver::step_timed(int n, double ms[3], int launches[3]) {
    if (n <= 0) raise(FV_ERR_BAD_ARG, "step_timed needs n > 0");
    ensure_history(n);
    const int per_step = viscous ? 1 : (general ? cfg.stages * (cfg.order == 2 ? 3 : 2) + (batch ? 1 : 0) : 2);
    const size_t need = persistent ? 2 : (size_t)n * per_step + 1;
    while (events.size() < need) {
        cudaEvent_t e;
        FV_CUDA(cudaEventCreate(&e));
        events.push_back(e);
    }
    std::vector<int> classes;
    classes.reserve(need);
    size_t pos = 0;
    if (persistent) reset_wait_error();
    FV_CUDA(cudaEventRecord(events[0], stream));
    launch_steps(n, &classes, &events, &pos);
    FV_CUDA(cudaGetLastError());
    FV_CUDA(cudaEventSynchronize(events[pos]));
    for (int k = 0; k < 3; ++k) { ms[k] = 0.0; launches[k] = 0; }
    for (size_t i = 0; i < classes.size(); ++i) {
        float t = 0.f;
        FV_CUDA(cudaEventElapsedTime(&t, events[i], events[i + 1]));
        ms[classes[i]] += t;
        launches[classes[i]] += 1;
    }
    steps_taken += n;
}

cudaGraphExec_t Solver::graph_for(int k) {
    auto it = graphs.find(k);
    if (it != graphs.end()) return it->second;
    cudaGraph_t g = nullptr;
    FV_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    launch_steps(k, nullptr, nullptr, nullptr);
    FV_CUDA(cudaStreamEndCapture(stream, &g));
    cudaGraphExec_t ge = nullptr;
    FV_CUDA(cudaGraphInstantiate(&ge, g, 0));
    cudaGraphDestroy(g);
    graphs[k] = ge;
    return ge;
}

void Solver::step_async(int n) {
    if (n < 0) raise(FV_ERR_BAD_ARG, "negative step count");
    ensure_history(std::min(n, 1 << 20));
    if (!mg.empty()) {
        // multigrid V-cycles: one smoothing iteration on this level, then
        // the coarse-grid correction (direct launches)
        for (int i = 0; i < n; ++i) {
            launch_step(nullptr, nullptr, nullptr);
            mg_cycle(0);
        }
        FV_CUDA(cudaGetLastError());
        steps_taken += n;
        return;
    }
    if (persistent) reset_wait_error();
    const int chunk = persistent ? kPersistChunk : kGraphChunk;
    int q = n / chunk, r = n % chunk;
    if (q) {
        cudaGraphExec_t ge = graph_for(chunk);
        for (int i = 0; i < q; ++i) FV_CUDA(cudaGraphLaunch(ge, stream));
    }
    if (r) FV_CUDA(cudaGraphLaunch(graph_for(r), stream));
    steps_taken += n;
}

void Solver::read_ctl(StepCtl& c) {
    FV_CUDA(cudaMemcpyAsync(&c, ctl, sizeof(c), cudaMemcpyDeviceToHost, stream));
    FV_CUDA(cudaStreamSynchronize(stream));
}

void Solver::history(int n, double* out) {
    if (n > hist_cap) raise(FV_ERR_BAD_ARG, "history longer than the recorded window");
    StepCtl c;
    read_ctl(c);
    std::vector<double> all(4 * (size_t)hist_cap);
    FV_CUDA(cudaMemcpy(all.data(), hist, all.size() * sizeof(double), cudaMemcpyDeviceToHost));
    for (int i = 0; i < n; ++i) {
        int s = c.step - n + i;
        int row = ((s % hist_cap) + hist_cap) % hist_cap;
        std::memcpy(out + 4 * i, all.data() + 4 * row, 4 * sizeof(double));
    }
}

// Device-order <-> reference-order permutation of the state, on the GPU so
// that host buffers cross PCIe/C2C once and untouched by the host.
__global__ void k_scatter_state(const St* __restrict__ U, St* __restrict__ out, const int* __restrict__ perm, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[perm[i]] = U[i];
}
__global__ void k_gather_state(const St* __restrict__ in, St* __restrict__ U, const int* __restrict__ perm, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) U[i] = in[perm[i]];
}

void Solver::download_field(double* out) {
    k_scatter_state<<<(N + 255) / 256, 256, 0, stream>>>(U, staging, d_perm, N);
    FV_CUDA(cudaGetLastError());
    FV_CUDA(cudaMemcpyAsync(out, staging, sizeof(St) * (size_t)N, cudaMemcpyDeviceToHost, stream));
    FV_CUDA(cudaStreamSynchronize(stream));
}

void Solver::upload_field(const void* in_ref_order) {
    FV_CUDA(cudaMemcpyAsync(staging, in_ref_order, sizeof(St) * (size_t)N, cudaMemcpyHostToDevice, stream));
    k_gather_state<<<(N + 255) / 256, 256, 0, stream>>>(staging, U, d_perm, N);
    FV_CUDA(cudaGetLastError());
    refresh_primitives();
    // residual() resets to zero (include/EulerFVMSolver.h:151-155)
    static const double z[4] = {0, 0, 0, 0};
    static const int zi = 0;
    FV_CUDA(cudaMemcpyAsync(reinterpret_cast<char*>(ctl) + offsetof(StepCtl, norms), z, sizeof(z),
                            cudaMemcpyHostToDevice, stream));
    FV_CUDA(cudaMemcpyAsync(reinterpret_cast<char*>(ctl) + offsetof(StepCtl, nonfinite), &zi, sizeof(zi),
                            cudaMemcpyHostToDevice, stream));
    FV_CUDA(cudaStreamSynchronize(stream));
}

void Solver::set_launch(int bg, int bf, int bc) {
    for (int b : {bg, bf, bc})
        if (b < kMinBlock || b > kMaxBlock || b % 32 != 0)
            raise(FV_ERR_BAD_ARG, "launch shape: 128..512 threads per block, a multiple of 32");
    if (!general || viscous) raise(FV_ERR_UNSUPPORTED, "launch shapes apply to the second-order / multi-stage path");
    FV_CUDA(cudaStreamSynchronize(stream));
    cfg.blk_grad = bg;
    cfg.blk_face = bf;
    cfg.blk_cell = bc;
    for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
    graphs.clear();
}

void Solver::freeze_limiter(bool on) {
    if (viscous) raise(FV_ERR_UNSUPPORTED, "limiter freezing: Euler solvers");
    if (!general || opt.order != 2 || opt.limiter == FV_LIM_NONE) return;  // no limiter to freeze
    FV_CUDA(cudaStreamSynchronize(stream));
    for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
    graphs.clear();
    if (!on) {
        psi_mode = 0;
        return;
    }
    if (!psi_buf) psi_buf = dalloc_owned<char>(4 * (size_t)N * (cfg.fp32 ? sizeof(float) : sizeof(double)));
    // capture: one gradient evaluation at the current state stores psi
    refresh_primitives();
    O2Args a = o2_args();
    a.psi_mode = 1;
    if (cfg.fp32) o2::launch_part_f32(a, cfg, 0, 0, stream);
    else o2::launch_part_f64(a, cfg, 0, 0, stream);
    FV_CUDA(cudaGetLastError());
    FV_CUDA(cudaStreamSynchronize(stream));
    psi_mode = 2;
}

void Solver::limiter_values(double* out_ref, const double* in_ref) {
    if (!general || opt.order != 2 || opt.limiter == FV_LIM_NONE)
        raise(FV_ERR_UNSUPPORTED, "limiter values: second order with a limiter");
    if (in_ref) {
        // import: freeze at the given values
        FV_CUDA(cudaStreamSynchronize(stream));
        for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
        graphs.clear();
        const size_t esz = cfg.fp32 ? sizeof(float) : sizeof(double);
        if (!psi_buf) psi_buf = dalloc_owned<char>(4 * (size_t)N * esz);
        std::vector<double> d(4 * (size_t)N);
        std::vector<float> f(cfg.fp32 ? 4 * (size_t)N : 0);
        for (int i = 0; i < N; ++i)
            for (int k = 0; k < 4; ++k) {
                const double v = in_ref[4 * (size_t)perm[i] + k];
                if (!(v >= 0.0 && v <= 1.0)) raise(FV_ERR_BAD_ARG, "limiter values must lie in [0, 1]");
                if (cfg.fp32) f[4 * (size_t)i + k] = (float)v;
                else d[4 * (size_t)i + k] = v;
            }
        h2d_sync(psi_buf, cfg.fp32 ? static_cast<const void*>(f.data()) : static_cast<const void*>(d.data()),
                 4 * (size_t)N * esz, stream);
        psi_mode = 2;
    }
    if (out_ref) {
        if (psi_mode != 2) raise(FV_ERR_BAD_ARG, "limiter values: the limiter is not frozen");
        FV_CUDA(cudaStreamSynchronize(stream));
        std::vector<double> d(4 * (size_t)N);
        if (cfg.fp32) {
            std::vector<float> f(4 * (size_t)N);
            FV_CUDA(cudaMemcpy(f.data(), psi_buf, sizeof(float) * f.size(), cudaMemcpyDeviceToHost));
            for (size_t i = 0; i < f.size(); ++i) d[i] = f[i];
        } else {
            FV_CUDA(cudaMemcpy(d.data(), psi_buf, sizeof(double) * d.size(), cudaMemcpyDeviceToHost));
        }
        for (int i = 0; i < N; ++i)
            for (int k = 0; k < 4; ++k) out_ref[4 * (size_t)perm[i] + k] = d[4 * (size_t)i + k];
    }
}

void Solver::autotune(int n, int out[3]) {
    if (n <= 0) raise(FV_ERR_BAD_ARG, "autotune needs n > 0");
    if (!general || viscous) raise(FV_ERR_UNSUPPORTED, "autotune applies to the second-order / multi-stage path");
    // save the state the trial steps change
    FV_CUDA(cudaStreamSynchronize(stream));
    StepCtl c0;
    read_ctl(c0);
    FV_CUDA(cudaMemcpyAsync(staging, U, sizeof(St) * (size_t)N, cudaMemcpyDeviceToDevice, stream));
    std::vector<int> act, it;
    std::vector<double> nrm;
    if (batch) {
        act.resize(n_inst); it.resize(n_inst); nrm.resize(4 * (size_t)n_inst);
        FV_CUDA(cudaMemcpy(act.data(), active, sizeof(int) * n_inst, cudaMemcpyDeviceToHost));
        FV_CUDA(cudaMemcpy(it.data(), inst_iter, sizeof(int) * n_inst, cudaMemcpyDeviceToHost));
        FV_CUDA(cudaMemcpy(nrm.data(), inst_norms, sizeof(double) * nrm.size(), cudaMemcpyDeviceToHost));
    }
    const int cand[3] = {128, 256, 512};
    double best[3] = {1e300, 1e300, 1e300};
    int pick[3] = {256, 256, 256};
    for (int b : cand) {
        set_launch(b, b, b);
        double ms[3];
        int l[3];
        step_timed(1, ms, l);  // warm-up at this shape
        step_timed(n, ms, l);
        for (int k = 0; k < 3; ++k)
            if (l[k] > 0 && ms[k] < best[k]) { best[k] = ms[k]; pick[k] = b; }
    }
    set_launch(pick[0], pick[1], pick[2]);
    // restore
    FV_CUDA(cudaMemcpyAsync(U, staging, sizeof(St) * (size_t)N, cudaMemcpyDeviceToDevice, stream));
    FV_CUDA(cudaMemcpyAsync(ctl, &c0, sizeof(c0), cudaMemcpyHostToDevice, stream));
    if (batch) {
        FV_CUDA(cudaMemcpyAsync(active, act.data(), sizeof(int) * n_inst, cudaMemcpyHostToDevice, stream));
        FV_CUDA(cudaMemcpyAsync(inst_iter, it.data(), sizeof(int) * n_inst, cudaMemcpyHostToDevice, stream));
        FV_CUDA(cudaMemcpyAsync(inst_norms, nrm.data(), sizeof(double) * nrm.size(), cudaMemcpyHostToDevice, stream));
    }
    refresh_primitives();
    FV_CUDA(cudaStreamSynchronize(stream));
    steps_taken -= (long long)3 * (n + 1);
    for (int k = 0; k < 3; ++k) out[k] = pick[k];
}

void Solver::set_cfl(double cfl) {
    FV_CUDA(cudaMemcpyAsync(reinterpret_cast<char*>(ctl) + offsetof(StepCtl, cfl), &cfl, sizeof(cfl),
                            cudaMemcpyHostToDevice, stream));
    FV_CUDA(cudaStreamSynchronize(stream));
}

void Solver::set_stream(void* s) {
    FV_CUDA(cudaStreamSynchronize(stream));
    for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
    graphs.clear();
    if (own_stream) cudaStreamDestroy(stream);
    if (s) {
        stream = static_cast<cudaStream_t>(s);
        own_stream = false;
    } else {
        FV_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        own_stream = true;
    }
    for (MGLevel& L : mg) L.s->set_stream(stream);  // coarse levels run on this stream
}

// compute_wall_traction + compute_wall_forces (src/WallTraction.cpp:95-217),
// domain total over the wall faces in reference face order.  Wall pressure
// is the owner cell's pressure (include/WallTraction.h:59-66); the viscous
// solver adds the wall shear from the corrected face gradients, the
// inviscid one has none.
void Solver::wall_forces(const double ref[7], double out[11], int instance) {
    const size_t nw = wall_faces.size();
    std::vector<double> tau(nw, 0.0), pw(nw, 0.0);
    if (viscous) {
        std::vector<double2> tp(nw);
        if (rans) {
            if (opt.strict) rans_launch_wall(rans_args(), ns_wall_faces, (int)nw, ns_wall_out, stream);
            else rans_launch_wall_fast(rans_args(), ns_wall_faces, (int)nw, ns_wall_out, stream);
        } else {
            if (opt.strict) ns_launch_wall(ns, ns_wall_faces, (int)nw, ns_wall_out, stream);
            else ns_launch_wall_fast(ns, ns_wall_faces, (int)nw, ns_wall_out, stream);
        }
        FV_CUDA(cudaGetLastError());
        if (nw) FV_CUDA(cudaMemcpyAsync(tp.data(), ns_wall_out, sizeof(double2) * nw, cudaMemcpyDeviceToHost, stream));
        FV_CUDA(cudaStreamSynchronize(stream));
        for (size_t i = 0; i < nw; ++i) { tau[i] = tp[i].x; pw[i] = tp[i].y; }
    } else {
        std::vector<double> f(4 * (size_t)N);
        download_field(f.data());
        for (size_t i = 0; i < nw; ++i) {
            const double* s = f.data() + 4 * (size_t)wall_faces[i].cell;
            double u = s[1] / s[0], v = s[2] / s[0];
            pw[i] = (gamma - 1.0) * (s[3] - 0.5 * s[0] * (u * u + v * v));
        }
    }
    double vmag = std::hypot(ref[1], ref[2]);
    double dx = ref[1] / vmag, dy = ref[2] / vmag;
    double lx = -dy, ly = dx;
    double qL = 0.5 * ref[0] * vmag * vmag * ref[4];
    double qL2 = qL * ref[4];
    double fd = 0, pd = 0, td = 0, lift = 0, mom = 0;
    size_t counted = 0;
    for (size_t i = 0; i < nw; ++i) {
        if (instance >= 0 && wall_inst[i] != instance) continue;
        ++counted;
        const WallFace& w = wall_faces[i];
        const double p = pw[i];
        const double tx = -w.ny, ty = w.nx;  // rotate90 (src/WallTraction.cpp:11-13)
        double fx = w.area * tau[i] * tx, fy = w.area * tau[i] * ty;
        double px = w.area * p * w.nx, py = w.area * p * w.ny;
        double rx = w.xm - ref[5], ry = w.ym - ref[6];
        double dfx = fx + px, dfy = fy + py;
        double fdi = fx * dx + fy * dy, pdi = px * dx + py * dy;
        fd += fdi;
        pd += pdi;
        td += fdi + pdi;
        lift += (fx + px) * lx + (fy + py) * ly;
        mom += rx * dfy - ry * dfx;
    }
    out[0] = fd; out[1] = pd; out[2] = td; out[3] = lift; out[4] = mom;
    out[5] = fd / qL; out[6] = pd / qL; out[7] = td / qL; out[8] = lift / qL; out[9] = mom / qL2;
    out[10] = (double)counted;
}

}  // namespace fvgb

// ===========================================================================
// C ABI
// ===========================================================================
using fvgb::Solver;
using fvgb::guarded;

extern "C" {

const char* fv_last_error(void) { return fvgb::last_error(); }
int fv_abi_version(void) { return 100; }
int fv_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

int fv_mesh_create_polygons(int32_t n_nodes, const double* xy, int32_t n_cells, const int64_t* cell_off,
                            const int32_t* cell_nodes, int32_t n_bedges, const int32_t* bedge_nodes,
                            const int32_t* bedge_patch, int32_t n_patches, int32_t reorder, fv_mesh_t* out) {
    return guarded([&] {
        if (!out) fvgb::raise(FV_ERR_BAD_ARG, "null output handle");
        auto m = std::make_unique<fv_mesh_s>();
        fvgb::build_from_polygons(m->h, n_nodes, xy, n_cells, cell_off, cell_nodes, n_bedges, bedge_nodes,
                                  bedge_patch, n_patches);
        m->h.build_device_layout(reorder);
        *out = m.release();
    });
}

int fv_mesh_create_faces(int32_t n_nodes, const double* xy, int32_t n_faces, const int32_t* face_nodes,
                         const int32_t* face_cells, const int32_t* face_patch, int32_t n_cells,
                         const int32_t* cell_face_off, const int32_t* cell_faces, const double* cell_geom,
                         int32_t n_patches, int32_t reorder, fv_mesh_t* out) {
    return guarded([&] {
        if (!out) fvgb::raise(FV_ERR_BAD_ARG, "null output handle");
        auto m = std::make_unique<fv_mesh_s>();
        fvgb::build_from_faces(m->h, n_nodes, xy, n_faces, face_nodes, face_cells, face_patch, n_cells,
                               cell_face_off, cell_faces, cell_geom, n_patches);
        m->h.build_device_layout(reorder);
        *out = m.release();
    });
}

int fv_mesh_counts(fv_mesh_t mesh, int64_t counts[5]) {
    return guarded([&] {
        if (!mesh || !counts) fvgb::raise(FV_ERR_BAD_ARG, "null argument");
        const HostMesh& h = mesh->h;
        counts[0] = h.n_cells;
        counts[1] = h.n_faces;
        counts[2] = h.n_faces - h.n_int_faces;
        counts[3] = h.n_patches;
        counts[4] = (int64_t)h.cf.size();
    });
}

int fv_mesh_export(fv_mesh_t mesh, int32_t* face_i32, double* face_f64, double* cell_f64, int32_t* cell_face_off,
                   int32_t* cell_faces) {
    return guarded([&] {
        if (!mesh) fvgb::raise(FV_ERR_BAD_ARG, "null mesh");
        const HostMesh& h = mesh->h;
        for (int32_t f = 0; f < h.n_faces; ++f) {
            if (face_i32) {
                int32_t* o = face_i32 + 5 * (size_t)f;
                o[0] = h.fn1[f]; o[1] = h.fn2[f]; o[2] = h.fl[f]; o[3] = h.fr[f]; o[4] = h.fpatch[f];
            }
            if (face_f64) {
                double* o = face_f64 + 5 * (size_t)f;
                o[0] = h.fnx[f]; o[1] = h.fny[f]; o[2] = h.farea[f]; o[3] = h.fxm[f]; o[4] = h.fym[f];
            }
        }
        for (int32_t c = 0; c < h.n_cells; ++c)
            if (cell_f64) {
                cell_f64[3 * (size_t)c] = h.vol[c];
                cell_f64[3 * (size_t)c + 1] = h.cx[c];
                cell_f64[3 * (size_t)c + 2] = h.cy[c];
            }
        if (cell_face_off) std::copy(h.cf_off.begin(), h.cf_off.end(), cell_face_off);
        if (cell_faces) std::copy(h.cf.begin(), h.cf.end(), cell_faces);
    });
}

int fv_mesh_permutation(fv_mesh_t mesh, int32_t* perm) {
    return guarded([&] {
        if (!mesh || !perm) fvgb::raise(FV_ERR_BAD_ARG, "null argument");
        std::copy(mesh->h.perm.begin(), mesh->h.perm.end(), perm);
    });
}

int fv_mesh_dataflow_plan(fv_mesh_t mesh, const int32_t* patch_types, int32_t blocks, int32_t counts[4],
                          int32_t* cell_off, int32_t* face_off, int32_t* faces, int32_t* dep_face_off,
                          int32_t* dep_face, int32_t* dep_cell_off, int32_t* dep_cell, int32_t* face_cells) {
    return guarded([&] {
        if (!mesh || !patch_types || !counts) fvgb::raise(FV_ERR_BAD_ARG, "null argument");
        if (blocks < 1) fvgb::raise(FV_ERR_BAD_ARG, "blocks must be >= 1");
        const fvgb::HostMesh& h = mesh->h;
        for (int p = 0; p < h.n_patches; ++p)
            if (patch_types[p] < FV_BC_WALL || patch_types[p] > FV_BC_NOSLIP)
                fvgb::raise(FV_ERR_BAD_ARG, "unknown boundary type");
        fvgb::DataflowPlan p;
        const bool ok = fvgb::dataflow_plan(h, patch_types, blocks, p);
        counts[0] = p.nb;
        counts[1] = (int32_t)p.dep_face.size();
        counts[2] = (int32_t)p.dep_cell.size();
        counts[3] = ok ? 1 : 0;
        auto put = [](const std::vector<int>& v, int32_t* out) {
            if (out) std::copy(v.begin(), v.end(), out);
        };
        put(p.cell_off, cell_off);
        put(p.face_off, face_off);
        put(p.faces, faces);
        put(p.dep_face_off, dep_face_off);
        put(p.dep_face, dep_face);
        put(p.dep_cell_off, dep_cell_off);
        put(p.dep_cell, dep_cell);
        if (face_cells)
            for (int f = 0; f < h.n_faces; ++f) {
                face_cells[2 * (size_t)f] = h.d_fl[f];
                face_cells[2 * (size_t)f + 1] = h.d_fr[f];
            }
    });
}

int fv_mesh_agglomerate(fv_mesh_t mesh, int32_t counts[2], int32_t* agg, double* coarse_cell_f64,
                        int32_t* coarse_face_i32, double* coarse_face_f64) {
    return guarded([&] {
        if (!mesh || !counts) fvgb::raise(FV_ERR_BAD_ARG, "null argument");
        std::vector<int32_t> a;
        HostMesh c;
        agglomerate(mesh->h, a, c);
        counts[0] = c.n_cells;
        counts[1] = c.n_faces;
        if (agg) std::copy(a.begin(), a.end(), agg);
        for (int32_t k = 0; k < c.n_cells && coarse_cell_f64; ++k) {
            coarse_cell_f64[3 * (size_t)k] = c.vol[k];
            coarse_cell_f64[3 * (size_t)k + 1] = c.cx[k];
            coarse_cell_f64[3 * (size_t)k + 2] = c.cy[k];
        }
        for (int32_t f = 0; f < c.n_faces; ++f) {
            if (coarse_face_i32) {
                int32_t* o = coarse_face_i32 + 3 * (size_t)f;
                o[0] = c.fl[f]; o[1] = c.fr[f]; o[2] = c.fpatch[f];
            }
            if (coarse_face_f64) {
                double* o = coarse_face_f64 + 3 * (size_t)f;
                o[0] = c.fnx[f]; o[1] = c.fny[f]; o[2] = c.farea[f];
            }
        }
    });
}

int fv_mesh_destroy(fv_mesh_t mesh) {
    delete mesh;
    return FV_OK;
}

void fv_options_default(fv_options_t* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->flux = FV_FLUX_RUSANOV;
    o->order = 1;
    o->gradient = FV_GRAD_LSQ;
    o->limiter = FV_LIM_VENKAT;
    o->venkat_k = 5.0;
    o->rk_stages = 1;
    o->dt_mode = FV_DT_GLOBAL;
    o->precision = FV_PREC_FP64;
    o->strict = 0;
    o->exact_tol = 1e-6;
    o->exact_max_iter = 20;
    o->viscous = 0;
    o->gas_constant = 287.0;
    o->mu = 0.0;
    o->prandtl = 0.72;
    o->prandtl_t = 0.9;
    o->initial_nut = 0.0;
    // SAModelConstants defaults (include/SpalartAllmaras.h:13-23)
    const double sa[9] = {0.1355, 0.622, 2.0 / 3.0, 0.41, 0.3, 2.0, 7.1, 0.7, 0.9};
    for (int i = 0; i < 9; ++i) o->sa[i] = sa[i];
}

int fv_solver_create(fv_mesh_t mesh, const fv_bc_t* bcs, int32_t n_bcs, double gamma, double cfl, const fv_ic_t* ic,
                     const fv_options_t* opt, fv_solver_t* out) {
    return guarded([&] {
        if (!mesh || !out || !ic || (!bcs && mesh->h.n_patches > 0)) fvgb::raise(FV_ERR_BAD_ARG, "null argument");
        fv_options_t o;
        if (opt) o = *opt;
        else fv_options_default(&o);
        auto s = std::make_unique<fv_solver_s>();
        s->s.init(mesh->h, bcs, n_bcs, gamma, cfl, *ic, o);
        *out = s.release();
    });
}

int fv_solver_destroy(fv_solver_t s) {
    delete s;
    return FV_OK;
}

int fv_solver_set_stream(fv_solver_t s, void* stream) {
    return guarded([&] {
        if (!s) fvgb::raise(FV_ERR_BAD_ARG, "null solver");
        s->s.set_stream(stream);
    });
}

int fv_step_async(fv_solver_t s, int32_t n) {
    return guarded([&] {
        if (!s) fvgb::raise(FV_ERR_BAD_ARG, "null solver");
        s->s.step_async(n);
    });
}

int fv_step(fv_solver_t s, int32_t n, double* history) {
    int rc = guarded([&] {
        if (!s) fvgb::raise(FV_ERR_BAD_ARG, "null solver");
        s->s.step_async(n);
        fvgb::StepCtl c;
        s->s.read_ctl(c);
        s->s.check_persistent();
        if (history && n > 0) s->s.history(n, history);
        if (c.nonfinite) fvgb::raise(FV_ERR_NONFINITE, "non-finite residual norm");
    });
    return rc;
}

int fv_step_timed(fv_solver_t s, int32_t n, double kernel_ms[3], int32_t launches[3]) {
    return guarded([&] {
        if (!s || !kernel_ms || !launches) fvgb::raise(FV_ERR_BAD_ARG, "null argument");
        int l[3];
        s->s.step_timed(n, kernel_ms, l);
        for (int k = 0; k < 3; ++k) launches[k] = l[k];
        fvgb::StepCtl c;
        s->s.read_ctl(c);
        s->s.check_persistent();
        if (c.nonfinite) fvgb::raise(FV_ERR_NONFINITE, "non-finite residual norm");
    });
}

int fv_get_history(fv_solver_t s, int32_t n, double* history) {
    return guarded([&] {
        if (!s || !history || n < 0) fvgb::raise(FV_ERR_BAD_ARG, "bad argument");
        s->s.history(n, history);
    });
}

int fv_get_field(fv_solver_t s, double* U) {
    return guarded([&] {
        if (!s || !U) fvgb::raise(FV_ERR_BAD_ARG, "null argument");
        s->s.download_field(U);
    });
}

int fv_set_field(fv_solver_t s, const double* U) {
    return guarded([&] {
        if (!s || !U) fvgb::raise(FV_ERR_BAD_ARG, "null argument");
        s->s.upload_field(U);
    });
}

int fv_get_residual(fv_solver_t s, double norms[4]) {
    return guarded([&] {
        if (!s || !norms) fvgb::raise(FV_ERR_BAD_ARG, "null argument");
        fvgb::StepCtl c;
        s->s.read_ctl(c);
        for (int k = 0; k < 4; ++k) norms[k] = c.norms[k];
    });
}

int fv_solver_set_launch(fv_solver_t s, const int32_t blocks[3]) {
    return guarded([&] {
        if (!s || !blocks) fvgb::raise(FV_ERR_BAD_ARG, "null argument");
        s->s.set_launch(blocks[0], blocks[1], blocks[2]);
    });
}

int fv_solver_set_persistent(fv_solver_t s, int32_t on) {
    return guarded([&] {
        if (!s) fvgb::raise(FV_ERR_BAD_ARG, "null solver");
        s->s.set_persistent(on);
    });
}

int fv_solver_persistent(fv_solver_t s, int32_t* on, int32_t* grid) {
    return guarded([&] {
        if (!s) fvgb::raise(FV_ERR_BAD_ARG, "null solver");
        const int form = s->s.persistent_form();
        if (on) *on = form;
        if (grid) *grid = form == 2 ? s->s.df_grid : s->s.p_grid;
    });
}

int fv_solver_set_wait_limit(fv_solver_t s, int64_t cycles, int32_t phantom_arrivals) {
    return guarded([&] {
        if (!s) fvgb::raise(FV_ERR_BAD_ARG, "null solver");
        s->s.set_wait_limit(cycles, phantom_arrivals);
    });
}

int fv_solver_freeze_limiter(fv_solver_t s, int32_t on) {
    return guarded([&] {
        if (!s) fvgb::raise(FV_ERR_BAD_ARG, "null solver");
        s->s.freeze_limiter(on != 0);
    });
}

int fv_solver_limiter_values(fv_solver_t s, double* psi_out, const double* psi_in) {
    return guarded([&] {
        if (!s) fvgb::raise(FV_ERR_BAD_ARG, "null solver");
        s->s.limiter_values(psi_out, psi_in);
    });
}

int fv_solver_autotune(fv_solver_t s, int32_t steps, int32_t blocks[3]) {
    return guarded([&] {
        if (!s) fvgb::raise(FV_ERR_BAD_ARG, "null solver");
        int b[3];
        s->s.autotune(steps, b);
        if (blocks)
            for (int k = 0; k < 3; ++k) blocks[k] = b[k];
    });
}

static void get_cell_scalar(Solver& v, const double* dev, double* out) {
    std::vector<double> d(v.N);
    FV_CUDA(cudaStreamSynchronize(v.stream));
    FV_CUDA(cudaMemcpy(d.data(), dev, sizeof(double) * v.N, cudaMemcpyDeviceToHost));
    for (int i = 0; i < v.N; ++i) out[v.perm[i]] = d[i];
}

int fv_get_nut(fv_solver_t s, double* nut) {
    return guarded([&] {
        if (!s || !nut) fvgb::raise(FV_ERR_BAD_ARG, "null argument");
        if (!s->s.rans) fvgb::raise(FV_ERR_UNSUPPORTED, "not a RANS-SA solver");
        get_cell_scalar(s->s, s->s.rs.nut, nut);
    });
}

int fv_set_nut(fv_solver_t s, const double* nut) {
    return guarded([&] {
        if (!s || !nut) fvgb::raise(FV_ERR_BAD_ARG, "null argument");
        Solver& v = s->s;
        if (!v.rans) fvgb::raise(FV_ERR_UNSUPPORTED, "not a RANS-SA solver");
        std::vector<double> d(v.N);
        for (int i = 0; i < v.N; ++i) d[i] = nut[v.perm[i]];
        FV_CUDA(cudaStreamSynchronize(v.stream));
        fvgb::h2d_sync(v.rs.nut, d.data(), sizeof(double) * v.N, v.stream);
        const double z = 0.0;
        fvgb::h2d_sync(v.rs.nut_norm, &z, sizeof(z), v.stream);
    });
}

int fv_get_nut_residual(fv_solver_t s, double* norm) {
    return guarded([&] {
        if (!s || !norm) fvgb::raise(FV_ERR_BAD_ARG, "null argument");
        if (!s->s.rans) fvgb::raise(FV_ERR_UNSUPPORTED, "not a RANS-SA solver");
        FV_CUDA(cudaStreamSynchronize(s->s.stream));
        FV_CUDA(cudaMemcpy(norm, s->s.rs.nut_norm, sizeof(double), cudaMemcpyDeviceToHost));
    });
}

int fv_get_wall_distance(fv_solver_t s, double* d) {
    return guarded([&] {
        if (!s || !d) fvgb::raise(FV_ERR_BAD_ARG, "null argument");
        if (!s->s.rans) fvgb::raise(FV_ERR_UNSUPPORTED, "not a RANS-SA solver");
        get_cell_scalar(s->s, s->s.rs.walld, d);
    });
}

int fv_set_cfl(fv_solver_t s, double cfl) {
    return guarded([&] {
        if (!s || !(cfl > 0.0)) fvgb::raise(FV_ERR_BAD_ARG, "bad argument");
        s->s.set_cfl(cfl);
    });
}

int fv_get_gamma(fv_solver_t s, double* g) {
    return guarded([&] {
        if (!s || !g) fvgb::raise(FV_ERR_BAD_ARG, "null argument");
        *g = s->s.gamma;
    });
}

int fv_device_state(fv_solver_t s, void** U_dev, void** stream) {
    return guarded([&] {
        if (!s) fvgb::raise(FV_ERR_BAD_ARG, "null solver");
        if (U_dev) *U_dev = s->s.U;
        if (stream) *stream = s->s.stream;
    });
}

int fv_wall_forces(fv_solver_t s, const double ref[7], double out[11]) {
    return guarded([&] {
        if (!s || !ref || !out) fvgb::raise(FV_ERR_BAD_ARG, "null argument");
        s->s.wall_forces(ref, out);
    });
}

// ---------------------------------------------------------------- batch ----
int fv_mesh_create_batch(int32_t n, const fv_mesh_t* meshes, int32_t reorder, fv_mesh_t* out) {
    return guarded([&] {
        if (n <= 0 || !meshes || !out) fvgb::raise(FV_ERR_BAD_ARG, "bad argument");
        std::vector<const HostMesh*> parts;
        for (int i = 0; i < n; ++i) {
            if (!meshes[i]) fvgb::raise(FV_ERR_BAD_ARG, "null mesh");
            parts.push_back(&meshes[i]->h);
        }
        auto m = std::make_unique<fv_mesh_s>();
        fvgb::concat_meshes(parts, m->h);
        m->h.build_device_layout(reorder);
        *out = m.release();
    });
}

int fv_batch_create(fv_mesh_t mesh, const fv_bc_t* bcs, int32_t n_bcs, const double* inst_freestream, double gamma,
                    double cfl, const fv_options_t* opt, fv_solver_t* out) {
    return guarded([&] {
        if (!mesh || !out || !inst_freestream || !opt) fvgb::raise(FV_ERR_BAD_ARG, "null argument");
        fv_ic_t ic;
        std::memset(&ic, 0, sizeof(ic));
        ic.rho = 1.0;
        ic.p = 1.0;
        auto s = std::make_unique<fv_solver_s>();
        s->s.init(mesh->h, bcs, n_bcs, gamma, cfl, ic, *opt, inst_freestream);
        *out = s.release();
    });
}

int fv_batch_set_tolerance(fv_solver_t s, double tol_rho) {
    return guarded([&] {
        if (!s || !s->s.batch) fvgb::raise(FV_ERR_BAD_ARG, "not a batched solver");
        s->s.tol = tol_rho;
        FV_CUDA(cudaStreamSynchronize(s->s.stream));
        for (auto& kv : s->s.graphs) cudaGraphExecDestroy(kv.second);  // the tolerance is a launch parameter
        s->s.graphs.clear();
    });
}

int fv_batch_status(fv_solver_t s, int32_t* active, int32_t* iterations, double* norms) {
    return guarded([&] {
        if (!s || !s->s.batch) fvgb::raise(FV_ERR_BAD_ARG, "not a batched solver");
        fvgb::Solver& v = s->s;
        FV_CUDA(cudaStreamSynchronize(v.stream));
        if (active) FV_CUDA(cudaMemcpy(active, v.active, sizeof(int) * v.n_inst, cudaMemcpyDeviceToHost));
        if (iterations) FV_CUDA(cudaMemcpy(iterations, v.inst_iter, sizeof(int) * v.n_inst, cudaMemcpyDeviceToHost));
        if (norms) FV_CUDA(cudaMemcpy(norms, v.inst_norms, sizeof(double) * 4 * v.n_inst, cudaMemcpyDeviceToHost));
    });
}

int fv_batch_set_active(fv_solver_t s, int32_t instance, int32_t active) {
    return guarded([&] {
        if (!s || !s->s.batch || instance < 0 || instance >= s->s.n_inst || (active != 0 && active != 1))
            fvgb::raise(FV_ERR_BAD_ARG, "bad argument");
        fvgb::Solver& v = s->s;
        const int a = active;
        FV_CUDA(cudaMemcpyAsync(v.active + instance, &a, sizeof(int), cudaMemcpyHostToDevice, v.stream));
        FV_CUDA(cudaStreamSynchronize(v.stream));
    });
}

int fv_batch_wall_forces(fv_solver_t s, int32_t instance, const double ref[7], double out[11]) {
    return guarded([&] {
        if (!s || !s->s.batch || !ref || !out || instance < 0 || instance >= s->s.n_inst)
            fvgb::raise(FV_ERR_BAD_ARG, "bad argument");
        s->s.wall_forces(ref, out, instance);
    });
}

}  // extern "C"
