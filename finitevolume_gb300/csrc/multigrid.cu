// Agglomeration multigrid for steady solves: the full approximation scheme
// (FAS) V-cycle over coarse levels built by agglomerate() (mesh_host.cpp).
// No reference counterpart: the reference advances its explicit scheme
// without convergence acceleration.
//
// After one smoothing iteration on level l, the residual R_l(U_l) (with
// the level's own forcing) is restricted: the coarse state is the
// volume-weighted mean U_c0 = sum V U / sum V and the coarse forcing
// P = sum R_l - R_c(U_c0), so that the coarse problem R_c(U_c) + P = 0 has
// U_c0 as its solution exactly when the finer residual vanishes; the
// coarse level (first order, SSP-RK3, local dt) is smoothed and corrected
// recursively, and the finer state gets U_l += relax (U_c - U_c0),
// injected cell by cell and halved (up to three times, then dropped) where
// it would change the density or pressure by more than a factor of two.  The converged finer solution is that of the
// scheme without multigrid: at convergence R_l = 0 and the corrections
// vanish.  Every kernel writes its own cell; the restriction sums each
// coarse cell's finer cells in a fixed order, so runs are bit reproducible.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "capi_internal.h"
#include "physics.cuh"

namespace fvgb {
const HostMesh& host_mesh_of(const fv_mesh_s* m);
}

namespace mgk {

using fvgb::St;

__global__ void k_restrict(int nc, const int* __restrict__ off, const int* __restrict__ fine,
                           const St* __restrict__ Uf, const St* __restrict__ Rf, const double* __restrict__ vf,
                           const double* __restrict__ vc, St* __restrict__ U0, St* __restrict__ Rr) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    double u[4] = {0, 0, 0, 0}, r[4] = {0, 0, 0, 0};
    for (int k = off[c]; k < off[c + 1]; ++k) {
        const int i = fine[k];
        const St a = Uf[i], b = Rf[i];
        const double v = vf[i];
        u[0] += v * a.r; u[1] += v * a.ru; u[2] += v * a.rv; u[3] += v * a.E;
        r[0] += b.r; r[1] += b.ru; r[2] += b.rv; r[3] += b.E;
    }
    const double iv = 1.0 / vc[c];
    St q;
    q.r = u[0] * iv; q.ru = u[1] * iv; q.rv = u[2] * iv; q.E = u[3] * iv;
    U0[c] = q;
    St s;
    s.r = r[0]; s.ru = r[1]; s.rv = r[2]; s.E = r[3];
    Rr[c] = s;
}

__global__ void k_forcing(int nc, const St* __restrict__ Rr, const St* __restrict__ Rc, St* __restrict__ P) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const St a = Rr[c], b = Rc[c];
    St p;
    p.r = a.r - b.r; p.ru = a.ru - b.ru; p.rv = a.rv - b.rv; p.E = a.E - b.E;
    P[c] = p;
}

__global__ void k_prolong(int nf, const int* __restrict__ coarse_of, const St* __restrict__ Uc,
                          const St* __restrict__ U0, St* __restrict__ Uf, double relax, double gamma,
                          const int* __restrict__ cell_inst, const int* __restrict__ active) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nf) return;
    if (active && !active[cell_inst[i]]) return;  // frozen batch instance
    const int c = coarse_of[i];
    const St a = Uc[c], b = U0[c], u = Uf[i];
    const double p0 = (gamma - 1.0) * (u.E - 0.5 * (u.ru * u.ru + u.rv * u.rv) / u.r);
    // the correction, halved until density and pressure stay within a
    // factor of two of their current values (none after three halvings)
    double w = relax;
    for (int t = 0; t < 4; ++t, w *= 0.5) {
        St n;
        n.r = u.r + w * (a.r - b.r);
        n.ru = u.ru + w * (a.ru - b.ru);
        n.rv = u.rv + w * (a.rv - b.rv);
        n.E = u.E + w * (a.E - b.E);
        const double p = (gamma - 1.0) * (n.E - 0.5 * (n.ru * n.ru + n.rv * n.rv) / n.r);
        if (n.r > 0.5 * u.r && n.r < 2.0 * u.r && p > 0.5 * p0 && p < 2.0 * p0) {
            Uf[i] = n;
            return;
        }
    }
}

}  // namespace mgk

namespace fvgb {

void Solver::eval_residual(St* out) {
    O2Args a = o2_args();
    a.resid = out;
    if (cfg.order == 2) {
        if (cfg.fp32) o2::launch_part_f32(a, cfg, 1, 0, stream);
        else o2::launch_part_f64(a, cfg, 1, 0, stream);
    }
    if (cfg.fp32) {
        o2::launch_part_f32(a, cfg, 1, 1, stream);
        o2::launch_residual_f32(a, stream);
    } else {
        o2::launch_part_f64(a, cfg, 1, 1, stream);
        o2::launch_residual_f64(a, stream);
    }
}

void Solver::mg_cycle(size_t level) {
    if (level >= mg.size()) return;
    MGLevel& L = mg[level];
    Solver& c = *L.s;
    const int B = 256;
    // batched: the coarse level skips the instances frozen on this level
    if (batch)
        FV_CUDA(cudaMemcpyAsync(c.active, active, sizeof(int) * n_inst, cudaMemcpyDeviceToDevice, stream));
    // finer residual at the smoothed state (with its own forcing)
    eval_residual(mg_resid);
    mgk::k_restrict<<<(c.N + B - 1) / B, B, 0, stream>>>(c.N, L.fine_off, L.fine, U, mg_resid, dm.vol, c.dm.vol,
                                                        L.U0, L.Rr);
    // coarse residual at the restricted state, without forcing
    FV_CUDA(cudaMemcpyAsync(c.U, L.U0, sizeof(St) * (size_t)c.N, cudaMemcpyDeviceToDevice, stream));
    c.forcing = nullptr;
    c.refresh_primitives();
    c.eval_residual(L.Rc);
    mgk::k_forcing<<<(c.N + B - 1) / B, B, 0, stream>>>(c.N, L.Rr, L.Rc, L.P);
    c.forcing = L.P;
    for (int k = 0; k < mg_smooth; ++k) {
        c.launch_step(nullptr, nullptr, nullptr);
        c.mg_cycle(0);
    }
    mgk::k_prolong<<<(N + B - 1) / B, B, 0, stream>>>(N, L.coarse_of, c.U, L.U0, U, mg_relax, gamma, cell_inst,
                                                      active);
    FV_CUDA(cudaGetLastError());
    refresh_primitives();
}

void Solver::enable_multigrid(const HostMesh& hm, int levels, int smooth, double relax) {
    if (!general || viscous) raise(FV_ERR_UNSUPPORTED, "multigrid: Euler solves on the second-order / multi-stage path");
    if (!cfg.local_dt) raise(FV_ERR_UNSUPPORTED, "multigrid: steady solves with local time stepping");
    if (levels < 0 || levels > 8 || smooth < 1 || !(relax > 0.0 && relax <= 1.0))
        raise(FV_ERR_BAD_ARG, "multigrid: 0..8 levels, smooth >= 1, 0 < relax <= 1");
    if (hm.n_cells != N) raise(FV_ERR_BAD_ARG, "mesh does not match the solver");
    FV_CUDA(cudaStreamSynchronize(stream));
    mg.clear();
    if (levels == 0) return;
    mg_smooth = smooth;
    mg_relax = relax;
    if (!mg_resid) mg_resid = dalloc_owned<St>(N);
    // boundary conditions as this solver has them
    std::vector<fv_bc_t> bcs(bc.n);
    for (int p = 0; p < bc.n; ++p) {
        fv_bc_t& b = bcs[p];
        std::memset(&b, 0, sizeof(b));
        b.type = bc.type[p];
        for (int k = 0; k < 4; ++k) b.state[k] = bc.st[p][k];
        b.wall_u = bc.wall_u[p];
        b.wall_v = bc.wall_v[p];
        b.isothermal = bc.isothermal[p];
        b.wall_T = bc.wall_T[p];
    }
    StepCtl c0;
    read_ctl(c0);
    fv_options_t o = opt;
    o.order = 1;
    o.rk_stages = 3;
    o.dt_mode = FV_DT_LOCAL;
    o.precision = FV_PREC_FP64;
    o.strict = 0;
    fv_ic_t ic;
    std::memset(&ic, 0, sizeof(ic));
    ic.rho = 1.0;
    ic.p = 1.0;
    const HostMesh* prev = &hm;
    std::vector<HostMesh> keep(levels);
    Solver* finer = this;
    for (int l = 0; l < levels; ++l) {
        std::vector<int32_t> agg;
        agglomerate(*prev, agg, keep[l]);
        if (keep[l].n_cells < 8 || keep[l].n_cells >= prev->n_cells) break;
        keep[l].build_device_layout(FV_REORDER_MORTON);
        MGLevel L;
        L.s.reset(new Solver());
        L.s->init(keep[l], bcs.data(), bc.n, gamma, c0.cfl, ic, o, batch ? inst_fs_host.data() : nullptr);
        L.s->set_stream(stream);
        Solver& cs = *L.s;
        const int nf = finer->N;
        const int nc = cs.N;
        L.n_fine = nf;
        // finer device cell -> coarse device cell
        std::vector<int> co(nf);
        for (int i = 0; i < nf; ++i) co[i] = keep[l].iperm[agg[prev->perm[i]]];
        std::vector<int> off(nc + 1, 0), fl(nf);
        for (int i = 0; i < nf; ++i) off[co[i] + 1] += 1;
        for (int cc = 0; cc < nc; ++cc) off[cc + 1] += off[cc];
        std::vector<int> pos(off.begin(), off.end() - 1);
        for (int i = 0; i < nf; ++i) fl[pos[co[i]]++] = i;
        L.coarse_of = finer->upload_owned(co);
        L.fine_off = finer->upload_owned(off);
        L.fine = finer->upload_owned(fl);
        L.U0 = finer->dalloc_owned<St>(nc);
        L.Rr = finer->dalloc_owned<St>(nc);
        L.P = finer->dalloc_owned<St>(nc);
        L.Rc = finer->dalloc_owned<St>(nc);
        if (!cs.mg_resid) cs.mg_resid = cs.dalloc_owned<St>(nc);
        cs.mg_smooth = smooth;
        cs.mg_relax = relax;
        finer->mg.push_back(std::move(L));
        Solver* next = finer->mg.back().s.get();
        finer = next;
        prev = &keep[l];
    }
    for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
    graphs.clear();
    FV_CUDA(cudaStreamSynchronize(stream));
}

}  // namespace fvgb

extern "C" int fv_solver_multigrid(fv_solver_t s, fv_mesh_t mesh, int32_t levels, int32_t smooth, double relax) {
    return fvgb::guarded([&] {
        if (!s || !mesh) fvgb::raise(FV_ERR_BAD_ARG, "null argument");
        s->s.enable_multigrid(fvgb::host_mesh_of(mesh), levels, smooth, relax);
    });
}
