// First-order explicit steps as one persistent, cooperative launch.
//
// The reference's step (src/EulerFVMSolver.cpp:58-112) needs every face flux
// before any cell update and, in its global-dt mode, the minimum over all
// faces of the CFL step (compute_dt, :133-162) before the first update.  The
// two-kernel path (euler_o1.cuh) makes those dependencies kernel boundaries,
// which on a 32k-cell mesh costs more than the arithmetic.  Here one launch
// of co-resident blocks (a cooperative launch) runs K steps.  Its
// grid-barrier form (k_o1_persistent) meets each dependency at a grid
// barrier:
//
//   prologue   per-cell primitives P = (u, v, p, c) of the current state
//   per step   face phase: fluxes (and the CFL candidate or lambda*A),
//                 block 0 also folds the previous step's norm partials
//              barrier
//              cell phase: signed gather, U += dt/V R, the new P, and one
//                 norm partial per 256-cell tile
//              barrier
//   epilogue   block 0 folds the last step's partials
//
// P is the reference's own per-side quantities (u = rho_u/rho, v, the
// pressure and sound speed expressions of EulerState.h:58-82), formed once
// per cell instead of once per face side; the fluxes read them instead of
// recomputing them.  In the strict build (--fmad=false, FV_STRICT_ORDER)
// every value is the same IEEE result as the reference's, so it stays
// bit-identical to the reference.  The default build spends fewer FP64-pipe
// instructions on the same quantities: 1/rho by fvconv::rcp_nr3 (three
// DFMA) and products with it instead of three divisions per cell, the
// normal velocity of the Rusanov flux from P instead of a division per face
// side, and the local-dt update factor dt/V = cfl / sum lambda A by one
// reciprocal, and the ghost states from P with short dependent chains
// (ghost_p); it agrees with the reference within 1e-10.  In both builds the
// norm partials are formed over the same 256-cell tiles and folded in the
// same order as k_cell_o1's, so the residual history is bit-identical to
// the two-kernel path too.
//
// With local dt a step has no global dependency, and the dataflow form
// (k_o1_dataflow, further down) replaces the grid barriers by waits on the
// few blocks that share faces with each block.
//
// The grid barrier is a counter plus a generation word.  Every wait (grid
// barrier or neighbour progress) is bounded (PersistCtl::limit, in SM clock
// cycles): a block that gives up sets PersistCtl::err and leaves, so the
// others give up at their next wait too and the launch always ends; the
// host reports FV_ERR_TIMEOUT.
//
// Included by kernels_fast.cu and kernels_strict.cu with FV_KNS defined,
// after euler_o1.cuh.
#pragma once

#include "euler_o1.cuh"
#include "fpconv.cuh"

namespace FV_KNS {

using fvgb::DfPlan;
using fvgb::PersistCtl;

struct Prim {
    double u, v, p, c;
};

__device__ __forceinline__ Prim prim_of(const St& s, double g) {
    Prim q;
#ifdef FV_STRICT_ORDER
    q.u = s.ru / s.r;
    q.v = s.rv / s.r;
    q.p = pressure(s, g);
    q.c = sqrt(g * q.p / s.r);  // sound_speed: sqrt(g * pressure / rho)
#else
    const double ir = fvconv::rcp_nr3(s.r);
    q.u = s.ru * ir;
    q.v = s.rv * ir;
    q.p = (g - 1.0) * (s.E - 0.5 * (s.ru * q.u + s.rv * q.v));
    q.c = sqrt(g * q.p * ir);
#endif
    return q;
}
// Loads of arrays this kernel itself writes (state, primitives, fluxes,
// wave-speed sums) bypass L1 (ld.global.cg): another block may have
// written them since this SM last cached the line, and only L2 is
// coherent across SMs.  The read-only path (__ldg) would be wrong here.
__device__ __forceinline__ St ld_state_cg(const St* U, int i) {
    const double2* p = reinterpret_cast<const double2*>(U + i);
    const double2 a = __ldcg(p), b = __ldcg(p + 1);
    return st_make(a.x, a.y, b.x, b.y);
}
__device__ __forceinline__ Prim ld_prim(const double4_32a* P, int i) {
    const double2* p = reinterpret_cast<const double2*>(P + i);
    const double2 a = __ldcg(p), b = __ldcg(p + 1);
    Prim o;
    o.u = a.x; o.v = a.y; o.p = b.x; o.c = b.y;
    return o;
}
__device__ __forceinline__ void st_prim(double4_32a* P, int i, const Prim& q) {
    double4_32a o;
    o.x = q.u; o.y = q.v; o.z = q.p; o.w = q.c;
    P[i] = o;
}

// phys_flux (EulerState.h:89-101) with u, v, p taken from P.
__device__ __forceinline__ St phys_flux_p(const St& s, const Prim& q, double nx, double ny) {
    const double Vn = q.u * nx + q.v * ny;
    St f;
    f.r = s.r * Vn;
    f.ru = s.ru * Vn + q.p * nx;
    f.rv = s.rv * Vn + q.p * ny;
    f.E = (s.E + q.p) * Vn;
    return f;
}

// rusanov (RusanovFlux.h:33-43) with the per-side primitives from P.
__device__ __forceinline__ St rusanov_p(const St& L, const Prim& PL, const St& R, const Prim& PR, double nx,
                                        double ny) {
#ifdef FV_STRICT_ORDER
    const double VnL = (L.ru * nx + L.rv * ny) / L.r;
    const double VnR = (R.ru * nx + R.rv * ny) / R.r;
#else
    const double VnL = PL.u * nx + PL.v * ny;
    const double VnR = PR.u * nx + PR.v * ny;
#endif
    const double Smax = rmax(fabs(VnL) + PL.c, fabs(VnR) + PR.c);
    const St FL = phys_flux_p(L, PL, nx, ny);
    const St FR = phys_flux_p(R, PR, nx, ny);
    return 0.5 * (FL + FR) - 0.5 * Smax * (R - L);
}

// hllc (HllcFlux.h:35-76) with the per-side primitives from P.
__device__ __forceinline__ St hllc_p1(const St& UL, const Prim& PL, const St& UR, const Prim& PR, double nx,
                                      double ny) {
    const double tx = -ny, ty = nx;
    const double rL = UL.r, rR = UR.r;
    const double VnL = PL.u * nx + PL.v * ny, VnR = PR.u * nx + PR.v * ny;
    const double VtL = PL.u * tx + PL.v * ty, VtR = PR.u * tx + PR.v * ty;
    const double pL = PL.p, pR = PR.p, cL = PL.c, cR = PR.c;
    const double SL = rmin(VnL - cL, VnR - cR);
    const double SR = rmax(VnL + cL, VnR + cR);
    if (SL >= 0.0) return phys_flux_p(UL, PL, nx, ny);
    if (SR <= 0.0) return phys_flux_p(UR, PR, nx, ny);
    const double Ss = (pR - pL + rL * VnL * (SL - VnL) - rR * VnR * (SR - VnR)) / (rL * (SL - VnL) - rR * (SR - VnR));
    const bool left = (Ss >= 0.0);
    const double SK = left ? SL : SR;
    const double rK = left ? rL : rR;
    const double VnK = left ? VnL : VnR;
    const double VtK = left ? VtL : VtR;
    const double pK = left ? pL : pR;
    const St& UK = left ? UL : UR;
    const Prim& PK = left ? PL : PR;
    const double factor = rK * (SK - VnK) / (SK - Ss);
    const double mn = factor * Ss;
    const double mt = factor * VtK;
    const double Es = factor * (UK.E / rK + (Ss - VnK) * (Ss + pK / (rK * (SK - VnK))));
    St Us;
    Us.r = factor;
    Us.ru = mn * nx - mt * ny;
    Us.rv = mn * ny + mt * nx;
    Us.E = Es;
    return phys_flux_p(UK, PK, nx, ny) + SK * (Us - UK);
}

template <int FLUX>
__device__ __forceinline__ St num_flux_p(const St& L, const Prim& PL, const St& R, const Prim& PR, double nx,
                                         double ny, double g, double tol, int maxit) {
    if constexpr (FLUX == FLUX_HLLC) return hllc_p1(L, PL, R, PR, nx, ny);
    else if constexpr (FLUX == FLUX_EXACT) return exact_riemann(L, R, nx, ny, g, tol, maxit);
    else return rusanov_p(L, PL, R, PR, nx, ny);
}

// face_smax (compute_dt's per-face max(|Vn| + c)) with P.
__device__ __forceinline__ double face_smax_p(const Prim& PL, const Prim& PR, bool interior, double nx, double ny) {
    double Smax = fabs(PL.u * nx + PL.v * ny) + PL.c;
    if (interior) Smax = rmax(Smax, fabs(PR.u * nx + PR.v * ny) + PR.c);
    return Smax;
}

#ifndef FV_STRICT_ORDER
// The characteristic farfield (physics.cuh, char_farfield) from the
// interior primitives P instead of the conserved state, returning the
// ghost's primitives too: its sound speed is |cb| (p_b = rho_b cb^2 / g),
// and the boundary density rho_s (cb^2 / (g s))^(1/(g-1)) with the upwind
// side's entropy s = p_s / rho_s^g is rho_s |cb / c_s|^(2/(g-1)), taken by
// pow_near1.  This is the longest dependent chain of the face phase and a
// few blocks own all the farfield faces, so no division, square root or
// library power depends on the interior state here.
__device__ __forceinline__ void char_farfield_p(const St& UL, const Prim& PL, const double* sinf, double nx,
                                                double ny, double g, St& UR, Prim& PR) {
    const double rf = sinf[0], irf = fvconv::rcp_nr3(rf), uf = sinf[1] * irf, vf = sinf[2] * irf;
    const double pf = (g - 1.0) * (sinf[3] - 0.5 * rf * (uf * uf + vf * vf));
    const double cf = sqrt(g * pf * irf);
    const double vni = PL.u * nx + PL.v * ny, vnf = uf * nx + vf * ny;
    const double ici = fvconv::rcp_nr3(PL.c), icf = fvconv::rcp_nr3(cf);  // off the chain
    if (vnf <= -cf) {  // supersonic inflow
        UR = st_make(sinf[0], sinf[1], sinf[2], sinf[3]);
        PR.u = uf; PR.v = vf; PR.p = pf; PR.c = cf;
        return;
    }
    if (vni >= PL.c) {  // supersonic outflow
        UR = UL;
        PR = PL;
        return;
    }
    const double k = 2.0 / (g - 1.0);
    const double Rp = vni + k * PL.c, Rm = vnf - k * cf;
    const double vnb = 0.5 * (Rp + Rm);
    const double cb = 0.25 * (g - 1.0) * (Rp - Rm);
    const bool out = vnb > 0.0;
    const double rs = out ? UL.r : rf, ics = out ? ici : icf;
    const double ut = out ? PL.u - vni * nx : uf - vnf * nx;
    const double vt = out ? PL.v - vni * ny : vf - vnf * ny;
    const double rb = rs * fvconv::pow_near1(fabs(cb) * ics, k);
    const double ub = ut + vnb * nx, vb = vt + vnb * ny;
    const double pb = rb * cb * cb * (1.0 / g);
    UR = st_make(rb, rb * ub, rb * vb, pb * (1.0 / (g - 1.0)) + 0.5 * rb * (ub * ub + vb * vb));
    PR.u = ub; PR.v = vb; PR.p = pb; PR.c = fabs(cb);
}

// Ghost state and its primitives from the interior state and primitives:
// the characteristic farfield above; the slip wall as the mirror image
// (density, pressure, sound speed and speed, hence E, unchanged, the
// normal velocity reversed); outflow the interior itself; the fixed
// farfield and the no-slip wall through ghost_state.  Same states as
// ghost_state + prim_of up to rounding, with short dependent chains.
__device__ __forceinline__ void ghost_p(const BCTable& bc, int patch, const St& UL, const Prim& PL, double nx,
                                        double ny, double g, St& UR, Prim& PR) {
    const int t = bc.type[patch];
    if (t == BC_CHAR) {
        char_farfield_p(UL, PL, bc.st[patch], nx, ny, g, UR, PR);
    } else if (t == BC_WALL) {
        const double Vn = PL.u * nx + PL.v * ny;
        PR.u = PL.u - 2.0 * Vn * nx;
        PR.v = PL.v - 2.0 * Vn * ny;
        PR.p = PL.p;
        PR.c = PL.c;
        UR = st_make(UL.r, UL.r * PR.u, UL.r * PR.v, UL.E);
    } else if (t == BC_OUTFLOW) {
        UR = UL;
        PR = PL;
    } else {
        UR = ghost_state(bc, patch, UL, nx, ny, g);
        PR = prim_of(UR, g);
    }
}
#endif

// One face of the face phase: the flux times the face length into ff[f]
// and, with local dt, lambda * length into dtf[f].  Returns the face's
// global-dt candidate cfl * (CFL length) / max(|Vn| + c) (DBL_MAX with
// local dt).
template <int FLUX, bool LOCAL>
__device__ __forceinline__ double face_phase_face(const O1Args& a, const double4_32a* P, int f, double g,
                                                  double cfl) {
    const int L = a.m.fl[f], R = a.m.fr[f];
    const double4_32a geo = a.m.fgeom[f];
    const St UL = ld_state_cg(a.U, L);
    const Prim PL = ld_prim(P, L);
    St UR;
    Prim PR;
    if (R >= 0) {
        UR = ld_state_cg(a.U, R);
        PR = ld_prim(P, R);
    } else {
#ifndef FV_STRICT_ORDER
        ghost_p(a.bc, a.m.fpatch[f], UL, PL, geo.x, geo.y, g, UR, PR);
#else
        UR = ghost_state(a.bc, a.m.fpatch[f], UL, geo.x, geo.y, g);
        PR = prim_of(UR, g);
#endif
    }
    const St Fl = num_flux_p<FLUX>(UL, PL, UR, PR, geo.x, geo.y, g, a.exact_tol, a.exact_max_iter);
    st_state(a.ff, f, geo.z * Fl);
    const double Smax = face_smax_p(PL, PR, R >= 0, geo.x, geo.y);
    if (LOCAL) {
        a.dtf[f] = Smax * geo.z;
        return DBL_MAX;
    }
    return cfl * geo.w / Smax;
}

// One cell of the cell phase: the signed gather of its face fluxes,
// U += dt/V R, the new primitives, and the squares of R for the norms.
template <bool LOCAL>
__device__ __forceinline__ void cell_phase_cell(const O1Args& a, double4_32a* P, int c, double g, double cfl,
                                                double dt_g, double& s0, double& s1, double& s2, double& s3) {
    double dt = dt_g;
    St Rs = st_make(0.0, 0.0, 0.0, 0.0);
    const int e0 = a.m.cf_off[c], e1 = a.m.cf_off[c + 1];
    double lam = 0.0;
    for (int e = e0; e < e1; ++e) {
        const int ent = a.m.cf[e];
        const int f = ent >> 1;
        Rs += flip_if(ld_state_cg(a.ff, f), ent);
        if (LOCAL) lam += __ldcg(a.dtf + f);
    }
    double coef;  // dt / V
#ifdef FV_STRICT_ORDER
    if (LOCAL) dt = cfl * a.m.vol[c] / lam;
    coef = dt / a.m.vol[c];
#else
    coef = LOCAL ? cfl * fvconv::rcp_nr3(lam) : dt / a.m.vol[c];
#endif
    s0 = Rs.r * Rs.r; s1 = Rs.ru * Rs.ru; s2 = Rs.rv * Rs.rv; s3 = Rs.E * Rs.E;
    const St u = ld_state_cg(a.U, c);
    const St un = u + coef * Rs;
    st_state(a.U, c, un);
    st_prim(P, c, prim_of(un, g));
}

// Grid barrier with a bounded wait.  Returns false (in every thread of the
// block) once any block has given up; the caller then returns.
__device__ __forceinline__ bool grid_barrier(PersistCtl* pc, unsigned int expected) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned int* vgen = &pc->gen;
        volatile int* verr = &pc->err;
        const unsigned int g0 = *vgen;  // read before arriving: gen cannot move until this block arrives
        __threadfence();
        const unsigned int arrived = atomicAdd(&pc->count, 1u);
        int good = 1;
        if (arrived == expected - 1) {
            atomicExch(&pc->count, 0u);
            __threadfence();
            atomicAdd(&pc->gen, 1u);
        } else {
            const long long t0 = clock64();
            while (*vgen == g0) {
                if (*verr || clock64() - t0 > pc->limit) {
                    atomicExch(&pc->err, 1);
                    good = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        ok = good && !*verr;
    }
    __syncthreads();
    return ok != 0;
}

// Block 0 folds one step's tile partials exactly as finish_norms' last
// block does (tiles strided over the block's threads, transposed warp sums,
// warps in order), records the history row and advances the step counter.
__device__ __forceinline__ void fold_step_norms(StepCtl* ctl, const double* partials, int n_tiles, double* hist,
                                                int hist_cap) {
    __shared__ double red[fvgb::kCellBlock / 32][4];
    constexpr int nw = fvgb::kCellBlock / 32;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double t[4] = {0.0, 0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < n_tiles; b += fvgb::kCellBlock) {
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
    }
    __syncthreads();
}

template <int FLUX, bool LOCAL>
__global__ void __launch_bounds__(fvgb::kCellBlock) k_o1_persistent(const O1Args a, double4_32a* __restrict__ P,
                                                                     PersistCtl* __restrict__ pc, int nsteps) {
    const double g = a.gamma;
    const int nb = gridDim.x;
    const unsigned int expected = (unsigned int)nb + (unsigned int)pc->phantom;
    const int n_tiles = (a.m.n_cells + fvgb::kCellBlock - 1) / fvgb::kCellBlock;
    const int F = a.m.n_faces, N = a.m.n_cells;

    // prologue: primitives of the current state; both dt slots armed
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += nb * blockDim.x)
        st_prim(P, c, prim_of(ld_state_cg(a.U, c), g));
    if (blockIdx.x == 0 && threadIdx.x < 2)
        pc->dt_slot[threadIdx.x] = (unsigned long long)__double_as_longlong(DBL_MAX);
    if (!grid_barrier(pc, expected)) return;

    for (int s = 0; s < nsteps; ++s) {
        const int slot = s & 1;
        if (blockIdx.x == 0 && s > 0) {
            fold_step_norms(a.ctl, a.partials, n_tiles, a.hist, a.hist_cap);
            if (threadIdx.x == 0) pc->dt_slot[slot ^ 1] = (unsigned long long)__double_as_longlong(DBL_MAX);
        }
        // face phase
        const double cfl = a.ctl->cfl;
        double cand = DBL_MAX;
        // each block takes an equal contiguous range of faces, so that every
        // SM (the grid is a multiple of the SM count) gets the same share
        const int f0 = (int)((long long)F * blockIdx.x / nb), f1 = (int)((long long)F * (blockIdx.x + 1) / nb);
        for (int f = f0 + threadIdx.x; f < f1; f += blockDim.x)
            cand = fmin(cand, face_phase_face<FLUX, LOCAL>(a, P, f, g, cfl));
        if (!LOCAL) {
            __shared__ double smin[fvgb::kCellBlock / 32];
            cand = warp_min(cand);
            if ((threadIdx.x & 31) == 0) smin[threadIdx.x >> 5] = cand;
            __syncthreads();
            if (threadIdx.x == 0) {
                double v = smin[0];
                for (int w = 1; w < fvgb::kCellBlock / 32; ++w) v = fmin(v, smin[w]);
                atomicMin(&pc->dt_slot[slot], (unsigned long long)__double_as_longlong(v));
            }
        }
        if (!grid_barrier(pc, expected)) return;

        // cell phase, one 256-cell tile at a time (the tiles of k_cell_o1)
        const double dt_g = LOCAL ? 0.0 : __longlong_as_double((long long)*(volatile unsigned long long*)&pc->dt_slot[slot]);
        for (int tile = blockIdx.x; tile < n_tiles; tile += nb) {
            const int c = tile * fvgb::kCellBlock + threadIdx.x;
            double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
            if (c < N) cell_phase_cell<LOCAL>(a, P, c, g, cfl, dt_g, s0, s1, s2, s3);
            // the tile's partial: finish_norms' block reduction
            __shared__ double red[fvgb::kCellBlock / 32][4];
            const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
            const double ws = warp_sum4(s0, s1, s2, s3);
            if ((lane & 7) == 0) red[w][lane >> 3] = ws;
            __syncthreads();
            if (threadIdx.x < 4) {
                double v = 0.0;
                for (int i = 0; i < fvgb::kCellBlock / 32; ++i) v += red[i][threadIdx.x];
                a.partials[tile * 4 + threadIdx.x] = v;
            }
            __syncthreads();
        }
        if (!grid_barrier(pc, expected)) return;
    }
    if (blockIdx.x == 0 && nsteps > 0) fold_step_norms(a.ctl, a.partials, n_tiles, a.hist, a.hist_cap);
}

// ---------------------------------------------------------------------------
// Dataflow form (local dt only).  The local-dt step has no global
// dependency inside a step, only the face -> cell -> face ones between
// neighbouring cells, so the grid barriers of k_o1_persistent are replaced
// by waits on the few blocks that share faces with this one (DfPlan).
// Blocks then drift against distant blocks instead of meeting at every
// phase, and a wait costs one L2 round trip to a neighbour's progress word.
// One block of kDfBlock threads per SM owns a contiguous range of whole
// cell warps (a Morton-ordered mesh keeps that range compact, so a block
// has a handful of neighbours).  The arithmetic per face and per cell is
// face_phase_face / cell_phase_cell, and the norm partials are formed per
// 32-cell warp and folded, after the last step, tile by tile in
// k_cell_o1's order: fields and residual histories are the same bits as
// the barrier form's.
//
// Progress words are published with st.release.gpu after a block barrier
// (the block's writes of the phase, gathered by bar.sync, are ordered
// before it) and polled with relaxed loads followed by one
// fence.acq_rel.gpu and a block barrier (the PTX release/acquire pattern;
// every data load of the next phase is an L2 load, ld.global.cg).

__device__ __forceinline__ unsigned int ld_relaxed_gpu(const unsigned int* p) {
    unsigned int v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Thread 0 waits until every block in deps[0..n) has published progress
// >= target, bounded by pc->limit cycles like the grid barrier (a wait that
// runs out, or sees pc->err set by another block, sets pc->err and ends
// the launch).  Returns false in every thread when the launch must end.
__device__ __forceinline__ bool df_wait(PersistCtl* pc, const unsigned int* prog, const int* deps, int n,
                                        unsigned int target) {
    __shared__ int ok;
    if (threadIdx.x == 0) {
        const volatile int* verr = &pc->err;
        const long long t0 = clock64();
        const long long lim = pc->limit;
        int good = 1;
        for (int i = 0; i < n && good; ++i) {
            const unsigned int* p = prog + (size_t)deps[i] * fvgb::kDfProgStride;
            for (unsigned int it = 0; ld_relaxed_gpu(p) < target; ++it) {
                if ((it & 31u) == 31u && (*verr || clock64() - t0 > lim)) {
                    good = 0;
                    break;
                }
            }
        }
        if (!good) atomicExch(&pc->err, 1);
        asm volatile("fence.acq_rel.gpu;" ::: "memory");
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

// All of this block's writes of the phase are done (block barrier), then
// its progress word moves with release semantics.
__device__ __forceinline__ void df_publish(unsigned int* prog, unsigned int v) {
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int* p = prog + (size_t)blockIdx.x * fvgb::kDfProgStride;
        asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
    }
}

// Fold of step s's per-warp partials in the order of fold_step_norms over
// k_cell_o1's tile partials: a tile's partial is the sum of its 8 warp sums
// in warp order (from 0.0; warps past the last cell add nothing, as their
// zero sums add nothing there), the tiles are strided over the first
// kCellBlock threads, then the transposed warp sums and the warps in order.
// The warp partials are staged in shared memory kDfBlock at a time (64
// tiles), so that the loads are one round of independent L2 reads.
__device__ __forceinline__ void df_fold(const O1Args& a, const DfPlan& d, int s, int row, bool last) {
    constexpr int nw = fvgb::kCellBlock / 32;
    constexpr int CH = fvgb::kDfBlock;
    __shared__ double2 wsm[CH][2];
    __shared__ double red[nw][4];
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    const int W = d.n_warps;
    const int n_tiles = (a.m.n_cells + fvgb::kCellBlock - 1) / fvgb::kCellBlock;
    const double* wp = d.wpart + (size_t)s * W * 4;
    double t[4] = {0.0, 0.0, 0.0, 0.0};
    for (int base = 0; base < W; base += CH) {
        if (base + tid < W) {
            const double2* p = reinterpret_cast<const double2*>(wp + 4 * (size_t)(base + tid));
            wsm[tid][0] = __ldcg(p);
            wsm[tid][1] = __ldcg(p + 1);
        }
        __syncthreads();
        if (tid < fvgb::kCellBlock) {
            // this thread's tile among the chunk's CH / nw tiles, if any
            const int t0 = base / nw;
            const int tile = t0 + (((tid - t0) % fvgb::kCellBlock) + fvgb::kCellBlock) % fvgb::kCellBlock;
            if (tile < t0 + CH / nw && tile < n_tiles) {
                double v[4] = {0.0, 0.0, 0.0, 0.0};
                for (int i = 0; i < nw; ++i) {
                    const int cw = tile * nw + i;
                    if (cw < W) {
                        const double2 x = wsm[cw - base][0], y = wsm[cw - base][1];
                        v[0] += x.x; v[1] += x.y; v[2] += y.x; v[3] += y.y;
                    }
                }
                t[0] += v[0]; t[1] += v[1]; t[2] += v[2]; t[3] += v[3];
            }
        }
        __syncthreads();
    }
    const double ts = warp_sum4(t[0], t[1], t[2], t[3]);
    if (w < nw && (lane & 7) == 0) red[w][lane >> 3] = ts;
    __syncthreads();
    if (tid == 0) {
        int bad = 0;
        for (int k = 0; k < 4; ++k) {
            double v = 0.0;
            for (int i = 0; i < nw; ++i) v += red[i][k];
            const double n = sqrt(v);
            if (!isfinite(n)) bad = 1;
            a.hist[row * 4 + k] = n;
            if (last) a.ctl->norms[k] = n;
        }
        if (bad) a.ctl->nonfinite = 1;
    }
    __syncthreads();
}

template <int FLUX>
__global__ void __launch_bounds__(fvgb::kDfBlock, 1) k_o1_dataflow(const O1Args a, double4_32a* __restrict__ P,
                                                                  PersistCtl* __restrict__ pc, const DfPlan d,
                                                                  int nsteps) {
    const double g = a.gamma;
    const int b = blockIdx.x, nb = gridDim.x;
    const unsigned int expected = (unsigned int)nb + (unsigned int)pc->phantom;
    const int N = a.m.n_cells;
    const int c0 = d.cell_off[b], c1 = d.cell_off[b + 1];
    const int fa = d.face_off[b], fz = d.face_off[b + 1];
    const int step0 = a.ctl->step;
    const double cfl = a.ctl->cfl;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int nwarps = fvgb::kDfBlock / 32;

    __shared__ int dep_f[fvgb::kDfMaxDeps], dep_c[fvgb::kDfMaxDeps];
    const int nf = d.dep_face_off[b + 1] - d.dep_face_off[b];
    const int nc = d.dep_cell_off[b + 1] - d.dep_cell_off[b];
    if (threadIdx.x < nf) dep_f[threadIdx.x] = d.dep_face[d.dep_face_off[b] + threadIdx.x];
    if (threadIdx.x < nc) dep_c[threadIdx.x] = d.dep_cell[d.dep_cell_off[b] + threadIdx.x];

    // prologue: primitives of the own cells, progress word reset
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) st_prim(P, c, prim_of(ld_state_cg(a.U, c), g));
    if (threadIdx.x == 0) d.prog[(size_t)b * fvgb::kDfProgStride] = 0u;
    if (!grid_barrier(pc, expected)) return;

    for (int s = 0; s < nsteps; ++s) {
        // face phase: the right cells' states of step s are final
        if (s > 0 && !df_wait(pc, d.prog, dep_f, nf, 2u * s)) return;
        for (int j = fa + threadIdx.x; j < fz; j += blockDim.x)
            face_phase_face<FLUX, true>(a, P, d.faces[j], g, cfl);
        df_publish(d.prog, 2u * s + 1u);

        // cell phase: every face of the own cells has its step-s flux and
        // no block still reads the own cells' step-s states
        if (!df_wait(pc, d.prog, dep_c, nc, 2u * s + 1u)) return;
        double* wp = d.wpart + (size_t)s * d.n_warps * 4;
        for (int cw = c0 / 32 + warp; cw * 32 < c1; cw += nwarps) {
            const int c = cw * 32 + lane;
            double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
            if (c < N) cell_phase_cell<true>(a, P, c, g, cfl, 0.0, s0, s1, s2, s3);
            const double ws = warp_sum4(s0, s1, s2, s3);
            if ((lane & 7) == 0) wp[(size_t)cw * 4 + (lane >> 3)] = ws;
        }
        df_publish(d.prog, 2u * s + 2u);
    }
    if (!grid_barrier(pc, expected)) return;
    // the launch's norms, steps strided over the blocks
    for (int s = b; s < nsteps; s += nb) df_fold(a, d, s, (step0 + s) % a.hist_cap, s == nsteps - 1);
    if (b == 0 && threadIdx.x == 0) a.ctl->step = step0 + nsteps;
}

template <int FLUX>
static int o1df_blocks_per_sm() {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_o1_dataflow<FLUX>, fvgb::kDfBlock, 0) != cudaSuccess)
        return 0;
    return nb;
}

template <int FLUX>
static cudaError_t launch_o1df(const O1Args& a, double4_32a* P, PersistCtl* pc, const DfPlan& d, int nsteps,
                               int grid, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(fvgb::kDfBlock);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_o1_dataflow<FLUX>, a, P, pc, d, nsteps);
}

template <int FLUX, bool LOCAL>
static int o1p_blocks_per_sm() {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_o1_persistent<FLUX, LOCAL>, fvgb::kCellBlock, 0) !=
        cudaSuccess)
        return 0;
    return nb;
}

template <int FLUX, bool LOCAL>
static cudaError_t launch_o1p(const O1Args& a, double4_32a* P, PersistCtl* pc, int nsteps, int grid,
                              cudaStream_t s) {
    // cudaLaunchKernelEx with the cooperative attribute: co-residency of all
    // blocks is guaranteed (or the launch fails), and the launch can be
    // captured into a CUDA graph.
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(fvgb::kCellBlock);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_o1_persistent<FLUX, LOCAL>, a, P, pc, nsteps);
}

}  // namespace FV_KNS

#ifdef FV_DEFINE_O1_LAUNCH
namespace fvgb {
namespace FV_KNS {
// Largest co-resident grid of the persistent kernel for this flux/dt mode.
int o1p_max_blocks_per_sm(int flux, int local) {
    switch (flux * 2 + (local ? 1 : 0)) {
        case 0: return ::FV_KNS::o1p_blocks_per_sm<0, false>();
        case 1: return ::FV_KNS::o1p_blocks_per_sm<0, true>();
        case 2: return ::FV_KNS::o1p_blocks_per_sm<1, false>();
        case 3: return ::FV_KNS::o1p_blocks_per_sm<1, true>();
        case 4: return ::FV_KNS::o1p_blocks_per_sm<2, false>();
        default: return ::FV_KNS::o1p_blocks_per_sm<2, true>();
    }
}
int o1df_max_blocks_per_sm(int flux) {
    switch (flux) {
        case 0: return ::FV_KNS::o1df_blocks_per_sm<0>();
        case 1: return ::FV_KNS::o1df_blocks_per_sm<1>();
        default: return ::FV_KNS::o1df_blocks_per_sm<2>();
    }
}
cudaError_t launch_o1_dataflow(const O1Args& a, double4_32a* P, PersistCtl* pc, const DfPlan& d, int nsteps,
                               int grid, cudaStream_t s) {
    switch (a.flux) {
        case 0: return ::FV_KNS::launch_o1df<0>(a, P, pc, d, nsteps, grid, s);
        case 1: return ::FV_KNS::launch_o1df<1>(a, P, pc, d, nsteps, grid, s);
        default: return ::FV_KNS::launch_o1df<2>(a, P, pc, d, nsteps, grid, s);
    }
}
cudaError_t launch_o1_persistent(const O1Args& a, double4_32a* P, PersistCtl* pc, int nsteps, int grid,
                                 cudaStream_t s) {
    switch (a.flux * 2 + (a.local_dt ? 1 : 0)) {
        case 0: return ::FV_KNS::launch_o1p<0, false>(a, P, pc, nsteps, grid, s);
        case 1: return ::FV_KNS::launch_o1p<0, true>(a, P, pc, nsteps, grid, s);
        case 2: return ::FV_KNS::launch_o1p<1, false>(a, P, pc, nsteps, grid, s);
        case 3: return ::FV_KNS::launch_o1p<1, true>(a, P, pc, nsteps, grid, s);
        case 4: return ::FV_KNS::launch_o1p<2, false>(a, P, pc, nsteps, grid, s);
        default: return ::FV_KNS::launch_o1p<2, true>(a, P, pc, nsteps, grid, s);
    }
}
}  // namespace FV_KNS
}  // namespace fvgb
#endif  // FV_DEFINE_O1_LAUNCH
