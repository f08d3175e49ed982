// Plain data shared by host code and the kernel translation units.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

namespace fvgb {

// Conserved state of one cell, AoS, one 32-byte sector: {rho, rho_u, rho_v, E}.
struct __align__(32) St {
    double r, ru, rv, E;
};

constexpr int kMaxPatches = 32;

struct BCTable {
    int n;
    int type[kMaxPatches];
    double st[kMaxPatches][4];  // conserved freestream state (farfield kinds)
    double wall_u[kMaxPatches], wall_v[kMaxPatches];
    int isothermal[kMaxPatches];
    double wall_T[kMaxPatches];
};

// Device mesh, device (reordered) numbering.  Faces [0, n_int_faces) are
// internal and sorted by owner; the rest are boundary faces sorted by patch.
struct DevMesh {
    int n_cells, n_faces, n_int_faces;
    const int* fl;          // [F] owner (cell_left)
    const int* fr;          // [F] neighbour or -1
    const int* fpatch;      // [F]
    const double4_32a* fgeom;  // [F] nx, ny, area, CFL length
    const double2* fmid;    // [F] face midpoint
    const int* cf_off;      // [N+1]
    const int* cf;          // entries: face << 1 | (cell is owner)
    const double* vol;      // [N]
    const double2* cxy;     // [N] centroid
};

// Per-solver control block in device memory.  Graph replays read the CFL
// number and step counter from here, so set_cfl never invalidates a graph.
struct StepCtl {
    unsigned long long dt_bits;  // global-dt min accumulator (positive double bits)
    unsigned int done_blocks;    // last-block-done counter of the cell pass
    int step;                    // steps taken since construction / set_field
    double cfl;
    double norms[4];             // last step's residual L2 norms
    int nonfinite;               // set when a norm is not finite
    int pad;
};

// Control block of the persistent first-order kernel: its grid barrier
// (arrival counter, generation, error flag), the bound on every wait in SM
// clock cycles, and the two global-dt min slots (alternating by step).
// `phantom` extra arrivals are waited for at every barrier; nothing ever
// makes them, so a positive value exercises the timeout path.
struct PersistCtl {
    unsigned int count;
    int err;
    unsigned int gen;
    int phantom;
    long long limit;
    unsigned long long dt_slot[2];
};

// Plan of the dataflow form of the persistent first-order kernel (local
// dt): block b owns the cells [cell_off[b], cell_off[b+1]) (whole 32-cell
// warps) and the faces whose left cell it owns (faces[face_off[b] ..
// face_off[b+1])).  Instead of grid barriers, each phase waits only for the
// blocks it shares faces with: the face phase of step s for the cell phase
// of step s-1 of dep_face's blocks (the owners of its faces' right cells),
// the cell phase for the face phase of step s of dep_cell's blocks (the
// owners of the other faces of its cells).  prog[b * kDfProgStride] is
// 2s+1 once block b has finished the face phase of step s and 2s+2 once it
// has finished the cell phase (one 128-byte line per block, so that the
// polls of one block's word do not hit the others').  Each warp of cells
// leaves the residual partial of every step of the launch in wpart; the
// norms are folded after the last step.
struct DfPlan {
    const int* faces;         // [F] face ids grouped by owning block
    const int* face_off;      // [nb+1]
    const int* cell_off;      // [nb+1]
    const int* dep_face;      // blocks the face phase waits for
    const int* dep_face_off;  // [nb+1]
    const int* dep_cell;      // blocks the cell phase waits for
    const int* dep_cell_off;  // [nb+1]
    unsigned int* prog;       // [nb * kDfProgStride]
    double* wpart;            // [max_steps * n_warps * 4] per-warp partials
    int n_warps;              // cell warps, ceil(N / 32)
    int max_steps;            // steps per launch (wpart capacity)
};
constexpr int kDfBlock = 512;          // threads per block (one block per SM)
constexpr int kDfProgStride = 32;      // progress words per block (128 bytes)
constexpr int kDfMaxDeps = 32;         // dependency list bound per block and phase
constexpr size_t kDfPartialBytes = 64u << 20;  // wpart budget (bounds steps per launch)

struct O1Args {
    DevMesh m;
    St* U;
    St* ff;            // [F] face fluxes (times face length)
    double* dtf;       // [F] per-face lambda * length (local dt)
    StepCtl* ctl;
    double* partials;  // [cell blocks * 4]
    double* hist;      // [hist_cap * 4]
    int hist_cap;
    BCTable bc;
    double gamma, exact_tol;
    int exact_max_iter;
    int flux;          // 0 Rusanov, 1 HLLC, 2 exact
    int local_dt;
};

struct O2Args {
    DevMesh m;
    const int* cnb;          // per entry: neighbour or -1-face
    // Reconstruction geometry in flux precision T (double or float arrays):
    const void* lsq;         // per entry LSQ weights (2 T)
    const void* lsq_sum;     // per cell sums of the LSQ weights (2 T)
    const void* gg;          // per entry Green-Gauss coefficients (4 T; double: double4_32a)
    const void* erf;         // per entry face offset (2 T)
    const void* frf;         // per face offsets from the owner / neighbour centroid (4 T)
    const void* eps2;        // per cell Venkatakrishnan (K h)^3, h = sqrt(volume) (T)
    const float4* fgeom32;   // FP32 mode: per face nx, ny, area, CFL length
    St* U;
    St* U0;
    void* W;                 // primitive copy: St (FP64) or float4 (FP32 flux)
    void* G;                 // limited gradients: 4 double2 or 2 float4 per cell
    void* ff;                // face fluxes: St or float4
    void* cs;                // per cell sound speed (cell-centred, for dt; T)
    double* dtf;             // per face lambda * length (local dt)
    double* dtv;             // per cell dt/volume of the current iteration
    StepCtl* ctl;
    double* partials;
    double* hist;
    int hist_cap;
    BCTable bc;
    double gamma, venkat_k, exact_tol;
    double igm1;             // 1 / (gamma - 1)
    float gamma32, igm1_32;  // the same constants rounded to float
    int exact_max_iter;
    // Batched solves (all null otherwise): instance of each cell, the
    // instance-active flags, per-instance freestream (4 conserved values),
    // per-cell squared residuals at stage 0.
    const int* cell_inst;
    const int* active;
    const double* inst_fs;
    double4_32a* r2;
    // Discrete-adjoint linearisation (FP64 only; null otherwise): the
    // unlimited gradients (4 double2 per cell) and the limiter values
    // (4 per cell) of k_grad.
    double2* lim_gu;
    double* lim_psi;
    // Limiter freezing: psi_mode 1 stores the limiter values ([4N], flux
    // precision) in psi_buf as they are computed; 2 reads them from there
    // instead of evaluating the limiter; 0 neither.
    void* psi_buf;
    int psi_mode;
    // FP64 live-limiter reconstruction (null otherwise): per cell-face
    // entry the unlimited increment g . (x_f - x_c) of the four primitives,
    // per cell the four limiter values, and per face the entries of its
    // owner and neighbour (-1 on a boundary face).  With psi_mode != 2
    // k_grad writes the first two instead of the limited gradients, and
    // k_face reconstructs W + psi * increment: the increments k_grad forms
    // for the limiter anyway are not formed a second time.
    St* d2;
    St* psi4;
    const int2* fe;
    // Multigrid (null otherwise): a forcing term added to every cell's
    // residual (coarse levels of the full-approximation scheme), and the
    // output of the residual-only pass.
    const St* forcing;
    St* resid;
};

// Second-order path configuration (validated by the solver).
struct O2Config {
    int fp32;      // 1: FP32 flux/gradient arithmetic
    int flux;      // 0 Rusanov, 1 HLLC, 2 exact
    int order;     // 1 or 2
    int gradient;  // 0 LSQ, 1 Green-Gauss
    int limiter;   // 0 none, 1 Barth-Jespersen, 2 Venkatakrishnan
    int stages;    // 1 or 3
    int local_dt;  // 1 local, 0 global
    // launch shapes (threads per block, 128..512, multiple of 32), chosen by
    // the autotuner; 256 by default
    int blk_grad, blk_face, blk_cell;
};

constexpr int kCellBlock = 256;
constexpr int kFaceBlock = 256;
constexpr int kMaxBlock = 512;  // largest tunable block of the second-order kernels
constexpr int kMinBlock = 128;  // smallest (sizes the norm partials)

namespace o2 {
void launch_prim_f64(const O2Args& a, cudaStream_t s);
void launch_prim_f32(const O2Args& a, cudaStream_t s);
// part 0: gradients + limiter (order 2 only), 1: face fluxes, 2: update.
void launch_part_f64(const O2Args& a, const O2Config& c, int stage, int part, cudaStream_t s);
void launch_part_f32(const O2Args& a, const O2Config& c, int stage, int part, cudaStream_t s);
// residual R(U) (+ forcing) per cell into a.resid, from the face fluxes of
// the last face pass; no update
void launch_residual_f64(const O2Args& a, cudaStream_t s);
void launch_residual_f32(const O2Args& a, cudaStream_t s);
void launch_batch_norms(const O2Args& a, int n_inst, const int* inst_off, double* inst_norms, int* inst_iter,
                        int* active, double tol, cudaStream_t s);
}  // namespace o2

// part 0: face pass, 1: cell pass.
namespace fast { void launch_o1_part(const O1Args& a, int part, cudaStream_t s); }
namespace strict { void launch_o1_part(const O1Args& a, int part, cudaStream_t s); }
// The persistent first-order kernel (cooperative launch of `grid` blocks of
// kCellBlock threads running nsteps steps) and its co-resident block count
// per SM; P holds the per-cell primitives.
namespace fast {
int o1p_max_blocks_per_sm(int flux, int local);
cudaError_t launch_o1_persistent(const O1Args& a, double4_32a* P, PersistCtl* pc, int nsteps, int grid,
                                 cudaStream_t s);
}  // namespace fast
namespace strict {
int o1p_max_blocks_per_sm(int flux, int local);
cudaError_t launch_o1_persistent(const O1Args& a, double4_32a* P, PersistCtl* pc, int nsteps, int grid,
                                 cudaStream_t s);
}  // namespace strict
// Its dataflow form for local dt (grid = the plan's block count, kDfBlock
// threads per block, at most one block per SM).
namespace fast {
int o1df_max_blocks_per_sm(int flux);
cudaError_t launch_o1_dataflow(const O1Args& a, double4_32a* P, PersistCtl* pc, const DfPlan& d, int nsteps,
                               int grid, cudaStream_t s);
}  // namespace fast
namespace strict {
int o1df_max_blocks_per_sm(int flux);
cudaError_t launch_o1_dataflow(const O1Args& a, double4_32a* P, PersistCtl* pc, const DfPlan& d, int nsteps,
                               int grid, cudaStream_t s);
}  // namespace strict

}  // namespace fvgb
