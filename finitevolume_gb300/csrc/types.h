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

struct O1Args {
    DevMesh m;
    St* U;
    St* ff;            // [F] face fluxes (times face length)
    double* dtf;       // [F] per-face CFL time step (local dt)
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

constexpr int kCellBlock = 256;
constexpr int kFaceBlock = 256;

namespace fast { void launch_o1_step(const O1Args& a, cudaStream_t s); }
namespace strict { void launch_o1_step(const O1Args& a, cudaStream_t s); }

}  // namespace fvgb
