// Solver state held behind an fv_solver_t handle.
#pragma once

#include <map>
#include <memory>
#include <vector>

#include <algorithm>

#include "../../include/fv_gb300.h"
#include "errors.h"
#include "mesh_host.h"
#include "ns.h"
#include "rans.h"
#include "types.h"

namespace fvgb {

struct WallFace {
    int cell;  // owner cell, reference numbering
    double nx, ny, area, xm, ym;
    int dev_face;  // the face's device index
};

struct Solver;

// One coarse level of the agglomeration multigrid (full approximation
// scheme): its own first-order solver on the agglomerated mesh and the
// transfer maps to the next finer level (device numbering of both).
struct MGLevel {
    std::unique_ptr<Solver> s;
    int n_fine = 0;
    int* fine_off = nullptr;   // [N_c + 1] CSR: coarse cell -> finer cells
    int* fine = nullptr;
    int* coarse_of = nullptr;  // [N_f] finer cell -> coarse cell
    St* U0 = nullptr;          // restricted state
    St* Rr = nullptr;          // restricted finer residual
    St* P = nullptr;           // forcing
    St* Rc = nullptr;          // coarse residual at the restricted state
};

// The dataflow form's partition of a mesh in device order (DfPlan's host
// side): nb blocks, the cells [cell_off[b], cell_off[b+1]) and the faces
// faces[face_off[b] .. face_off[b+1]) of block b, and the blocks its face
// and cell phases wait for.
struct DataflowPlan {
    int nb = 0;
    std::vector<int> cell_off, face_off, faces, dep_face_off, dep_face, dep_cell_off, dep_cell;
};
// Builds the plan over min(sms, cell warps) blocks; patch_type[p] is the
// FV_BC_* of patch p.  False when a block would wait for more than
// kDfMaxDeps blocks in one phase (the plan is still filled in).
bool dataflow_plan(const HostMesh& hm, const int* patch_type, int sms, DataflowPlan& p);

struct Solver {
    static constexpr int kGraphChunk = 32;

    fv_options_t opt{};
    double gamma = 1.4;
    int N = 0, F = 0, n_cell_blocks = 0;
    std::vector<int32_t> perm;  // device cell -> reference cell
    std::vector<WallFace> wall_faces;
    BCTable bc{};
    DevMesh dm{};

    St* U = nullptr;
    St* staging = nullptr;     // reference-order copy for get/set field
    int* d_perm = nullptr;     // device cell -> reference cell
    St* ff = nullptr;
    double* dtf = nullptr;
    double* partials = nullptr;
    double* hist = nullptr;
    int hist_cap = 0;
    StepCtl* ctl = nullptr;
    long long steps_taken = 0;

    // Batched steady solves (one mesh per instance, concatenated)
    bool batch = false;
    int n_inst = 0;
    std::vector<int32_t> group_off;   // instance cell ranges (same in both numberings)
    std::vector<int> wall_inst;       // instance of each entry of wall_faces
    int* cell_inst = nullptr;
    int* active = nullptr;
    int* inst_off = nullptr;
    int* inst_iter = nullptr;
    double* inst_fs = nullptr;
    std::vector<double> inst_fs_host;   // the same, host copy (coarse multigrid levels)
    double* inst_norms = nullptr;
    double4_32a* r2 = nullptr;
    double tol = -1.0;                // density-norm tolerance; < 0 never freezes

    // Navier-Stokes path (and RANS-SA on top of it)
    bool viscous = false;
    bool rans = false;
    RansArgs rs{};
    double* nut_hist = nullptr;
    NSArgs ns{};
    int* ns_wall_faces = nullptr;   // device indices of the wall faces, reference order
    double2* ns_wall_out = nullptr; // (tau_wall, p) per wall face

    // second-order / multi-stage path
    bool general = false;           // false: reference-mode first-order kernels
    O2Config cfg{};
    St* U0 = nullptr;
    void* W = nullptr;
    void* G = nullptr;
    void* cs = nullptr;             // sound speed, flux precision
    double* dtv = nullptr;
    const int* cnb = nullptr;
    // reconstruction geometry in flux precision (see O2Args)
    const void* lsq = nullptr;
    const void* lsq_sum = nullptr;
    const void* gg = nullptr;
    const void* erf = nullptr;
    const void* frf = nullptr;
    const void* eps2 = nullptr;
    const float4* fgeom32 = nullptr;
    const St* forcing = nullptr;    // multigrid coarse levels: FAS forcing term
    void* psi_buf = nullptr;        // frozen limiter values [4N], flux precision
    St* d2 = nullptr;               // FP64 live limiter: per-entry increments [E] (O2Args::d2)
    St* psi4 = nullptr;             //   and per-cell limiter values [N]
    int2* fe = nullptr;             //   owner / neighbour entry per face [F]
    int psi_mode = 0;               // 0 evaluated, 2 frozen (see O2Args)

    // Persistent first-order path (order 1, forward Euler, FP64 Euler): one
    // cooperative launch runs a chunk of steps (euler_o1p.cuh).
    bool persistent = false;        // in use
    bool persistent_ok = false;     // available (device and scheme)
    int p_grid = 0;                 // co-resident blocks of the launch
    PersistCtl* pctl = nullptr;
    double4_32a* Pc = nullptr;      // per-cell primitives u, v, p, c
    // Its dataflow form (local dt): neighbour waits instead of grid
    // barriers, one block per SM (DfPlan).  Used unless barrier_form.
    bool dataflow_ok = false;
    bool barrier_form = false;
    int df_grid = 0;
    DfPlan dfp{};
    static constexpr int kPersistChunk = 256;
    static constexpr long long kDefaultWaitCycles = 2000000000LL;  // ~1 s at 2 GHz

    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::map<int, cudaGraphExec_t> graphs;
    std::vector<void*> owned;
    std::vector<cudaEvent_t> events;  // step_timed event pool

    void init(const HostMesh& hm, const fv_bc_t* bcs, int n_bcs, double g, double cfl, const fv_ic_t& ic,
              const fv_options_t& o, const double* batch_freestream = nullptr);
    void ensure_history(int n);
    O1Args o1_args() const;
    RansArgs rans_args() const;
    O2Args o2_args() const;
    void refresh_primitives();
    void launch_step(std::vector<int>* classes, std::vector<cudaEvent_t>* events, size_t* ev_pos);
    // k steps: one persistent launch, or k x launch_step
    void launch_steps(int k, std::vector<int>* classes, std::vector<cudaEvent_t>* events, size_t* ev_pos);
    // 0 two-kernel path, 1 persistent (dataflow form where planned), 2
    // persistent barrier form
    void set_persistent(int mode);
    // 0 two-kernel path, 1 barrier form, 2 dataflow form
    int persistent_form() const;
    void build_dataflow(const HostMesh& hm, int sms);
    void set_wait_limit(long long cycles, int phantom);
    // FV_ERR_TIMEOUT if a persistent launch gave up at a wait since the
    // last reset_wait_error (called at the start of every step call)
    void check_persistent();
    void reset_wait_error();
    void step_timed(int n, double ms[3], int launches[3]);
    cudaGraphExec_t graph_for(int k);
    void step_async(int n);
    void read_ctl(StepCtl& c);
    void history(int n, double* out);
    void download_field(double* out);
    void upload_field(const void* in_ref_order);
    void set_cfl(double cfl);
    // launch shapes of the second-order kernels (gradients, faces, cells)
    void set_launch(int bg, int bf, int bc);
    // time each kernel class at 128/256/512 threads per block for n steps
    // (state restored afterwards) and keep the fastest shape per class
    void autotune(int n, int out[3]);
    void set_stream(void* s);
    // Freeze the limiter at the current state (its values are captured and
    // reused by every later gradient evaluation) or release it.
    void freeze_limiter(bool on);
    // Frozen limiter values [N x 4], reference cell order: copy out (out_ref)
    // and/or freeze at given values (in_ref, each in [0, 1]).
    void limiter_values(double* out_ref, const double* in_ref);
    void wall_forces(const double ref[7], double out[11], int instance = -1);

    // Agglomeration multigrid (steady solves with local time stepping):
    // `levels` coarse levels below this solver, smoothed `smooth` RK
    // iterations each per V-cycle; corrections scaled by `relax`.
    std::vector<MGLevel> mg;
    St* mg_resid = nullptr;
    int mg_smooth = 1;
    double mg_relax = 1.0;
    void enable_multigrid(const HostMesh& hm, int levels, int smooth, double relax);
    template <typename T>
    T* dalloc_owned(size_t n) {
        void* p = nullptr;
        FV_CUDA(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)));
        owned.push_back(p);
        return static_cast<T*>(p);
    }
    template <typename T>
    T* upload_owned(const std::vector<T>& v) {
        T* p = dalloc_owned<T>(v.size());
        if (!v.empty()) h2d_sync(p, v.data(), v.size() * sizeof(T), stream);
        return p;
    }
    void eval_residual(St* out);
    void mg_cycle(size_t level);
    ~Solver();
};

}  // namespace fvgb
