// fv_step_noalloc: one first-order step on caller-owned device memory,
// with every work array in a fixed, file-scope device array instead of a
// cudaMalloc.
//
// Some callers cannot let a library allocate device memory: a host
// application that owns a fixed device-memory budget and hands out all of
// it through its own pool, code that runs while other threads are capturing
// CUDA graphs in relaxed capture mode (an allocation there is an illegal
// operation), or an embedded/real-time caller that allocates everything at
// start-up and forbids allocation (and its latency and failure modes) in
// the solve loop.  They keep the mesh and the state in their own device
// buffers and call this entry point, which calls no cudaMalloc, cudaFree or
// any allocating library routine.
//
// The scratch (face fluxes, block partial sums, the step control block)
// lives in g_noalloc_scratch below: about 4 MiB that every GPU which loads
// this library holds until the process exits.  All calls share it; the
// control block is re-armed by a kernel at the start of every call, and the
// other regions are fully overwritten before they are read.  Calls whose
// GPU work overlaps (on different streams, or from different threads)
// therefore race on the scratch and must be serialised by the caller.
#include <algorithm>
#include <cfloat>
#include <cstring>
#include <exception>

#include "../../include/fv_gb300.h"
#include "errors.h"
#include "types.h"

namespace fvgb {
namespace {

constexpr int kMaxBlocks = (FV_NOALLOC_MAX_CELLS + kCellBlock - 1) / kCellBlock;
constexpr size_t kFluxOff = 0;
constexpr size_t kFluxBytes = sizeof(St) * (size_t)FV_NOALLOC_MAX_FACES;
constexpr size_t kPartOff = kFluxOff + kFluxBytes;
constexpr size_t kPartBytes = sizeof(double) * 4 * (size_t)kMaxBlocks;
constexpr size_t kHistOff = kPartOff + kPartBytes;
constexpr size_t kHistBytes = 256;
constexpr size_t kCtlOff = kHistOff + kHistBytes;
constexpr size_t kCheckOff = kCtlOff + 256;
constexpr size_t kScratchBytes = kCheckOff + 256;
static_assert(sizeof(StepCtl) <= 256, "control block must fit its slot");

// The fixed scratch.  In host code the name is only a stand-in for the
// device symbol: its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Device address of the scratch in the current context.  It is resolved on
// every call (cudaGetSymbolAddress allocates nothing), so it stays right
// after a cudaDeviceReset or under a context the caller made current
// itself.  The first call in a context may load the module: make it
// before any stream capture.
unsigned char* scratch_in_current_context() {
    void* p = nullptr;
    cudaError_t rc = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (rc != cudaSuccess || !p)
        raise(FV_ERR_CUDA, std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(rc));
    return static_cast<unsigned char*>(p);
}

// Checks the caller's device mesh before any step kernel reads it: every
// face's cells in range (right = -1 only with a patch), every boundary
// face's patch in [0, n_bcs), the CSR offsets non-decreasing from 0 and
// every entry naming a face.  Bits of *bad: 1 patch, 2 cell index, 4 CSR.
__global__ void k_noalloc_check(const fv_noalloc_mesh_t m, int n_bcs, int* bad) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int b = 0;
    if (i < m.n_faces) {
        const int L = m.face_left[i], R = m.face_right[i];
        if (L < 0 || L >= m.n_cells || R < -1 || R >= m.n_cells) b |= 2;
        if (R < 0) {
            const int p = m.face_patch[i];
            if (p < 0 || p >= n_bcs) b |= 1;
        }
    }
    if (i < m.n_cells) {
        const int e0 = m.cell_face_off[i], e1 = m.cell_face_off[i + 1];
        if (e1 < e0 || (i == 0 && e0 != 0)) b |= 4;
    }
    if (i == 0) {
        const int e1 = m.cell_face_off[m.n_cells];
        if (e1 < 0) b |= 4;
    }
    if (b) atomicOr(bad, b);
}

__global__ void k_noalloc_check_entries(const fv_noalloc_mesh_t m, int* bad) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < m.cell_face_off[m.n_cells] && (unsigned)(m.cell_faces[e] >> 1) >= (unsigned)m.n_faces) atomicOr(bad, 4);
}

__global__ void k_noalloc_arm(StepCtl* ctl, double cfl, int* bad) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        *bad = 0;
        ctl->dt_bits = (unsigned long long)__double_as_longlong(DBL_MAX);
        ctl->done_blocks = 0u;
        ctl->step = 0;
        ctl->cfl = cfl;
        for (int k = 0; k < 4; ++k) ctl->norms[k] = 0.0;
        ctl->nonfinite = 0;
    }
}

}  // namespace
}  // namespace fvgb

extern "C" int fv_step_noalloc(const fv_noalloc_mesh_t* mesh, const fv_bc_t* bcs, int32_t n_bcs, double gamma,
                               double cfl, int32_t flux, double* U, double norms[4], void* stream) {
    using namespace fvgb;
    try {
        if (!mesh || !U || !norms || (!bcs && n_bcs > 0)) raise(FV_ERR_BAD_ARG, "fv_step_noalloc: null argument");
        if (mesh->n_cells <= 0 || mesh->n_faces <= 0) raise(FV_ERR_BAD_ARG, "fv_step_noalloc: empty mesh");
        if (mesh->n_faces > FV_NOALLOC_MAX_FACES || mesh->n_cells > FV_NOALLOC_MAX_CELLS)
            raise(FV_ERR_BAD_ARG, "fv_step_noalloc: mesh has " + std::to_string(mesh->n_cells) + " cells and " +
                                      std::to_string(mesh->n_faces) + " faces; the fixed scratch holds at most " +
                                      std::to_string(FV_NOALLOC_MAX_CELLS) + " cells and " +
                                      std::to_string(FV_NOALLOC_MAX_FACES) + " faces");
        if (!mesh->face_left || !mesh->face_right || !mesh->face_patch || !mesh->face_geom || !mesh->cell_face_off ||
            !mesh->cell_faces || !mesh->cell_volume)
            raise(FV_ERR_BAD_ARG, "fv_step_noalloc: null mesh array");
        if (reinterpret_cast<uintptr_t>(mesh->face_geom) % 32 || reinterpret_cast<uintptr_t>(U) % 32)
            raise(FV_ERR_BAD_ARG, "fv_step_noalloc: face_geom and U must be 32-byte aligned");
        if (n_bcs < 0 || n_bcs > kMaxPatches) raise(FV_ERR_BAD_ARG, "fv_step_noalloc: n_bcs must be 0..32");
        if (flux < FV_FLUX_RUSANOV || flux > FV_FLUX_EXACT) raise(FV_ERR_BAD_ARG, "fv_step_noalloc: unknown flux");
        if (!(gamma > 1.0) || !(cfl > 0.0)) raise(FV_ERR_BAD_ARG, "fv_step_noalloc: gamma must be > 1, cfl > 0");

        unsigned char* base = scratch_in_current_context();
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        O1Args a;
        std::memset(&a, 0, sizeof(a));
        a.m.n_cells = mesh->n_cells;
        a.m.n_faces = mesh->n_faces;
        a.m.fl = mesh->face_left;
        a.m.fr = mesh->face_right;
        a.m.fpatch = mesh->face_patch;
        a.m.fgeom = reinterpret_cast<const double4_32a*>(mesh->face_geom);
        a.m.cf_off = mesh->cell_face_off;
        a.m.cf = mesh->cell_faces;
        a.m.vol = mesh->cell_volume;
        a.U = reinterpret_cast<St*>(U);
        a.ff = reinterpret_cast<St*>(base + kFluxOff);
        a.dtf = nullptr;  // global dt only
        a.partials = reinterpret_cast<double*>(base + kPartOff);
        a.hist = reinterpret_cast<double*>(base + kHistOff);
        a.hist_cap = 1;
        a.ctl = reinterpret_cast<StepCtl*>(base + kCtlOff);
        a.bc.n = n_bcs;
        for (int p = 0; p < n_bcs; ++p) {
            if (bcs[p].type < FV_BC_WALL || bcs[p].type > FV_BC_NOSLIP)
                raise(FV_ERR_BAD_ARG, "fv_step_noalloc: unknown boundary type");
            a.bc.type[p] = bcs[p].type;
            for (int k = 0; k < 4; ++k) a.bc.st[p][k] = bcs[p].state[k];
            a.bc.wall_u[p] = bcs[p].wall_u;
            a.bc.wall_v[p] = bcs[p].wall_v;
        }
        a.gamma = gamma;
        a.exact_tol = 1e-6;
        a.exact_max_iter = 20;
        a.flux = flux;
        a.local_dt = 0;

        int* bad = reinterpret_cast<int*>(base + kCheckOff);
        k_noalloc_arm<<<1, 32, 0, s>>>(a.ctl, cfl, bad);
        const int n_chk = std::max(mesh->n_faces, mesh->n_cells);
        k_noalloc_check<<<(n_chk + 255) / 256, 256, 0, s>>>(*mesh, n_bcs, bad);
        FV_CUDA(cudaGetLastError());
        int bad_h = 0;
        FV_CUDA(cudaMemcpyAsync(&bad_h, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
        FV_CUDA(cudaStreamSynchronize(s));
        if (!(bad_h & 4)) {
            // the entries are only walked once the offsets are known sane
            int n_ent = 0;
            FV_CUDA(cudaMemcpyAsync(&n_ent, mesh->cell_face_off + mesh->n_cells, sizeof(int), cudaMemcpyDeviceToHost, s));
            FV_CUDA(cudaStreamSynchronize(s));
            if (n_ent > 0) {
                k_noalloc_check_entries<<<(n_ent + 255) / 256, 256, 0, s>>>(*mesh, bad);
                FV_CUDA(cudaGetLastError());
                FV_CUDA(cudaMemcpyAsync(&bad_h, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
                FV_CUDA(cudaStreamSynchronize(s));
            }
        }
        if (bad_h & 1) raise(FV_ERR_BAD_ARG, "fv_step_noalloc: a boundary face's patch is outside [0, n_bcs)");
        if (bad_h & 2) raise(FV_ERR_BAD_ARG, "fv_step_noalloc: a face's cell index is out of range");
        if (bad_h & 4) raise(FV_ERR_BAD_ARG, "fv_step_noalloc: cell_face_off / cell_faces are not a valid CSR");
        fast::launch_o1_part(a, 0, s);
        fast::launch_o1_part(a, 1, s);
        FV_CUDA(cudaGetLastError());
        StepCtl c;
        FV_CUDA(cudaMemcpyAsync(&c, a.ctl, sizeof(c), cudaMemcpyDeviceToHost, s));
        FV_CUDA(cudaStreamSynchronize(s));
        for (int k = 0; k < 4; ++k) norms[k] = c.norms[k];
        if (c.nonfinite) raise(FV_ERR_NONFINITE, "fv_step_noalloc: non-finite residual norm");
        return FV_OK;
    } catch (const Error& e) {
        set_last_error(e.msg);
        return e.code;
    } catch (const std::exception& e) {  // no exception crosses the C ABI
        set_last_error(e.what());
        return FV_ERR_BAD_ARG;
    }
}
