// Checkpoint files in the reference's binary layout (include/Checkpoint.h:26-46):
//   0  "FVMCKPT\0"   8  u32 version (2)   12 u32 equation tag
//   16 u64 cell_count 24 i64 step_index   32 u64 build_number
//   40 payload: raw native doubles (Euler/NS: cell_count x {rho, rho_u,
//      rho_v, E}; Diffusion: cell_count x phi; RANS: U then extra scalars).
// The format itself has to be identical so that runs resume across the two
// codes; the reading/writing code here is this library's own.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <exception>
#include <string>

#include "../../include/fv_gb300.h"
#include "errors.h"

namespace {

constexpr char kMagic[8] = {'F', 'V', 'M', 'C', 'K', 'P', 'T', '\0'};
constexpr uint32_t kVersion = 2;

int64_t doubles_per_cell(int32_t eq) {
    switch (eq) {
        case FV_CKPT_DIFFUSION:
        case FV_CKPT_ADVECTION_DIFFUSION: return 1;
        case FV_CKPT_EULER:
        case FV_CKPT_NAVIER_STOKES: return 4;
        case FV_CKPT_RANS_SA: return 5;
        case FV_CKPT_RANS_SST: return 6;
        default: return -1;
    }
}

bool is_flow(int32_t eq) { return eq == FV_CKPT_EULER || eq == FV_CKPT_NAVIER_STOKES || eq == FV_CKPT_RANS_SA || eq == FV_CKPT_RANS_SST; }

struct File {
    FILE* f;
    explicit File(FILE* p) : f(p) {}
    ~File() {
        if (f) std::fclose(f);
    }
};

template <typename Fn>
int guard(Fn&& fn) {
    try {
        fn();
        return FV_OK;
    } catch (const fvgb::Error& e) {
        fvgb::set_last_error(e.msg);
        return e.code;
    } catch (const std::exception& e) {  // no exception crosses the C ABI
        fvgb::set_last_error(e.what());
        return FV_ERR_BAD_ARG;
    }
}

}  // namespace

extern "C" {

int fv_checkpoint_write(const char* path, int32_t equation, int64_t step_index, uint64_t build_number,
                        int64_t cell_count, const double* payload) {
    return guard([&] {
        const int64_t per = doubles_per_cell(equation);
        if (!path || !payload || per < 0 || cell_count < 0) fvgb::raise(FV_ERR_BAD_ARG, "fv_checkpoint_write: bad argument");
        File f(std::fopen(path, "wb"));
        if (!f.f) fvgb::raise(FV_ERR_BAD_ARG, std::string("fv_checkpoint_write: cannot open ") + path);
        const uint32_t ver = kVersion, tag = (uint32_t)equation;
        const uint64_t cells = (uint64_t)cell_count;
        bool ok = std::fwrite(kMagic, 1, 8, f.f) == 8 && std::fwrite(&ver, 4, 1, f.f) == 1 &&
                  std::fwrite(&tag, 4, 1, f.f) == 1 && std::fwrite(&cells, 8, 1, f.f) == 1 &&
                  std::fwrite(&step_index, 8, 1, f.f) == 1 && std::fwrite(&build_number, 8, 1, f.f) == 1;
        const size_t n = (size_t)(per * cell_count);
        ok = ok && (n == 0 || std::fwrite(payload, sizeof(double), n, f.f) == n);
        if (!ok || std::fflush(f.f) != 0) fvgb::raise(FV_ERR_BAD_ARG, std::string("fv_checkpoint_write: write failed: ") + path);
    });
}

int fv_checkpoint_read(const char* path, int32_t expected_equation, int64_t expected_cell_count, int64_t* step_index,
                       uint64_t* build_number, double* payload) {
    return guard([&] {
        if (!path || !payload || expected_cell_count < 0 ||
            (expected_equation >= 0 && doubles_per_cell(expected_equation) < 0))
            fvgb::raise(FV_ERR_BAD_ARG, "fv_checkpoint_read: bad argument");
        File f(std::fopen(path, "rb"));
        if (!f.f) fvgb::raise(FV_ERR_BAD_ARG, std::string("fv_checkpoint_read: cannot open ") + path);
        char magic[8];
        uint32_t ver = 0, tag = 0;
        uint64_t cells = 0, build = 0;
        int64_t step = 0;
        if (std::fread(magic, 1, 8, f.f) != 8 || std::memcmp(magic, kMagic, 8) != 0)
            fvgb::raise(FV_ERR_BAD_ARG, "fv_checkpoint_read: not a checkpoint (bad magic)");
        if (std::fread(&ver, 4, 1, f.f) != 1 || ver != kVersion)
            fvgb::raise(FV_ERR_BAD_ARG, "fv_checkpoint_read: unsupported format version");
        if (std::fread(&tag, 4, 1, f.f) != 1 || std::fread(&cells, 8, 1, f.f) != 1 ||
            std::fread(&step, 8, 1, f.f) != 1 || std::fread(&build, 8, 1, f.f) != 1)
            fvgb::raise(FV_ERR_BAD_ARG, "fv_checkpoint_read: truncated header");
        // expected_equation < 0: any flow equation, reading its state block
        // (Checkpoint::read_flow_field, include/Checkpoint.h:140-142).
        if (expected_equation >= 0 ? (int32_t)tag != expected_equation : !is_flow((int32_t)tag))
            fvgb::raise(FV_ERR_BAD_ARG, "fv_checkpoint_read: checkpoint is for another equation set");
        if ((int64_t)cells != expected_cell_count)
            fvgb::raise(FV_ERR_BAD_ARG, "fv_checkpoint_read: cell count does not match the mesh");
        const int64_t per = expected_equation >= 0 ? doubles_per_cell(expected_equation) : 4;
        const size_t n = (size_t)(per * expected_cell_count);
        if (n && std::fread(payload, sizeof(double), n, f.f) != n)
            fvgb::raise(FV_ERR_BAD_ARG, "fv_checkpoint_read: truncated payload");
        if (step_index) *step_index = step;
        if (build_number) *build_number = build;
    });
}

}  // extern "C"
