// Status codes and the thread-local last-error message of the C ABI.
#pragma once

#include <string>

namespace fvgb {

struct Error {
    int code;
    std::string msg;
};

[[noreturn]] void raise(int code, const std::string& msg);
void set_last_error(const std::string& msg);
const char* last_error();

}  // namespace fvgb

#define FV_CUDA(call)                                                                        \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            ::fvgb::raise(2, std::string(#call) + ": " + cudaGetErrorString(e_));          \
    } while (0)

#ifdef __CUDACC__
namespace fvgb {
// Host -> device upload that has landed when it returns.  A plain
// cudaMemcpy from pageable memory may return once the bytes are staged,
// before the DMA reaches the device, and kernels on a non-blocking stream
// are not ordered after the legacy stream; copying on `s` and waiting for
// `s` closes that gap whatever stream later reads the data.
inline void h2d_sync(void* dst, const void* src, size_t bytes, cudaStream_t s = cudaStreamLegacy) {
    if (!bytes) return;
    FV_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
    FV_CUDA(cudaStreamSynchronize(s));
}
}  // namespace fvgb
#endif
