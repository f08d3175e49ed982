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
