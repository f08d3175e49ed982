#include "errors.h"

namespace fvgb {

namespace {
thread_local std::string g_last;
}

void raise(int code, const std::string& msg) { throw Error{code, msg}; }
void set_last_error(const std::string& msg) { g_last = msg; }
const char* last_error() { return g_last.c_str(); }

}  // namespace fvgb
