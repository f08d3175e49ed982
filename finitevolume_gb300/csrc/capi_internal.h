// Shared by the translation units that implement the C ABI: the opaque
// solver handle and the exception-to-status wrapper of every entry point.
#pragma once

#include <exception>
#include <new>

#include "../../include/fv_gb300.h"
#include "errors.h"
#include "mesh_host.h"
#include "solver.h"

struct fv_solver_s {
    fvgb::Solver s;
};

namespace fvgb {

template <typename Fn>
int guarded(Fn&& fn) {
    try {
        fn();
        return FV_OK;
    } catch (const Error& e) {
        set_last_error(e.msg);
        return e.code;
    } catch (const MeshError& e) {
        set_last_error(e.msg);
        return e.code;
    } catch (const std::bad_alloc&) {
        set_last_error("host allocation failed");
        return FV_ERR_BAD_ARG;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return FV_ERR_BAD_ARG;
    }
}

}  // namespace fvgb
