// Internal declarations shared by the host-side translation units of
// liblbm_gb300.so (not installed, not part of the ABI).
#pragma once
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <exception>
#include <new>
#include <string>
#include <vector>

#include "lbm_gb300.h"

namespace lbm {

// Records the message for lbm_last_error() and returns the status.
lbm_status fail(lbm_status s, const char* fmt, ...);
void clear_error();

// Temporary device memory from the device's stream-ordered pool, allocated
// and freed in the order of `stream` (a cudaStream_t).  The pool keeps up to
// a few GB between uses, so a lattice or geometry build does not go back to
// the driver for every scratch array.  cudaFree of such memory does not wait
// for the device: callers synchronise first.
lbm_status dev_alloc(void** p, size_t bytes, void* stream, const char* what);
void dev_free(void* p, void* stream);

// Runs f (returning lbm_status) so that no C++ exception crosses the C ABI:
// an allocation failure becomes LBM_ERR_NOMEM, any other exception
// LBM_ERR_STATE with its message.
template <class F>
lbm_status guarded(const char* what, F&& f) {
    try {
        return f();
    } catch (const std::bad_alloc&) {
        return fail(LBM_ERR_NOMEM, "%s: out of host memory", what);
    } catch (const std::exception& e) {
        return fail(LBM_ERR_STATE, "%s: %s", what, e.what());
    }
}

// Triangle array helpers (host).
using TriVec = std::vector<lbm_tri>;
lbm_status to_c_array(const TriVec& v, lbm_tri** out, size_t* n);

// Marching-tetrahedra mesher over an implicit function given at grid vertices.
struct CapsuleSet;
lbm_status mesh_capsules(const double* seg, size_t nseg, const double lo[3], const double hi[3], double h,
                         uint64_t seed, TriVec& out);

}  // namespace lbm
