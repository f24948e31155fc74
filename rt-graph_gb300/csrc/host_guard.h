// Host-side allocation failures at the C boundary (shared by the CUDA and the host-only
// sources of the library).
#pragma once

#include <new>
#include <stdexcept>

#include "rtg.h"

namespace rtg {

// The body of a C entry point that allocates host memory: a failed host allocation
// (std::bad_alloc, or std::length_error for a size no vector can hold) comes back as
// RTG_ERR_OOM instead of leaving through the C boundary as an exception.
template <class F> rtg_status host_alloc_guard(F &&body) {
    try {
        return body();
    } catch (const std::bad_alloc &) {
        return RTG_ERR_OOM;
    } catch (const std::length_error &) {
        return RTG_ERR_OOM;
    }
}

}  // namespace rtg
