// The library's device allocations go through device_malloc, so a test can make them fail
// (amdg_debug_fail_device_allocations) and check that every call reports AMDG_ERR_NOMEM.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace amdg {
cudaError_t device_malloc_raw(void** p, size_t bytes);
template <class T>
cudaError_t device_malloc(T** p, size_t bytes) {
    return device_malloc_raw(reinterpret_cast<void**>(p), bytes);
}
}  // namespace amdg
