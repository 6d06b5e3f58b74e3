// CUDA error reporting for the entry points of the C ABI; the host-only entry points
// (errors, uniforms) are in host.cpp.
#include <cuda_runtime.h>

#include "vrt_internal.h"

namespace vrt {

int cuda_error(cudaError_t e, const char* what) {
    cudaGetLastError();  // clear a non-sticky error so later calls do not report it again
    return set_error(VRT_ECUDA, "%s: %s (%d)", what, cudaGetErrorString(e), (int)e);
}

}  // namespace vrt
