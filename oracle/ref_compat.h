/*
 * Force-included (nvcc -include) when the reference's own CUDA sources are
 * compiled by oracle/ref_build.py.  TEST INFRASTRUCTURE ONLY.
 *
 * The reference (src/cuda/rectv.cu:149-197,250) calls
 * cudaMemPrefetchAsync(ptr, bytes, int device, stream), the signature of
 * CUDA <= 12.  CUDA 13 takes a cudaMemLocation and a flags word instead.  This
 * overload maps the old call onto the new one (device ordinal -> device
 * location, cudaCpuDeviceId -> host location) so that the reference's sources
 * compile unchanged.
 */
#pragma once
#include <cuda_runtime.h>

#if defined(CUDART_VERSION) && CUDART_VERSION >= 13000
static inline cudaError_t cudaMemPrefetchAsync(const void *ptr, size_t bytes, int device, cudaStream_t stream) {
    cudaMemLocation loc;
    if (device == cudaCpuDeviceId) {
        loc.type = cudaMemLocationTypeHost;
        loc.id = 0;
    } else {
        loc.type = cudaMemLocationTypeDevice;
        loc.id = device;
    }
    return cudaMemPrefetchAsync(ptr, bytes, loc, 0u, stream);
}
#endif
