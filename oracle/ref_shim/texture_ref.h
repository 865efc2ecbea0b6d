// Stand-in for CUDA's texture reference API (test infrastructure: the
// reference-pin cubin of interactions_gpu.cu only).  CUDA 12 removed texture
// references (texture<T, 1, mode> objects at file scope, cudaBindTexture,
// tex1Dfetch on them) and cudaThreadSynchronize; the reference's interaction
// kernels use them.  Here a texture reference becomes a device global holding
// the bound pointer and element count, and tex1Dfetch reads the bound linear
// memory, returning zero outside the bound range as a bound linear texture
// does.  The binding happens on the device (a setter kernel beside the
// reference code), so the host stubs below only keep the reference's host
// functions compiling.
#pragma once

#include <climits>
#include <cuda_runtime.h>

template <class T, int dim = 1, enum cudaTextureReadMode mode = cudaReadModeElementType>
struct texture_ref_shim {
    const T *ptr;
    long long count;
};

#define texture __device__ texture_ref_shim

template <class T, int dim, enum cudaTextureReadMode mode>
__device__ __forceinline__ T tex1Dfetch(const texture_ref_shim<T, dim, mode> &t, int i) {
    if (i < 0 || (long long)i >= t.count) return T{};
    return t.ptr[i];
}

template <class T, int dim, enum cudaTextureReadMode mode>
inline cudaError_t cudaBindTexture(size_t *, const texture_ref_shim<T, dim, mode> &, const void *, size_t = UINT_MAX) {
    return cudaSuccess;
}

template <class T, int dim, enum cudaTextureReadMode mode>
inline cudaError_t cudaUnbindTexture(const texture_ref_shim<T, dim, mode> &) {
    return cudaSuccess;
}

#define cudaThreadSynchronize cudaDeviceSynchronize

// binds one texture stand-in on the device: `bytes` of linear memory at p
template <class T, int dim, enum cudaTextureReadMode mode>
__device__ __forceinline__ void texture_ref_bind(texture_ref_shim<T, dim, mode> &t, const void *p,
                                                 unsigned long long bytes) {
    t.ptr = (const T *)p;
    t.count = p ? (long long)(bytes / sizeof(T)) : 0;
}
