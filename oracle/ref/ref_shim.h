// ref_shim.h -- lets the reference's CUDA device headers compile as plain
// host C++ (g++) so that its own intersection and mask-table code can be run
// on the CPU as a cross-check of the oracle.  Nothing from the reference is
// copied: ref_driver.cpp includes the reference headers where they lie.
//
// The shim supplies: empty CUDA execution-space qualifiers, the launch
// built-ins (threadIdx/blockIdx/blockDim; ref_driver.cpp runs one "thread" per
// call), the few device intrinsics the headers use (with CUDA's saturating
// conversion semantics), a point-sampled stand-in for the removed texture
// reference API, and a float max() with device fmaxf semantics at global
// scope (on the device the reference's float max() calls resolve there).
#pragma once

#include <algorithm>
#include <cassert>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <vector>

#include <cuda_runtime.h>

using std::abs;

#undef __device__
#undef __host__
#undef __global__
#undef __shared__
#undef __forceinline__
#define __device__
#define __host__
#define __global__
#define __shared__
#define __forceinline__ inline

struct RefDim3 {
    unsigned x, y, z;
};
extern RefDim3 threadIdx, blockIdx, blockDim, gridDim;

inline int __float_as_int(float f) {
    int i;
    std::memcpy(&i, &f, 4);
    return i;
}
inline float __int_as_float(int i) {
    float f;
    std::memcpy(&f, &i, 4);
    return f;
}
inline int __float2int_rd(float x) {
    if (std::isnan(x)) return 0;
    if (x >= 2147483648.0f) return INT_MAX;
    if (x < -2147483648.0f) return INT_MIN;
    return (int)std::floor(x);
}
inline int __float2int_rn(float x) {
    if (std::isnan(x)) return 0;
    if (x >= 2147483648.0f) return INT_MAX;
    if (x < -2147483648.0f) return INT_MIN;
    return (int)std::nearbyint(x);
}
inline int __popc(unsigned x) { return __builtin_popcount(x); }

// Device fmaxf semantics (NaN ignored, +0 preferred) for float max().
inline float max(float a, float b) {
    if (std::isnan(a)) return b;
    if (std::isnan(b)) return a;
    if (a > b) return a;
    if (b > a) return b;
    return std::signbit(a) ? b : a;
}

inline unsigned max(unsigned a, unsigned b) { return a > b ? a : b; }

template <class T>
inline T __ldg(const T *p) {
    return *p;
}

// Texture references were removed from CUDA 12; this stand-in keeps the
// reference's declarations compiling and samples like a clamped, point-
// filtered, normalised-coordinate 2D texture: texel = clamp(floor(u * w)).
template <class T, int dim = 1, enum cudaTextureReadMode mode = cudaReadModeElementType>
struct texture {
    int normalized = 0;
    enum cudaTextureFilterMode filterMode = cudaFilterModePoint;
    enum cudaTextureAddressMode addressMode[3] = {cudaAddressModeClamp, cudaAddressModeClamp,
                                                  cudaAddressModeClamp};
    const T *ptr = nullptr;
    size_t w = 0, h = 0, pitch = 0;
};
template <class T, int dim, enum cudaTextureReadMode mode>
inline cudaError_t cudaBindTexture2D(size_t *offset, texture<T, dim, mode> &t, const void *p,
                                     const cudaChannelFormatDesc &, size_t w, size_t h, size_t pitch) {
    if (offset) *offset = 0;
    t.ptr = (const T *)p;
    t.w = w;
    t.h = h;
    t.pitch = pitch;
    return cudaSuccess;
}
template <class T, int dim, enum cudaTextureReadMode mode>
inline T tex2D(const texture<T, dim, mode> &t, float u, float v) {
    long ix = __float2int_rd(u * (float)t.w), iy = __float2int_rd(v * (float)t.h);
    ix = std::min<long>(std::max<long>(ix, 0), (long)t.w - 1);
    iy = std::min<long>(std::max<long>(iy, 0), (long)t.h - 1);
    return *(const T *)((const char *)t.ptr + iy * t.pitch + ix * sizeof(T));
}
