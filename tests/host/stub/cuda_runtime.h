/* Host stand-in for <cuda_runtime.h>: lets the device headers
 * (libffrs_gb300/csrc/rs256_device.cuh, rsi16_device.cuh) compile as plain
 * C++ so that CPU tests can run their algorithms against the oracle.  Only
 * what those headers use; warp intrinsics come from warp_emu.h. */
#pragma once
#include <cstddef>
#include <cstdint>
#define __device__
#define __host__
#define __forceinline__ inline
#define __noinline__
static inline unsigned __funnelshift_r(unsigned lo, unsigned hi, unsigned shift) {
    return (unsigned)((((unsigned long long)hi << 32) | lo) >> (shift & 31));
}
#define __align__(n) alignas(n)
struct uint4 {
    unsigned x, y, z, w;
};
typedef struct CUstream_st *cudaStream_t;
template <typename T>
static inline T min(T a, T b) {
    return a < b ? a : b;
}
template <typename T>
static inline T max(T a, T b) {
    return a < b ? b : a;
}
struct HostDim3 {
    unsigned x = 0, y = 0, z = 0;
};
static HostDim3 threadIdx, blockDim;
static inline uint4 make_uint4(unsigned x, unsigned y, unsigned z, unsigned w) { return uint4{x, y, z, w}; }
static inline unsigned __umulhi(unsigned a, unsigned b) { return (unsigned)(((unsigned long long)a * b) >> 32); }
static inline unsigned __brev(unsigned x) {
    unsigned r = 0;
    for (int i = 0; i < 32; ++i) r |= ((x >> i) & 1u) << (31 - i);
    return r;
}
template <typename T>
static inline T __ldg(const T *p) {
    return *p;
}
static inline size_t __cvta_generic_to_shared(const void *p) { return (size_t)p; }
