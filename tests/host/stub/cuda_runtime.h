/* Host stand-in for <cuda_runtime.h>: lets the per-thread RS256 decoder
 * (libffrs_gb300/csrc/rs256_device.cuh) compile as plain C++ so that a CPU
 * test can run it against the oracle.  Only what that header uses. */
#pragma once
#include <cstddef>
#include <cstdint>
#define __device__
#define __host__
#define __forceinline__ inline
static inline unsigned __funnelshift_r(unsigned lo, unsigned hi, unsigned shift) {
    return (unsigned)((((unsigned long long)hi << 32) | lo) >> (shift & 31));
}
#define __align__(n) alignas(n)
struct uint4 {
    unsigned x, y, z, w;
};
struct HostDim3 {
    unsigned x = 0, y = 0, z = 0;
};
static HostDim3 threadIdx, blockDim;
