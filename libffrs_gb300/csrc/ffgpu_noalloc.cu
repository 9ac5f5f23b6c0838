// C ABI: RS256 decode that allocates nothing.
//
// ffgpu_rs256_decode allocates its scratch (the bitsliced syndrome planes,
// then the Berlekamp-Massey records: 36 bytes per block at ecc_len 32) from
// the stream-ordered pool on every call.  Some callers cannot allocate on their hot path: a
// framework that reserved all device memory up front and hands out buffers
// itself (the pool allocation would fail or compete with it), and real-time
// callers that must not see an allocation stall or an out-of-memory error in
// the middle of a repair loop.  This entry point runs the same kernels on a
// fixed scratch array compiled into the library instead.
//
// Limits and rules:
// * the scratch is kNoAllocScratchBytes (18 MiB): up to 524,288 blocks per
//   call at ecc_len 32 and 1,048,576 at ecc_len 16; larger requests are
//   rejected with FFGPU_EINVAL, as are codes and buffers the bitsliced
//   kernels do not cover (ecc_len 16 or 32, primitive 2, polynomial 0x11d,
//   4-byte aligned data and parity);
// * nothing in the scratch has to start at zero: the syndrome kernel writes
//   every plane word of every group before the Berlekamp-Massey kernel reads
//   it, and that kernel writes every record word the Chien kernel reads;
// * there is one scratch per device for the whole process, so calls that can
//   overlap on the device -- from different streams, or from different host
//   threads -- race on it; callers must order them (one stream, or events);
// * the scratch address is looked up once per device with
//   cudaGetSymbolAddress; make the first call on a device outside any stream
//   capture;
// * the scratch used is the current device's: the stream must belong to the
//   current device (checked), and a code switched to the table decoder
//   (ffgpu_rs256_set_table_only) is rejected.
#include <cuda_runtime.h>

#include <mutex>

#include "common.cuh"
#include "handles.h"
#include "rs256.cuh"

using namespace ffgpu;

namespace {

constexpr size_t kNoAllocScratchBytes = (size_t)18 << 20;
__device__ __align__(256) uint8_t g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_addr_mu;
void *g_addr[kMaxDevices] = {};

void *scratch_address() {
    int dev = 0;
    FFGPU_CHECK_CUDA(cudaGetDevice(&dev));
    FFGPU_REQUIRE(dev >= 0 && dev < kMaxDevices, "device index out of range");
    std::lock_guard<std::mutex> lk(g_addr_mu);
    if (!g_addr[dev]) FFGPU_CHECK_CUDA(cudaGetSymbolAddress(&g_addr[dev], g_noalloc_scratch));
    return g_addr[dev];
}

}  // namespace

extern "C" {

int ffgpu_rs256_decode_noalloc(const ffgpu_rs256 *code, uint8_t *data, uint8_t *parity, size_t nblocks,
                               size_t message_len, uint8_t *status, void *stream) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        const Rs256Code &c = *code->code;
        FFGPU_REQUIRE(message_len >= 1 && message_len + (size_t)c.ecc <= 255, "block_len must be <= 255");
        FFGPU_REQUIRE(c.fast && (c.ecc == 16 || c.ecc == 32),
                      "decode without allocation covers ecc_len 16 and 32 with primitive 2 and polynomial 0x11d");
        FFGPU_REQUIRE(!c.table_only,
                      "decode without allocation runs the bitsliced kernels; this code is set to the table decoder "
                      "(ffgpu_rs256_set_table_only)");
        FFGPU_REQUIRE((((uintptr_t)data | (uintptr_t)parity) & 3) == 0,
                      "decode without allocation needs 4-byte aligned data and parity");
        const size_t need = rs256_fast_scratch_bytes(c.ecc, nblocks);
        if (need > kNoAllocScratchBytes)
            throw Error(FFGPU_EINVAL, "decode without allocation: " + std::to_string(nblocks) + " blocks need " +
                                          std::to_string(need) + " bytes of scratch, the fixed scratch holds " +
                                          std::to_string(kNoAllocScratchBytes) + "; split the request");
        if (nblocks == 0) return;
        int dev = 0;
        FFGPU_CHECK_CUDA(cudaGetDevice(&dev));
        if (stream) {
            int sdev = dev;
            FFGPU_CHECK_CUDA(cudaStreamGetDevice((cudaStream_t)stream, &sdev));
            FFGPU_REQUIRE(sdev == dev, "decode without allocation: the stream belongs to another device than the "
                                       "current one, whose scratch array the call would use");
        }
        void *scratch = scratch_address();
        if (!rs256_fast_decode_with(c, data, parity, nblocks, (int)message_len, status, scratch, (cudaStream_t)stream))
            throw Error(FFGPU_EINVAL, "decode without allocation: request not covered by the bitsliced kernels");
    });
}

}  // extern "C"
