// RS256 code object shared by the table kernels (rs256.cu) and the bitsliced
// kernels (rs256_bitsliced.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "gf256.h"

namespace ffgpu {

struct Rs256Code {
    GF256Host gf;
    int ecc;
    int primitive, polynomial;
    int W = 1;  // 32-bit words holding one remainder (power of two >= ecc/4)
    uint8_t generator[256];
    uint8_t roots[256];
    std::vector<uint32_t> lut_words;
    uint32_t *d_lut = nullptr;
    uint8_t *d_exp512 = nullptr;
    uint8_t *d_log256 = nullptr;
    bool fast = false;       // bitsliced kernels available for this code
    void *fast_state = nullptr;
    bool table_only = false;  // force the table kernels (cross-checks)

    Rs256Code(int ecc, int primitive, int polynomial);
    ~Rs256Code();
    Rs256Code(const Rs256Code &) = delete;
    Rs256Code &operator=(const Rs256Code &) = delete;
};

void rs256_encode(const Rs256Code &c, const uint8_t *data, size_t nblocks, int msg_len, uint8_t *parity,
                  cudaStream_t st);
void rs256_decode(const Rs256Code &c, uint8_t *data, uint8_t *parity, size_t nblocks, int msg_len, uint8_t *status,
                  cudaStream_t st);
void rs256_encode_table(const Rs256Code &c, const uint8_t *data, size_t nblocks, int msg_len, uint8_t *parity,
                        cudaStream_t st);
void rs256_decode_table(const Rs256Code &c, uint8_t *data, uint8_t *parity, size_t nblocks, int msg_len,
                        uint8_t *status, uint8_t *synds, cudaStream_t st);

// syndromes (ecc bytes per block, S_0 first), bitsliced kernel when it covers
// the request, else the table kernel
void rs256_synds(const Rs256Code &c, const uint8_t *data, const uint8_t *parity, size_t nblocks, int msg_len,
                 uint8_t *synds, cudaStream_t st);
bool rs256_fast_synds(const Rs256Code &c, const uint8_t *data, const uint8_t *parity, size_t nblocks, int msg_len,
                      uint8_t *synds, cudaStream_t st);

// bitsliced fast path (rs256_bitsliced.cu); the *_encode/_decode functions
// return false when they do not cover the request
bool rs256_fast_init(Rs256Code &c);
void rs256_fast_free(Rs256Code &c);
bool rs256_fast_encode(const Rs256Code &c, const uint8_t *data, size_t nblocks, int msg_len, uint8_t *parity,
                       cudaStream_t st);
bool rs256_fast_decode(const Rs256Code &c, uint8_t *data, uint8_t *parity, size_t nblocks, int msg_len,
                       uint8_t *status, cudaStream_t st);
// the bitsliced decode on caller-provided scratch of rs256_fast_scratch_bytes
// bytes (4-byte aligned); returns false when the request is not covered
size_t rs256_fast_scratch_bytes(int ecc, size_t nblocks);
bool rs256_fast_decode_with(const Rs256Code &c, uint8_t *data, uint8_t *parity, size_t nblocks, int msg_len,
                            uint8_t *status, void *scratch, cudaStream_t st);

}  // namespace ffgpu
