// RS256: Reed-Solomon over GF(2^8) -- code objects and the table-driven
// kernels that serve every (ecc_len, primitive, polynomial, length).
//
// Encoder (reed_solomon.hpp:169-297): a byte-serial LFSR over the row table
// lut[v] = v * x^ecc mod g held in shared memory as 32-bit words, one thread
// per block.  The reference's slicing-by-N loops combine N rows of this same
// linear table, so for a field the parity is identical.
//
// Decoder (reed_solomon.hpp:559-595): one thread per block.  The remainder
// R = r(x) * x^ecc mod g is formed with the same LFSR; R == 0 exactly when all
// syndromes vanish.  Otherwise S_j = r(a^j) = sum_m R[m] a^{-j(m+1)}, followed
// by the reference's Berlekamp-Massey (:655-702), its root search over
// positions [0, size + ecc) (:516-537), Forney (:704-743) and the in-place
// correction (:583-592).  A block whose decode fails is left untouched.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "common.cuh"
#include "gf256.h"
#include "rs256.cuh"
#include "rs256_device.cuh"

namespace ffgpu {

template <int W>
__global__ void __launch_bounds__(128) rs256_encode_table_kernel(const uint8_t *__restrict__ data, size_t nblocks,
                                                                 int msg_len, const uint32_t *__restrict__ lut,
                                                                 int ecc, uint8_t *__restrict__ parity) {
    extern __shared__ __align__(16) uint32_t smem[];
    uint32_t *s_lut = smem;
    uint8_t *s_data = reinterpret_cast<uint8_t *>(smem + 256 * W);
    for (int i = threadIdx.x; i < 256 * W; i += blockDim.x) s_lut[i] = lut[i];
    const size_t first = (size_t)blockIdx.x * blockDim.x;
    const size_t nb = min((size_t)blockDim.x, nblocks - first);
    stage_bytes(s_data, data + first * (size_t)msg_len, nb * (size_t)msg_len);
    __syncthreads();
    if (threadIdx.x >= nb) return;
    rs256_encode_one<W>(s_data + (size_t)threadIdx.x * msg_len, msg_len, s_lut,
                        parity + (first + threadIdx.x) * (size_t)ecc, ecc);
}

// Per-thread decode scratch, interleaved across threads so that lock-step
// accesses of a warp fall on consecutive bytes: in shared memory after the
// tables (gscratch == NULL, decode_scratch_bytes(ecc) for each of the CTA's
// threads), else in global memory (256-byte columns across the launch).
template <int W>
__global__ void __launch_bounds__(128) rs256_decode_table_kernel(uint8_t *__restrict__ data,
                                                                 uint8_t *__restrict__ parity, size_t nblocks,
                                                                 int msg_len, const uint32_t *__restrict__ lut,
                                                                 const uint8_t *__restrict__ exp512,
                                                                 const uint8_t *__restrict__ log256, int ecc,
                                                                 uint8_t *__restrict__ status,
                                                                 uint8_t *__restrict__ synds_out,
                                                                 uint8_t *__restrict__ gscratch) {
    extern __shared__ __align__(16) uint32_t smem[];
    uint32_t *s_lut = smem;
    uint8_t *ex = reinterpret_cast<uint8_t *>(smem + 256 * W);
    uint8_t *lg = ex + 512;
    for (int i = threadIdx.x; i < 256 * W; i += blockDim.x) s_lut[i] = lut[i];
    for (int i = threadIdx.x; i < 512; i += blockDim.x) ex[i] = exp512[i];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) lg[i] = log256[i];
    __syncthreads();
    const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t nthreads = (size_t)gridDim.x * blockDim.x;
    const DecodeScratchG sc = gscratch ? DecodeScratchG(gscratch, tid, nthreads)
                                       : DecodeScratchG(reinterpret_cast<uint8_t *>(lg + 256), threadIdx.x,
                                                        blockDim.x, ecc);
    for (size_t blk = tid; blk < nblocks; blk += nthreads)
        decode_one<W>(data + blk * (size_t)msg_len, parity + blk * (size_t)ecc, msg_len, ecc, s_lut, ex, lg, sc,
                      status ? status + blk : nullptr, synds_out ? synds_out + blk * (size_t)ecc : nullptr);
}

// ---------------------------------------------------------------- host

static int bucket_words(int ecc) {
    const int w = (ecc + 3) / 4;
    int b = 1;
    while (b < w) b *= 2;
    return b;
}

Rs256Code::Rs256Code(int ecc_, int primitive_, int polynomial_)
    : gf((uint8_t)primitive_, (uint8_t)(polynomial_ & 0xff)), ecc(ecc_), primitive(primitive_),
      polynomial(polynomial_) {
    FFGPU_REQUIRE(ecc_ >= 1 && ecc_ <= 254, "ecc_len must be in [1, 254]");
    FFGPU_REQUIRE(gf.is_field(), "primitive does not generate GF(2^8) with this polynomial");
    rs256_generator(gf, ecc, generator, roots);
    std::vector<uint8_t> lut;
    rs256_lut(gf, ecc, generator, lut);
    W = bucket_words(ecc);
    lut_words.assign((size_t)256 * W, 0);
    for (int v = 0; v < 256; ++v)
        for (int j = 0; j < ecc; ++j)
            lut_words[(size_t)v * W + j / 4] |= (uint32_t)lut[(size_t)v * ecc + j] << (8 * (j % 4));
    uint8_t exp512[512], log256[256];
    for (int i = 0; i < 512; ++i) exp512[i] = gf.exp[i % 255];
    std::memcpy(log256, gf.log, 256);
    FFGPU_CHECK_CUDA(cudaMalloc(&d_lut, lut_words.size() * 4));
    FFGPU_CHECK_CUDA(cudaMalloc(&d_exp512, 512));
    FFGPU_CHECK_CUDA(cudaMalloc(&d_log256, 256));
    FFGPU_CHECK_CUDA(cudaMemcpy(d_lut, lut_words.data(), lut_words.size() * 4, cudaMemcpyHostToDevice));
    FFGPU_CHECK_CUDA(cudaMemcpy(d_exp512, exp512, 512, cudaMemcpyHostToDevice));
    FFGPU_CHECK_CUDA(cudaMemcpy(d_log256, log256, 256, cudaMemcpyHostToDevice));
    fast = rs256_fast_init(*this);
}

Rs256Code::~Rs256Code() {
    rs256_fast_free(*this);
    if (d_lut) cudaFree(d_lut);
    if (d_exp512) cudaFree(d_exp512);
    if (d_log256) cudaFree(d_log256);
}

template <int W>
static void launch_encode_table(const Rs256Code &c, const uint8_t *data, size_t nblocks, int msg_len, uint8_t *parity,
                                cudaStream_t st) {
    const unsigned threads = 128;
    const size_t smem = (size_t)256 * W * 4 + (size_t)threads * msg_len + 16;
    // once per process (a thread-safe static initialiser)
    static const bool attr = [] {
        FFGPU_CHECK_CUDA(cudaFuncSetAttribute(rs256_encode_table_kernel<W>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              200 * 1024));
        return true;
    }();
    (void)attr;
    KernelTimer kt_timer("rs256_encode_table_kernel", st);
    rs256_encode_table_kernel<W><<<grid_for(nblocks, threads), threads, smem, st>>>(data, nblocks, msg_len, c.d_lut,
                                                                                    c.ecc, parity);
    check_launch("rs256_encode_table_kernel");
}

template <int W>
static void launch_decode_table(const Rs256Code &c, uint8_t *data, uint8_t *parity, size_t nblocks, int msg_len,
                                uint8_t *status, uint8_t *synds, cudaStream_t st) {
    const unsigned threads = 128;
    const size_t tables = (size_t)256 * W * 4 + 768;
    const size_t sm_scratch = decode_scratch_bytes(c.ecc) * threads;
    const bool in_smem = tables + sm_scratch <= 100 * 1024;  // ecc <= 64
    const size_t smem = tables + (in_smem ? sm_scratch : 0);
    static const bool attr = [] {
        FFGPU_CHECK_CUDA(cudaFuncSetAttribute(rs256_decode_table_kernel<W>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              200 * 1024));
        return true;
    }();
    (void)attr;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t grid = std::min<size_t>(grid_for(nblocks, threads), (size_t)(sms > 0 ? sms : 132) * 8);
    void *scratch = nullptr;
    if (!in_smem) FFGPU_CHECK_CUDA(cudaMallocAsync(&scratch, grid * threads * kDecodeScratchBytes, st));
    KernelTimer kt_timer("rs256_decode_table_kernel", st);
    rs256_decode_table_kernel<W><<<(unsigned)grid, threads, smem, st>>>(data, parity, nblocks, msg_len, c.d_lut,
                                                                        c.d_exp512, c.d_log256, c.ecc, status, synds,
                                                                        (uint8_t *)scratch);
    cudaError_t le = cudaGetLastError();
    if (scratch) cudaFreeAsync(scratch, st);
    if (le != cudaSuccess) throw Error(FFGPU_ECUDA, std::string("rs256_decode_table_kernel: ") + cudaGetErrorString(le));
    launched();
}

#define FFGPU_W_DISPATCH(W, CALL)          \
    switch (W) {                           \
        case 1: { constexpr int w_ = 1; CALL; } break;   \
        case 2: { constexpr int w_ = 2; CALL; } break;   \
        case 4: { constexpr int w_ = 4; CALL; } break;   \
        case 8: { constexpr int w_ = 8; CALL; } break;   \
        case 16: { constexpr int w_ = 16; CALL; } break; \
        case 32: { constexpr int w_ = 32; CALL; } break; \
        default: { constexpr int w_ = 64; CALL; } break; \
    }

void rs256_encode_table(const Rs256Code &c, const uint8_t *data, size_t nblocks, int msg_len, uint8_t *parity,
                        cudaStream_t st) {
    if (nblocks == 0) return;
    FFGPU_W_DISPATCH(c.W, (launch_encode_table<w_>(c, data, nblocks, msg_len, parity, st)));
}

void rs256_decode_table(const Rs256Code &c, uint8_t *data, uint8_t *parity, size_t nblocks, int msg_len,
                        uint8_t *status, uint8_t *synds, cudaStream_t st) {
    if (nblocks == 0) return;
    FFGPU_W_DISPATCH(c.W, (launch_decode_table<w_>(c, data, parity, nblocks, msg_len, status, synds, st)));
}

void rs256_encode(const Rs256Code &c, const uint8_t *data, size_t nblocks, int msg_len, uint8_t *parity,
                  cudaStream_t st) {
    if (nblocks == 0) return;
    if (c.fast && rs256_fast_encode(c, data, nblocks, msg_len, parity, st)) return;
    rs256_encode_table(c, data, nblocks, msg_len, parity, st);
}

void rs256_synds(const Rs256Code &c, const uint8_t *data, const uint8_t *parity, size_t nblocks, int msg_len,
                 uint8_t *synds, cudaStream_t st) {
    if (nblocks == 0) return;
    if (c.fast && rs256_fast_synds(c, data, parity, nblocks, msg_len, synds, st)) return;
    rs256_decode_table(c, const_cast<uint8_t *>(data), const_cast<uint8_t *>(parity), nblocks, msg_len, nullptr,
                       synds, st);
}

void rs256_decode(const Rs256Code &c, uint8_t *data, uint8_t *parity, size_t nblocks, int msg_len, uint8_t *status,
                  cudaStream_t st) {
    if (nblocks == 0) return;
    if (c.fast && rs256_fast_decode(c, data, parity, nblocks, msg_len, status, st)) return;
    rs256_decode_table(c, data, parity, nblocks, msg_len, status, nullptr, st);
}

}  // namespace ffgpu
