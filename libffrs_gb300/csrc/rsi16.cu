// RSi16 kernels.  One warp owns one block at a time (persistent warps); the
// block and the reference's repair scratch (ntt_len + 6 * ecc words,
// libffrs/rsi16v_impl.hpp:122-168) live in a per-warp workspace in shared
// memory when it fits, else in global memory.  Every polynomial operation of
// the reference's W = 1 code path is mirrored step for step with its uint32
// length arithmetic; the vector loops inside each step are spread over the 32
// lanes with __syncwarp() between dependent steps.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <type_traits>
#include <vector>

#include "common.cuh"
#include "rsi16.cuh"

#include "rsi16_device.cuh"
#include "rsi16_bt.cuh"

namespace ffgpu {

// ---------------------------------------------------------------- host tables

uint32_t Rsi16Code::rbo(uint32_t i) const {
    uint16_t b = (uint16_t)i;
    b = (uint16_t)(((b >> 1) & 0x5555) | ((b & 0x5555) << 1));
    b = (uint16_t)(((b >> 2) & 0x3333) | ((b & 0x3333) << 2));
    b = (uint16_t)(((b >> 4) & 0x0f0f) | ((b & 0x0f0f) << 4));
    b = (uint16_t)((b >> 8) | (b << 8));
    return (uint32_t)(b >> rbo_shift);
}

static uint32_t neg(uint32_t a) { return a == 0 ? 0 : 0x10001u - a; }

// the twiddles of the one-block-per-thread kernels (rsi16_bt.cuh), with their
// Shoup companions
template <int N>
static BtTw<N> bt_twiddles(const Rsi16Code &c) {
    BtTw<N> tw;
    for (int i = 0; i < N / 2; ++i) {
        tw.ct[i] = c.roots_ecc[i];
        tw.gs[i] = c.roots_i_ecc[i];
    }
    for (int i = 0; i < N; ++i) tw.mix[i] = c.ecc_mix[i];
    auto shoup = [](uint32_t w) { return (uint32_t)(((uint64_t)w << 32) / 0x10001u); };
    for (int i = 0; i < N / 2; ++i) {
        tw.ct_s[i] = shoup(tw.ct[i]);
        tw.gs_s[i] = shoup(tw.gs[i]);
    }
    for (int i = 0; i < N; ++i) tw.mix_s[i] = shoup(tw.mix[i]);
    return tw;
}

Rsi16Code::Rsi16Code(size_t block_len_, size_t ecc_len, uint32_t primitive_)
    : primitive(primitive_), block_len(block_len_), ecc(ecc_len) {
    if (ecc_len < 2 || (ecc_len & (ecc_len - 1)))
        throw Error(FFGPU_EASSERT, "ecc_len must be a power of 2: " + std::to_string(ecc_len));
    if (block_len_ < ecc_len || block_len_ % ecc_len)
        throw Error(FFGPU_EASSERT, "block_len must be a multiple of ecc_len. block_len: " + std::to_string(block_len_) +
                                       " ecc_len: " + std::to_string(ecc_len));
    if (block_len_ > 65536) throw Error(FFGPU_EASSERT, "block_len must be <= 65536");
    // GF(65537) exp/log built with gf_mul_mod (libffrs/galois.hpp:133-144, 239-250)
    exp_.assign(65537, 0);
    log_.assign(65537, 0);
    uint32_t x = 1;
    for (uint32_t i = 0; i < 65537; ++i) {
        exp_[i] = x;
        log_[x] = i;
        uint64_t prod = (uint64_t)x * primitive;
        x = (prod > 0xffffffffull ? 1u : (uint32_t)prod) % 0x10001u;
    }
    // PyGFi16 ctor check (libffrs/pygfi16.hpp:53-58)
    if (!(pow(primitive, 32768) == 65536 && pow(primitive, 65536) == 1))
        throw Error(FFGPU_EASSERT, std::to_string(primitive) + " is not a primitive element of GF(65537)");
    message_len = block_len - ecc;
    ecc_mask = (uint32_t)(ecc - 1);
    pntt_blocks = block_len / ecc;
    size_t lg = 0;
    while (((size_t)1 << lg) < block_len) ++lg;
    if (lg == 0) lg = 1;
    ntt_len = (size_t)1 << lg;
    rbo_shift = 16u - (unsigned)__builtin_ctzl(ntt_len);
    ntt_len_i = inv((uint32_t)ntt_len);
    ecc_len_i = inv((uint32_t)ecc);
    ecc2_len_i = inv((uint32_t)(ecc * 2));
    root = pow(primitive, (uint32_t)(65536 / ntt_len));
    if (pow(root, (uint32_t)ntt_len) != 1 || pow(root, (uint32_t)(ntt_len / 2)) != 65536)
        throw Error(FFGPU_EASSERT, "ntt root of unity sanity check failed");
    const uint32_t root_i = inv(root);
    roots_ntt.resize(ntt_len);
    roots_i_ntt.resize(ntt_len);
    for (size_t i = 0; i < ntt_len; ++i) {
        roots_ntt[i] = pow(root, (uint32_t)i);
        roots_i_ntt[i] = pow(root_i, (uint32_t)i);
    }
    rbo_ecc.resize(ecc);
    for (size_t i = 0; i < ecc; ++i) rbo_ecc[i] = rbo((uint32_t)(i * (ntt_len / ecc)));
    const uint32_t er = pow(primitive, (uint32_t)(65536 / ecc));
    if (pow(er, (uint32_t)ecc) != 1 || pow(er, (uint32_t)(ecc / 2)) != 65536)
        throw Error(FFGPU_EASSERT, "ntt root of unity sanity check failed");
    const uint32_t er_i = inv(er);
    roots_ecc.resize(ecc);
    roots_i_ecc.resize(ecc);
    for (size_t i = 0; i < ecc; ++i) {
        roots_ecc[i] = pow(er, (uint32_t)i);
        roots_i_ecc[i] = pow(er_i, (uint32_t)i);
    }
    const uint32_t er2 = pow(primitive, (uint32_t)(65536 / (ecc * 2)));
    if (pow(er2, (uint32_t)(ecc * 2)) != 1 || pow(er2, (uint32_t)ecc) != 65536)
        throw Error(FFGPU_EASSERT, "ntt root of unity sanity check failed");
    const uint32_t er2_i = inv(er2);
    roots_ecc2.resize(ecc * 2);
    roots_i_ecc2.resize(ecc * 2);
    for (size_t i = 0; i < ecc * 2; ++i) {
        roots_ecc2[i] = pow(er2, (uint32_t)i);
        roots_i_ecc2[i] = pow(er2_i, (uint32_t)i);
    }
    pntt_shift.resize(block_len);
    for (size_t i = 0; i < block_len; ++i) {
        size_t blk = (i / ecc) * ecc, j = i - blk;
        pntt_shift[i] = pow(root, (uint32_t)(j * rbo((uint32_t)blk)));
    }
    pintt_shift.resize(ntt_len);
    for (size_t i = 0; i < ntt_len; ++i) {
        size_t blk = (i / ecc) * ecc, j = i - blk;
        pintt_shift[i] = div(pow(root_i, (uint32_t)(j * rbo((uint32_t)blk))), (uint32_t)ntt_len);
    }
    ecc_mix.resize(ecc);
    const uint32_t w = roots_ntt[rbo((uint32_t)(block_len - ecc))];
    const uint32_t w_i = inv(w);
    for (size_t i = 0; i < ecc; ++i) ecc_mix[i] = neg(div(pow(w_i, (uint32_t)i), (uint32_t)ecc));

    auto shoup = [](const std::vector<uint32_t> &v) {
        std::vector<uint32_t> o(v.size());
        for (size_t i = 0; i < v.size(); ++i) o[i] = (uint32_t)(((uint64_t)v[i] << 32) / 0x10001u);
        return o;
    };
    pntt_shift_s = shoup(pntt_shift);
    pintt_shift_s = shoup(pintt_shift);

    // one device allocation for all tables
    std::vector<uint32_t> all;
    auto put = [&](const std::vector<uint32_t> &v) {
        size_t off = all.size();
        all.insert(all.end(), v.begin(), v.end());
        while (all.size() % 32) all.push_back(0);
        return off;
    };
    std::vector<uint32_t> inv_tab(65537);
    for (uint32_t a = 0; a < 65537; ++a) inv_tab[a] = inv(a);
    const size_t o_rn = put(roots_ntt), o_re = put(roots_ecc), o_rie = put(roots_i_ecc), o_re2 = put(roots_ecc2),
                 o_rie2 = put(roots_i_ecc2), o_ps = put(pntt_shift), o_pis = put(pintt_shift), o_rbo = put(rbo_ecc),
                 o_mix = put(ecc_mix), o_inv = put(inv_tab), o_pss = put(pntt_shift_s), o_piss = put(pintt_shift_s);
    // the block-per-thread twiddles of ecc 32 / 64, for launches that cannot
    // take them as a kernel parameter (the mixed batch)
    std::vector<uint32_t> btw;
    if (ecc == 64 || ecc == 32) {
        if (ecc == 64) {
            const BtTw<64> tw = bt_twiddles<64>(*this);
            btw.assign((const uint32_t *)&tw, (const uint32_t *)&tw + sizeof tw / 4);
        } else {
            const BtTw<32> tw = bt_twiddles<32>(*this);
            btw.assign((const uint32_t *)&tw, (const uint32_t *)&tw + sizeof tw / 4);
        }
    }
    const size_t o_btw = btw.empty() ? 0 : put(btw);
    FFGPU_CHECK_CUDA(cudaMalloc(&d_tables, all.size() * 4));
    FFGPU_CHECK_CUDA(cudaMemcpy(d_tables, all.data(), all.size() * 4, cudaMemcpyHostToDevice));
    dev.roots_ntt = d_tables + o_rn;
    dev.roots_ecc = d_tables + o_re;
    dev.roots_i_ecc = d_tables + o_rie;
    dev.roots_ecc2 = d_tables + o_re2;
    dev.roots_i_ecc2 = d_tables + o_rie2;
    dev.pntt_shift = d_tables + o_ps;
    dev.pintt_shift = d_tables + o_pis;
    dev.rbo_ecc = d_tables + o_rbo;
    dev.ecc_mix = d_tables + o_mix;
    dev.inv_tab = d_tables + o_inv;
    dev.pntt_shift_s = d_tables + o_pss;
    dev.bt_tw = btw.empty() ? nullptr : d_tables + o_btw;
    dev.pintt_shift_s = d_tables + o_piss;
    dev.block_len = (uint32_t)block_len;
    dev.message_len = (uint32_t)message_len;
    dev.ecc = (uint32_t)ecc;
    dev.ntt_len = (uint32_t)ntt_len;
    dev.pntt_blocks = (uint32_t)pntt_blocks;
    dev.ecc_mask = ecc_mask;
    dev.rbo_shift = rbo_shift;
    dev.ecc_len_i = ecc_len_i;
    dev.ecc2_len_i = ecc2_len_i;
    dev.temp_len = (uint32_t)(ntt_len + 6 * ecc);
}

Rsi16Code::~Rsi16Code() {
    if (d_tables) cudaFree(d_tables);
}

// ---------------------------------------------------------------- kernels

struct WarpCtx {
    int lane, warp_global, nwarps;
    uint32_t *ws;
};

__device__ __forceinline__ WarpCtx warp_ctx(uint32_t *gscratch, uint32_t ws_words) {
    extern __shared__ uint32_t smem_ws[];
    WarpCtx w;
    w.lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    w.warp_global = blockIdx.x * (blockDim.x >> 5) + wib;
    w.nwarps = gridDim.x * (blockDim.x >> 5);
    w.ws = gscratch ? gscratch + (size_t)w.warp_global * ws_words : smem_ws + (size_t)wib * ws_words;
    return w;
}

// EPL > 0: ecc == 32 * EPL, the transforms run on registers
template <int EPL>
__global__ void rsi16_encode_warp_kernel(Rsi16Dev c, BlockView v, size_t nblocks, uint32_t *gscratch,
                                         uint32_t ws_words) {
    WarpCtx w = warp_ctx(gscratch, ws_words);
    if constexpr (EPL > 0) {
        RegTw<EPL> tw;
        reg_twiddles<EPL>(c, w.lane, tw);
        // two blocks per pass (a lone last block pairs with itself)
        for (size_t b = 2 * (size_t)w.warp_global; b < nblocks; b += 2 * (size_t)w.nwarps)
            rsi16_encode_pair_reg<EPL>(c, v, b, b + 1 < nblocks ? b + 1 : b, tw, w.lane);
    } else {
        for (size_t b = w.warp_global; b < nblocks; b += w.nwarps) rsi16_encode_block(c, v, b, w.ws, w.lane);
    }
}

// ecc = N: one block per thread (rsi16_bt.cuh), 32 blocks per warp.  Blocks
// are contiguous uint16 words (message_len words of message, N of parity).
template <int N>
__global__ void __launch_bounds__(128, N == 64 ? 3 : 4) rsi16_encode_bt_kernel(Rsi16Dev c, const __grid_constant__ BtTw<N> tw,
                                                                 const uint16_t *__restrict__ msg,
                                                                 uint16_t *__restrict__ par, size_t nblocks) {
    extern __shared__ __align__(16) uint8_t bt_smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, wpc = blockDim.x >> 5;
    uint8_t *bufs = bt_smem + wib * bt_warp_smem<N>();
    const size_t ntiles = (nblocks + 31) / 32;
    for (size_t t = (size_t)blockIdx.x * wpc + wib; t < ntiles; t += (size_t)gridDim.x * wpc)
        bt_encode_tile<N>(c, tw, bufs, msg, par, t * 32, nblocks, lane);
}

// syndromes of block b go to synds[(b / out_group) * out_gstride + (b % out_group) * ecc]
__global__ void rsi16_synd_warp_kernel(Rsi16Dev c, BlockView v, size_t nblocks, uint32_t *synds, size_t out_group,
                                       size_t out_gstride, uint32_t *gscratch, uint32_t ws_words) {
    WarpCtx w = warp_ctx(gscratch, ws_words);
    for (size_t b = w.warp_global; b < nblocks; b += w.nwarps) {
        w_gather(c, v, b, w.ws, true, w.lane);
        w_pntt(c, w.ws, c.pntt_blocks, w.lane);
        uint32_t *o = synds + (b / out_group) * out_gstride + (b % out_group) * c.ecc;
        for (uint32_t k = w.lane; k < c.ecc; k += 32) o[k] = w.ws[k];
        __syncwarp();
    }
}

// ecc = N < 32: 32 / N blocks per warp pass, the transforms on registers
template <int N>
__global__ void __launch_bounds__(128) rsi16_encode_sub_kernel(Rsi16Dev c, BlockView v, size_t nblocks) {
    constexpr int G = 32 / N;
    const int lane = threadIdx.x & 31;
    SubTw<N> tw;
    sub_twiddles<N>(c, lane % N, tw);
    const size_t warp = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const size_t nw = ((size_t)gridDim.x * blockDim.x) >> 5;
    for (size_t b0 = warp * G; b0 < nblocks; b0 += nw * G) rsi16_encode_sub_pass<N>(c, v, b0, nblocks, tw, lane);
}

// syndromes, ecc = N < 32 (output layout as rsi16_synd_warp_kernel)
template <int N>
__global__ void __launch_bounds__(128) rsi16_synd_sub_kernel(Rsi16Dev c, BlockView v, size_t nblocks,
                                                             uint32_t *synds, size_t out_group, size_t out_gstride) {
    constexpr int G = 32 / N;
    const int lane = threadIdx.x & 31, e = lane % N, s = lane / N;
    SubTw<N> tw;
    sub_twiddles<N>(c, e, tw);
    const size_t warp = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const size_t nw = ((size_t)gridDim.x * blockDim.x) >> 5;
    for (size_t b0 = warp * G; b0 < nblocks; b0 += nw * G) {
        const size_t b = b0 + s;
        const bool act = b < nblocks;
        const uint32_t a = sub_pntt<N>(c, v, act ? b : b0, act, c.pntt_blocks, true, tw, e);
        if (act) synds[(b / out_group) * out_gstride + (b % out_group) * N + e] = a;
    }
}

// syndromes, ecc = 32 * EPL: two blocks per warp pass on registers
template <int EPL>
__global__ void __launch_bounds__(128) rsi16_synd_reg_kernel(Rsi16Dev c, BlockView v, size_t nblocks,
                                                             uint32_t *synds, size_t out_group, size_t out_gstride) {
    const int lane = threadIdx.x & 31;
    RegTw<EPL> tw;
    reg_twiddles<EPL>(c, lane, tw);
    const size_t warp = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const size_t nw = ((size_t)gridDim.x * blockDim.x) >> 5;
    for (size_t b = 2 * warp; b < nblocks; b += 2 * nw) {
        const size_t b1 = b + 1 < nblocks ? b + 1 : b;
        uint32_t a0[EPL], a1[EPL];
        reg_pntt2<EPL>(c, v, b, b1, c.pntt_blocks, true, tw, lane, a0, a1);
        uint32_t *o0 = synds + (b / out_group) * out_gstride + (b % out_group) * c.ecc;
        uint32_t *o1 = synds + (b1 / out_group) * out_gstride + (b1 % out_group) * c.ecc;
#pragma unroll
        for (int h = 0; h < EPL; ++h) {
            o0[lane * EPL + h] = a0[h];
            o1[lane * EPL + h] = a1[h];
        }
    }
}

// blocks repaired by the bounded-distance path / by the step-for-step mirror
__device__ unsigned long long g_repair_fast_blocks, g_repair_mirror_blocks;

template <int EPL>
__global__ void rsi16_repair_warp_kernel(Rsi16Dev c, BlockView v, size_t nblocks, uint8_t *status,
                                         const uint8_t *active, uint32_t *gscratch, uint32_t ws_words) {
    WarpCtx w = warp_ctx(gscratch, ws_words);
    RegTw<EPL ? EPL : 1> tw;
    if constexpr (EPL > 0) reg_twiddles<EPL>(c, w.lane, tw);
    unsigned long long nfast = 0, nmirror = 0;
    for (size_t b = w.warp_global; b < nblocks; b += w.nwarps) {
        if (active && !active[b]) continue;
        if (rsi16_repair_bm_block_t<EPL>(c, v, b, w.ws, status, tw, w.lane)) {
            ++nfast;
        } else {
            rsi16_repair_block(c, v, b, w.ws, status, w.lane);
            ++nmirror;
        }
    }
    if (w.lane == 0 && (nfast | nmirror)) {
        atomicAdd(&g_repair_fast_blocks, nfast);
        atomicAdd(&g_repair_mirror_blocks, nmirror);
    }
}

// ecc 32 and 64: batches of 32 blocks per warp, syndromes warp-wide,
// Berlekamp-Massey one block per lane, roots and Forney warp-wide.  Warps take
// batches from a counter, so that a warp busy with a block the
// bounded-distance path does not accept (the step-for-step mirror, about 10^5
// instructions on one warp, on its workspace slice of mirror_ws) takes fewer
// batches.  The warp workspace in shared memory is the batch's syndrome
// columns [ecc][33], locator columns [ecc/2 + 1][33] and the finishing scratch
// (two root lists of ecc + 1 words, Omega and C').

template <int EPL>
__global__ void __launch_bounds__(128, 4) rsi16_repair_batch_kernel(Rsi16Dev c, BlockView v, size_t nblocks,
                                                                 uint8_t *status, const uint8_t *active,
                                                                 uint32_t ws_words, unsigned int *next_batch,
                                                                 uint32_t *mirror_ws, uint32_t mirror_words) {
    constexpr int T = 16 * EPL;
    WarpCtx w = warp_ctx(nullptr, ws_words);
    RegTw<EPL> tw;
    reg_twiddles<EPL>(c, w.lane, tw);
    uint32_t *mws = mirror_ws + (size_t)w.warp_global * mirror_words;
    const size_t nbatches = (nblocks + 31) / 32;
    unsigned long long nfast = 0, nmirror = 0;
    for (;;) {
        unsigned int bi = 0;
        if (w.lane == 0) bi = atomicAdd(next_batch, 1u);
        bi = __shfl_sync(0xffffffffu, bi, 0);
        if (bi >= nbatches) break;
        const size_t base = (size_t)bi * 32;
        rsi16_repair32<EPL>(c, v, base, (int)min((size_t)32, nblocks - base), status, active, tw, w.lane, w.ws, mws,
                            nfast, nmirror);
    }
    if (w.lane == 0 && (nfast | nmirror)) {
        atomicAdd(&g_repair_fast_blocks, nfast);
        atomicAdd(&g_repair_mirror_blocks, nmirror);
    }
}

// ecc = N: the repair with one block per thread (bt_repair_tile); warps take
// tiles of 32 blocks from a counter, blocks the bounded-distance path does
// not accept go to the step-for-step mirror on the warp's slice of mirror_ws.
template <int N>
__global__ void __launch_bounds__(128, N == 64 ? 3 : 4) rsi16_repair_bt_kernel(Rsi16Dev c, const __grid_constant__ BtTw<N> tw,
                                                                 BlockView v, size_t nblocks, uint8_t *status,
                                                                 const uint8_t *active, unsigned int *next_tile,
                                                                 uint32_t *mirror_ws, uint32_t mirror_words) {
    extern __shared__ __align__(16) uint32_t bt_rsmem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, wpc = blockDim.x >> 5;
    uint32_t *ws = bt_rsmem + wib * BtRepairSmem<N>::kWords;
    uint32_t *mws = mirror_ws + ((size_t)blockIdx.x * wpc + wib) * mirror_words;
    uint16_t *msg = (uint16_t *)v.msg, *par = (uint16_t *)v.par;
    const size_t ntiles = (nblocks + 31) / 32;
    unsigned long long nfast = 0, nmirror = 0;
    for (;;) {
        unsigned int t = 0;
        if (lane == 0) t = atomicAdd(next_tile, 1u);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= ntiles) break;
        const size_t blk0 = (size_t)t * 32;
        for (uint32_t m = bt_repair_tile<N>(c, tw, msg, par, blk0, nblocks, status, active, ws, lane, nfast); m;
             m &= m - 1) {
            __syncwarp();
            rsi16_repair_block(c, v, blk0 + (__ffs(m) - 1), mws, status, lane);
            ++nmirror;
        }
    }
    const unsigned int f = __reduce_add_sync(0xffffffffu, (unsigned int)nfast);
    if (lane == 0 && (f | nmirror)) {
        atomicAdd(&g_repair_fast_blocks, (unsigned long long)f);
        atomicAdd(&g_repair_mirror_blocks, nmirror);
    }
}

void rsi16_repair_counters(uint64_t *fast, uint64_t *mirror, bool reset) {
    unsigned long long f = 0, m = 0;
    FFGPU_CHECK_CUDA(cudaDeviceSynchronize());
    FFGPU_CHECK_CUDA(cudaMemcpyFromSymbol(&f, g_repair_fast_blocks, sizeof f));
    FFGPU_CHECK_CUDA(cudaMemcpyFromSymbol(&m, g_repair_mirror_blocks, sizeof m));
    if (fast) *fast = f;
    if (mirror) *mirror = m;
    if (reset) {
        const unsigned long long z = 0;
        FFGPU_CHECK_CUDA(cudaMemcpyToSymbol(g_repair_fast_blocks, &z, sizeof z));
        FFGPU_CHECK_CUDA(cudaMemcpyToSymbol(g_repair_mirror_blocks, &z, sizeof z));
    }
}

__global__ void rsi16_repair_known_warp_kernel(Rsi16Dev c, BlockView v, size_t nblocks, const uint32_t *pos,
                                               const uint32_t *pos_off, const uint32_t *pos_cnt,
                                               uint32_t count_all, const uint8_t *active, uint8_t *status,
                                               uint32_t *gscratch, uint32_t ws_words) {
    WarpCtx w = warp_ctx(gscratch, ws_words);
    for (size_t b = w.warp_global; b < nblocks; b += w.nwarps) {
        if (active && !active[b]) continue;
        rsi16_repair_known_block(c, v, b, pos + (pos_off ? pos_off[b] : 0), pos_cnt ? pos_cnt[b] : count_all,
                                 w.ws, status, w.lane);
    }
}

__global__ void rsi16_sugiyama_kernel(Rsi16Dev c, const uint32_t *synds, size_t nblocks, uint32_t *locator,
                                      uint32_t *evaluator, uint8_t *status, uint32_t *gscratch, uint32_t ws_words) {
    WarpCtx w = warp_ctx(gscratch, ws_words);
    const int lane = w.lane;
    const uint32_t ecc = c.ecc;
    uint32_t *temp = w.ws;
    Scratch s{temp, c.temp_len};
    for (size_t b = w.warp_global; b < nblocks; b += w.nwarps) {
        // py_sugiyama layout (pyrsi16.hpp:653-664): a1 | r1 | temp4
        w_fill(temp, 0, c.temp_len, lane);
        for (uint32_t k = lane; k < ecc; k += 32) temp[ecc + k] = synds[b * ecc + k];
        __syncwarp();
        uint32_t n = 0;
        int st = w_sugiyama(c, s, temp, temp + ecc, temp + 2 * ecc, &n, lane);
        for (uint32_t k = lane; k < ecc; k += 32) {
            locator[b * ecc + k] = temp[k];
            evaluator[b * ecc + k] = temp[ecc + k];
        }
        if (lane == 0) status[b] = st ? FFGPU_STATUS_ASSERT : 0;
        __syncwarp();
    }
}

__global__ void rsi16_roots_kernel(Rsi16Dev c, const uint32_t *poly, uint8_t *is_zero, uint32_t *gscratch) {
    const int lane = threadIdx.x & 31;
    uint32_t *b = gscratch;
    for (uint32_t k = lane; k < c.ntt_len; k += 32) b[k] = k < c.ecc ? poly[k] : 0u;
    __syncwarp();
    w_pintt(c, b, lane);
    for (uint32_t k = lane; k < c.block_len; k += 32) is_zero[k] = b[k] == 0;
}

__global__ void rsi16_mix_kernel(Rsi16Dev c, uint32_t *vecs, size_t nvec) {
    const int lane = threadIdx.x & 31;
    const size_t wg = (size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const size_t nw = (size_t)gridDim.x * (blockDim.x >> 5);
    for (size_t i = wg; i < nvec; i += nw) w_mix(c, vecs + i * c.ecc, lane);
}

// ---------------------------------------------------------------- launches

namespace {

// A launch shape.  Workspaces that do not fit in shared memory come from a
// stream-ordered allocation, freed on the same stream after the launch, so
// that launches on concurrent streams (or inside a captured graph) each get
// their own.
struct Launch {
    unsigned grid = 0, threads = 0;
    size_t smem = 0;
    uint32_t *gscratch = nullptr;
    uint32_t ws_words = 0;
    cudaStream_t st;
    explicit Launch(cudaStream_t s) : st(s) {}
    ~Launch() {
        if (gscratch) cudaFreeAsync(gscratch, st);
    }
    Launch(const Launch &) = delete;
    Launch &operator=(const Launch &) = delete;
};

int num_sms() {
    static const int n = [] {  // once per process (a thread-safe static initialiser)
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        return v > 0 ? v : 132;
    }();
    return n;
}

template <typename K>
void plan(Launch &L, K kernel, size_t nblocks, uint32_t ws_words) {
    L.threads = 128;
    const unsigned warps_per_cta = L.threads / 32;
    const size_t want_warps = nblocks ? nblocks : 1;
    size_t max_ctas = (size_t)num_sms() * 8;
    size_t ctas = std::min(max_ctas, (want_warps + warps_per_cta - 1) / warps_per_cta);
    if (ctas == 0) ctas = 1;
    L.grid = (unsigned)ctas;
    L.ws_words = ws_words;
    const size_t smem = (size_t)warps_per_cta * ws_words * 4;
    if (smem <= 64 * 1024) {
        L.smem = smem;
        FFGPU_CHECK_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024));
    } else {
        L.smem = 0;
        FFGPU_CHECK_CUDA(cudaMallocAsync((void **)&L.gscratch, (size_t)ctas * warps_per_cta * ws_words * 4, L.st));
    }
}

}  // namespace

// register-NTT width for this code (0: the shared-memory transforms)
static int reg_epl(const Rsi16Code &c) { return (c.ecc == 32 || c.ecc == 64 || c.ecc == 128) ? (int)(c.ecc / 32) : 0; }

template <int EPL>
static void launch_encode(const Rsi16Code &c, const BlockView &v, size_t nblocks, cudaStream_t st) {
    Launch L(st);
    plan(L, rsi16_encode_warp_kernel<EPL>, nblocks, EPL ? 0u : (uint32_t)c.block_len);
    KernelTimer kt_timer("rsi16_encode_warp_kernel", st);
    rsi16_encode_warp_kernel<EPL><<<L.grid, L.threads, L.smem, st>>>(c.dev, v, nblocks, L.gscratch, L.ws_words);
    check_launch("rsi16_encode_warp_kernel");
}

// sub-warp transform width for this code (0: none)
static int sub_n(const Rsi16Code &c) { return (c.ecc == 2 || c.ecc == 4 || c.ecc == 8 || c.ecc == 16) ? (int)c.ecc : 0; }

// CTAs of 128 threads for nwarps warps of work
static unsigned warp_grid(size_t nwarps) {
    return (unsigned)std::max<size_t>(1, std::min<size_t>((size_t)num_sms() * 16, (nwarps + 3) / 4));
}

template <int N>
static void launch_encode_sub(const Rsi16Code &c, const BlockView &v, size_t nblocks, cudaStream_t st) {
    KernelTimer kt_timer("rsi16_encode_sub_kernel", st);
    rsi16_encode_sub_kernel<N><<<warp_grid((nblocks + 32 / N - 1) / (32 / N)), 128, 0, st>>>(c.dev, v, nblocks);
    check_launch("rsi16_encode_sub_kernel");
}

template <int N>
static void launch_synd_sub(const Rsi16Code &c, const BlockView &v, size_t nblocks, uint32_t *synds,
                            size_t out_group, size_t out_gstride, cudaStream_t st) {
    KernelTimer kt_timer("rsi16_synd_sub_kernel", st);
    rsi16_synd_sub_kernel<N><<<warp_grid((nblocks + 32 / N - 1) / (32 / N)), 128, 0, st>>>(
        c.dev, v, nblocks, synds, out_group, out_gstride);
    check_launch("rsi16_synd_sub_kernel");
}

template <int EPL>
static void launch_synd_reg(const Rsi16Code &c, const BlockView &v, size_t nblocks, uint32_t *synds,
                            size_t out_group, size_t out_gstride, cudaStream_t st) {
    KernelTimer kt_timer("rsi16_synd_reg_kernel", st);
    rsi16_synd_reg_kernel<EPL><<<warp_grid((nblocks + 1) / 2), 128, 0, st>>>(c.dev, v, nblocks, synds, out_group,
                                                                             out_gstride);
    check_launch("rsi16_synd_reg_kernel");
}

// The one-block-per-thread kernels apply to ecc 32 and 64 on contiguous
// uint16 blocks whose rows start on 16-byte boundaries (message_len is a
// multiple of ecc, so every row does when the base pointers do).
static bool bt_view(const Rsi16Code &c, const BlockView &v) {
    return (c.ecc == 64 || c.ecc == 32) && c.pntt_blocks >= 2 && v.group == 1 && v.msg16 && v.par16 && v.msg_estride == 1 &&
           v.par_estride == 1 && v.msg_gstride == c.message_len && v.par_gstride == c.ecc &&
           ((uintptr_t)v.msg & 15) == 0 && ((uintptr_t)v.par & 15) == 0 && ((uintptr_t)c.dev.pntt_shift & 15) == 0;
}


template <int N>
static void launch_encode_bt(const Rsi16Code &c, const BlockView &v, size_t nblocks, cudaStream_t st) {
    const size_t ntiles = (nblocks + 31) / 32;
    const unsigned grid = (unsigned)std::max<size_t>(1, std::min<size_t>((ntiles + 3) / 4, (size_t)num_sms() * 24));
    KernelTimer kt_timer("rsi16_encode_bt_kernel", st);
    rsi16_encode_bt_kernel<N><<<grid, 128, 4 * bt_warp_smem<N>(), st>>>(
        c.dev, bt_twiddles<N>(c), (const uint16_t *)v.msg, (uint16_t *)v.par, nblocks);
    check_launch("rsi16_encode_bt_kernel");
}

void rsi16_encode(const Rsi16Code &c, const BlockView &v, size_t nblocks, cudaStream_t st) {
    if (!nblocks) return;
    if (bt_view(c, v)) {
        if (c.ecc == 64)
            launch_encode_bt<64>(c, v, nblocks, st);
        else
            launch_encode_bt<32>(c, v, nblocks, st);
        return;
    }
    switch (reg_epl(c)) {
        case 1: launch_encode<1>(c, v, nblocks, st); return;
        case 2: launch_encode<2>(c, v, nblocks, st); return;
        case 4: launch_encode<4>(c, v, nblocks, st); return;
        default: break;
    }
    switch (sub_n(c)) {
        case 2: launch_encode_sub<2>(c, v, nblocks, st); return;
        case 4: launch_encode_sub<4>(c, v, nblocks, st); return;
        case 8: launch_encode_sub<8>(c, v, nblocks, st); return;
        case 16: launch_encode_sub<16>(c, v, nblocks, st); return;
        default: launch_encode<0>(c, v, nblocks, st); return;
    }
}

void rsi16_synd(const Rsi16Code &c, const BlockView &v, size_t nblocks, uint32_t *synds, cudaStream_t st) {
    rsi16_synd_grouped(c, v, nblocks, synds, nblocks ? nblocks : 1, 0, st);
}

void rsi16_synd_grouped(const Rsi16Code &c, const BlockView &v, size_t nblocks, uint32_t *synds, size_t out_group,
                        size_t out_gstride, cudaStream_t st) {
    if (!nblocks) return;
    switch (reg_epl(c)) {
        case 1: launch_synd_reg<1>(c, v, nblocks, synds, out_group, out_gstride, st); return;
        case 2: launch_synd_reg<2>(c, v, nblocks, synds, out_group, out_gstride, st); return;
        case 4: launch_synd_reg<4>(c, v, nblocks, synds, out_group, out_gstride, st); return;
        default: break;
    }
    switch (sub_n(c)) {
        case 2: launch_synd_sub<2>(c, v, nblocks, synds, out_group, out_gstride, st); return;
        case 4: launch_synd_sub<4>(c, v, nblocks, synds, out_group, out_gstride, st); return;
        case 8: launch_synd_sub<8>(c, v, nblocks, synds, out_group, out_gstride, st); return;
        case 16: launch_synd_sub<16>(c, v, nblocks, synds, out_group, out_gstride, st); return;
        default: break;
    }
    Launch L(st);
    plan(L, rsi16_synd_warp_kernel, nblocks, (uint32_t)c.block_len);
    KernelTimer kt_timer("rsi16_synd_warp_kernel", st);
    rsi16_synd_warp_kernel<<<L.grid, L.threads, L.smem, st>>>(c.dev, v, nblocks, synds, out_group, out_gstride,
                                                              L.gscratch, L.ws_words);
    check_launch("rsi16_synd_warp_kernel");
}

template <int N>
static void launch_repair_bt(const Rsi16Code &c, const BlockView &v, size_t nblocks, uint8_t *status,
                             const uint8_t *active, cudaStream_t st) {
    const size_t smem = 4 * (size_t)BtRepairSmem<N>::kWords * 4;  // four warps per CTA
    const size_t ntiles = (nblocks + 31) / 32;
    const unsigned grid =
        (unsigned)std::max<size_t>(1, std::min<size_t>((ntiles + 3) / 4, (size_t)num_sms() * (N == 64 ? 3 : 4)));
    // the tile counter and the mirror workspaces (one per warp), stream-ordered
    const uint32_t mwords = c.dev.temp_len + 1;
    const size_t mbytes = 256 + (size_t)grid * 4 * mwords * 4;
    void *scratch = nullptr;
    FFGPU_CHECK_CUDA(cudaMallocAsync(&scratch, mbytes, st));
    FFGPU_CHECK_CUDA(cudaMemsetAsync(scratch, 0, 4, st));
    static const bool attr = [] {
        FFGPU_CHECK_CUDA(cudaFuncSetAttribute(rsi16_repair_bt_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)(4 * BtRepairSmem<N>::kWords * 4)));
        return true;
    }();
    (void)attr;
    {
        KernelTimer kt_timer("rsi16_repair_bt_kernel", st);
        rsi16_repair_bt_kernel<N><<<grid, 128, smem, st>>>(c.dev, bt_twiddles<N>(c), v, nblocks, status, active,
                                                          (unsigned int *)scratch,
                                                          (uint32_t *)((char *)scratch + 256), mwords);
    }
    cudaError_t e = cudaGetLastError();
    cudaFreeAsync(scratch, st);
    if (e != cudaSuccess) throw Error(FFGPU_ECUDA, std::string("rsi16_repair_bt_kernel: ") + cudaGetErrorString(e));
    launched();
}

void rsi16_repair(const Rsi16Code &c, const BlockView &v, size_t nblocks, uint8_t *status, cudaStream_t st,
                  const uint8_t *active) {
    if (!nblocks) return;
    if (bt_view(c, v)) {
        if (c.ecc == 64)
            launch_repair_bt<64>(c, v, nblocks, status, active, st);
        else
            launch_repair_bt<32>(c, v, nblocks, status, active, st);
        return;
    }
    auto go = [&](auto epl) {
        constexpr int E = decltype(epl)::value;
        if constexpr (E == 1 || E == 2) {
            const uint32_t ws = (uint32_t)((c.ecc + c.ecc / 2 + 1) * kColStride + 3 * c.ecc + 4);
            const size_t smem = 4 * (size_t)ws * 4;  // four warps per CTA
            const size_t batches = (nblocks + 31) / 32;
            const int per_sm = std::max(1, (int)((220 * 1024) / (smem + 1024)));
            const unsigned grid =
                (unsigned)std::max<size_t>(1, std::min<size_t>((batches + 3) / 4, (size_t)num_sms() * per_sm));
            // the batch counter and the mirror workspaces (one per warp),
            // stream-ordered so that concurrent calls on other streams get
            // their own
            const uint32_t mwords = c.dev.temp_len + 1;
            const size_t mbytes = 256 + (size_t)grid * 4 * mwords * 4;
            void *scratch = nullptr;
            FFGPU_CHECK_CUDA(cudaMallocAsync(&scratch, mbytes, st));
            FFGPU_CHECK_CUDA(cudaMemsetAsync(scratch, 0, 4, st));
            FFGPU_CHECK_CUDA(cudaFuncSetAttribute(rsi16_repair_batch_kernel<E>,
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            {
                KernelTimer kt_timer("rsi16_repair_batch_kernel", st);
                rsi16_repair_batch_kernel<E><<<grid, 128, smem, st>>>(
                    c.dev, v, nblocks, status, active, ws, (unsigned int *)scratch,
                    (uint32_t *)((char *)scratch + 256), mwords);
            }
            cudaError_t e = cudaGetLastError();
            cudaFreeAsync(scratch, st);
            if (e != cudaSuccess)
                throw Error(FFGPU_ECUDA, std::string("rsi16_repair_batch_kernel: ") + cudaGetErrorString(e));
            launched();
            return;
        }
        Launch L(st);
        plan(L, rsi16_repair_warp_kernel<E>, nblocks, c.dev.temp_len + 1);
        KernelTimer kt_timer("rsi16_repair_warp_kernel", st);
        rsi16_repair_warp_kernel<E><<<L.grid, L.threads, L.smem, st>>>(c.dev, v, nblocks, status, active,
                                                                       L.gscratch, L.ws_words);
        check_launch("rsi16_repair_warp_kernel");
    };
    switch (reg_epl(c)) {
        case 1: go(std::integral_constant<int, 1>{}); break;
        case 2: go(std::integral_constant<int, 2>{}); break;
        case 4: go(std::integral_constant<int, 4>{}); break;
        default: go(std::integral_constant<int, 0>{}); break;
    }
}

void rsi16_repair_known(const Rsi16Code &c, const BlockView &v, size_t nblocks, const uint32_t *pos,
                        const uint32_t *pos_off, const uint32_t *pos_cnt, uint32_t count_all, const uint8_t *active,
                        uint8_t *status, cudaStream_t st) {
    if (!nblocks) return;
    Launch L(st);
    plan(L, rsi16_repair_known_warp_kernel, nblocks, c.dev.temp_len + 1);
    KernelTimer kt_timer("rsi16_repair_known_warp_kernel", st);
    rsi16_repair_known_warp_kernel<<<L.grid, L.threads, L.smem, st>>>(c.dev, v, nblocks, pos, pos_off, pos_cnt,
                                                                         count_all, active, status, L.gscratch,
                                                                         L.ws_words);
    check_launch("rsi16_repair_known_warp_kernel");
}

void rsi16_sugiyama(const Rsi16Code &c, const uint32_t *synds, size_t nblocks, uint32_t *locator, uint32_t *evaluator,
                    uint8_t *status, cudaStream_t st) {
    if (!nblocks) return;
    Launch L(st);
    plan(L, rsi16_sugiyama_kernel, nblocks, c.dev.temp_len + 1);
    KernelTimer kt_timer("rsi16_sugiyama_kernel", st);
    rsi16_sugiyama_kernel<<<L.grid, L.threads, L.smem, st>>>(c.dev, synds, nblocks, locator, evaluator, status,
                                                             L.gscratch, L.ws_words);
    check_launch("rsi16_sugiyama_kernel");
}

void rsi16_roots(const Rsi16Code &c, const uint32_t *poly, uint8_t *is_zero, cudaStream_t st) {
    uint32_t *scratch = nullptr;
    FFGPU_CHECK_CUDA(cudaMallocAsync((void **)&scratch, c.ntt_len * 4 + 128, st));
    rsi16_roots_kernel<<<1, 32, 0, st>>>(c.dev, poly, is_zero, scratch);
    cudaFreeAsync(scratch, st);
    check_launch("rsi16_roots_kernel");
}

void rsi16_mix_ecc(const Rsi16Code &c, uint32_t *vecs, size_t nvec, cudaStream_t st) {
    if (!nvec) return;
    const unsigned grid = (unsigned)std::min<size_t>((nvec + 3) / 4, (size_t)num_sms() * 8);
    KernelTimer kt_timer("rsi16_mix_kernel", st);
    rsi16_mix_kernel<<<grid, 128, 0, st>>>(c.dev, vecs, nvec);
    check_launch("rsi16_mix_kernel");
}

}  // namespace ffgpu
