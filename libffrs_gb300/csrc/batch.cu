// Fused batch path: requests of mixed codes (RS256, RSi16, CIRC16), uneven
// geometries and both directions are served by one launch sequence.  RS256
// and RSi16 requests are cut into work items, grouped into classes (RS256 by
// the width of the LFSR remainder, RSi16), and each class is served by one
// persistent launch on its own forked stream: an RS256 CTA (four warps) or an
// RSi16 warp pulls the next item from the class's counter; items are ordered
// longest first so the tail stays short.  The sequence can be captured once
// in a CUDA graph and replayed.  The schedule -- RS256 blocks per item, RSi16
// blocks per item and CTAs per SM -- is chosen by timing candidate plans on
// the batch itself (decode buffers are restored after every trial).
//
// Each item runs the same per-block device code as the standalone kernels
// (rs256_device.cuh, rsi16_device.cuh), so the bytes are identical to the
// plain per-request path.
//
// CIRC16 requests are not items: one codeword's encode or CircRepair is a
// chain of stages that each spread over hundreds of rows, which one CTA would
// walk alone.  Their codewords are gathered (one copy kernel) into contiguous
// arrays per code and direction, run through circ16_encode /
// circ16_repair_many (every stage one launch over all of them) and scattered
// back, on a high-priority side stream beside the persistent kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "circ16.cuh"
#include "common.cuh"
#include "handles.h"
#include "rs256_device.cuh"
#include "rsi16_device.cuh"
#include "rsi16_bt.cuh"

namespace ffgpu {

enum : uint8_t {
    BK_RS256_ENC = 0,
    BK_RS256_DEC = 1,
    BK_RSI16_ENC = 2,
    BK_RSI16_DEC = 3,
    BK_CIRC16_ENC = 4,
    BK_CIRC16_DEC = 5
};

constexpr int kBatchThreads = 128;
constexpr int kBatchWarps = kBatchThreads / 32;

struct BatchCode {
    // RS256
    const uint32_t *lut;
    const uint8_t *exp512, *log256;
    int W, ecc;
    // RSi16
    Rsi16Dev rsi;
};

struct BatchItem {
    uint8_t kind;
    uint8_t lane_bm;  // RSi16 repair by 32-block batches with a Berlekamp-Massey per lane
    uint8_t bt;       // RSi16 ecc 32 / 64 on 16-byte aligned blocks: one block per thread
    uint8_t pad;
    uint32_t code;
    uint32_t nblocks;
    int32_t msg_len;
    void *msg;
    void *par;
    uint8_t *status;
};

struct BatchArgs {
    const BatchItem *items;
    uint32_t nitems;
    const BatchCode *codes;
    uint32_t *counter;
    uint8_t *rs_scratch;   // per CTA: kBatchThreads * kDecodeScratchBytes
    uint32_t ws_words;     // RSi16 workspace words per warp (shared memory)
};

// ---------------------------------------------------------------- item bodies

template <int W>
__device__ void rs256_enc_item(const BatchCode &c, const BatchItem &it, uint32_t *sm) {
    uint32_t *s_lut = sm;
    uint8_t *s_data = reinterpret_cast<uint8_t *>(sm + 256 * W);
    for (int i = threadIdx.x; i < 256 * W; i += kBatchThreads) s_lut[i] = c.lut[i];
    const int ml = it.msg_len;
    const uint8_t *data = static_cast<const uint8_t *>(it.msg);
    uint8_t *par = static_cast<uint8_t *>(it.par);
    for (uint32_t b0 = 0; b0 < it.nblocks; b0 += kBatchThreads) {
        const int nb = (int)min((uint32_t)kBatchThreads, it.nblocks - b0);
        __syncthreads();  // table ready, previous chunk consumed
        for (int i = threadIdx.x; i < nb * ml; i += kBatchThreads) s_data[i] = data[(size_t)b0 * ml + i];
        __syncthreads();
        if ((int)threadIdx.x < nb)
            rs256_encode_one<W>(s_data + (size_t)threadIdx.x * ml, ml, s_lut,
                                par + (size_t)(b0 + threadIdx.x) * c.ecc, c.ecc);
    }
}

template <int W>
__device__ void rs256_dec_item(const BatchCode &c, const BatchItem &it, uint32_t *sm, uint8_t *scratch) {
    uint32_t *s_lut = sm;
    uint8_t *ex = reinterpret_cast<uint8_t *>(sm + 256 * W);
    uint8_t *lg = ex + 512;
    for (int i = threadIdx.x; i < 256 * W; i += kBatchThreads) s_lut[i] = c.lut[i];
    for (int i = threadIdx.x; i < 512; i += kBatchThreads) ex[i] = c.exp512[i];
    for (int i = threadIdx.x; i < 256; i += kBatchThreads) lg[i] = c.log256[i];
    __syncthreads();
    // scratch in shared memory after the tables for ecc <= 64 (W <= 16),
    // else this CTA's slice of global memory
    const DecodeScratchG sc = W <= 16 ? DecodeScratchG(lg + 256, threadIdx.x, kBatchThreads, c.ecc)
                                      : DecodeScratchG(scratch, threadIdx.x, kBatchThreads);
    const int ml = it.msg_len;
    uint8_t *data = static_cast<uint8_t *>(it.msg);
    uint8_t *par = static_cast<uint8_t *>(it.par);
    for (uint32_t b = threadIdx.x; b < it.nblocks; b += kBatchThreads)
        decode_one<W>(data + (size_t)b * ml, par + (size_t)b * c.ecc, ml, c.ecc, s_lut, ex, lg, sc, it.status + b,
                      nullptr);
}


// A whole RSi16 item on the calling warp: repairs by 32-block batches with a
// Berlekamp-Massey per lane (ecc 32, 64) or block by block, encodes two
// blocks per pass on registers (ecc 32..128), 32/ecc blocks per pass on the
// sub-warp transforms (ecc 2..16) or block by block.
template <int EPL>
__device__ void rsi16_item_t(const Rsi16Dev &c, const BatchItem &it, uint32_t *ws, bool decode) {
    const int lane = threadIdx.x & 31;
    const BlockView v = contiguous_view(it.msg, true, c.message_len, it.par, true, c.ecc);
    const size_t nb = it.nblocks;
    RegTw<EPL ? EPL : 1> tw;
    if constexpr (EPL > 0) reg_twiddles<EPL>(c, lane, tw);
    if (decode) {
        if constexpr (EPL == 1 || EPL == 2) {
            if (it.lane_bm) {
                unsigned long long nf = 0, nm = 0;
                for (size_t base = 0; base < nb; base += 32)
                    rsi16_repair32<EPL>(c, v, base, (int)min((size_t)32, nb - base), it.status, nullptr, tw, lane, ws,
                                        ws, nf, nm);
                return;
            }
        }
        for (size_t b = 0; b < nb; ++b)
            if (!rsi16_repair_bm_block_t<EPL>(c, v, b, ws, it.status, tw, lane))
                rsi16_repair_block(c, v, b, ws, it.status, lane);
    } else if constexpr (EPL > 0) {
        for (size_t b = 0; b < nb; b += 2) rsi16_encode_pair_reg<EPL>(c, v, b, b + 1 < nb ? b + 1 : b, tw, lane);
    } else {
        for (size_t b = 0; b < nb; ++b) rsi16_encode_block(c, v, b, ws, lane);
    }
}

template <int N>
__device__ void rsi16_encode_item_sub(const Rsi16Dev &c, const BatchItem &it) {
    const int lane = threadIdx.x & 31;
    const BlockView v = contiguous_view(it.msg, true, c.message_len, it.par, true, c.ecc);
    SubTw<N> tw;
    sub_twiddles<N>(c, lane % N, tw);
    for (size_t b0 = 0; b0 < it.nblocks; b0 += 32 / N) rsi16_encode_sub_pass<N>(c, v, b0, it.nblocks, tw, lane);
}

// A whole RSi16 ecc-N item on the calling warp with one block per lane
// (rsi16_bt.cuh), 32 blocks at a time.  The code's twiddles are copied to the
// end of the warp's workspace; the tile's columns and staging buffers start
// at its beginning, and so does the step-for-step mirror, which runs after
// the tile's columns are dead.  Encode and repair are separate functions, not
// inlined, so that each gets the registers of its own path.
template <int N>
__device__ __forceinline__ BtTwShared<N> bt_item_twiddles(const Rsi16Dev &c, uint32_t *ws, uint32_t ws_words) {
    constexpr int TW = (int)(sizeof(BtTw<N>) / 4);
    uint32_t *twp = ws + ws_words - TW;
    for (int i = threadIdx.x & 31; i < TW; i += 32) twp[i] = c.bt_tw[i];
    __syncwarp();
    return BtTwShared<N>{(uint32_t)__cvta_generic_to_shared(twp)};
}

template <int N>
__device__ __noinline__ void rsi16_bt_enc_item(const Rsi16Dev &c, const BatchItem &it, uint32_t *ws,
                                               uint32_t ws_words) {
    const int lane = threadIdx.x & 31;
    const BtTwShared<N> tw = bt_item_twiddles<N>(c, ws, ws_words);
    for (size_t blk0 = 0; blk0 < it.nblocks; blk0 += 32)
        bt_encode_tile<N>(c, tw, reinterpret_cast<uint8_t *>(ws), static_cast<const uint16_t *>(it.msg),
                          static_cast<uint16_t *>(it.par), blk0, it.nblocks, lane);
    __syncwarp();  // the twiddles are read before the next item overwrites them
}

template <int N>
__device__ __noinline__ void rsi16_bt_dec_item(const Rsi16Dev &c, const BatchItem &it, uint32_t *ws,
                                               uint32_t ws_words) {
    const int lane = threadIdx.x & 31;
    const BtTwShared<N> tw = bt_item_twiddles<N>(c, ws, ws_words);
    uint16_t *msg = static_cast<uint16_t *>(it.msg), *par = static_cast<uint16_t *>(it.par);
    unsigned long long nf = 0;
    for (size_t blk0 = 0; blk0 < it.nblocks; blk0 += 32) {
        for (uint32_t m = bt_repair_tile<N>(c, tw, msg, par, blk0, it.nblocks, it.status, nullptr, ws, lane, nf); m;
             m &= m - 1) {
            __syncwarp();
            rsi16_repair_block(c, contiguous_view(it.msg, true, c.message_len, it.par, true, c.ecc),
                               blk0 + (__ffs(m) - 1), ws, it.status, lane);
        }
    }
    __syncwarp();
}

__device__ void rsi16_item(const Rsi16Dev &c, const BatchItem &it, uint32_t *ws, bool decode) {
    switch (c.ecc) {
        case 32: rsi16_item_t<1>(c, it, ws, decode); return;
        case 64: rsi16_item_t<2>(c, it, ws, decode); return;
        case 128: rsi16_item_t<4>(c, it, ws, decode); return;
        default: break;
    }
    if (!decode) {
        switch (c.ecc) {
            case 2: rsi16_encode_item_sub<2>(c, it); return;
            case 4: rsi16_encode_item_sub<4>(c, it); return;
            case 8: rsi16_encode_item_sub<8>(c, it); return;
            case 16: rsi16_encode_item_sub<16>(c, it); return;
            default: break;
        }
    }
    rsi16_item_t<0>(c, it, ws, decode);
}

// Byte ranges copied one CTA per range (ranges of at most kSegBytes): the
// gather of CIRC16 codewords into the repair arrays and their scatter back.
struct CopySeg {
    const uint8_t *src;
    uint8_t *dst;
    uint64_t bytes;
};
constexpr size_t kSegBytes = 64 * 1024;

__global__ void __launch_bounds__(256) seg_copy_kernel(const CopySeg *segs) {
    const CopySeg sg = segs[blockIdx.x];
    if ((((uintptr_t)sg.src | (uintptr_t)sg.dst | sg.bytes) & 15) == 0) {
        const uint4 *s4 = reinterpret_cast<const uint4 *>(sg.src);
        uint4 *d4 = reinterpret_cast<uint4 *>(sg.dst);
        for (size_t i = threadIdx.x; i < sg.bytes / 16; i += blockDim.x) d4[i] = s4[i];
    } else {
        for (size_t i = threadIdx.x; i < sg.bytes; i += blockDim.x) sg.dst[i] = sg.src[i];
    }
}

// Item classes, one persistent launch each with its own registers, shared
// memory and CTAs per SM: RS256 items by the width W of their LFSR remainder
// (W <= 4: ecc <= 16; W <= 16: ecc <= 64; wider), then the RSi16 items.
constexpr int kClasses = 5;
constexpr int kClsRsi16 = 3;
constexpr int kClsRsi16Bt = 4;  // RSi16 ecc 32 / 64 items, one block per thread (its own register budget)

__host__ __device__ constexpr int rs256_class(int W) { return W <= 4 ? 0 : (W <= 16 ? 1 : 2); }

#define FFGPU_BATCH_W_CLS(CLS, W, CALL)                                    \
    if constexpr (CLS == 0) {                                              \
        switch (W) {                                                       \
            case 1: { constexpr int w_ = 1; CALL; } break;                 \
            case 2: { constexpr int w_ = 2; CALL; } break;                 \
            default: { constexpr int w_ = 4; CALL; } break;                \
        }                                                                  \
    } else if constexpr (CLS == 1) {                                       \
        switch (W) {                                                       \
            case 8: { constexpr int w_ = 8; CALL; } break;                 \
            default: { constexpr int w_ = 16; CALL; } break;               \
        }                                                                  \
    } else {                                                               \
        switch (W) {                                                       \
            case 32: { constexpr int w_ = 32; CALL; } break;               \
            default: { constexpr int w_ = 64; CALL; } break;               \
        }                                                                  \
    }

template <int CLS>
__global__ void __launch_bounds__(kBatchThreads) batch_kernel(BatchArgs a) {
    extern __shared__ __align__(16) uint32_t sm[];
    if constexpr (CLS == kClsRsi16 || CLS == kClsRsi16Bt) {
        // RSi16 items are warp-sized: every warp pulls whole items
        const int lane = threadIdx.x & 31;
        uint32_t *wws = sm + (size_t)(threadIdx.x >> 5) * a.ws_words;
        for (;;) {
            uint32_t idx = 0;
            if (lane == 0) idx = atomicAdd(a.counter, 1u);
            idx = __shfl_sync(0xffffffffu, idx, 0);
            if (idx >= a.nitems) break;
            const BatchItem it = a.items[idx];
            const Rsi16Dev &c = a.codes[it.code].rsi;
            if constexpr (CLS == kClsRsi16Bt) {
                const bool dec = it.kind == BK_RSI16_DEC;
                if (c.ecc == 64 && dec)
                    rsi16_bt_dec_item<64>(c, it, wws, a.ws_words);
                else if (c.ecc == 64)
                    rsi16_bt_enc_item<64>(c, it, wws, a.ws_words);
                else if (dec)
                    rsi16_bt_dec_item<32>(c, it, wws, a.ws_words);
                else
                    rsi16_bt_enc_item<32>(c, it, wws, a.ws_words);
            } else {
                rsi16_item(c, it, wws, it.kind == BK_RSI16_DEC);
            }
        }
        return;
    }
    __shared__ uint32_t s_idx;
    uint8_t *rs_scratch = a.rs_scratch + (size_t)blockIdx.x * kBatchThreads * kDecodeScratchBytes;
    for (;;) {
        __syncthreads();  // every thread has read s_idx and finished the last item
        if (threadIdx.x == 0) s_idx = atomicAdd(a.counter, 1u);
        __syncthreads();
        const uint32_t idx = s_idx;
        if (idx >= a.nitems) break;
        const BatchItem it = a.items[idx];
        const BatchCode &c = a.codes[it.code];
        if (it.kind == BK_RS256_ENC) {
            FFGPU_BATCH_W_CLS(CLS, c.W, (rs256_enc_item<w_>(c, it, sm)));
        } else {
            FFGPU_BATCH_W_CLS(CLS, c.W, (rs256_dec_item<w_>(c, it, sm, rs_scratch)));
        }
    }
}

}  // namespace ffgpu

// ---------------------------------------------------------------- host side

using namespace ffgpu;

struct ffgpu_batch {
    struct Req {
        uint8_t kind;
        const void *handle;
        void *a, *b;
        uint8_t *status;
        size_t nblocks, msg_len;
    };
    std::vector<Req> reqs;
    // plan
    std::vector<BatchCode> codes;
    std::vector<const void *> code_keys;
    // items by class (rs256_class, kClsRsi16), each served by its own
    // persistent launch
    struct ItemClass {
        std::vector<BatchItem> items;
        DeviceBuffer d_items;
        size_t smem = 0;
        uint32_t ws_words = 0;
        unsigned grid = 0;
        int per_sm = 0;
    };
    ItemClass cls[kClasses];
    DeviceBuffer d_codes, d_counter, d_rs_scratch, d_backup;
    int tile_rs = 512, tile_rsi = 8, ctas_rs = 0, ctas_rsi = 0;
    bool planned = false;
    // CIRC16 requests: per code and direction, the codewords' place in the
    // gathered arrays (words of d_cmsg / d_cecc, entries of d_cst, bytes of
    // d_cws)
    struct CircGroup {
        ffgpu_circ16 *handle;
        bool decode;
        size_t ncw, moff, eoff, soff, ws_off;
    };
    std::vector<CircGroup> circ;
    size_t n_gather = 0, n_scatter = 0;
    DeviceBuffer d_cmsg, d_cecc, d_cst, d_cws, d_segs;
    // the plan's table uploads, staged in page-locked memory and copied on
    // the plan's stream (ev_stage: the last staged copies, waited for before
    // the staging is rewritten)
    struct Upload {
        void *dst;
        std::vector<uint8_t> bytes;
    };
    std::vector<Upload> uploads;
    PinnedBuffer h_stage;
    cudaEvent_t ev_stage = nullptr;
    // side streams of the class launches (index 0 unused: the caller's) and
    // of the CIRC16 chain
    cudaStream_t side[kClasses] = {}, circ_st = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join[kClasses] = {}, ev_cfork = nullptr, ev_cjoin = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int graph_kernels = 1;
    std::mutex mu;

    ~ffgpu_batch() {
        drop_graph();
        if (ev_stage) {
            cudaEventSynchronize(ev_stage);
            cudaEventDestroy(ev_stage);
        }
        for (int k = 1; k < kClasses; ++k) {
            if (side[k]) cudaStreamDestroy(side[k]);
            if (ev_join[k]) cudaEventDestroy(ev_join[k]);
        }
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (circ_st) cudaStreamDestroy(circ_st);
        if (ev_cfork) cudaEventDestroy(ev_cfork);
        if (ev_cjoin) cudaEventDestroy(ev_cjoin);
    }
    void drop_graph() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
    }
};

namespace {

int sm_count_b() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 132;
}

uint32_t code_index(ffgpu_batch &B, const void *key, const BatchCode &bc) {
    for (size_t i = 0; i < B.code_keys.size(); ++i)
        if (B.code_keys[i] == key) return (uint32_t)i;
    B.code_keys.push_back(key);
    B.codes.push_back(bc);
    return (uint32_t)(B.codes.size() - 1);
}

// relative cost of one item, for the longest-first order
double item_cost(const ffgpu_batch &B, const BatchItem &it) {
    const BatchCode &c = B.codes[it.code];
    switch (it.kind) {
        case BK_RS256_ENC: return (double)it.nblocks * it.msg_len * (1 + c.ecc / 8.0);
        case BK_RS256_DEC: return (double)it.nblocks * (it.msg_len + c.ecc) * (4 + c.ecc);
        case BK_RSI16_ENC: return (double)it.nblocks * c.rsi.block_len * 8;
        default: return (double)it.nblocks * c.rsi.block_len * (40 + c.rsi.ecc);
    }
}

void add_segs(std::vector<CopySeg> &v, const void *src, void *dst, size_t bytes) {
    for (size_t o = 0; o < bytes; o += kSegBytes)
        v.push_back({static_cast<const uint8_t *>(src) + o, static_cast<uint8_t *>(dst) + o,
                     (uint64_t)std::min(kSegBytes, bytes - o)});
}

size_t circ_group(ffgpu_batch &B, const ffgpu_batch::Req &r) {
    const bool dec = r.kind == BK_CIRC16_DEC;
    for (size_t g = 0; g < B.circ.size(); ++g)
        if (B.circ[g].handle == r.handle && B.circ[g].decode == dec) return g;
    B.circ.push_back({const_cast<ffgpu_circ16 *>(static_cast<const ffgpu_circ16 *>(r.handle)), dec, 0, 0, 0, 0, 0});
    return B.circ.size() - 1;
}

// Gathered arrays, workspaces and copy ranges of the CIRC16 requests: an
// encode gathers messages and scatters ecc; a repair gathers and scatters
// both, and scatters the status.
void queue_upload(ffgpu_batch &B, void *dst, const void *src, size_t n) {
    const uint8_t *p = static_cast<const uint8_t *>(src);
    B.uploads.push_back({dst, std::vector<uint8_t>(p, p + n)});
}

// Copies the queued tables to the device on `st` through the page-locked
// staging buffer: the host never waits for the device, except for the
// previous plan's staged copies before their buffer is reused.
void flush_uploads(ffgpu_batch &B, cudaStream_t st) {
    size_t total = 0;
    for (const auto &u : B.uploads) total += (u.bytes.size() + 15) & ~(size_t)15;
    if (total) {
        if (!B.ev_stage) FFGPU_CHECK_CUDA(cudaEventCreateWithFlags(&B.ev_stage, cudaEventDisableTiming));
        else FFGPU_CHECK_CUDA(cudaEventSynchronize(B.ev_stage));
        uint8_t *h = static_cast<uint8_t *>(B.h_stage.get(total));
        size_t off = 0;
        for (const auto &u : B.uploads) {
            std::memcpy(h + off, u.bytes.data(), u.bytes.size());
            FFGPU_CHECK_CUDA(cudaMemcpyAsync(u.dst, h + off, u.bytes.size(), cudaMemcpyHostToDevice, st));
            off += (u.bytes.size() + 15) & ~(size_t)15;
        }
        FFGPU_CHECK_CUDA(cudaEventRecord(B.ev_stage, st));
    }
    B.uploads.clear();
}

void plan_circ(ffgpu_batch &B) {
    B.circ.clear();
    B.n_gather = B.n_scatter = 0;
    for (const auto &r : B.reqs)
        if (r.kind == BK_CIRC16_ENC || r.kind == BK_CIRC16_DEC) B.circ[circ_group(B, r)].ncw += r.nblocks;
    if (B.circ.empty()) return;
    size_t mw = 0, ew = 0, sw = 0, ws = 0;
    for (auto &g : B.circ) {
        const Circ16Code &c = *g.handle->code;
        g.moff = mw;
        g.eoff = ew;
        g.soff = sw;
        g.ws_off = ws;
        mw += (g.ncw * c.message_len + 127) & ~(size_t)127;
        ew += (g.ncw * c.ecc_len + 127) & ~(size_t)127;
        sw += g.decode ? (g.ncw + 255) & ~(size_t)255 : 0;
        const size_t wb = g.decode ? circ16_repair_many_ws_bytes(c, g.ncw) : circ16_encode_ws_bytes(c, g.ncw);
        ws += (wb + 255) & ~(size_t)255;
    }
    uint16_t *cm = static_cast<uint16_t *>(B.d_cmsg.get(mw * 2));
    uint16_t *ce = static_cast<uint16_t *>(B.d_cecc.get(ew * 2));
    uint8_t *cs = static_cast<uint8_t *>(B.d_cst.get(std::max<size_t>(sw, 1)));
    B.d_cws.get(ws);
    std::vector<CopySeg> gat, sca;
    std::vector<size_t> next(B.circ.size(), 0);
    for (const auto &r : B.reqs) {
        if (r.kind != BK_CIRC16_ENC && r.kind != BK_CIRC16_DEC) continue;
        const size_t g = circ_group(B, r);
        const auto &cg = B.circ[g];
        const Circ16Code &c = *cg.handle->code;
        uint16_t *dm = cm + cg.moff + next[g] * c.message_len;
        uint16_t *de = ce + cg.eoff + next[g] * c.ecc_len;
        uint8_t *ds = cs + cg.soff + next[g];
        next[g] += r.nblocks;
        const size_t mb = r.nblocks * c.message_len * 2, eb = r.nblocks * c.ecc_len * 2;
        add_segs(gat, r.a, dm, mb);
        if (cg.decode) {
            add_segs(gat, r.b, de, eb);
            add_segs(sca, dm, r.a, mb);
            if (r.status) add_segs(sca, ds, r.status, r.nblocks);
        }
        add_segs(sca, de, r.b, eb);
    }
    B.n_gather = gat.size();
    B.n_scatter = sca.size();
    gat.insert(gat.end(), sca.begin(), sca.end());
    B.d_segs.get(gat.size() * sizeof(CopySeg));
    queue_upload(B, B.d_segs.ptr, gat.data(), gat.size() * sizeof(CopySeg));
}

// The CIRC16 chain: gather, encode / repair per group, scatter.
void launch_circ(ffgpu_batch &B, cudaStream_t st) {
    const CopySeg *segs = static_cast<const CopySeg *>(B.d_segs.ptr);
    {
        KernelTimer kt_timer("seg_copy_kernel", st);
        seg_copy_kernel<<<(unsigned)B.n_gather, 256, 0, st>>>(segs);
    }
    check_launch("seg_copy_kernel");
    for (const auto &cg : B.circ) {
        Circ16Code &c = *cg.handle->code;
        uint16_t *m = static_cast<uint16_t *>(B.d_cmsg.ptr) + cg.moff;
        uint16_t *e = static_cast<uint16_t *>(B.d_cecc.ptr) + cg.eoff;
        void *w = static_cast<char *>(B.d_cws.ptr) + cg.ws_off;
        if (cg.decode)
            circ16_repair_many(c, m, e, cg.ncw, static_cast<uint8_t *>(B.d_cst.ptr) + cg.soff, st, w);
        else
            circ16_encode(c, m, cg.ncw, e, st, w);
    }
    {
        KernelTimer kt_timer("seg_copy_kernel", st);
        seg_copy_kernel<<<(unsigned)B.n_scatter, 256, 0, st>>>(segs + B.n_gather);
    }
    check_launch("seg_copy_kernel");
}

// Occupancy-limited grid of one class's persistent launch: ctas CTAs per SM
// (0: as many as fit), at most one CTA per item.
template <int CLS>
void size_class(ffgpu_batch::ItemClass &k, int ctas) {
    FFGPU_REQUIRE(k.smem <= 220 * 1024, "batch needs more shared memory per CTA than the device has");
    FFGPU_CHECK_CUDA(
        cudaFuncSetAttribute(batch_kernel<CLS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k.smem));
    int occ = 0;
    FFGPU_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batch_kernel<CLS>, kBatchThreads, k.smem));
    occ = std::max(occ, 1);
    k.per_sm = ctas > 0 ? std::min(ctas, occ) : occ;
    k.grid = (unsigned)std::max<size_t>(1, std::min<size_t>((size_t)sm_count_b() * k.per_sm, k.items.size()));
}

// The tables go to the device on `st`: launches of the plan must follow on
// the same stream (or after a synchronisation of it).
void build_plan(ffgpu_batch &B, int tile_rs, int tile_rsi, int ctas_rs, int ctas_rsi, cudaStream_t st) {
    B.drop_graph();
    B.uploads.clear();
    B.codes.clear();
    B.code_keys.clear();
    for (auto &K : B.cls) {
        K.items.clear();
        K.smem = 0;
        K.ws_words = 0;
    }
    auto &K1 = B.cls[kClsRsi16];
    auto &K2 = B.cls[kClsRsi16Bt];
    uint32_t ws_words = 0, ws_words_bt = 0;
    bool any_rs_dec = false;
    for (const auto &r : B.reqs) {
        BatchCode bc{};
        if (r.kind == BK_RS256_ENC || r.kind == BK_RS256_DEC) {
            const Rs256Code &c = *static_cast<const ffgpu_rs256 *>(r.handle)->code;
            bc.lut = c.d_lut;
            bc.exp512 = c.d_exp512;
            bc.log256 = c.d_log256;
            bc.W = c.W;
            bc.ecc = c.ecc;
            const uint32_t ci = code_index(B, r.handle, bc);
            auto &K = B.cls[rs256_class(c.W)];
            for (size_t b0 = 0; b0 < r.nblocks; b0 += (size_t)tile_rs) {
                BatchItem it{};
                it.kind = r.kind;
                it.code = ci;
                it.nblocks = (uint32_t)std::min<size_t>((size_t)tile_rs, r.nblocks - b0);
                it.msg_len = (int32_t)r.msg_len;
                it.msg = static_cast<uint8_t *>(r.a) + b0 * r.msg_len;
                it.par = static_cast<uint8_t *>(r.b) + b0 * (size_t)c.ecc;
                it.status = r.status ? r.status + b0 : nullptr;
                K.items.push_back(it);
            }
            if (r.kind == BK_RS256_ENC)
                K.smem = std::max(K.smem, (size_t)256 * c.W * 4 + (size_t)kBatchThreads * r.msg_len);
            else {
                const size_t sc = c.W <= 16 ? decode_scratch_bytes(c.ecc) * kBatchThreads : 0;
                K.smem = std::max(K.smem, (size_t)256 * c.W * 4 + 768 + sc);
                any_rs_dec |= c.W > 16;  // only the widest class keeps its scratch in global memory
            }
        } else if (r.kind == BK_RSI16_ENC || r.kind == BK_RSI16_DEC) {
            const Rsi16Code &c = *static_cast<const ffgpu_rsi16 *>(r.handle)->code;
            bc.rsi = c.dev;
            const uint32_t ci = code_index(B, r.handle, bc);
            // repair items of 8 blocks or more run a Berlekamp-Massey per lane
            // (one lane per block); the tile trades lanes busy per warp
            // against warps busy per batch
            // ecc 32 / 64 on 16-byte aligned buffers: one block per thread,
            // 64 blocks per item (rows stay aligned: message_len is a
            // multiple of ecc)
            const bool bt = (c.ecc == 32 || c.ecc == 64) && c.pntt_blocks >= 2 && c.dev.bt_tw &&
                            ((uintptr_t)r.a & 15) == 0 && ((uintptr_t)r.b & 15) == 0;
            const size_t tile = bt ? 64 : (size_t)tile_rsi;
            const bool lane_bm = !bt && r.kind == BK_RSI16_DEC && (c.ecc == 32 || c.ecc == 64) && tile >= 8;
            for (size_t b0 = 0; b0 < r.nblocks; b0 += tile) {
                BatchItem it{};
                it.kind = r.kind;
                it.code = ci;
                it.nblocks = (uint32_t)std::min<size_t>(tile, r.nblocks - b0);
                it.lane_bm = lane_bm && it.nblocks >= 8;
                it.bt = bt;
                it.msg = static_cast<uint16_t *>(r.a) + b0 * c.message_len;
                it.par = static_cast<uint16_t *>(r.b) + b0 * c.ecc;
                it.status = r.status ? r.status + b0 : nullptr;
                (bt ? K2 : K1).items.push_back(it);
            }
            if (!bt)
                ws_words = std::max(ws_words, r.kind == BK_RSI16_DEC ? c.dev.temp_len + 1 : (uint32_t)c.block_len);
            if (lane_bm)  // the batch's columns (the mirror overlays them)
                ws_words = std::max(ws_words, (uint32_t)((c.ecc + c.ecc / 2 + 1) * kColStride + 3 * c.ecc + 4));
            if (bt) {
                // the tile's columns and staging (or the mirror) at the start,
                // the twiddles at the end
                const uint32_t tw = c.ecc == 64 ? (uint32_t)(sizeof(BtTw<64>) / 4) : (uint32_t)(sizeof(BtTw<32>) / 4);
                const uint32_t tile_words = c.ecc == 64 ? (uint32_t)BtRepairSmem<64>::kWords
                                                        : (uint32_t)BtRepairSmem<32>::kWords;
                const uint32_t lead = std::max(tile_words, r.kind == BK_RSI16_DEC ? c.dev.temp_len + 1 : 0u);
                ws_words_bt = std::max(ws_words_bt, ((lead + 3) & ~3u) + tw);
            }
        }
    }
    plan_circ(B);
    // longest first within each class
    for (auto &K : B.cls) {
        std::vector<std::pair<double, size_t>> order(K.items.size());
        for (size_t i = 0; i < K.items.size(); ++i) order[i] = {-item_cost(B, K.items[i]), i};
        std::stable_sort(order.begin(), order.end());
        std::vector<BatchItem> sorted(K.items.size());
        for (size_t i = 0; i < order.size(); ++i) sorted[i] = K.items[order[i].second];
        K.items.swap(sorted);
    }
    K1.ws_words = (ws_words + 3) & ~3u;
    K1.smem = (size_t)kBatchWarps * K1.ws_words * 4;
    K2.ws_words = (ws_words_bt + 3) & ~3u;
    K2.smem = (size_t)kBatchWarps * K2.ws_words * 4;
    size_class<0>(B.cls[0], ctas_rs);
    size_class<1>(B.cls[1], ctas_rs);
    size_class<2>(B.cls[2], ctas_rs);
    size_class<kClsRsi16>(K1, ctas_rsi);
    size_class<kClsRsi16Bt>(K2, 0);
    B.tile_rs = tile_rs;
    B.tile_rsi = tile_rsi;
    B.ctas_rs = ctas_rs;
    B.ctas_rsi = ctas_rsi;

    B.d_codes.get(std::max<size_t>(1, B.codes.size()) * sizeof(BatchCode));
    B.d_counter.get(kClasses * 32 * 4);
    // global decode scratch: one slice per CTA of the widest RS256 class
    // (the narrower ones keep theirs in shared memory)
    if (any_rs_dec) B.d_rs_scratch.get((size_t)B.cls[2].grid * kBatchThreads * kDecodeScratchBytes);
    for (auto &K : B.cls) {
        K.d_items.get(std::max<size_t>(1, K.items.size()) * sizeof(BatchItem));
        if (!K.items.empty()) queue_upload(B, K.d_items.ptr, K.items.data(), K.items.size() * sizeof(BatchItem));
    }
    if (!B.codes.empty()) queue_upload(B, B.d_codes.ptr, B.codes.data(), B.codes.size() * sizeof(BatchCode));
    flush_uploads(B, st);
    B.planned = true;
}

template <int CLS>
void launch_class(ffgpu_batch &B, cudaStream_t st, bool timed) {
    const auto &K = B.cls[CLS];
    if (K.items.empty()) return;
    uint32_t *counter = static_cast<uint32_t *>(B.d_counter.ptr) + CLS * 32;
    FFGPU_CHECK_CUDA(cudaMemsetAsync(counter, 0, 4, st));
    BatchArgs a;
    a.items = static_cast<const BatchItem *>(K.d_items.ptr);
    a.nitems = (uint32_t)K.items.size();
    a.codes = static_cast<const BatchCode *>(B.d_codes.ptr);
    a.counter = counter;
    a.rs_scratch = static_cast<uint8_t *>(B.d_rs_scratch.ptr);
    a.ws_words = K.ws_words;
    if (timed) {
        KernelTimer kt_timer(CLS < kClsRsi16 ? "batch_kernel_rs256" : "batch_kernel_rsi16", st);
        batch_kernel<CLS><<<K.grid, kBatchThreads, K.smem, st>>>(a);
    } else {
        batch_kernel<CLS><<<K.grid, kBatchThreads, K.smem, st>>>(a);
    }
    check_launch("batch_kernel");
}

// which: bit k the items of class k, bit 5 the CIRC16 chain (the autotuner
// times the RS256 classes and the RSi16 classes apart)
constexpr int kRunRs256 = 7, kRunRsi16 = 8 | 16, kRunCirc = 32, kRunAll = 63;
// The class launches run side by side (class k > 0 on side stream k, forked
// from and joined back into st), so that one class's tail overlaps the
// others' work.
void launch_classes(ffgpu_batch &B, cudaStream_t st, bool timed, int which);

void launch_plan(ffgpu_batch &B, cudaStream_t st, bool timed, int which = kRunAll) {
    // the CIRC16 chain (many short dependent launches) on a high-priority
    // side stream, beside the class launches
    const bool circ = (which & kRunCirc) && !B.circ.empty();
    if (circ) {
        if (!B.circ_st) {
            int lo = 0, hi = 0;
            FFGPU_CHECK_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
            FFGPU_CHECK_CUDA(cudaStreamCreateWithPriority(&B.circ_st, cudaStreamNonBlocking, hi));
            FFGPU_CHECK_CUDA(cudaEventCreateWithFlags(&B.ev_cfork, cudaEventDisableTiming));
            FFGPU_CHECK_CUDA(cudaEventCreateWithFlags(&B.ev_cjoin, cudaEventDisableTiming));
        }
        FFGPU_CHECK_CUDA(cudaEventRecord(B.ev_cfork, st));
        FFGPU_CHECK_CUDA(cudaStreamWaitEvent(B.circ_st, B.ev_cfork, 0));
        launch_circ(B, B.circ_st);
        FFGPU_CHECK_CUDA(cudaEventRecord(B.ev_cjoin, B.circ_st));
    }
    launch_classes(B, st, timed, which);
    if (circ) FFGPU_CHECK_CUDA(cudaStreamWaitEvent(st, B.ev_cjoin, 0));
}

void launch_classes(ffgpu_batch &B, cudaStream_t st, bool timed, int which) {
    int run[kClasses], n = 0;
    for (int k = 0; k < kClasses; ++k)
        if ((which & (1 << k)) && !B.cls[k].items.empty()) run[n++] = k;
    if (!n) return;
    if (n > 1) {
        if (!B.side[1]) {
            for (int k = 1; k < kClasses; ++k)
                FFGPU_CHECK_CUDA(cudaStreamCreateWithFlags(&B.side[k], cudaStreamNonBlocking));
            FFGPU_CHECK_CUDA(cudaEventCreateWithFlags(&B.ev_fork, cudaEventDisableTiming));
            for (int k = 1; k < kClasses; ++k)
                FFGPU_CHECK_CUDA(cudaEventCreateWithFlags(&B.ev_join[k], cudaEventDisableTiming));
        }
        FFGPU_CHECK_CUDA(cudaEventRecord(B.ev_fork, st));
    }
    for (int i = 0; i < n; ++i) {
        const int k = run[i];
        cudaStream_t s = i == 0 ? st : B.side[i];
        if (i > 0) FFGPU_CHECK_CUDA(cudaStreamWaitEvent(s, B.ev_fork, 0));
        switch (k) {
            case 0: launch_class<0>(B, s, timed); break;
            case 1: launch_class<1>(B, s, timed); break;
            case 2: launch_class<2>(B, s, timed); break;
            case kClsRsi16: launch_class<kClsRsi16>(B, s, timed); break;
            default: launch_class<kClsRsi16Bt>(B, s, timed); break;
        }
        if (i > 0) FFGPU_CHECK_CUDA(cudaEventRecord(B.ev_join[i], s));
    }
    for (int i = 1; i < n; ++i) FFGPU_CHECK_CUDA(cudaStreamWaitEvent(st, B.ev_join[i], 0));
}

// RS256 / RSi16 decode requests are repaired in place: save / restore them
// around the autotuner's trials (which leave the CIRC16 chain out)
struct Region {
    void *p;
    size_t n;
};

std::vector<Region> decode_regions(const ffgpu_batch &B) {
    std::vector<Region> v;
    for (const auto &r : B.reqs) {
        if (r.kind == BK_RS256_DEC) {
            const Rs256Code &c = *static_cast<const ffgpu_rs256 *>(r.handle)->code;
            v.push_back({r.a, r.nblocks * r.msg_len});
            v.push_back({r.b, r.nblocks * (size_t)c.ecc});
        } else if (r.kind == BK_RSI16_DEC) {
            const Rsi16Code &c = *static_cast<const ffgpu_rsi16 *>(r.handle)->code;
            v.push_back({r.a, r.nblocks * c.message_len * 2});
            v.push_back({r.b, r.nblocks * c.ecc * 2});
        }
    }
    return v;
}

void copy_regions(ffgpu_batch &B, const std::vector<Region> &rs, bool save, cudaStream_t st) {
    uint8_t *bk = static_cast<uint8_t *>(B.d_backup.ptr);
    size_t off = 0;
    for (const auto &r : rs) {
        if (save)
            FFGPU_CHECK_CUDA(cudaMemcpyAsync(bk + off, r.p, r.n, cudaMemcpyDeviceToDevice, st));
        else
            FFGPU_CHECK_CUDA(cudaMemcpyAsync(r.p, bk + off, r.n, cudaMemcpyDeviceToDevice, st));
        off += r.n;
    }
}

// Times candidate schedules of each item class on the batch itself (the
// decode inputs restored before every run) and keeps the fastest: RS256
// blocks per item x CTAs per SM for the RS256 launch, RSi16 blocks per item x
// CTAs per SM for the RSi16 launch.
void autotune(ffgpu_batch &B, cudaStream_t st) {
    const auto regions = decode_regions(B);
    size_t total = 0;
    for (const auto &r : regions) total += r.n;
    if (total) B.d_backup.get(total);
    copy_regions(B, regions, true, st);
    cudaEvent_t e0, e1;
    FFGPU_CHECK_CUDA(cudaEventCreate(&e0));
    FFGPU_CHECK_CUDA(cudaEventCreate(&e1));
    auto trial = [&](int which) {
        float ms = 0.f;
        for (int rep = 0; rep < 2; ++rep) {  // the first run warms up
            copy_regions(B, regions, false, st);
            FFGPU_CHECK_CUDA(cudaEventRecord(e0, st));
            launch_plan(B, st, false, which);
            FFGPU_CHECK_CUDA(cudaEventRecord(e1, st));
            FFGPU_CHECK_CUDA(cudaEventSynchronize(e1));
            FFGPU_CHECK_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        }
        return ms;
    };
    const int tiles_rs[] = {128, 512, 2048};
    const int tiles_rsi[] = {2, 4, 8, 16, 32};
    const int ctas[] = {1, 2, 4, 0};
    int bt_rs = B.tile_rs, bt_rsi = B.tile_rsi, bc_rs = B.ctas_rs, bc_rsi = B.ctas_rsi;
    bool any_rs = false;
    for (int k = 0; k < kClsRsi16; ++k) any_rs |= !B.cls[k].items.empty();
    if (any_rs) {
        float best = 1e30f;
        for (int t : tiles_rs)
            for (int cps : ctas) {
                build_plan(B, t, bt_rsi, cps, bc_rsi, st);
                const float ms = trial(kRunRs256);
                if (ms < best) {
                    best = ms;
                    bt_rs = t;
                    bc_rs = cps;
                }
            }
    }
    if (!B.cls[kClsRsi16].items.empty()) {
        float best = 1e30f;
        for (int t : tiles_rsi)
            for (int cps : ctas) {
                build_plan(B, bt_rs, t, bc_rs, cps, st);
                const float ms = trial(kRunRsi16);
                if (ms < best) {
                    best = ms;
                    bt_rsi = t;
                    bc_rsi = cps;
                }
            }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    copy_regions(B, regions, false, st);
    FFGPU_CHECK_CUDA(cudaStreamSynchronize(st));
    build_plan(B, bt_rs, bt_rsi, bc_rs, bc_rsi, st);
}

}  // namespace

extern "C" {

int ffgpu_batch_create(ffgpu_batch **out) {
    return guarded([&] {
        FFGPU_REQUIRE(out, "out is NULL");
        *out = new ffgpu_batch();
    });
}

int ffgpu_batch_destroy(ffgpu_batch *b) {
    return guarded([&] { delete b; });
}

int ffgpu_batch_clear(ffgpu_batch *b) {
    return guarded([&] {
        FFGPU_REQUIRE(b, "batch is NULL");
        std::lock_guard<std::mutex> lk(b->mu);
        b->reqs.clear();
        b->planned = false;
        b->drop_graph();
    });
}

int ffgpu_batch_add_rs256(ffgpu_batch *b, const ffgpu_rs256 *code, int op, uint8_t *data, uint8_t *parity,
                          size_t nblocks, size_t message_len, uint8_t *status) {
    return guarded([&] {
        FFGPU_REQUIRE(b && code, "batch or code is NULL");
        FFGPU_REQUIRE(op == FFGPU_OP_ENCODE || op == FFGPU_OP_DECODE, "op must be FFGPU_OP_ENCODE or FFGPU_OP_DECODE");
        const Rs256Code &c = *code->code;
        FFGPU_REQUIRE(message_len >= 1 && message_len + (size_t)c.ecc <= 255,
                      "message_len + ecc_len must be in [ecc_len + 1, 255]");
        FFGPU_REQUIRE(op == FFGPU_OP_ENCODE || status, "decode needs a status array");
        std::lock_guard<std::mutex> lk(b->mu);
        b->reqs.push_back({op == FFGPU_OP_ENCODE ? BK_RS256_ENC : BK_RS256_DEC, code, data, parity, status, nblocks,
                           message_len});
        b->planned = false;
    });
}

int ffgpu_batch_add_rsi16(ffgpu_batch *b, const ffgpu_rsi16 *code, int op, uint16_t *msg, uint16_t *parity,
                          size_t nblocks, uint8_t *status) {
    return guarded([&] {
        FFGPU_REQUIRE(b && code, "batch or code is NULL");
        FFGPU_REQUIRE(op == FFGPU_OP_ENCODE || op == FFGPU_OP_DECODE, "op must be FFGPU_OP_ENCODE or FFGPU_OP_DECODE");
        FFGPU_REQUIRE(op == FFGPU_OP_ENCODE || status, "decode needs a status array");
        std::lock_guard<std::mutex> lk(b->mu);
        b->reqs.push_back({op == FFGPU_OP_ENCODE ? BK_RSI16_ENC : BK_RSI16_DEC, code, msg, parity, status, nblocks, 0});
        b->planned = false;
    });
}

int ffgpu_batch_add_circ16(ffgpu_batch *b, const ffgpu_circ16 *code, int op, uint16_t *msg, uint16_t *ecc,
                           size_t nblocks, uint8_t *status) {
    return guarded([&] {
        FFGPU_REQUIRE(b && code, "batch or code is NULL");
        FFGPU_REQUIRE(op == FFGPU_OP_ENCODE || op == FFGPU_OP_DECODE, "op must be FFGPU_OP_ENCODE or FFGPU_OP_DECODE");
        FFGPU_REQUIRE(op == FFGPU_OP_ENCODE || status, "decode needs a status array");
        std::lock_guard<std::mutex> lk(b->mu);
        b->reqs.push_back({op == FFGPU_OP_ENCODE ? BK_CIRC16_ENC : BK_CIRC16_DEC, code, msg, ecc,
                           op == FFGPU_OP_ENCODE ? nullptr : status, nblocks, 0});
        b->planned = false;
    });
}

int ffgpu_batch_plan(ffgpu_batch *b, int autotune_on, void *stream) {
    return guarded([&] {
        FFGPU_REQUIRE(b, "batch is NULL");
        std::lock_guard<std::mutex> lk(b->mu);
        cudaStream_t st = (cudaStream_t)stream;
        // the work list is rewritten: no launch of this batch may be in flight
        FFGPU_CHECK_CUDA(cudaStreamSynchronize(st));
        if (autotune_on)
            autotune(*b, st);
        else
            build_plan(*b, b->tile_rs, b->tile_rsi, b->ctas_rs, b->ctas_rsi, st);
    });
}

int ffgpu_batch_capture(ffgpu_batch *b, void *stream) {
    return guarded([&] {
        FFGPU_REQUIRE(b, "batch is NULL");
        std::lock_guard<std::mutex> lk(b->mu);
        cudaStream_t st = (cudaStream_t)stream;
        if (!b->planned) build_plan(*b, b->tile_rs, b->tile_rsi, b->ctas_rs, b->ctas_rsi, st);
        // the tables are on the device before any replay reads them
        if (b->ev_stage) FFGPU_CHECK_CUDA(cudaEventSynchronize(b->ev_stage));
        b->drop_graph();
        cudaStream_t cap = st;
        bool own = false;
        if (!cap) {  // the legacy default stream cannot be captured
            FFGPU_CHECK_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
            own = true;
        }
        FFGPU_CHECK_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
        try {
            launch_plan(*b, cap, false);
        } catch (...) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(cap, &g);
            if (g) cudaGraphDestroy(g);
            if (own) cudaStreamDestroy(cap);
            throw;
        }
        FFGPU_CHECK_CUDA(cudaStreamEndCapture(cap, &b->graph));
        if (own) cudaStreamDestroy(cap);
        size_t nn = 0;
        FFGPU_CHECK_CUDA(cudaGraphGetNodes(b->graph, nullptr, &nn));
        std::vector<cudaGraphNode_t> nodes(nn);
        if (nn) FFGPU_CHECK_CUDA(cudaGraphGetNodes(b->graph, nodes.data(), &nn));
        b->graph_kernels = 0;
        for (auto n : nodes) {
            cudaGraphNodeType t;
            if (cudaGraphNodeGetType(n, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++b->graph_kernels;
        }
        FFGPU_CHECK_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
    });
}

int ffgpu_batch_launch(ffgpu_batch *b, void *stream) {
    return guarded([&] {
        FFGPU_REQUIRE(b, "batch is NULL");
        std::lock_guard<std::mutex> lk(b->mu);
        cudaStream_t st = (cudaStream_t)stream;
        if (b->exec) {
            KernelTimer kt_timer("batch_kernel", st);
            FFGPU_CHECK_CUDA(cudaGraphLaunch(b->exec, st));
            launched(b->graph_kernels);
            return;
        }
        if (!b->planned) build_plan(*b, b->tile_rs, b->tile_rsi, b->ctas_rs, b->ctas_rsi, st);
        // a plan made on another stream: its table uploads come first
        if (b->ev_stage) FFGPU_CHECK_CUDA(cudaStreamWaitEvent(st, b->ev_stage, 0));
        launch_plan(*b, st, true);
    });
}

int ffgpu_batch_info(const ffgpu_batch *b, int *tile_rs256, int *tile_rsi16, int *ctas_per_sm, size_t *items,
                     unsigned *grid) {
    return guarded([&] {
        FFGPU_REQUIRE(b, "batch is NULL");
        if (tile_rs256) *tile_rs256 = b->tile_rs;
        if (tile_rsi16) *tile_rsi16 = b->tile_rsi;
        // the first RS256 launch's CTAs per SM (the RSi16 launch's when there
        // are no RS256 items); items and grids of all launches together
        int k = 0;
        while (k < kClsRsi16 && b->cls[k].items.empty()) ++k;
        size_t n = 0;
        unsigned g = 0;
        for (const auto &K : b->cls) {
            n += K.items.size();
            g += K.items.empty() ? 0 : K.grid;
        }
        if (ctas_per_sm) *ctas_per_sm = b->cls[k].per_sm;
        if (items) *items = n;
        if (grid) *grid = g;
    });
}

}  // extern "C"
