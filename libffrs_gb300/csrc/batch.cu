// Fused batch path: requests of mixed codes (RS256, RSi16, CIRC16), uneven
// geometries and both directions are cut into work items and served by ONE
// persistent launch.  Every CTA (four warps) pulls the next item from a global
// counter; items are ordered longest first so the tail stays short.  The
// launch can be captured once in a CUDA graph and replayed.  The schedule --
// RS256 blocks per item, RSi16 blocks per item and CTAs per SM -- is chosen by
// timing candidate plans on the batch itself (decode buffers are restored
// after every trial).
//
// Each item runs the same per-block device code as the standalone kernels
// (rs256_device.cuh, rsi16_device.cuh), so the bytes are identical to the
// plain per-request path.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "circ16_device.cuh"
#include "common.cuh"
#include "handles.h"
#include "rs256_device.cuh"
#include "rsi16_device.cuh"

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
    // RSi16, or the inner code of a CIRC16
    Rsi16Dev rsi;
    // CIRC16: outer code and geometry (pycirc16.hpp:46-65)
    Rsi16Dev rso;
    uint32_t c_message_len, c_ecc_len, c_rso_interleave, c_rso_ieccl, c_rsi_ieccl, c_inner_rows, c_outer_rows;
    uint32_t c_rsi_total;
    CircDims cd;
    // CircRepair workspace (word offsets) and the saved message after it
    uint32_t o_rso, o_rsi, o_syn, o_blk, o_bsyn, o_zpos, o_zoff, o_zcnt, o_zact, o_vec, o_flag, o_locs, o_lcnt, o_poff,
        o_pcnt, o_kn, o_un, o_st, o_save;
};

struct BatchItem {
    uint8_t kind;
    uint8_t pad[3];
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
    uint32_t *circ_tmp;    // per CTA: circ_tmp_words
    size_t circ_tmp_words;
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
    const DecodeScratchG sc(scratch, threadIdx.x, kBatchThreads);
    const int ml = it.msg_len;
    uint8_t *data = static_cast<uint8_t *>(it.msg);
    uint8_t *par = static_cast<uint8_t *>(it.par);
    for (uint32_t b = threadIdx.x; b < it.nblocks; b += kBatchThreads)
        decode_one<W>(data + (size_t)b * ml, par + (size_t)b * c.ecc, ml, c.ecc, s_lut, ex, lg, sc, it.status + b,
                      nullptr);
}

#define FFGPU_BATCH_W(W, CALL)                       \
    switch (W) {                                     \
        case 1: { constexpr int w_ = 1; CALL; } break;   \
        case 2: { constexpr int w_ = 2; CALL; } break;   \
        case 4: { constexpr int w_ = 4; CALL; } break;   \
        case 8: { constexpr int w_ = 8; CALL; } break;   \
        case 16: { constexpr int w_ = 16; CALL; } break; \
        case 32: { constexpr int w_ = 32; CALL; } break; \
        default: { constexpr int w_ = 64; CALL; } break; \
    }

template <int EPL>
__device__ void rsi16_item_t(const Rsi16Dev &c, const BatchItem &it, uint32_t *ws, bool decode) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const BlockView v = contiguous_view(it.msg, true, c.message_len, it.par, true, c.ecc);
    RegTw<EPL ? EPL : 1> tw;
    if constexpr (EPL > 0) reg_twiddles<EPL>(c, lane, tw);
    for (uint32_t b = warp; b < it.nblocks; b += kBatchWarps) {
        if (decode) {
            if (!rsi16_repair_bm_block_t<EPL>(c, v, b, ws, it.status, tw, lane))
                rsi16_repair_block(c, v, b, ws, it.status, lane);
        } else if constexpr (EPL > 0) {
            rsi16_encode_block_reg<EPL>(c, v, b, tw, lane);
        } else {
            rsi16_encode_block(c, v, b, ws, lane);
        }
    }
}

__device__ void rsi16_item(const Rsi16Dev &c, const BatchItem &it, uint32_t *ws, bool decode) {
    switch (c.ecc) {
        case 32: rsi16_item_t<1>(c, it, ws, decode); break;
        case 64: rsi16_item_t<2>(c, it, ws, decode); break;
        case 128: rsi16_item_t<4>(c, it, ws, decode); break;
        default: rsi16_item_t<0>(c, it, ws, decode); break;
    }
}

// One CIRC16 codeword (circ16_encode for a single block): the outer code over
// the interleaved columns into untruncated words, their uint16 copy into the
// ecc, then the inner code over the message rows and over the outer parity rows.
__device__ void circ16_enc_item(const BatchCode &c, const BatchItem &it, uint32_t *ws, uint32_t *tmp) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint16_t *ecc = static_cast<uint16_t *>(it.par);
    const uint32_t I = c.c_rso_interleave;
    const BlockView vo{it.msg, 0, 1, I, tmp, 0, 1, I, I, true, false};
    for (uint32_t b = warp; b < I; b += kBatchWarps) rsi16_encode_block(c.rso, vo, b, ws, lane);
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < c.c_rso_ieccl; i += kBatchThreads) ecc[i] = (uint16_t)tmp[i];
    const BlockView vi{it.msg, 0, c.rsi.message_len, 1, ecc + c.c_rso_ieccl, 0, c.rsi.ecc, 1, c.c_inner_rows,
                       true, true};
    for (uint32_t b = warp; b < c.c_inner_rows; b += kBatchWarps) rsi16_encode_block(c.rsi, vi, b, ws, lane);
    const BlockView vio{tmp, 0, c.rsi.message_len, 1, ecc + c.c_rso_ieccl + c.c_rsi_ieccl, 0, c.rsi.ecc, 1,
                        c.c_outer_rows, false, true};
    for (uint32_t b = warp; b < c.c_outer_rows; b += kBatchWarps) rsi16_encode_block(c.rsi, vio, b, ws, lane);
}

// One CIRC16 codeword repaired inside the CTA: CircRepair (pycirc16.hpp:135-335)
// stage by stage, each stage spread over the four warps with a barrier after
// it, exactly as the per-request pipeline of stage kernels.  A column whose
// outer repair raises (status 0xFF) ends the reference's column loop there:
// the columns from it on get their saved words back and the ecc is not
// written; the block's status is 0 or 0xFF.
__device__ void circ16_dec_item(const BatchCode &c, const BatchItem &it, uint32_t *ws, uint32_t *W,
                                uint32_t *s_first) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, tid = threadIdx.x;
    const Rsi16Dev &ri = c.rsi, &ro = c.rso;
    const CircDims d = c.cd;
    uint16_t *msg = static_cast<uint16_t *>(it.msg), *ecc = static_cast<uint16_t *>(it.par);
    uint32_t *rso_ecc = W + c.o_rso, *rsi_ecc = W + c.o_rsi, *synd = W + c.o_syn, *blocks = W + c.o_blk,
             *bsyn = W + c.o_bsyn, *zpos = W + c.o_zpos, *zoff = W + c.o_zoff, *zcnt = W + c.o_zcnt,
             *vecs = W + c.o_vec, *locs = W + c.o_locs, *lcnt = W + c.o_lcnt, *poff = W + c.o_poff,
             *pcnt = W + c.o_pcnt;
    uint8_t *zact = reinterpret_cast<uint8_t *>(W + c.o_zact), *flag = reinterpret_cast<uint8_t *>(W + c.o_flag),
            *kn = reinterpret_cast<uint8_t *>(W + c.o_kn), *un = reinterpret_cast<uint8_t *>(W + c.o_un),
            *cst = reinterpret_cast<uint8_t *>(W + c.o_st);
    uint16_t *save = reinterpret_cast<uint16_t *>(W + c.o_save);
    const uint32_t I = c.c_rso_interleave, n_oz = d.interleave * ro.ecc, n_iz = d.interleave * ro.block_len;
    // load_ecc (pycirc16.hpp:159-163), and a copy of the message
    for (uint32_t i = tid; i < c.c_message_len; i += kBatchThreads) save[i] = msg[i];
    for (uint32_t i = tid; i < c.c_rso_ieccl; i += kBatchThreads) rso_ecc[i] = ecc[i];
    for (uint32_t i = tid; i < c.c_rsi_total; i += kBatchThreads) rsi_ecc[i] = ecc[c.c_rso_ieccl + i];
    __syncthreads();
    // compute_rsi_synd (pycirc16.hpp:165-181)
    const BlockView vmsg{msg, 0, ri.message_len, 1, rsi_ecc, 0, ri.ecc, 1, c.c_inner_rows, true, false};
    for (uint32_t b = warp; b < c.c_inner_rows; b += kBatchWarps)
        rsi16_synd_block(ri, vmsg, b, ws, synd + (size_t)b * ri.ecc, lane);
    const BlockView vrso{rso_ecc, 0, ri.message_len, 1, rsi_ecc + c.c_rsi_ieccl, 0, ri.ecc, 1, c.c_outer_rows,
                         false, false};
    for (uint32_t b = warp; b < c.c_outer_rows; b += kBatchWarps)
        rsi16_synd_block(ri, vrso, b, ws, synd + c.c_rsi_ieccl + (size_t)b * ri.ecc, lane);
    __syncthreads();
    // repair_outer_zeros
    for (uint32_t k = warp; k < n_oz; k += kBatchWarps)
        outer_zeros_prepare_item(d, rso_ecc, rsi_ecc, synd, blocks, zpos, zoff, zcnt, zact, k, lane);
    __syncthreads();
    const BlockView vblk{blocks, 0, ri.block_len, 1, blocks + ri.message_len, 0, ri.block_len, 1, n_oz, false, false};
    for (uint32_t b = warp; b < n_oz; b += kBatchWarps)
        if (zact[b]) rsi16_repair_known_block(ri, vblk, b, zpos + zoff[b], zcnt[b], ws, nullptr, lane);
    __syncthreads();
    for (uint32_t b = warp; b < n_oz; b += kBatchWarps) rsi16_synd_block(ri, vblk, b, ws, bsyn + (size_t)b * ri.ecc, lane);
    __syncthreads();
    for (uint32_t k = warp; k < n_oz; k += kBatchWarps)
        outer_zeros_commit_item(d, rso_ecc, rsi_ecc, synd, blocks, bsyn, zpos, zcnt, zact, k, lane);
    __syncthreads();
    // repair_inner_zeros
    for (uint32_t k = warp; k < n_iz; k += kBatchWarps) inner_zeros_prepare_item(d, rsi_ecc, synd, vecs, flag, k, lane);
    __syncthreads();
    for (uint32_t k = warp; k < n_iz; k += kBatchWarps) w_mix(ri, vecs + (size_t)k * ri.ecc, lane);
    __syncthreads();
    for (uint32_t k = warp; k < n_iz; k += kBatchWarps) inner_zeros_commit_item(d, rsi_ecc, synd, vecs, flag, k, lane);
    __syncthreads();
    // find_error_locations, then the outer repairs
    for (uint32_t k = warp; k < d.interleave; k += kBatchWarps) find_locations_item(d, synd, locs, lcnt, k, lane);
    if (tid == 0) *s_first = 0xffffffffu;
    __syncthreads();
    for (uint32_t col = tid; col < I; col += kBatchThreads) {
        outer_modes_col(d, lcnt, poff, pcnt, kn, un, col, 0);
        cst[col] = 0;
    }
    __syncthreads();
    const BlockView vcol = interleaved_view(msg, true, ro.message_len, rso_ecc, false, ro.ecc, I);
    for (uint32_t col = warp; col < I; col += kBatchWarps) {
        if (kn[col])
            rsi16_repair_known_block(ro, vcol, col, locs + poff[col], pcnt[col], ws, cst, lane);
        else if (un[col] && !rsi16_repair_bm_block(ro, vcol, col, ws, cst, lane))
            rsi16_repair_block(ro, vcol, col, ws, cst, lane);
    }
    __syncthreads();
    for (uint32_t col = tid; col < I; col += kBatchThreads)
        if (cst[col] == FFGPU_STATUS_ASSERT) atomicMin(s_first, col);
    // recompute_inner_ecc (pycirc16.hpp:320-324)
    const BlockView vre{msg, 0, ri.message_len, 1, rsi_ecc, 0, ri.ecc, 1, c.c_inner_rows, true, false};
    for (uint32_t b = warp; b < c.c_inner_rows; b += kBatchWarps) rsi16_encode_block(ri, vre, b, ws, lane);
    const BlockView vreo{rso_ecc, 0, ri.message_len, 1, rsi_ecc + c.c_rsi_ieccl, 0, ri.ecc, 1, c.c_outer_rows,
                         false, false};
    for (uint32_t b = warp; b < c.c_outer_rows; b += kBatchWarps) rsi16_encode_block(ri, vreo, b, ws, lane);
    __syncthreads();
    const uint32_t first = *s_first;
    if (first == 0xffffffffu) {
        // dump_ecc (pycirc16.hpp:326-330)
        for (uint32_t i = tid; i < c.c_rso_ieccl; i += kBatchThreads) ecc[i] = (uint16_t)rso_ecc[i];
        for (uint32_t i = tid; i < c.c_rsi_total; i += kBatchThreads) ecc[c.c_rso_ieccl + i] = (uint16_t)rsi_ecc[i];
    } else {
        const uint32_t ncol = I - first;
        for (uint32_t i = tid; i < ro.message_len * ncol; i += kBatchThreads) {
            const uint32_t r = i / ncol, col = first + i % ncol;
            msg[(size_t)r * I + col] = save[(size_t)r * I + col];
        }
    }
    if (tid == 0 && it.status) *it.status = first == 0xffffffffu ? 0 : FFGPU_STATUS_ASSERT;
}

__global__ void __launch_bounds__(kBatchThreads) batch_kernel(BatchArgs a) {
    extern __shared__ __align__(16) uint32_t sm[];
    __shared__ uint32_t s_idx, s_first;
    uint8_t *rs_scratch = a.rs_scratch + (size_t)blockIdx.x * kBatchThreads * kDecodeScratchBytes;
    uint32_t *ctmp = a.circ_tmp + (size_t)blockIdx.x * a.circ_tmp_words;
    uint32_t *ws = sm + (size_t)(threadIdx.x >> 5) * a.ws_words;
    for (;;) {
        __syncthreads();  // every thread has read s_idx and finished the last item
        if (threadIdx.x == 0) s_idx = atomicAdd(a.counter, 1u);
        __syncthreads();
        const uint32_t idx = s_idx;
        if (idx >= a.nitems) break;
        const BatchItem it = a.items[idx];
        const BatchCode &c = a.codes[it.code];
        switch (it.kind) {
            case BK_RS256_ENC:
                FFGPU_BATCH_W(c.W, (rs256_enc_item<w_>(c, it, sm)));
                break;
            case BK_RS256_DEC:
                FFGPU_BATCH_W(c.W, (rs256_dec_item<w_>(c, it, sm, rs_scratch)));
                break;
            case BK_RSI16_ENC:
                rsi16_item(c.rsi, it, ws, false);
                break;
            case BK_RSI16_DEC:
                rsi16_item(c.rsi, it, ws, true);
                break;
            case BK_CIRC16_ENC:
                circ16_enc_item(c, it, ws, ctmp);
                break;
            case BK_CIRC16_DEC:
                circ16_dec_item(c, it, ws, ctmp, &s_first);
                break;
            default:
                break;
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
    std::vector<BatchItem> items;
    DeviceBuffer d_items, d_codes, d_counter, d_rs_scratch, d_circ_tmp, d_backup;
    size_t smem = 0, circ_tmp_words = 0;
    uint32_t ws_words = 0;
    unsigned grid = 0;
    int tile_rs = 512, tile_rsi = 8, ctas_per_sm = 0;
    bool planned = false;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::mutex mu;

    ~ffgpu_batch() { drop_graph(); }
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
        case BK_RSI16_DEC: return (double)it.nblocks * c.rsi.block_len * (40 + c.rsi.ecc);
        case BK_CIRC16_DEC:
            return ((double)c.c_rso_interleave * c.rso.block_len +
                    (double)(c.c_inner_rows + c.c_outer_rows) * c.rsi.block_len) * 40;
        default:
            return ((double)c.c_rso_interleave * c.rso.block_len +
                    (double)(c.c_inner_rows + c.c_outer_rows) * c.rsi.block_len) * 8;
    }
}

void build_plan(ffgpu_batch &B, int tile_rs, int tile_rsi, int ctas_per_sm) {
    B.drop_graph();
    B.codes.clear();
    B.code_keys.clear();
    B.items.clear();
    size_t smem = 0;
    uint32_t ws_words = 0;
    size_t circ_words = 0;
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
            for (size_t b0 = 0; b0 < r.nblocks; b0 += (size_t)tile_rs) {
                BatchItem it{};
                it.kind = r.kind;
                it.code = ci;
                it.nblocks = (uint32_t)std::min<size_t>((size_t)tile_rs, r.nblocks - b0);
                it.msg_len = (int32_t)r.msg_len;
                it.msg = static_cast<uint8_t *>(r.a) + b0 * r.msg_len;
                it.par = static_cast<uint8_t *>(r.b) + b0 * (size_t)c.ecc;
                it.status = r.status ? r.status + b0 : nullptr;
                B.items.push_back(it);
            }
            if (r.kind == BK_RS256_ENC)
                smem = std::max(smem, (size_t)256 * c.W * 4 + (size_t)kBatchThreads * r.msg_len);
            else {
                smem = std::max(smem, (size_t)256 * c.W * 4 + 768);
                any_rs_dec = true;
            }
        } else if (r.kind == BK_RSI16_ENC || r.kind == BK_RSI16_DEC) {
            const Rsi16Code &c = *static_cast<const ffgpu_rsi16 *>(r.handle)->code;
            bc.rsi = c.dev;
            const uint32_t ci = code_index(B, r.handle, bc);
            for (size_t b0 = 0; b0 < r.nblocks; b0 += (size_t)tile_rsi) {
                BatchItem it{};
                it.kind = r.kind;
                it.code = ci;
                it.nblocks = (uint32_t)std::min<size_t>((size_t)tile_rsi, r.nblocks - b0);
                it.msg = static_cast<uint16_t *>(r.a) + b0 * c.message_len;
                it.par = static_cast<uint16_t *>(r.b) + b0 * c.ecc;
                it.status = r.status ? r.status + b0 : nullptr;
                B.items.push_back(it);
            }
            ws_words = std::max(ws_words, r.kind == BK_RSI16_DEC ? c.dev.temp_len + 1 : (uint32_t)c.block_len);
        } else {
            const Circ16Code &c = *static_cast<const ffgpu_circ16 *>(r.handle)->code;
            bc.rsi = c.rsi->dev;
            bc.rso = c.rso->dev;
            bc.c_message_len = (uint32_t)c.message_len;
            bc.c_ecc_len = (uint32_t)c.ecc_len;
            bc.c_rso_interleave = (uint32_t)c.rso_interleave;
            bc.c_rso_ieccl = (uint32_t)c.rso_ieccl;
            bc.c_rsi_ieccl = (uint32_t)c.rsi_ieccl;
            bc.c_inner_rows = (uint32_t)c.inner_rows;
            bc.c_outer_rows = (uint32_t)c.outer_rows;
            bc.c_rsi_total = (uint32_t)c.rsi_total;
            bc.cd = circ16_dims(c);
            const CircLayout lay = circ16_layout(c);
            bc.o_rso = (uint32_t)lay.o_rso;
            bc.o_rsi = (uint32_t)lay.o_rsi;
            bc.o_syn = (uint32_t)lay.o_syn;
            bc.o_blk = (uint32_t)lay.o_blk;
            bc.o_bsyn = (uint32_t)lay.o_bsyn;
            bc.o_zpos = (uint32_t)lay.o_zpos;
            bc.o_zoff = (uint32_t)lay.o_zoff;
            bc.o_zcnt = (uint32_t)lay.o_zcnt;
            bc.o_zact = (uint32_t)lay.o_zact;
            bc.o_vec = (uint32_t)lay.o_vec;
            bc.o_flag = (uint32_t)lay.o_flag;
            bc.o_locs = (uint32_t)lay.o_locs;
            bc.o_lcnt = (uint32_t)lay.o_lcnt;
            bc.o_poff = (uint32_t)lay.o_poff;
            bc.o_pcnt = (uint32_t)lay.o_pcnt;
            bc.o_kn = (uint32_t)lay.o_kn;
            bc.o_un = (uint32_t)lay.o_un;
            bc.o_st = (uint32_t)lay.o_st;
            bc.o_save = (uint32_t)lay.words;
            const uint32_t ci = code_index(B, r.handle, bc);
            for (size_t b = 0; b < r.nblocks; ++b) {
                BatchItem it{};
                it.kind = r.kind;
                it.code = ci;
                it.nblocks = 1;
                it.msg = static_cast<uint16_t *>(r.a) + b * c.message_len;
                it.par = static_cast<uint16_t *>(r.b) + b * c.ecc_len;
                it.status = r.status ? r.status + b : nullptr;
                B.items.push_back(it);
            }
            if (r.kind == BK_CIRC16_DEC) {
                ws_words = std::max(ws_words, std::max(c.rsi->dev.temp_len, c.rso->dev.temp_len) + 1);
                circ_words = std::max(circ_words, lay.words + (c.message_len + 1) / 2);
            } else {
                ws_words = std::max(ws_words, (uint32_t)std::max(c.rsi->block_len, c.rso->block_len));
                circ_words = std::max(circ_words, c.rso_ieccl);
            }
        }
    }
    // longest first
    std::vector<std::pair<double, size_t>> order(B.items.size());
    for (size_t i = 0; i < B.items.size(); ++i) order[i] = {-item_cost(B, B.items[i]), i};
    std::stable_sort(order.begin(), order.end());
    std::vector<BatchItem> sorted(B.items.size());
    for (size_t i = 0; i < order.size(); ++i) sorted[i] = B.items[order[i].second];
    B.items.swap(sorted);

    ws_words = (ws_words + 3) & ~3u;
    B.ws_words = ws_words;
    B.smem = std::max(smem, (size_t)kBatchWarps * ws_words * 4);
    FFGPU_REQUIRE(B.smem <= 220 * 1024, "batch needs more shared memory per CTA than the device has");
    FFGPU_CHECK_CUDA(cudaFuncSetAttribute(batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)B.smem));
    int occ = 0;
    FFGPU_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batch_kernel, kBatchThreads, B.smem));
    occ = std::max(occ, 1);
    const int per_sm = ctas_per_sm > 0 ? std::min(ctas_per_sm, occ) : occ;
    B.grid = (unsigned)std::max<size_t>(1, std::min<size_t>((size_t)sm_count_b() * per_sm, B.items.size()));
    B.tile_rs = tile_rs;
    B.tile_rsi = tile_rsi;
    B.ctas_per_sm = per_sm;
    B.circ_tmp_words = (circ_words + 63) & ~(size_t)63;

    B.d_items.get(std::max<size_t>(1, B.items.size()) * sizeof(BatchItem));
    B.d_codes.get(std::max<size_t>(1, B.codes.size()) * sizeof(BatchCode));
    B.d_counter.get(256);
    if (any_rs_dec) B.d_rs_scratch.get((size_t)B.grid * kBatchThreads * kDecodeScratchBytes);
    if (B.circ_tmp_words) B.d_circ_tmp.get((size_t)B.grid * B.circ_tmp_words * 4);
    if (!B.items.empty())
        FFGPU_CHECK_CUDA(cudaMemcpy(B.d_items.ptr, B.items.data(), B.items.size() * sizeof(BatchItem),
                                    cudaMemcpyHostToDevice));
    if (!B.codes.empty())
        FFGPU_CHECK_CUDA(cudaMemcpy(B.d_codes.ptr, B.codes.data(), B.codes.size() * sizeof(BatchCode),
                                    cudaMemcpyHostToDevice));
    B.planned = true;
}

void launch_plan(ffgpu_batch &B, cudaStream_t st, bool timed) {
    FFGPU_CHECK_CUDA(cudaMemsetAsync(B.d_counter.ptr, 0, 4, st));
    BatchArgs a;
    a.items = static_cast<const BatchItem *>(B.d_items.ptr);
    a.nitems = (uint32_t)B.items.size();
    a.codes = static_cast<const BatchCode *>(B.d_codes.ptr);
    a.counter = static_cast<uint32_t *>(B.d_counter.ptr);
    a.rs_scratch = static_cast<uint8_t *>(B.d_rs_scratch.ptr);
    a.circ_tmp = static_cast<uint32_t *>(B.d_circ_tmp.ptr);
    a.circ_tmp_words = B.circ_tmp_words;
    a.ws_words = B.ws_words;
    if (timed) {
        KernelTimer kt_timer("batch_kernel", st);
        batch_kernel<<<B.grid, kBatchThreads, B.smem, st>>>(a);
        check_launch("batch_kernel");
    } else {
        batch_kernel<<<B.grid, kBatchThreads, B.smem, st>>>(a);
        check_launch("batch_kernel");
    }
}

// decode requests are repaired in place: save / restore them around trials
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
        } else if (r.kind == BK_CIRC16_DEC) {
            const Circ16Code &c = *static_cast<const ffgpu_circ16 *>(r.handle)->code;
            v.push_back({r.a, r.nblocks * c.message_len * 2});
            v.push_back({r.b, r.nblocks * c.ecc_len * 2});
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

void autotune(ffgpu_batch &B, cudaStream_t st) {
    const auto regions = decode_regions(B);
    size_t total = 0;
    for (const auto &r : regions) total += r.n;
    if (total) B.d_backup.get(total);
    copy_regions(B, regions, true, st);
    cudaEvent_t e0, e1;
    FFGPU_CHECK_CUDA(cudaEventCreate(&e0));
    FFGPU_CHECK_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    int bt_rs = 512, bt_rsi = 8, bt_cta = 0;
    const int tiles_rs[] = {128, 512, 2048};
    const int tiles_rsi[] = {2, 8, 32};
    const int ctas[] = {1, 2, 0};
    for (int trs : tiles_rs)
        for (int tri : tiles_rsi)
            for (int cps : ctas) {
                build_plan(B, trs, tri, cps);
                float ms = 0.f;
                for (int rep = 0; rep < 2; ++rep) {  // the first run warms up
                    copy_regions(B, regions, false, st);
                    FFGPU_CHECK_CUDA(cudaEventRecord(e0, st));
                    launch_plan(B, st, false);
                    FFGPU_CHECK_CUDA(cudaEventRecord(e1, st));
                    FFGPU_CHECK_CUDA(cudaEventSynchronize(e1));
                    FFGPU_CHECK_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                }
                if (ms < best) {
                    best = ms;
                    bt_rs = trs;
                    bt_rsi = tri;
                    bt_cta = cps;
                }
            }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    copy_regions(B, regions, false, st);
    FFGPU_CHECK_CUDA(cudaStreamSynchronize(st));
    build_plan(B, bt_rs, bt_rsi, bt_cta);
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
            build_plan(*b, b->tile_rs, b->tile_rsi, b->ctas_per_sm);
    });
}

int ffgpu_batch_capture(ffgpu_batch *b, void *stream) {
    return guarded([&] {
        FFGPU_REQUIRE(b, "batch is NULL");
        std::lock_guard<std::mutex> lk(b->mu);
        if (!b->planned) build_plan(*b, b->tile_rs, b->tile_rsi, b->ctas_per_sm);
        b->drop_graph();
        cudaStream_t st = (cudaStream_t)stream;
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
            launched();
            return;
        }
        if (!b->planned) build_plan(*b, b->tile_rs, b->tile_rsi, b->ctas_per_sm);
        launch_plan(*b, st, true);
    });
}

int ffgpu_batch_info(const ffgpu_batch *b, int *tile_rs256, int *tile_rsi16, int *ctas_per_sm, size_t *items,
                     unsigned *grid) {
    return guarded([&] {
        FFGPU_REQUIRE(b, "batch is NULL");
        if (tile_rs256) *tile_rs256 = b->tile_rs;
        if (tile_rsi16) *tile_rsi16 = b->tile_rsi;
        if (ctas_per_sm) *ctas_per_sm = b->ctas_per_sm;
        if (items) *items = b->items.size();
        if (grid) *grid = b->grid;
    });
}

}  // extern "C"
