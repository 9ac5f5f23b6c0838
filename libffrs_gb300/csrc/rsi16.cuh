// RSi16: Reed-Solomon over GF(65537) with NTT-based encode and an NTT-domain
// Sugiyama decoder.  Code object (host tables + device copies) and the kernel
// entry points used by the C ABI and by the CIRC16 pipeline.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

namespace ffgpu {

// Device view of one RSi16 code: every table the reference's NTT / RSi16v
// constructors build (libffrs/ntt.hpp:55-123, libffrs/rsi16v_impl.hpp:68-86).
struct Rsi16Dev {
    const uint32_t *roots_ntt, *roots_ecc, *roots_i_ecc, *roots_ecc2, *roots_i_ecc2;
    const uint32_t *pntt_shift, *pintt_shift, *rbo_ecc, *ecc_mix;
    // floor(w 2^32 / p) of every pntt_shift / pintt_shift entry w (the
    // Shoup companions used by the one-block-per-thread kernels)
    const uint32_t *pntt_shift_s, *pintt_shift_s;
    // ecc 32 / 64: the BtTw of the block-per-thread kernels, else NULL
    const uint32_t *bt_tw;
    const uint32_t *inv_tab;  // inverse of every field element (inv(0) == 1, as the reference's table)
    uint32_t block_len, message_len, ecc, ntt_len, pntt_blocks, ecc_mask, rbo_shift;
    uint32_t ecc_len_i, ecc2_len_i;
    uint32_t temp_len;  // ntt_len + 6 * ecc: the reference's repair scratch
};

struct Rsi16Code {
    uint32_t primitive;
    size_t block_len, message_len, ecc, ntt_len, pntt_blocks;
    uint32_t root, ecc_mask;
    unsigned rbo_shift;
    std::vector<uint32_t> exp_, log_;
    std::vector<uint32_t> roots_ntt, roots_i_ntt, roots_ecc, roots_i_ecc, roots_ecc2, roots_i_ecc2;
    std::vector<uint32_t> pntt_shift, pintt_shift, rbo_ecc, ecc_mix;
    std::vector<uint32_t> pntt_shift_s, pintt_shift_s;
    uint32_t ntt_len_i, ecc_len_i, ecc2_len_i;
    uint32_t *d_tables = nullptr;
    Rsi16Dev dev{};

    Rsi16Code(size_t block_len, size_t ecc_len, uint32_t primitive);
    ~Rsi16Code();
    Rsi16Code(const Rsi16Code &) = delete;
    Rsi16Code &operator=(const Rsi16Code &) = delete;

    uint32_t rbo(uint32_t i) const;
    uint32_t inv(uint32_t a) const { return exp_[65536u - log_[a]]; }
    uint32_t pow(uint32_t a, uint32_t e) const { return exp_[(uint32_t)(log_[a] * e) % 65536u]; }
    uint32_t div(uint32_t a, uint32_t b) const {
        if (!a) return 0;
        uint32_t r = log_[a] + 65536u - log_[b];
        if (r >= 65536u) r -= 65536u;
        return exp_[r];
    }
};

// A strided view of one family of blocks.  Block b belongs to group
// g = b / group and column j = b % group; element k of its message lives at
// msg[g * msg_gstride + j * msg_bstride + k * msg_estride] (same for parity).
// Contiguous blocks use group = 1 and gstride = message_len (or ecc_len);
// the columns of interleaved blocks (pyrsi16.hpp:323-361) use group =
// interleave, bstride = 1, estride = interleave.  msg16 / par16 select uint16
// (else uint32) words.
struct BlockView {
    void *msg;
    size_t msg_gstride, msg_bstride, msg_estride;
    void *par;
    size_t par_gstride, par_bstride, par_estride;
    size_t group;
    bool msg16, par16;
    __host__ __device__ size_t moff(size_t b, size_t k) const {
        return (b / group) * msg_gstride + (b % group) * msg_bstride + k * msg_estride;
    }
    __host__ __device__ size_t poff(size_t b, size_t k) const {
        return (b / group) * par_gstride + (b % group) * par_bstride + k * par_estride;
    }
};

__host__ __device__ inline BlockView contiguous_view(void *msg, bool msg16, size_t message_len, void *par, bool par16, size_t ecc) {
    return BlockView{msg, message_len, 0, 1, par, ecc, 0, 1, 1, msg16, par16};
}
__host__ __device__ inline BlockView interleaved_view(void *msg, bool msg16, size_t message_len, void *par, bool par16, size_t ecc,
                                  size_t interleave) {
    return BlockView{msg, message_len * interleave, 1, interleave, par, ecc * interleave, 1, interleave,
                     interleave, msg16, par16};
}

// Encode nblocks blocks of the view (parity written into the view's parity).
void rsi16_encode(const Rsi16Code &c, const BlockView &v, size_t nblocks, cudaStream_t st);
// Syndromes (ecc uint32 per block) of nblocks blocks of the view.
void rsi16_synd(const Rsi16Code &c, const BlockView &v, size_t nblocks, uint32_t *synds, cudaStream_t st);
// The same with the syndromes of block b at
// synds + (b / out_group) * out_gstride + (b % out_group) * ecc_len.
void rsi16_synd_grouped(const Rsi16Code &c, const BlockView &v, size_t nblocks, uint32_t *synds, size_t out_group,
                        size_t out_gstride, cudaStream_t st);
// Unknown-location repair in place; status per block (RepairStatus or 0xFF).
// A non-NULL active array restricts the repair to blocks with active[b] != 0.
void rsi16_repair(const Rsi16Code &c, const BlockView &v, size_t nblocks, uint8_t *status, cudaStream_t st,
                  const uint8_t *active = nullptr);
// Known-location repair in place with per-block position lists: positions of
// block b are pos[pos_off[b] .. pos_off[b] + pos_cnt[b]) (block positions,
// not RBO).  A NULL active array repairs every block; otherwise only blocks
// with active[b] != 0.
// pos_off == NULL: every block uses pos[0 ..); pos_cnt == NULL: every block
// has count_all positions.
void rsi16_repair_known(const Rsi16Code &c, const BlockView &v, size_t nblocks, const uint32_t *pos,
                        const uint32_t *pos_off, const uint32_t *pos_cnt, uint32_t count_all, const uint8_t *active,
                        uint8_t *status, cudaStream_t st);
// Sugiyama on raw syndrome vectors (debug surface of the binding).
void rsi16_sugiyama(const Rsi16Code &c, const uint32_t *synds, size_t nblocks, uint32_t *locator, uint32_t *evaluator,
                    uint8_t *status, cudaStream_t st);
// pintt_ecc zeros of one polynomial (debug surface of the binding).
void rsi16_roots(const Rsi16Code &c, const uint32_t *poly, uint8_t *is_zero, cudaStream_t st);
// blocks the unknown-location repair kernel served by the bounded-distance
// path and by the step-for-step mirror since load (or the last reset);
// synchronises the device
void rsi16_repair_counters(uint64_t *fast, uint64_t *mirror, bool reset);
// mix_ecc on nvec ecc-word vectors in place (used by the CIRC16 heuristics).
void rsi16_mix_ecc(const Rsi16Code &c, uint32_t *vecs, size_t nvec, cudaStream_t st);

}  // namespace ffgpu
