// CIRC16 code object and pipeline entry points (circ16.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>

#include "common.cuh"
#include "rsi16.cuh"

namespace ffgpu {

struct Circ16Code {
    std::unique_ptr<Rsi16Code> rsi, rso;
    size_t interleave, rso_interleave;
    size_t block_len, message_len, rso_ieccl, rsi_ieccl, rsio_len, ecc_len;
    size_t inner_rows, outer_rows, rsi_total;
    DeviceBuffer enc_tmp, rep_ws;

    Circ16Code(size_t inner_block_len, size_t inner_ecc_len, size_t outer_block_len, size_t outer_ecc_len,
               size_t interleave, uint32_t primitive);
};

// Word offsets of the CircRepair workspace of one block (every array 64-word
// aligned); `words` is the total.
struct CircLayout {
    size_t o_rso, o_rsi, o_syn, o_blk, o_bsyn, o_zpos, o_zoff, o_zcnt, o_zact, o_vec, o_flag, o_locs, o_lcnt, o_poff,
        o_pcnt, o_kn, o_un, o_st, words;
};
CircLayout circ16_layout(const Circ16Code &c);

// ws: circ16_encode_ws_bytes(c, nblocks) bytes of workspace, or NULL for the
// code's own.
void circ16_encode(Circ16Code &c, const uint16_t *msg, size_t nblocks, uint16_t *ecc, cudaStream_t st,
                   void *ws = nullptr);
size_t circ16_encode_ws_bytes(const Circ16Code &c, size_t nblocks);
// Repair of one block up to (not including) the ecc write-back.  With
// stop_after_find the pipeline stops after the error-row search and copies
// the rows of group find_k to locs_out / lcnt_out (host pointers).
void circ16_repair_one(Circ16Code &c, uint16_t *msg, uint16_t *ecc, cudaStream_t st, bool stop_after_find,
                       size_t find_k, uint32_t *locs_out, uint32_t *lcnt_out, uint8_t *col_status);
void circ16_dump_ecc(Circ16Code &c, uint16_t *ecc, cudaStream_t st);
// ncw codewords in place, every repair stage as one launch over all of them;
// status[cw] 0 or FFGPU_STATUS_ASSERT (NULL: not written).
void circ16_repair_many(Circ16Code &c, uint16_t *msg, uint16_t *ecc, size_t ncw, uint8_t *status, cudaStream_t st,
                        void *ws = nullptr);
size_t circ16_repair_many_ws_bytes(const Circ16Code &c, size_t ncw);

}  // namespace ffgpu
