// CIRC16: cross-interleaved code of two RSi16 codes (libffrs/pycirc16.hpp).
//
// Encode (pycirc16.hpp:352-363) is three RSi16 encodes over strided views:
// outer parity of the interleaved columns (kept untruncated as uint32, since
// the reference encodes rsio from that GFT buffer), inner parity of the
// message rows, and inner parity of the outer-parity rows.
//
// Repair (CircRepair, pycirc16.hpp:135-335) runs as a short sequence of
// kernels with every decision taken on the device.  The interleave groups k
// touch disjoint rows and columns, so all of them advance together; within a
// group the reference's order is kept: outer-zero repair, inner-zero repair,
// error-row search, outer erasure (or unknown-location) repair, inner parity
// recomputation, write-back with 16-bit truncation.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <vector>

#include "circ16.cuh"
#include "circ16_device.cuh"
#include "common.cuh"

namespace ffgpu {

Circ16Code::Circ16Code(size_t ib, size_t ie, size_t ob, size_t oe, size_t interleave_, uint32_t primitive)
    : interleave(interleave_) {
    FFGPU_REQUIRE(interleave_ >= 1, "interleave must be positive");
    rsi = std::make_unique<Rsi16Code>(ib, ie, primitive);
    rso = std::make_unique<Rsi16Code>(ob, oe, primitive);
    rso_interleave = rsi->message_len * interleave;
    block_len = ib * ob * interleave;
    message_len = rso->message_len * rso_interleave;
    rso_ieccl = rso->ecc * rso_interleave;
    rsi_ieccl = rsi->ecc * rso->message_len * interleave;
    rsio_len = rsi->ecc * rso->ecc * interleave;
    ecc_len = rso_ieccl + rsi_ieccl + rsio_len;
    inner_rows = rso->message_len * interleave;
    outer_rows = rso->ecc * interleave;
    rsi_total = rsi->ecc * rso->block_len * interleave;
}

// ---------------------------------------------------------------- small kernels

__global__ void k_widen(const uint16_t *__restrict__ a, uint32_t *__restrict__ b, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        b[i] = a[i];
}
__global__ void k_narrow(const uint32_t *__restrict__ a, uint16_t *__restrict__ b, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        b[i] = (uint16_t)a[i];
}
// per-block narrow: nblocks segments of n words, src stride ss, dst stride ds
__global__ void k_narrow_strided(const uint32_t *__restrict__ a, size_t ss, uint16_t *__restrict__ b, size_t ds,
                                 size_t n, size_t nblocks) {
    const size_t total = n * nblocks;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const size_t blk = i / n, j = i - blk * n;
        b[blk * ds + j] = (uint16_t)a[blk * ss + j];
    }
}

__global__ void k_outer_zeros_prepare(CircDims d, const uint32_t *rso_ecc, const uint32_t *rsi_ecc,
                                      const uint32_t *synd, uint32_t *blocks, uint32_t *zpos, uint32_t *zoff,
                                      uint32_t *zcnt, uint8_t *active) {
    outer_zeros_prepare_item(d, rso_ecc, rsi_ecc, synd, blocks, zpos, zoff, zcnt, active,
                             blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), threadIdx.x & 31);
}

__global__ void k_outer_zeros_commit(CircDims d, uint32_t *rso_ecc, uint32_t *rsi_ecc, uint32_t *synd,
                                     const uint32_t *blocks, const uint32_t *blk_synd, const uint32_t *zpos,
                                     const uint32_t *zcnt, const uint8_t *active) {
    outer_zeros_commit_item(d, rso_ecc, rsi_ecc, synd, blocks, blk_synd, zpos, zcnt, active,
                            blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), threadIdx.x & 31);
}

__global__ void k_inner_zeros_prepare(CircDims d, const uint32_t *rsi_ecc, const uint32_t *synd, uint32_t *vecs,
                                      uint8_t *flag) {
    inner_zeros_prepare_item(d, rsi_ecc, synd, vecs, flag, blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5),
                             threadIdx.x & 31);
}

__global__ void k_inner_zeros_commit(CircDims d, uint32_t *rsi_ecc, uint32_t *synd, const uint32_t *vecs,
                                     const uint8_t *flag) {
    inner_zeros_commit_item(d, rsi_ecc, synd, vecs, flag, blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5),
                            threadIdx.x & 31);
}

__global__ void k_find_locations(CircDims d, const uint32_t *synd, uint32_t *locs, uint32_t *lcnt) {
    find_locations_item(d, synd, locs, lcnt, blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), threadIdx.x & 31);
}

__global__ void k_outer_modes(CircDims d, const uint32_t *lcnt, uint32_t *pos_off, uint32_t *pos_cnt, uint8_t *known,
                              uint8_t *unknown) {
    outer_modes_col(d, lcnt, pos_off, pos_cnt, known, unknown, blockIdx.x * blockDim.x + threadIdx.x, 0);
}

// ---------------------------------------------------------------- host side

static unsigned g1(size_t n) { return (unsigned)std::min<size_t>((n + 255) / 256, 4096); }

CircDims circ16_dims(const Circ16Code &c) {
    CircDims d;
    d.ri_ml = (uint32_t)c.rsi->message_len;
    d.ri_ecc = (uint32_t)c.rsi->ecc;
    d.ri_bl = (uint32_t)c.rsi->block_len;
    d.ro_ml = (uint32_t)c.rso->message_len;
    d.ro_ecc = (uint32_t)c.rso->ecc;
    d.ro_bl = (uint32_t)c.rso->block_len;
    d.interleave = (uint32_t)c.interleave;
    d.rso_interleave = (uint32_t)c.rso_interleave;
    return d;
}

CircLayout circ16_layout(const Circ16Code &c) {
    const Rsi16Code &ri = *c.rsi, &ro = *c.rso;
    const size_t n_oz = c.interleave * ro.ecc, n_iz = c.interleave * ro.block_len;
    size_t off = 0;
    auto take = [&](size_t words) {
        size_t o = off;
        off += (words + 63) & ~(size_t)63;
        return o;
    };
    CircLayout L;
    L.o_rso = take(c.rso_ieccl);
    L.o_rsi = take(c.rsi_total);
    L.o_syn = take(c.rsi_total);
    L.o_blk = take(n_oz * ri.block_len);
    L.o_bsyn = take(n_oz * ri.ecc);
    L.o_zpos = take(n_oz * ri.ecc);
    L.o_zoff = take(n_oz);
    L.o_zcnt = take(n_oz);
    L.o_zact = take(n_oz / 4 + 1);
    L.o_vec = take(n_iz * ri.ecc);
    L.o_flag = take(n_iz / 4 + 1);
    L.o_locs = take(c.interleave * ro.block_len);
    L.o_lcnt = take(c.interleave);
    L.o_poff = take(c.rso_interleave);
    L.o_pcnt = take(c.rso_interleave);
    L.o_kn = take(c.rso_interleave / 4 + 1);
    L.o_un = take(c.rso_interleave / 4 + 1);
    L.o_st = take(c.rso_interleave / 4 + 1);
    L.words = off;
    return L;
}

void circ16_encode(Circ16Code &c, const uint16_t *msg, size_t nblocks, uint16_t *ecc, cudaStream_t st) {
    if (!nblocks) return;
    const Rsi16Code &ri = *c.rsi, &ro = *c.rso;
    uint32_t *tmp = (uint32_t *)c.enc_tmp.get(nblocks * c.rso_ieccl * 4);
    // outer code over the interleaved columns -> untruncated uint32 parity
    BlockView vo{(void *)msg, c.message_len, 1, c.rso_interleave, tmp, c.rso_ieccl, 1, c.rso_interleave,
                 c.rso_interleave, true, false};
    rsi16_encode(ro, vo, nblocks * c.rso_interleave, st);
    k_narrow_strided<<<g1(nblocks * c.rso_ieccl), 256, 0, st>>>(tmp, c.rso_ieccl, ecc, c.ecc_len, c.rso_ieccl,
                                                                 nblocks);
    check_launch("k_narrow_strided");
    // inner code over the message rows
    BlockView vi{(void *)msg, c.message_len, ri.message_len, 1, ecc + c.rso_ieccl, c.ecc_len, ri.ecc, 1,
                 c.inner_rows, true, true};
    rsi16_encode(ri, vi, nblocks * c.inner_rows, st);
    // inner code over the outer parity rows
    BlockView vio{tmp, c.rso_ieccl, ri.message_len, 1, ecc + c.rso_ieccl + c.rsi_ieccl, c.ecc_len, ri.ecc, 1,
                  c.outer_rows, false, true};
    rsi16_encode(ri, vio, nblocks * c.outer_rows, st);
}

// One CIRC16 block in place.  Returns through *assert_col the first outer
// column (in the reference's k-major order) whose repair raised, or SIZE_MAX.
void circ16_repair_one(Circ16Code &c, uint16_t *msg, uint16_t *ecc, cudaStream_t st, bool stop_after_find,
                       size_t find_k, uint32_t *locs_out, uint32_t *lcnt_out, uint8_t *col_status) {
    const Rsi16Code &ri = *c.rsi, &ro = *c.rso;
    const CircDims d = circ16_dims(c);
    const size_t n_oz = c.interleave * ro.ecc, n_iz = c.interleave * ro.block_len;
    const CircLayout lay = circ16_layout(c);
    const size_t o_rso = lay.o_rso, o_rsi = lay.o_rsi, o_syn = lay.o_syn, o_blk = lay.o_blk, o_bsyn = lay.o_bsyn,
                 o_zpos = lay.o_zpos, o_zoff = lay.o_zoff, o_zcnt = lay.o_zcnt, o_zact = lay.o_zact, o_vec = lay.o_vec,
                 o_flag = lay.o_flag, o_locs = lay.o_locs, o_lcnt = lay.o_lcnt, o_poff = lay.o_poff,
                 o_pcnt = lay.o_pcnt, o_kn = lay.o_kn, o_un = lay.o_un, o_st = lay.o_st;
    uint32_t *W = (uint32_t *)c.rep_ws.get(lay.words * 4);
    uint32_t *rso_ecc = W + o_rso, *rsi_ecc = W + o_rsi, *synd = W + o_syn;
    uint32_t *blocks = W + o_blk, *bsyn = W + o_bsyn, *zpos = W + o_zpos, *zoff = W + o_zoff, *zcnt = W + o_zcnt;
    uint8_t *zact = (uint8_t *)(W + o_zact);
    uint32_t *vecs = W + o_vec;
    uint8_t *flag = (uint8_t *)(W + o_flag);
    uint32_t *locs = W + o_locs, *lcnt = W + o_lcnt, *poff = W + o_poff, *pcnt = W + o_pcnt;
    uint8_t *kn = (uint8_t *)(W + o_kn), *un = (uint8_t *)(W + o_un), *cst = (uint8_t *)(W + o_st);
    const unsigned wpb = 4;  // warps per CTA for the per-item kernels

    // load_ecc (pycirc16.hpp:159-163)
    k_widen<<<g1(c.rso_ieccl), 256, 0, st>>>(ecc, rso_ecc, c.rso_ieccl);
    check_launch("k_widen");
    k_widen<<<g1(c.rsi_total), 256, 0, st>>>(ecc + c.rso_ieccl, rsi_ecc, c.rsi_total);
    check_launch("k_widen");
    // compute_rsi_synd (pycirc16.hpp:165-181)
    BlockView vmsg{msg, 0, ri.message_len, 1, rsi_ecc, 0, ri.ecc, 1, c.inner_rows, true, false};
    rsi16_synd(ri, vmsg, c.inner_rows, synd, st);
    BlockView vrso{rso_ecc, 0, ri.message_len, 1, rsi_ecc + c.rsi_ieccl, 0, ri.ecc, 1, c.outer_rows, false, false};
    rsi16_synd(ri, vrso, c.outer_rows, synd + c.rsi_ieccl, st);
    // repair_outer_zeros for every k
    k_outer_zeros_prepare<<<(unsigned)((n_oz + wpb - 1) / wpb), wpb * 32, 0, st>>>(d, rso_ecc, rsi_ecc, synd, blocks,
                                                                                   zpos, zoff, zcnt, zact);
    check_launch("k_outer_zeros_prepare");
    BlockView vblk{blocks, 0, ri.block_len, 1, blocks + ri.message_len, 0, ri.block_len, 1, n_oz, false, false};
    rsi16_repair_known(ri, vblk, n_oz, zpos, zoff, zcnt, 0, zact, nullptr, st);
    rsi16_synd(ri, vblk, n_oz, bsyn, st);
    k_outer_zeros_commit<<<(unsigned)((n_oz + wpb - 1) / wpb), wpb * 32, 0, st>>>(d, rso_ecc, rsi_ecc, synd, blocks,
                                                                                  bsyn, zpos, zcnt, zact);
    check_launch("k_outer_zeros_commit");
    // repair_inner_zeros for every k
    k_inner_zeros_prepare<<<(unsigned)((n_iz + wpb - 1) / wpb), wpb * 32, 0, st>>>(d, rsi_ecc, synd, vecs, flag);
    check_launch("k_inner_zeros_prepare");
    rsi16_mix_ecc(ri, vecs, n_iz, st);
    k_inner_zeros_commit<<<(unsigned)((n_iz + wpb - 1) / wpb), wpb * 32, 0, st>>>(d, rsi_ecc, synd, vecs, flag);
    check_launch("k_inner_zeros_commit");
    // find_error_locations for every k
    k_find_locations<<<(unsigned)((c.interleave + wpb - 1) / wpb), wpb * 32, 0, st>>>(d, synd, locs, lcnt);
    check_launch("k_find_locations");
    if (stop_after_find) {
        FFGPU_CHECK_CUDA(cudaMemcpyAsync(lcnt_out, lcnt + find_k, 4, cudaMemcpyDeviceToHost, st));
        FFGPU_CHECK_CUDA(cudaMemcpyAsync(locs_out, locs + find_k * ro.block_len, ro.block_len * 4,
                                         cudaMemcpyDeviceToHost, st));
        return;
    }
    // repair_outer_errors for every k (pycirc16.hpp:289-305)
    k_outer_modes<<<g1(c.rso_interleave), 256, 0, st>>>(d, lcnt, poff, pcnt, kn, un);
    check_launch("k_outer_modes");
    FFGPU_CHECK_CUDA(cudaMemsetAsync(cst, 0, c.rso_interleave, st));
    BlockView vcol = interleaved_view(msg, true, ro.message_len, rso_ecc, false, ro.ecc, c.rso_interleave);
    rsi16_repair_known(ro, vcol, c.rso_interleave, locs, poff, pcnt, 0, kn, cst, st);
    rsi16_repair(ro, vcol, c.rso_interleave, cst, st, un);
    // recompute_inner_ecc (pycirc16.hpp:320-324)
    BlockView vre{msg, 0, ri.message_len, 1, rsi_ecc, 0, ri.ecc, 1, c.inner_rows, true, false};
    rsi16_encode(ri, vre, c.inner_rows, st);
    BlockView vreo{rso_ecc, 0, ri.message_len, 1, rsi_ecc + c.rsi_ieccl, 0, ri.ecc, 1, c.outer_rows, false, false};
    rsi16_encode(ri, vreo, c.outer_rows, st);
    if (col_status) FFGPU_CHECK_CUDA(cudaMemcpyAsync(col_status, cst, c.rso_interleave, cudaMemcpyDeviceToHost, st));
}

// dump_ecc (pycirc16.hpp:326-330), kept separate so that a raising repair can
// skip it as the reference does
void circ16_dump_ecc(Circ16Code &c, uint16_t *ecc, cudaStream_t st) {
    const Rsi16Code &ri = *c.rsi, &ro = *c.rso;
    (void)ri;
    (void)ro;
    uint32_t *W = (uint32_t *)c.rep_ws.ptr;
    const size_t o_rsi = (c.rso_ieccl + 63) & ~(size_t)63;
    k_narrow<<<g1(c.rso_ieccl), 256, 0, st>>>(W, ecc, c.rso_ieccl);
    check_launch("k_narrow");
    k_narrow<<<g1(c.rsi_total), 256, 0, st>>>(W + o_rsi, ecc + c.rso_ieccl, c.rsi_total);
    check_launch("k_narrow");
}

}  // namespace ffgpu
