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

// ---------------------------------------------------------------- many codewords
//
// The stage kernels over ncw codewords at once: item i of codeword cw is the
// global item cw * nitems + i, and every per-codeword array is a slice of a
// codeword-major array.  Position offsets (zoff, pos_off) are made global, so
// that one known-location repair launch serves every codeword.

struct CircMany {
    size_t rso_n, rsi_n, n_oz, n_iz;  // words per codeword of rso_ecc / rsi_ecc (and synd), item counts
};

__global__ void km_widen(const uint16_t *__restrict__ ecc, size_t ecc_len, size_t rso_n, size_t rsi_n,
                         uint32_t *__restrict__ rso, uint32_t *__restrict__ rsi, size_t ncw) {
    const size_t per = rso_n + rsi_n, total = per * ncw;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const size_t cw = i / per, j = i - cw * per;
        const uint32_t w = ecc[cw * ecc_len + j];
        if (j < rso_n)
            rso[cw * rso_n + j] = w;
        else
            rsi[cw * rsi_n + (j - rso_n)] = w;
    }
}

__global__ void km_outer_zeros_prepare(CircDims d, CircMany m, size_t ncw, const uint32_t *rso_ecc,
                                       const uint32_t *rsi_ecc, const uint32_t *synd, uint32_t *blocks,
                                       uint32_t *zpos, uint32_t *zoff, uint32_t *zcnt, uint8_t *active) {
    const size_t gi = blockIdx.x * (size_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (gi >= ncw * m.n_oz) return;
    const size_t cw = gi / m.n_oz;
    outer_zeros_prepare_item(d, rso_ecc + cw * m.rso_n, rsi_ecc + cw * m.rsi_n, synd + cw * m.rsi_n,
                             blocks + cw * m.n_oz * d.ri_bl, zpos + cw * m.n_oz * d.ri_ecc, zoff + cw * m.n_oz,
                             zcnt + cw * m.n_oz, active + cw * m.n_oz, (uint32_t)(gi - cw * m.n_oz), lane);
    if (lane == 0) zoff[gi] += (uint32_t)(cw * m.n_oz * d.ri_ecc);
}

__global__ void km_outer_zeros_commit(CircDims d, CircMany m, size_t ncw, uint32_t *rso_ecc, uint32_t *rsi_ecc,
                                      uint32_t *synd, const uint32_t *blocks, const uint32_t *blk_synd,
                                      const uint32_t *zpos, const uint32_t *zcnt, const uint8_t *active) {
    const size_t gi = blockIdx.x * (size_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
    if (gi >= ncw * m.n_oz) return;
    const size_t cw = gi / m.n_oz;
    outer_zeros_commit_item(d, rso_ecc + cw * m.rso_n, rsi_ecc + cw * m.rsi_n, synd + cw * m.rsi_n,
                            blocks + cw * m.n_oz * d.ri_bl, blk_synd + cw * m.n_oz * d.ri_ecc,
                            zpos + cw * m.n_oz * d.ri_ecc, zcnt + cw * m.n_oz, active + cw * m.n_oz,
                            (uint32_t)(gi - cw * m.n_oz), threadIdx.x & 31);
}

__global__ void km_inner_zeros_prepare(CircDims d, CircMany m, size_t ncw, const uint32_t *rsi_ecc,
                                       const uint32_t *synd, uint32_t *vecs, uint8_t *flag) {
    const size_t gi = blockIdx.x * (size_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
    if (gi >= ncw * m.n_iz) return;
    const size_t cw = gi / m.n_iz;
    inner_zeros_prepare_item(d, rsi_ecc + cw * m.rsi_n, synd + cw * m.rsi_n, vecs + cw * m.n_iz * d.ri_ecc,
                             flag + cw * m.n_iz, (uint32_t)(gi - cw * m.n_iz), threadIdx.x & 31);
}

__global__ void km_inner_zeros_commit(CircDims d, CircMany m, size_t ncw, uint32_t *rsi_ecc, uint32_t *synd,
                                      const uint32_t *vecs, const uint8_t *flag) {
    const size_t gi = blockIdx.x * (size_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
    if (gi >= ncw * m.n_iz) return;
    const size_t cw = gi / m.n_iz;
    inner_zeros_commit_item(d, rsi_ecc + cw * m.rsi_n, synd + cw * m.rsi_n, vecs + cw * m.n_iz * d.ri_ecc,
                            flag + cw * m.n_iz, (uint32_t)(gi - cw * m.n_iz), threadIdx.x & 31);
}

__global__ void km_find_locations(CircDims d, CircMany m, size_t ncw, const uint32_t *synd, uint32_t *locs,
                                  uint32_t *lcnt) {
    const size_t gi = blockIdx.x * (size_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
    if (gi >= ncw * d.interleave) return;
    const size_t cw = gi / d.interleave;
    find_locations_item(d, synd + cw * m.rsi_n, locs + cw * (size_t)d.interleave * d.ro_bl, lcnt + cw * d.interleave,
                        (uint32_t)(gi - cw * d.interleave), threadIdx.x & 31);
}

__global__ void km_outer_modes(CircDims d, size_t ncw, const uint32_t *lcnt, uint32_t *pos_off, uint32_t *pos_cnt,
                               uint8_t *known, uint8_t *unknown) {
    const size_t gi = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (gi >= ncw * d.rso_interleave) return;
    const size_t cw = gi / d.rso_interleave, o = cw * d.rso_interleave;
    outer_modes_col(d, lcnt + cw * d.interleave, pos_off + o, pos_cnt + o, known + o, unknown + o,
                    (uint32_t)(gi - o), 0);
    pos_off[gi] += (uint32_t)(cw * (size_t)d.interleave * d.ro_bl);
}

// Per codeword (one CTA): the first outer column whose repair raised, in the
// reference's column order.  With one, the columns from it on get their
// original words back, the ecc is left as it was and the status is
// FFGPU_STATUS_ASSERT; otherwise the ecc is written back (16-bit truncation,
// dump_ecc, pycirc16.hpp:326-330) and the status is 0.
__global__ void km_finish(CircDims d, CircMany m, size_t ncw, const uint8_t *col_status, uint16_t *msg,
                          const uint16_t *saved, size_t message_len, uint16_t *ecc, size_t ecc_len,
                          const uint32_t *rso_ecc, const uint32_t *rsi_ecc, uint8_t *status) {
    const size_t cw = blockIdx.x;
    if (cw >= ncw) return;
    __shared__ uint32_t first;
    if (threadIdx.x == 0) first = d.rso_interleave;
    __syncthreads();
    const uint8_t *cs = col_status + cw * d.rso_interleave;
    for (uint32_t c = threadIdx.x; c < d.rso_interleave; c += blockDim.x)
        if (cs[c] == FFGPU_STATUS_ASSERT) atomicMin(&first, c);
    __syncthreads();
    const uint32_t f = first;
    if (f < d.rso_interleave) {
        const size_t ncols = d.rso_interleave - f;
        for (size_t i = threadIdx.x; i < (size_t)d.ro_ml * ncols; i += blockDim.x) {
            const size_t r = i / ncols, col = f + (i - r * ncols);
            const size_t at = cw * message_len + r * d.rso_interleave + col;
            msg[at] = saved[at];
        }
        if (threadIdx.x == 0 && status) status[cw] = FFGPU_STATUS_ASSERT;
        return;
    }
    uint16_t *e = ecc + cw * ecc_len;
    for (size_t j = threadIdx.x; j < m.rso_n + m.rsi_n; j += blockDim.x)
        e[j] = (uint16_t)(j < m.rso_n ? rso_ecc[cw * m.rso_n + j] : rsi_ecc[cw * m.rsi_n + (j - m.rso_n)]);
    if (threadIdx.x == 0 && status) status[cw] = 0;
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

void circ16_encode(Circ16Code &c, const uint16_t *msg, size_t nblocks, uint16_t *ecc, cudaStream_t st, void *ws) {
    if (!nblocks) return;
    const Rsi16Code &ri = *c.rsi, &ro = *c.rso;
    uint32_t *tmp = (uint32_t *)(ws ? ws : c.enc_tmp.get(circ16_encode_ws_bytes(c, nblocks)));
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

size_t circ16_encode_ws_bytes(const Circ16Code &c, size_t nblocks) { return nblocks * c.rso_ieccl * 4; }

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

// Codeword-major workspace of circ16_repair_many: byte offsets of every
// stage array for ncw codewords.
struct ManyLayout {
    size_t o_rso, o_rsi, o_syn, o_blk, o_bsyn, o_zpos, o_zoff, o_zcnt, o_zact, o_vec, o_flag, o_locs, o_lcnt, o_poff,
        o_pcnt, o_kn, o_un, o_st, o_save, bytes;
};

static ManyLayout many_layout(const Circ16Code &c, size_t ncw) {
    const Rsi16Code &ri = *c.rsi, &ro = *c.rso;
    const size_t rso_n = c.rso_ieccl, rsi_n = c.rsi_total, n_oz = c.interleave * ro.ecc,
                 n_iz = c.interleave * ro.block_len;
    ManyLayout L;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off += (bytes + 255) & ~(size_t)255;
        return o;
    };
    L.o_rso = take(ncw * rso_n * 4);
    L.o_rsi = take(ncw * rsi_n * 4);
    L.o_syn = take(ncw * rsi_n * 4);
    L.o_blk = take(ncw * n_oz * ri.block_len * 4);
    L.o_bsyn = take(ncw * n_oz * ri.ecc * 4);
    L.o_zpos = take(ncw * n_oz * ri.ecc * 4);
    L.o_zoff = take(ncw * n_oz * 4);
    L.o_zcnt = take(ncw * n_oz * 4);
    L.o_zact = take(ncw * n_oz);
    L.o_vec = take(ncw * n_iz * ri.ecc * 4);
    L.o_flag = take(ncw * n_iz);
    L.o_locs = take(ncw * c.interleave * ro.block_len * 4);
    L.o_lcnt = take(ncw * c.interleave * 4);
    L.o_poff = take(ncw * c.rso_interleave * 4);
    L.o_pcnt = take(ncw * c.rso_interleave * 4);
    L.o_kn = take(ncw * c.rso_interleave);
    L.o_un = take(ncw * c.rso_interleave);
    L.o_st = take(ncw * c.rso_interleave);
    L.o_save = take(ncw * c.message_len * 2);
    L.bytes = off;
    return L;
}

size_t circ16_repair_many_ws_bytes(const Circ16Code &c, size_t ncw) { return many_layout(c, ncw).bytes; }

// ncw codewords in place (device pointers): the stages of circ16_repair_one,
// each one launch over every codeword.  status[cw] is 0 or
// FFGPU_STATUS_ASSERT as in ffgpu_circ16_repair.  ws: a workspace of
// circ16_repair_many_ws_bytes(c, ncw) bytes, or NULL for the code's own.
void circ16_repair_many(Circ16Code &c, uint16_t *msg, uint16_t *ecc, size_t ncw, uint8_t *status, cudaStream_t st,
                        void *ws) {
    if (!ncw) return;
    const Rsi16Code &ri = *c.rsi, &ro = *c.rso;
    const CircDims d = circ16_dims(c);
    CircMany m;
    m.rso_n = c.rso_ieccl;
    m.rsi_n = c.rsi_total;
    m.n_oz = c.interleave * ro.ecc;
    m.n_iz = c.interleave * ro.block_len;
    const ManyLayout L = many_layout(c, ncw);
    char *W = (char *)(ws ? ws : c.rep_ws.get(L.bytes));
    const size_t o_rso = L.o_rso, o_rsi = L.o_rsi, o_syn = L.o_syn, o_blk = L.o_blk, o_bsyn = L.o_bsyn,
                 o_zpos = L.o_zpos, o_zoff = L.o_zoff, o_zcnt = L.o_zcnt, o_zact = L.o_zact, o_vec = L.o_vec,
                 o_flag = L.o_flag, o_locs = L.o_locs, o_lcnt = L.o_lcnt, o_poff = L.o_poff, o_pcnt = L.o_pcnt,
                 o_kn = L.o_kn, o_un = L.o_un, o_st = L.o_st, o_save = L.o_save;
    uint32_t *rso_ecc = (uint32_t *)(W + o_rso), *rsi_ecc = (uint32_t *)(W + o_rsi), *synd = (uint32_t *)(W + o_syn);
    uint32_t *blocks = (uint32_t *)(W + o_blk), *bsyn = (uint32_t *)(W + o_bsyn), *zpos = (uint32_t *)(W + o_zpos);
    uint32_t *zoff = (uint32_t *)(W + o_zoff), *zcnt = (uint32_t *)(W + o_zcnt);
    uint8_t *zact = (uint8_t *)(W + o_zact), *flag = (uint8_t *)(W + o_flag);
    uint32_t *vecs = (uint32_t *)(W + o_vec), *locs = (uint32_t *)(W + o_locs), *lcnt = (uint32_t *)(W + o_lcnt);
    uint32_t *poff = (uint32_t *)(W + o_poff), *pcnt = (uint32_t *)(W + o_pcnt);
    uint8_t *kn = (uint8_t *)(W + o_kn), *un = (uint8_t *)(W + o_un), *cst = (uint8_t *)(W + o_st);
    uint16_t *saved = (uint16_t *)(W + o_save);
    const unsigned wpb = 4;  // warps per CTA of the per-item kernels
    auto items = [&](size_t n) { return (unsigned)((n + wpb - 1) / wpb); };

    FFGPU_CHECK_CUDA(cudaMemcpyAsync(saved, msg, ncw * c.message_len * 2, cudaMemcpyDeviceToDevice, st));
    // load_ecc (pycirc16.hpp:159-163)
    {
        KernelTimer kt_timer("km_widen", st);
        km_widen<<<g1(ncw * (m.rso_n + m.rsi_n)), 256, 0, st>>>(ecc, c.ecc_len, m.rso_n, m.rsi_n, rso_ecc, rsi_ecc, ncw);
    }
    check_launch("km_widen");
    // compute_rsi_synd (pycirc16.hpp:165-181): message rows, then outer parity rows
    BlockView vmsg{msg, c.message_len, ri.message_len, 1, rsi_ecc, m.rsi_n, ri.ecc, 1, c.inner_rows, true, false};
    rsi16_synd_grouped(ri, vmsg, ncw * c.inner_rows, synd, c.inner_rows, m.rsi_n, st);
    BlockView vrso{rso_ecc, m.rso_n, ri.message_len, 1, rsi_ecc + c.rsi_ieccl, m.rsi_n, ri.ecc, 1, c.outer_rows,
                   false, false};
    rsi16_synd_grouped(ri, vrso, ncw * c.outer_rows, synd + c.rsi_ieccl, c.outer_rows, m.rsi_n, st);
    // repair_outer_zeros for every codeword and k
    {
        KernelTimer kt_timer("km_outer_zeros_prepare", st);
        km_outer_zeros_prepare<<<items(ncw * m.n_oz), wpb * 32, 0, st>>>(d, m, ncw, rso_ecc, rsi_ecc, synd, blocks, zpos,
                                                                         zoff, zcnt, zact);
    }
    check_launch("km_outer_zeros_prepare");
    BlockView vblk{blocks, m.n_oz * ri.block_len, ri.block_len, 1, blocks + ri.message_len, m.n_oz * ri.block_len,
                   ri.block_len, 1, m.n_oz, false, false};
    rsi16_repair_known(ri, vblk, ncw * m.n_oz, zpos, zoff, zcnt, 0, zact, nullptr, st);
    rsi16_synd(ri, vblk, ncw * m.n_oz, bsyn, st);
    {
        KernelTimer kt_timer("km_outer_zeros_commit", st);
        km_outer_zeros_commit<<<items(ncw * m.n_oz), wpb * 32, 0, st>>>(d, m, ncw, rso_ecc, rsi_ecc, synd, blocks, bsyn,
                                                                        zpos, zcnt, zact);
    }
    check_launch("km_outer_zeros_commit");
    // repair_inner_zeros for every codeword and k
    {
        KernelTimer kt_timer("km_inner_zeros_prepare", st);
        km_inner_zeros_prepare<<<items(ncw * m.n_iz), wpb * 32, 0, st>>>(d, m, ncw, rsi_ecc, synd, vecs, flag);
    }
    check_launch("km_inner_zeros_prepare");
    rsi16_mix_ecc(ri, vecs, ncw * m.n_iz, st);
    {
        KernelTimer kt_timer("km_inner_zeros_commit", st);
        km_inner_zeros_commit<<<items(ncw * m.n_iz), wpb * 32, 0, st>>>(d, m, ncw, rsi_ecc, synd, vecs, flag);
    }
    check_launch("km_inner_zeros_commit");
    // find_error_locations, then repair_outer_errors (pycirc16.hpp:283-305)
    {
        KernelTimer kt_timer("km_find_locations", st);
        km_find_locations<<<items(ncw * c.interleave), wpb * 32, 0, st>>>(d, m, ncw, synd, locs, lcnt);
    }
    check_launch("km_find_locations");
    {
        KernelTimer kt_timer("km_outer_modes", st);
        km_outer_modes<<<g1(ncw * c.rso_interleave), 256, 0, st>>>(d, ncw, lcnt, poff, pcnt, kn, un);
    }
    check_launch("km_outer_modes");
    FFGPU_CHECK_CUDA(cudaMemsetAsync(cst, 0, ncw * c.rso_interleave, st));
    BlockView vcol = interleaved_view(msg, true, ro.message_len, rso_ecc, false, ro.ecc, c.rso_interleave);
    rsi16_repair_known(ro, vcol, ncw * c.rso_interleave, locs, poff, pcnt, 0, kn, cst, st);
    rsi16_repair(ro, vcol, ncw * c.rso_interleave, cst, st, un);
    // recompute_inner_ecc (pycirc16.hpp:320-324)
    BlockView vre{msg, c.message_len, ri.message_len, 1, rsi_ecc, m.rsi_n, ri.ecc, 1, c.inner_rows, true, false};
    rsi16_encode(ri, vre, ncw * c.inner_rows, st);
    BlockView vreo{rso_ecc, m.rso_n, ri.message_len, 1, rsi_ecc + c.rsi_ieccl, m.rsi_n, ri.ecc, 1, c.outer_rows,
                   false, false};
    rsi16_encode(ri, vreo, ncw * c.outer_rows, st);
    // raising codewords restored, the others' ecc written back
    {
        KernelTimer kt_timer("km_finish", st);
        km_finish<<<(unsigned)ncw, 256, 0, st>>>(d, m, ncw, cst, msg, saved, c.message_len, ecc, c.ecc_len, rso_ecc,
                                                 rsi_ecc, status);
    }
    check_launch("km_finish");
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
