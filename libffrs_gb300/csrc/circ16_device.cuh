// CIRC16 repair stages as per-item device routines (one warp per item, or one
// thread per column), shared by the stage kernels (circ16.cu) and the fused
// batch kernel, which runs a whole CircRepair (pycirc16.hpp:135-335) inside
// one CTA.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace ffgpu {

struct Circ16Code;
struct CircDims {
    uint32_t ri_ml, ri_ecc, ri_bl;          // inner code
    uint32_t ro_ml, ro_ecc, ro_bl;          // outer code
    uint32_t interleave, rso_interleave;
    __device__ uint32_t rso_off(uint32_t k, uint32_t row) const { return rso_interleave * row + k * ri_ml; }
    __device__ uint32_t rsi_off(uint32_t k, uint32_t row) const { return (row * interleave + k) * ri_ecc; }
};

CircDims circ16_dims(const Circ16Code &c);

// repair_outer_zeros, part 1 (pycirc16.hpp:183-217): one warp per (k, outer
// parity row r).  Rows with non-zero inner syndromes collect the positions
// holding 0 (outer parity words first, then inner parity words) and, when
// there are 1..ecc of them, stage the inner block for an erasure repair.
static __device__ void outer_zeros_prepare_item(CircDims d, const uint32_t *rso_ecc, const uint32_t *rsi_ecc,
                                      const uint32_t *synd, uint32_t *blocks, uint32_t *zpos, uint32_t *zoff,
                                      uint32_t *zcnt, uint8_t *active, uint32_t item, int lane) {
    const uint32_t nitems = d.interleave * d.ro_ecc;
    if (item >= nitems) return;
    const uint32_t k = item / d.ro_ecc, r = item % d.ro_ecc;
    const uint32_t row = d.ro_ml + r;
    const uint32_t io = d.rsi_off(k, row), ro = d.rso_off(k, r);
    bool nz = false;
    for (uint32_t j = lane; j < d.ri_ecc; j += 32) nz |= synd[io + j] != 0;
    const bool has = __any_sync(0xffffffffu, nz);
    uint32_t *pl = zpos + (size_t)item * d.ri_ecc;
    uint32_t count = 0;
    if (has) {
        for (uint32_t j0 = 0; j0 < d.ri_bl; j0 += 32) {
            const uint32_t j = j0 + lane;
            bool z = false;
            if (j < d.ri_ml)
                z = rso_ecc[ro + j] == 0;
            else if (j < d.ri_bl)
                z = rsi_ecc[io + (j - d.ri_ml)] == 0;
            const uint32_t m = __ballot_sync(0xffffffffu, z);
            if (z) {
                const uint32_t idx = count + __popc(m & ((1u << lane) - 1u));
                if (idx < d.ri_ecc) pl[idx] = j;
            }
            count += __popc(m);
        }
    }
    const bool act = has && count > 0 && count <= d.ri_ecc;
    uint32_t *blk = blocks + (size_t)item * d.ri_bl;
    if (act)
        for (uint32_t j = lane; j < d.ri_bl; j += 32)
            blk[j] = j < d.ri_ml ? rso_ecc[ro + j] : rsi_ecc[io + (j - d.ri_ml)];
    if (lane == 0) {
        zoff[item] = item * d.ri_ecc;
        zcnt[item] = act ? count : 0;
        active[item] = act ? 1 : 0;
    }
}

// repair_outer_zeros, part 2 (pycirc16.hpp:221-231): keep the repair only when
// every erased position came out as 0 (mod 2^16), then store the repaired
// inner block and its fresh syndromes.
static __device__ void outer_zeros_commit_item(CircDims d, uint32_t *rso_ecc, uint32_t *rsi_ecc, uint32_t *synd,
                                     const uint32_t *blocks, const uint32_t *blk_synd, const uint32_t *zpos,
                                     const uint32_t *zcnt, const uint8_t *active, uint32_t item, int lane) {
    const uint32_t nitems = d.interleave * d.ro_ecc;
    if (item >= nitems || !active[item]) return;
    const uint32_t k = item / d.ro_ecc, r = item % d.ro_ecc;
    const uint32_t row = d.ro_ml + r;
    const uint32_t io = d.rsi_off(k, row), ro = d.rso_off(k, r);
    const uint32_t *blk = blocks + (size_t)item * d.ri_bl;
    const uint32_t *pl = zpos + (size_t)item * d.ri_ecc;
    bool bad = false;
    for (uint32_t z = lane; z < zcnt[item]; z += 32) bad |= (blk[pl[z]] & 0xffffu) != 0;
    if (__any_sync(0xffffffffu, bad)) return;
    for (uint32_t j = lane; j < d.ri_bl; j += 32) {
        if (j < d.ri_ml)
            rso_ecc[ro + j] = blk[j];
        else
            rsi_ecc[io + (j - d.ri_ml)] = blk[j];
    }
    for (uint32_t j = lane; j < d.ri_ecc; j += 32) synd[io + j] = blk_synd[(size_t)item * d.ri_ecc + j];
}

// repair_inner_zeros, part 1 (pycirc16.hpp:242-251)
static __device__ void inner_zeros_prepare_item(CircDims d, const uint32_t *rsi_ecc, const uint32_t *synd, uint32_t *vecs,
                                      uint8_t *flag, uint32_t item, int lane) {
    const uint32_t nitems = d.interleave * d.ro_bl;
    if (item >= nitems) return;
    const uint32_t k = item / d.ro_bl, row = item % d.ro_bl;
    const uint32_t io = d.rsi_off(k, row);
    bool nz = false, zero = false;
    for (uint32_t j = lane; j < d.ri_ecc; j += 32) {
        nz |= synd[io + j] != 0;
        zero |= rsi_ecc[io + j] == 0;
    }
    const bool f = __any_sync(0xffffffffu, nz) && __any_sync(0xffffffffu, zero);
    for (uint32_t j = lane; j < d.ri_ecc; j += 32) vecs[(size_t)item * d.ri_ecc + j] = f ? synd[io + j] : 0u;
    if (lane == 0) flag[item] = f;
}

// repair_inner_zeros, part 2 (pycirc16.hpp:252-256)
static __device__ void inner_zeros_commit_item(CircDims d, uint32_t *rsi_ecc, uint32_t *synd, const uint32_t *vecs,
                                     const uint8_t *flag, uint32_t item, int lane) {
    const uint32_t nitems = d.interleave * d.ro_bl;
    if (item >= nitems || !flag[item]) return;
    const uint32_t k = item / d.ro_bl, row = item % d.ro_bl;
    const uint32_t io = d.rsi_off(k, row);
    const uint32_t *v = vecs + (size_t)item * d.ri_ecc;
    bool bad = false;
    for (uint32_t j = lane; j < d.ri_ecc; j += 32) bad |= (v[j] & 0xffffu) != 0;
    if (__any_sync(0xffffffffu, bad)) return;
    for (uint32_t j = lane; j < d.ri_ecc; j += 32) {
        rsi_ecc[io + j] = v[j];
        synd[io + j] = 0;
    }
}

// find_error_locations + repair_outer_errors dispatch (pycirc16.hpp:283-305):
// one warp per group k lists the outer rows whose inner syndromes are still
// non-zero, then every outer column of the group is marked for a known-
// location repair (count <= outer ecc_len) or an unknown-location repair.
static __device__ void find_locations_item(CircDims d, const uint32_t *synd, uint32_t *locs, uint32_t *lcnt, uint32_t k, int lane) {
    if (k >= d.interleave) return;
    uint32_t count = 0;
    for (uint32_t i = 0; i < d.ro_bl; ++i) {
        const uint32_t io = d.rsi_off(k, i);
        bool nz = false;
        for (uint32_t j = lane; j < d.ri_ecc; j += 32) nz |= synd[io + j] != 0;
        if (__any_sync(0xffffffffu, nz)) {
            if (lane == 0) locs[(size_t)k * d.ro_bl + count] = i;
            ++count;
        }
    }
    if (lane == 0) lcnt[k] = count;
}

static __device__ void outer_modes_col(CircDims d, const uint32_t *lcnt, uint32_t *pos_off, uint32_t *pos_cnt, uint8_t *known,
                              uint8_t *unknown, uint32_t c, int lane) {
    if (c >= d.rso_interleave) return;
    const uint32_t k = c / d.ri_ml;
    const uint32_t n = lcnt[k];
    pos_off[c] = k * d.ro_bl;
    pos_cnt[c] = n;
    known[c] = n > 0 && n <= d.ro_ecc;
    unknown[c] = n > d.ro_ecc;
}


}  // namespace ffgpu
