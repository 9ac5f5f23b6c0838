// RSi16 device code shared by the standalone kernels (rsi16.cu), the CIRC16
// pipeline and the fused batch kernel: GF(65537) arithmetic, warp-wide NTTs
// and the polynomial steps of the reference's W = 1 code path, block I/O
// through a BlockView, and the one-block routines a warp runs (encode,
// syndromes, unknown- and known-location repair).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/ffgpu.h"
#include "rsi16.cuh"

namespace ffgpu {

// ---------------------------------------------------------------- field ops

// GF(65537) on canonical values in [0, 65536] (libffrs/galois.hpp:258-346).
// The product x = a b <= 2^32 is taken to 64 bits (one wide multiply-add);
// with 2^16 = -1 and 2^32 = 1 (mod p), x = x0 + x1 2^16 + x2 2^32 reduces to
// x0 - x1 + x2 in [-65535, 65536], and one conditional add of p makes it
// canonical (65536 * 65536 = 2^32 gives x0 = x1 = 0, x2 = 1).
static __device__ __forceinline__ uint32_t fmul(uint32_t a, uint32_t b) {
    const uint64_t x = (uint64_t)a * b;
    const uint32_t lo = (uint32_t)x;
    const int32_t r = (int32_t)(lo & 0xffffu) - (int32_t)(lo >> 16) + (int32_t)(x >> 32);
    return (uint32_t)(r < 0 ? r + 0x10001 : r);
}
static __device__ __forceinline__ uint32_t fadd(uint32_t a, uint32_t b) {
    uint32_t r = a + b;
    return r >= 0x10001u ? r - 0x10001u : r;
}
static __device__ __forceinline__ uint32_t fsub(uint32_t a, uint32_t b) {
    uint32_t r = a - b;
    return ((int32_t)r < 0) ? r + 0x10001u : r;
}
static __device__ __forceinline__ uint32_t fneg(uint32_t a) { return a ? 0x10001u - a : 0u; }
// Inverse by Fermat (a^65535) with the reference table's inv(0) == 1
// (galois.hpp:98-101: _exp[65536 - _log[0]] == _exp[65536] == 1).
static __device__ __forceinline__ uint32_t finv(uint32_t a) {
    if (a == 0) return 1u;
    uint32_t t = a;                                // a^1
    uint32_t u = fmul(fmul(t, t), t);              // a^3
    uint32_t v = u;
#pragma unroll
    for (int i = 0; i < 2; ++i) v = fmul(v, v);
    v = fmul(v, u);                                // a^15
    uint32_t w = v;
#pragma unroll
    for (int i = 0; i < 4; ++i) w = fmul(w, w);
    w = fmul(w, v);                                // a^255
    uint32_t z = w;
#pragma unroll
    for (int i = 0; i < 8; ++i) z = fmul(z, z);
    return fmul(z, w);                             // a^65535
}
// div(a, b) == a * inv(b), div(0, b) == 0, div(a, 0) == a (galois.hpp:187-196)
static __device__ __forceinline__ uint32_t fdiv(uint32_t a, uint32_t b) { return a ? fmul(a, finv(b)) : 0u; }

// ---------------------------------------------------------------- warp NTTs

// ct_butterfly (libffrs/ntt.hpp:225-249): RBO input, normal order output
static __device__ void w_ct(const uint32_t *__restrict__ roots, uint32_t *x, uint32_t n, int lane) {
    for (uint32_t stride = 1, ef = n >> 1; stride < n; stride <<= 1, ef >>= 1) {
        for (uint32_t b = lane; b < (n >> 1); b += 32) {
            const uint32_t i = b & (stride - 1);
            const uint32_t j = ((b - i) << 1) + i;
            const uint32_t a = x[j], bb = x[j + stride];
            const uint32_t m = i ? fmul(bb, roots[ef * i]) : bb;
            x[j] = fadd(a, m);
            x[j + stride] = fsub(a, m);
        }
        __syncwarp();
    }
}

// gs_butterfly (libffrs/ntt.hpp:280-302): normal order input, RBO output
static __device__ void w_gs(const uint32_t *__restrict__ roots, uint32_t *x, uint32_t n, int lane) {
    for (uint32_t stride = n >> 1, ef = 0; stride > 0; stride >>= 1, ++ef) {
        for (uint32_t b = lane; b < (n >> 1); b += 32) {
            const uint32_t i = b & (stride - 1);
            const uint32_t j = ((b - i) << 1) + i;
            const uint32_t a = x[j], bb = x[j + stride];
            x[j] = fadd(a, bb);
            const uint32_t d = fsub(a, bb);
            x[j + stride] = i ? fmul(d, roots[i << ef]) : d;
        }
        __syncwarp();
    }
}

static __device__ __forceinline__ void w_nttr(const Rsi16Dev &c, uint32_t *x, int lane) { w_gs(c.roots_ecc, x, c.ecc, lane); }
static __device__ __forceinline__ void w_inttr(const Rsi16Dev &c, uint32_t *x, int lane) {
    w_ct(c.roots_i_ecc, x, c.ecc, lane);
    for (uint32_t k = lane; k < c.ecc; k += 32) x[k] = fmul(x[k], c.ecc_len_i);
    __syncwarp();
}

// NTT::pntt (libffrs/ntt.hpp:133-152) over nchunks chunks, in place; the
// result is x[0 .. ecc).  nchunks == 0 still transforms chunk 0, as the
// reference's pntt_message does when block_len == ecc_len.
static __device__ void w_pntt(const Rsi16Dev &c, uint32_t *x, uint32_t nchunks, int lane) {
    const uint32_t ecc = c.ecc;
    w_ct(c.roots_ecc, x, ecc, lane);
    for (uint32_t k = lane; k < ecc; k += 32) x[k] = fmul(x[k], c.pntt_shift[k]);
    __syncwarp();
    for (uint32_t ch = 1; ch < nchunks; ++ch) {
        uint32_t *p = x + (size_t)ch * ecc;
        w_ct(c.roots_ecc, p, ecc, lane);
        for (uint32_t k = lane; k < ecc; k += 32) {
            const uint32_t v = fmul(p[k], c.pntt_shift[(size_t)ch * ecc + k]);
            p[k] = v;
            x[k] = fadd(x[k], v);
        }
        __syncwarp();
    }
}

// RSi16v::_mix_ecc (libffrs/rsi16v_impl.hpp:100-119)
static __device__ void w_mix(const Rsi16Dev &c, uint32_t *x, int lane) {
    for (uint32_t k = lane; k < c.ecc; k += 32) x[k] = fmul(x[k], c.ecc_mix[k]);
    __syncwarp();
    w_gs(c.roots_i_ecc, x, c.ecc, lane);
}

// NTT::pintt_ecc (libffrs/ntt.hpp:206-220)
static __device__ void w_pintt(const Rsi16Dev &c, uint32_t *b, int lane) {
    const uint32_t ecc = c.ecc, nch = c.block_len / ecc;
    for (uint32_t i = 1; i < nch; ++i) {
        uint32_t *p = b + (size_t)i * ecc;
        for (uint32_t k = lane; k < ecc; k += 32) p[k] = fmul(b[k], c.pintt_shift[(size_t)i * ecc + k]);
        __syncwarp();
        w_gs(c.roots_i_ecc, p, ecc, lane);
    }
    for (uint32_t k = lane; k < ecc; k += 32) b[k] = fmul(b[k], c.pintt_shift[k]);
    __syncwarp();
    w_gs(c.roots_i_ecc, b, ecc, lane);
}

// vec::poly::len for W = 1 (libffrs/simd.hpp:339-361): index of the last
// non-zero word in r[0 .. n), plus one
static __device__ uint32_t w_poly_len(const uint32_t *r, uint32_t n, int lane) {
    uint32_t best = 0;
    for (uint32_t k = lane; k < n; k += 32)
        if (r[k]) best = k + 1;
    return __reduce_max_sync(0xffffffffu, best);
}

static __device__ __forceinline__ bool w_all_zero(const uint32_t *r, uint32_t n, int lane) {
    bool nz = false;
    for (uint32_t k = lane; k < n; k += 32) nz |= (r[k] != 0);
    return !__any_sync(0xffffffffu, nz);
}

static __device__ __forceinline__ void w_copy(uint32_t *dst, const uint32_t *src, uint32_t n, int lane) {
    for (uint32_t k = lane; k < n; k += 32) dst[k] = src[k];
    __syncwarp();
}
static __device__ __forceinline__ void w_fill(uint32_t *dst, uint32_t v, uint32_t n, int lane) {
    for (uint32_t k = lane; k < n; k += 32) dst[k] = v;
    __syncwarp();
}

// in-scratch guard: a length that would make the reference run past its
// scratch buffer is reported as an assertion instead of being executed
struct Scratch {
    uint32_t *base;
    uint32_t size;
    __device__ bool ok(const uint32_t *p, uint32_t n) const {
        return p >= base && (uint64_t)(p - base) + n <= size;
    }
};

enum { ST_OK = 0, ST_ASSERT = -1 };

// NTT::_reverse_ntt_vec (libffrs/ntt.hpp:343-354).  Index i pairs with
// k = rbo_ecc[ecc - rbo_ecc[i]] (an involution on [1, ecc)); the sequential
// loop swaps each pair once at the smaller index and then scales every index
// by its own twiddles, so each pair is handled by one lane here.
static __device__ __forceinline__ uint32_t rev_scale(const Rsi16Dev &c, uint32_t i, uint32_t shift) {
    const uint32_t j = c.rbo_ecc[i];
    return fmul(c.roots_i_ecc[j], c.roots_ecc[(shift * j) & c.ecc_mask]);
}
static __device__ void w_reverse_ntt_vec(const Rsi16Dev &c, uint32_t *v, uint32_t shift, int lane) {
    const uint32_t ecc = c.ecc;
    for (uint32_t i = 1 + lane; i < ecc; i += 32) {
        const uint32_t k = c.rbo_ecc[ecc - c.rbo_ecc[i]];
        if (k < i) continue;
        if (k == i) {
            v[i] = fmul(v[i], rev_scale(c, i, shift));
        } else {
            const uint32_t vi = v[i], vk = v[k];
            v[i] = fmul(vk, rev_scale(c, i, shift));
            v[k] = fmul(vi, rev_scale(c, k, shift));
        }
    }
    __syncwarp();
}

// NTT::poly_inv_mod_xn_rev (libffrs/ntt.hpp:363-469), W = 1
static __device__ int w_poly_inv(const Rsi16Dev &c, const Scratch &s, uint32_t *g, uint32_t g_len, uint32_t g0,
                          uint32_t a_len, uint32_t *a, int lane) {
    const uint32_t ecc = c.ecc;
    const uint32_t a0 = finv(g0);
    w_fill(a, a0, ecc, lane);
    uint32_t l = 2;
    const uint32_t a_max = a_len;
    while (l < a_len) {
        if (g_len + l - 2 > ecc) return ST_ASSERT;
        for (uint32_t k = lane; k < ecc; k += 32) {
            const uint32_t ai = a[k];
            a[k] = fmul(ai, fsub(2, fmul(ai, g[k])));
        }
        __syncwarp();
        w_inttr(c, a, lane);
        if (l > ecc) return ST_ASSERT;
        for (uint32_t k = l + lane; k < ecc; k += 32) a[k] = 0;
        __syncwarp();
        w_nttr(c, a, lane);
        l *= 2;
    }
    for (uint32_t k = lane; k < ecc; k += 32) {
        const uint32_t ai = a[k];
        g[k] = fmul(ai, fsub(2, fmul(ai, g[k])));
    }
    __syncwarp();
    w_inttr(c, a, lane);
    w_inttr(c, g, lane);
    w_copy(a, g, ecc, lane);
    if (l > ecc) return ST_ASSERT;
    for (uint32_t k = l + lane; k < ecc; k += 32) a[k] = 0;
    __syncwarp();
    if (!s.ok(a, a_max)) return ST_ASSERT;
    // std::reverse(&a[0], &a[a_max])
    {
        const uint32_t half = a_max / 2;
        for (uint32_t k = lane; k < half; k += 32) {
            const uint32_t x = a[k], y = a[a_max - 1 - k];
            a[k] = y;
            a[a_max - 1 - k] = x;
        }
        __syncwarp();
    }
    if (a_len > ecc) return ST_ASSERT;
    for (uint32_t k = a_len + lane; k < ecc; k += 32) a[k] = 0;
    __syncwarp();
    w_nttr(c, a, lane);
    return ST_OK;
}

// NTT::poly_div_ntt (libffrs/ntt.hpp:471-564), W = 1
static __device__ int w_poly_div(const Rsi16Dev &c, const Scratch &s, const uint32_t *f, uint32_t f_len, const uint32_t *g,
                          uint32_t g_len, uint32_t f0, uint32_t g0, uint32_t *t, uint32_t *q, uint32_t *q_len_out,
                          int lane) {
    const uint32_t ecc = c.ecc;
    const uint32_t q_len = f_len - g_len + 1;
    if (!(g_len > 0)) return ST_ASSERT;
    if (f_len < g_len) {
        w_fill(q, 0, ecc, lane);
        *q_len_out = 0;
        return ST_OK;
    }
    w_copy(t, g, ecc, lane);
    w_reverse_ntt_vec(c, t, g_len, lane);
    int st = w_poly_inv(c, s, t, g_len, g0, q_len, q, lane);
    if (st) return st;
    for (uint32_t k = lane; k < ecc; k += 32) t[k] = fmul(fsub(f[k], f0), q[k]);
    __syncwarp();
    w_inttr(c, t, lane);
    const uint32_t right_n = min(q_len, ecc - g_len);
    if (!s.ok(t + g_len, right_n) || !s.ok(q, right_n)) return ST_ASSERT;
    if (!s.ok(t, q_len - right_n) || !s.ok(q + right_n, q_len - right_n)) return ST_ASSERT;
    // std::copy_n(&t[g_len], right_n, &q[0]); std::copy_n(&t[0], q_len - right_n, &q[right_n])
    if (q_len <= ecc) {  // q and t are disjoint ecc-word arrays
        for (uint32_t k = lane; k < q_len; k += 32) q[k] = (k < right_n) ? t[g_len + k] : t[k - right_n];
        __syncwarp();
    } else {  // overlapping copies: keep the reference's sequential order
        if (lane == 0) {
            for (uint32_t k = 0; k < right_n; ++k) q[k] = t[g_len + k];
            for (uint32_t k = 0; k < q_len - right_n; ++k) q[right_n + k] = t[k];
        }
        __syncwarp();
    }
    if (q_len > ecc && !s.ok(q, q_len)) return ST_ASSERT;
    for (uint32_t k = q_len + lane; k < ecc; k += 32) q[k] = 0;
    __syncwarp();
    w_nttr(c, q, lane);
    *q_len_out = q_len;
    return ST_OK;
}

// RSi16v::_sugiyama (libffrs/rsi16v_impl.hpp:271-440), W = 1.  a1 = ws + ecc,
// r1 = ws (the syndromes), temp4 = ws + 2 ecc, as in _repair.
static __device__ int w_sugiyama(const Rsi16Dev &c, const Scratch &s, uint32_t *a1, uint32_t *r1, uint32_t *temp4,
                          uint32_t *a1_len_out, int lane) {
    const uint32_t ecc = c.ecc, mask = c.ecc_mask;
    w_fill(temp4, 0, 4 * ecc, lane);
    w_fill(a1, 0, ecc, lane);
    uint32_t a1_len;
    uint32_t q_len = 0, t_len = 0;
    uint32_t *q = temp4, *t = temp4 + ecc, *a2 = temp4 + 2 * ecc, *r2 = temp4 + 3 * ecc;
    uint32_t a2_len = 1;
    w_fill(a2, 1, ecc, lane);
    uint32_t r1_len = w_poly_len(r1, ecc, lane);
    w_copy(r2, r1, ecc, lane);
    uint32_t r2_len = r1_len;
    uint32_t r2l = r2[0];
    const uint32_t lanes = (r1_len != 0) ? 0xffffffffu : 0u;
    {
        const uint32_t r1h = r1[(r1_len - 1) & mask];
        const uint32_t r1h2 = r1[(uint32_t)(r1_len - 2) & mask];
        const uint32_t a11 = fneg(finv(r1h));
        const uint32_t a10 = fmul(r1h2, fmul(a11, a11));
        __syncwarp();
        if (lane == 0) {
            a1[1] = a11;
            a1[0] = a10;
        }
        a1_len = 2 & lanes;
        // r1[i] = a10 * r1[i] (all i), then r1[i] += a11 * r2[i-1] (i >= 1);
        // r2 still holds the original r1, so both updates fuse
        for (uint32_t k = lane; k < ecc; k += 32) {
            uint32_t v = fmul(a10, r1[k]);
            if (k >= 1) v = fadd(v, fmul(a11, r2[k - 1]));
            r1[k] = v;
        }
        __syncwarp();
        r1_len = w_poly_len(r1, ecc - 1, lane) & lanes;
        for (uint32_t k = r1_len + lane; k < ecc; k += 32) r1[k] = 0;
        __syncwarp();
        w_nttr(c, a1, lane);
        w_nttr(c, r2, lane);
    }
    uint32_t cond = (r1_len >= ecc / 2) ? 0xffffffffu : 0u;
    if (cond) {
        for (uint32_t it = 1; it < ecc / 2; ++it) {
            const uint32_t r1h = r1[(r1_len - 1) & mask];
            const uint32_t r1l = r1[0];
            __syncwarp();
            w_nttr(c, r1, lane);
            int st = w_poly_div(c, s, r2, r2_len & cond, r1, r1_len, r2l, r1h, t, q, &q_len, lane);
            if (st) return st;
            // t = q * a1; q = q * r1; t = a2 - t; q = r2 - q  (pointwise, fused)
            for (uint32_t k = lane; k < ecc; k += 32) {
                const uint32_t qk = q[k];
                t[k] = fsub(a2[k], fmul(qk, a1[k]));
                q[k] = fsub(r2[k], fmul(qk, r1[k]));
            }
            __syncwarp();
            t_len = q_len + a1_len - 1;
            t_len = a2_len > t_len ? a2_len : t_len;
            uint32_t ql = q_len + r1_len - 1;
            q_len = r2_len > ql ? r2_len : ql;
            w_copy(a2, a1, ecc, lane);
            a2_len = a1_len;
            w_copy(r2, r1, ecc, lane);
            r2_len = r1_len;
            r2l = r1l;
            cond = (r1_len >= ecc / 2) ? 0xffffffffu : 0u;
            if (!cond) {
                w_inttr(c, r1, lane);
                break;
            }
            w_copy(a1, t, ecc, lane);
            w_copy(r1, q, ecc, lane);
            a1_len = t_len;
            r1_len = q_len;
            w_inttr(c, r1, lane);
            if (!s.ok(r1, r1_len & cond)) return ST_ASSERT;
            r1_len = w_poly_len(r1, r1_len & cond, lane);
        }
    }
    w_inttr(c, a1, lane);
    if (!s.ok(a1, a1_len & lanes)) return ST_ASSERT;
    a1_len = w_poly_len(a1, a1_len & lanes, lane);
    const uint32_t a10i = finv(a1[0]);
    __syncwarp();
    for (uint32_t k = lane; k < ecc; k += 32) {
        a1[k] = fmul(a1[k], a10i);
        r1[k] = fmul(r1[k], a10i);
    }
    __syncwarp();
    *a1_len_out = a1_len & lanes;
    return ST_OK;
}

static __device__ __forceinline__ uint32_t eval_poly(const uint32_t *r, uint32_t n, uint32_t x) {
    uint32_t sum = 0;
    for (uint32_t i = n; i-- > 0;) sum = fadd(fmul(sum, x), r[i]);
    return sum;
}

// ---------------------------------------------------------------- block I/O

static __device__ __forceinline__ uint32_t ld_word(const void *base, bool w16, size_t idx) {
    return w16 ? (uint32_t)((const uint16_t *)base)[idx] : ((const uint32_t *)base)[idx];
}
static __device__ __forceinline__ void st_word(void *base, bool w16, size_t idx, uint32_t v) {
    if (w16)
        ((uint16_t *)base)[idx] = (uint16_t)v;
    else
        ((uint32_t *)base)[idx] = v;
}

// block b -> ws[0 .. block_len): message words then parity words (or zeros)
static __device__ void w_gather(const Rsi16Dev &c, const BlockView &v, size_t b, uint32_t *ws, bool with_parity, int lane) {
    for (uint32_t k = lane; k < c.message_len; k += 32)
        ws[k] = ld_word(v.msg, v.msg16, v.moff(b, k));
    for (uint32_t k = lane; k < c.ecc; k += 32)
        ws[c.message_len + k] = with_parity ? ld_word(v.par, v.par16, v.poff(b, k)) : 0u;
    __syncwarp();
}

static __device__ __forceinline__ void put_pos(const Rsi16Dev &c, const BlockView &v, size_t b, uint32_t pos, uint32_t val) {
    if (pos < c.message_len)
        st_word(v.msg, v.msg16, v.moff(b, pos), val);
    else
        st_word(v.par, v.par16, v.poff(b, pos - c.message_len), val);
}
static __device__ __forceinline__ uint32_t get_pos(const Rsi16Dev &c, const BlockView &v, size_t b, uint32_t pos) {
    if (pos < c.message_len) return ld_word(v.msg, v.msg16, v.moff(b, pos));
    return ld_word(v.par, v.par16, v.poff(b, pos - c.message_len));
}

// ---------------------------------------------------------------- register NTTs
//
// For ecc = 32 * EPL (EPL = 1, 2, 4) a warp keeps one ecc-point vector in
// registers: lane L holds elements e = L * EPL + h.  Butterfly partners closer
// than EPL are in the same lane, the others in lane L ^ (stride / EPL) (one
// shuffle).  The butterflies are the reference's ct_butterfly / gs_butterfly
// (ntt.hpp:225-302) with the twiddle of each element preloaded per stage;
// the twiddle of index 0 is 1, and fmul(x, 1) == x, so every element takes
// the same path.

template <int EPL>
struct RegTw {
    uint32_t ct[7][EPL];  // roots_ecc[ef * (e & (stride - 1))], stride = 1, 2, ...
    uint32_t gs[7][EPL];  // roots_i_ecc[(e & (stride - 1)) << ef], stride = n/2, n/4, ...
};

// log2 of the register-transform length 32 * EPL
template <int EPL>
constexpr int reg_log() {
    return EPL == 1 ? 5 : (EPL == 2 ? 6 : 7);
}

// (every stage loop below has one constant trip count, so that it unrolls
// completely and the twiddle arrays stay in registers)
template <int EPL>
static __device__ __forceinline__ void reg_twiddles(const Rsi16Dev &c, int lane, RegTw<EPL> &tw) {
    constexpr int LOG = reg_log<EPL>();
    constexpr uint32_t n = 32 * EPL;
#pragma unroll
    for (int st = 0; st < LOG; ++st) {
        const uint32_t stride = 1u << st, ef = (n >> 1) >> st;
#pragma unroll
        for (int h = 0; h < EPL; ++h) tw.ct[st][h] = c.roots_ecc[ef * ((lane * EPL + h) & (stride - 1))];
    }
#pragma unroll
    for (int st = 0; st < LOG; ++st) {
        const uint32_t stride = (n >> 1) >> st, ef = (uint32_t)st;
#pragma unroll
        for (int h = 0; h < EPL; ++h) tw.gs[st][h] = c.roots_i_ecc[((lane * EPL + h) & (stride - 1)) << ef];
    }
}

// ct_butterfly on registers: RBO input, normal order output
template <int EPL>
static __device__ __forceinline__ void reg_ct(uint32_t (&x)[EPL], const RegTw<EPL> &tw, int lane) {
    constexpr int LOG = reg_log<EPL>();
#pragma unroll
    for (int st = 0; st < LOG; ++st) {
        const int stride = 1 << st;
        if (stride < EPL) {
#pragma unroll
            for (int h = 0; h < EPL; ++h) {
                if (h & stride) continue;
                const uint32_t a = x[h], m = fmul(x[h + stride], tw.ct[st][h]);
                x[h] = fadd(a, m);
                x[h + stride] = fsub(a, m);
            }
        } else {
            const int lm = stride / EPL;
            const bool upper = (lane & lm) != 0;
#pragma unroll
            for (int h = 0; h < EPL; ++h) {
                const uint32_t p = __shfl_xor_sync(0xffffffffu, x[h], lm);
                const uint32_t m = fmul(upper ? x[h] : p, tw.ct[st][h]);
                x[h] = upper ? fsub(p, m) : fadd(x[h], m);
            }
        }
    }
}

// gs_butterfly on registers: normal order input, RBO output
template <int EPL>
static __device__ __forceinline__ void reg_gs(uint32_t (&x)[EPL], const RegTw<EPL> &tw, int lane) {
    constexpr int LOG = reg_log<EPL>();
    constexpr int n = 32 * EPL;
#pragma unroll
    for (int st = 0; st < LOG; ++st) {
        const int stride = (n >> 1) >> st;
        if (stride < EPL) {
#pragma unroll
            for (int h = 0; h < EPL; ++h) {
                if (h & stride) continue;
                const uint32_t a = x[h], bb = x[h + stride];
                x[h] = fadd(a, bb);
                x[h + stride] = fmul(fsub(a, bb), tw.gs[st][h + stride]);
            }
        } else {
            const int lm = stride / EPL;
            const bool upper = (lane & lm) != 0;
#pragma unroll
            for (int h = 0; h < EPL; ++h) {
                const uint32_t p = __shfl_xor_sync(0xffffffffu, x[h], lm);
                x[h] = upper ? fmul(fsub(p, x[h]), tw.gs[st][h]) : fadd(x[h], p);
            }
        }
    }
}

// gs_butterfly on two vectors at once
template <int EPL>
static __device__ __forceinline__ void reg_gs2(uint32_t (&x)[EPL], uint32_t (&y)[EPL], const RegTw<EPL> &tw,
                                               int lane) {
    constexpr int LOG = reg_log<EPL>();
    constexpr int n = 32 * EPL;
#pragma unroll
    for (int st = 0; st < LOG; ++st) {
        const int stride = (n >> 1) >> st;
        if (stride < EPL) {
#pragma unroll
            for (int h = 0; h < EPL; ++h) {
                if (h & stride) continue;
                const uint32_t a = x[h], bb = x[h + stride];
                const uint32_t a2 = y[h], bb2 = y[h + stride];
                x[h] = fadd(a, bb);
                x[h + stride] = fmul(fsub(a, bb), tw.gs[st][h + stride]);
                y[h] = fadd(a2, bb2);
                y[h + stride] = fmul(fsub(a2, bb2), tw.gs[st][h + stride]);
            }
        } else {
            const int lm = stride / EPL;
            const bool upper = (lane & lm) != 0;
#pragma unroll
            for (int h = 0; h < EPL; ++h) {
                const uint32_t p = __shfl_xor_sync(0xffffffffu, x[h], lm);
                const uint32_t p2 = __shfl_xor_sync(0xffffffffu, y[h], lm);
                x[h] = upper ? fmul(fsub(p, x[h]), tw.gs[st][h]) : fadd(x[h], p);
                y[h] = upper ? fmul(fsub(p2, y[h]), tw.gs[st][h]) : fadd(y[h], p2);
            }
        }
    }
}

// NTT::pntt (ntt.hpp:133-152) of block b over nchunks chunks (at least chunk
// 0): S = sum_ch ct(chunk_ch) * pntt_shift_ch.  Words past the message are the
// parity (with_parity) or zeros.
template <int EPL>
static __device__ __forceinline__ void reg_pntt(const Rsi16Dev &c, const BlockView &v, size_t b, uint32_t nchunks,
                                                bool with_parity, const RegTw<EPL> &tw, int lane,
                                                uint32_t (&acc)[EPL]) {
    constexpr uint32_t n = 32 * EPL;
    const size_t mb = (b / v.group) * v.msg_gstride + (b % v.group) * v.msg_bstride;
    const size_t pb = (b / v.group) * v.par_gstride + (b % v.group) * v.par_bstride;
    const uint32_t nch = nchunks ? nchunks : 1;
    for (uint32_t ch = 0; ch < nch; ++ch) {
        uint32_t x[EPL];
#pragma unroll
        for (int h = 0; h < EPL; ++h) {
            const uint32_t k = ch * n + lane * EPL + h;
            uint32_t w = 0;
            if (k < c.message_len)
                w = ld_word(v.msg, v.msg16, mb + (size_t)k * v.msg_estride);
            else if (with_parity && k < c.block_len)
                w = ld_word(v.par, v.par16, pb + (size_t)(k - c.message_len) * v.par_estride);
            x[h] = w;
        }
        reg_ct<EPL>(x, tw, lane);
#pragma unroll
        for (int h = 0; h < EPL; ++h) {
            const uint32_t y = fmul(x[h], c.pntt_shift[ch * n + lane * EPL + h]);
            acc[h] = ch ? fadd(acc[h], y) : y;
        }
    }
}

// ct_butterfly on two vectors at once (twice the independent work per stage)
template <int EPL>
static __device__ __forceinline__ void reg_ct2(uint32_t (&x)[EPL], uint32_t (&y)[EPL], const RegTw<EPL> &tw,
                                               int lane) {
    constexpr int LOG = reg_log<EPL>();
#pragma unroll
    for (int st = 0; st < LOG; ++st) {
        const int stride = 1 << st;
        if (stride < EPL) {
#pragma unroll
            for (int h = 0; h < EPL; ++h) {
                if (h & stride) continue;
                const uint32_t a = x[h], m = fmul(x[h + stride], tw.ct[st][h]);
                const uint32_t a2 = y[h], m2 = fmul(y[h + stride], tw.ct[st][h]);
                x[h] = fadd(a, m);
                x[h + stride] = fsub(a, m);
                y[h] = fadd(a2, m2);
                y[h + stride] = fsub(a2, m2);
            }
        } else {
            const int lm = stride / EPL;
            const bool upper = (lane & lm) != 0;
#pragma unroll
            for (int h = 0; h < EPL; ++h) {
                const uint32_t p = __shfl_xor_sync(0xffffffffu, x[h], lm);
                const uint32_t p2 = __shfl_xor_sync(0xffffffffu, y[h], lm);
                const uint32_t m = fmul(upper ? x[h] : p, tw.ct[st][h]);
                const uint32_t m2 = fmul(upper ? y[h] : p2, tw.ct[st][h]);
                x[h] = upper ? fsub(p, m) : fadd(x[h], m);
                y[h] = upper ? fsub(p2, m2) : fadd(y[h], m2);
            }
        }
    }
}

// reg_pntt of two blocks b0, b1 of the same view at once
template <int EPL>
static __device__ __forceinline__ void reg_pntt2(const Rsi16Dev &c, const BlockView &v, size_t b0, size_t b1,
                                                 uint32_t nchunks, bool with_parity, const RegTw<EPL> &tw,
                                                 int lane, uint32_t (&acc0)[EPL], uint32_t (&acc1)[EPL]) {
    constexpr uint32_t n = 32 * EPL;
    const size_t mb0 = (b0 / v.group) * v.msg_gstride + (b0 % v.group) * v.msg_bstride;
    const size_t pb0 = (b0 / v.group) * v.par_gstride + (b0 % v.group) * v.par_bstride;
    const size_t mb1 = (b1 / v.group) * v.msg_gstride + (b1 % v.group) * v.msg_bstride;
    const size_t pb1 = (b1 / v.group) * v.par_gstride + (b1 % v.group) * v.par_bstride;
    const uint32_t nch = nchunks ? nchunks : 1;
    for (uint32_t ch = 0; ch < nch; ++ch) {
        uint32_t x[EPL], y[EPL];
#pragma unroll
        for (int h = 0; h < EPL; ++h) {
            const uint32_t k = ch * n + lane * EPL + h;
            uint32_t w0 = 0, w1 = 0;
            if (k < c.message_len) {
                w0 = ld_word(v.msg, v.msg16, mb0 + (size_t)k * v.msg_estride);
                w1 = ld_word(v.msg, v.msg16, mb1 + (size_t)k * v.msg_estride);
            } else if (with_parity && k < c.block_len) {
                w0 = ld_word(v.par, v.par16, pb0 + (size_t)(k - c.message_len) * v.par_estride);
                w1 = ld_word(v.par, v.par16, pb1 + (size_t)(k - c.message_len) * v.par_estride);
            }
            x[h] = w0;
            y[h] = w1;
        }
        reg_ct2<EPL>(x, y, tw, lane);
#pragma unroll
        for (int h = 0; h < EPL; ++h) {
            const uint32_t sh = c.pntt_shift[ch * n + lane * EPL + h];
            const uint32_t r0 = fmul(x[h], sh), r1 = fmul(y[h], sh);
            acc0[h] = ch ? fadd(acc0[h], r0) : r0;
            acc1[h] = ch ? fadd(acc1[h], r1) : r1;
        }
    }
}

// parity of blocks b0 and b1 at once (b1 == b0 is allowed)
template <int EPL>
static __device__ __forceinline__ void rsi16_encode_pair_reg(const Rsi16Dev &c, const BlockView &v, size_t b0,
                                                             size_t b1, const RegTw<EPL> &tw, int lane) {
    uint32_t a0[EPL], a1[EPL];
    reg_pntt2<EPL>(c, v, b0, b1, c.pntt_blocks - 1, false, tw, lane, a0, a1);
#pragma unroll
    for (int h = 0; h < EPL; ++h) {
        const uint32_t m = c.ecc_mix[lane * EPL + h];
        a0[h] = fmul(a0[h], m);
        a1[h] = fmul(a1[h], m);
    }
    reg_gs2<EPL>(a0, a1, tw, lane);
    const size_t p0 = (b0 / v.group) * v.par_gstride + (b0 % v.group) * v.par_bstride;
    const size_t p1 = (b1 / v.group) * v.par_gstride + (b1 % v.group) * v.par_bstride;
#pragma unroll
    for (int h = 0; h < EPL; ++h) {
        st_word(v.par, v.par16, p0 + (size_t)(lane * EPL + h) * v.par_estride, a0[h]);
        st_word(v.par, v.par16, p1 + (size_t)(lane * EPL + h) * v.par_estride, a1[h]);
    }
}

// parity of block b with the vector in registers
template <int EPL>
static __device__ __forceinline__ void rsi16_encode_block_reg(const Rsi16Dev &c, const BlockView &v, size_t b,
                                                              const RegTw<EPL> &tw, int lane) {
    uint32_t acc[EPL];
    reg_pntt<EPL>(c, v, b, c.pntt_blocks - 1, false, tw, lane, acc);
#pragma unroll
    for (int h = 0; h < EPL; ++h) acc[h] = fmul(acc[h], c.ecc_mix[lane * EPL + h]);
    reg_gs<EPL>(acc, tw, lane);
    const size_t pb = (b / v.group) * v.par_gstride + (b % v.group) * v.par_bstride;
#pragma unroll
    for (int h = 0; h < EPL; ++h) st_word(v.par, v.par16, pb + (size_t)(lane * EPL + h) * v.par_estride, acc[h]);
}

// ---------------------------------------------------------------- sub-warp register NTTs
//
// For ecc = N < 32 (N = 2, 4, 8, 16) a warp transforms 32 / N blocks at once:
// lane L holds element e = L % N of the block in slot L / N.  Every butterfly
// partner is lane L ^ stride with stride < N, inside the slot's N lanes, so
// one shuffle per stage serves every slot.  Twiddles as in RegTw with
// EPL = 1 over an N-point transform.

template <int N>
constexpr int sub_log() {
    return N == 2 ? 1 : (N == 4 ? 2 : (N == 8 ? 3 : 4));
}

template <int N>
struct SubTw {
    uint32_t ct[sub_log<N>()];
    uint32_t gs[sub_log<N>()];
};

template <int N>
static __device__ __forceinline__ void sub_twiddles(const Rsi16Dev &c, int e, SubTw<N> &tw) {
    constexpr int LOG = sub_log<N>();
#pragma unroll
    for (int st = 0; st < LOG; ++st) {
        const uint32_t stride = 1u << st, ef = (uint32_t)(N >> 1) >> st;
        tw.ct[st] = c.roots_ecc[ef * ((uint32_t)e & (stride - 1))];
    }
#pragma unroll
    for (int st = 0; st < LOG; ++st) {
        const uint32_t stride = (uint32_t)(N >> 1) >> st;
        tw.gs[st] = c.roots_i_ecc[((uint32_t)e & (stride - 1)) << st];
    }
}

// ct_butterfly of each slot's vector: RBO input, normal order output
template <int N>
static __device__ __forceinline__ uint32_t sub_ct(uint32_t x, const SubTw<N> &tw, int e) {
    constexpr int LOG = sub_log<N>();
#pragma unroll
    for (int st = 0; st < LOG; ++st) {
        const int stride = 1 << st;
        const bool upper = (e & stride) != 0;
        const uint32_t p = __shfl_xor_sync(0xffffffffu, x, stride);
        const uint32_t m = fmul(upper ? x : p, tw.ct[st]);
        x = upper ? fsub(p, m) : fadd(x, m);
    }
    return x;
}

// gs_butterfly of each slot's vector: normal order input, RBO output
template <int N>
static __device__ __forceinline__ uint32_t sub_gs(uint32_t x, const SubTw<N> &tw, int e) {
    constexpr int LOG = sub_log<N>();
#pragma unroll
    for (int st = 0; st < LOG; ++st) {
        const int stride = (N >> 1) >> st;
        const bool upper = (e & stride) != 0;
        const uint32_t p = __shfl_xor_sync(0xffffffffu, x, stride);
        x = upper ? fmul(fsub(p, x), tw.gs[st]) : fadd(x, p);
    }
    return x;
}

// NTT::pntt (ntt.hpp:133-152) of the block b in this lane's slot over nchunks
// chunks (at least chunk 0); element e of the result.  act false: the slot
// has no block (zeros, no loads; its lanes still take part in the shuffles).
template <int N>
static __device__ __forceinline__ uint32_t sub_pntt(const Rsi16Dev &c, const BlockView &v, size_t b, bool act,
                                                    uint32_t nchunks, bool with_parity, const SubTw<N> &tw, int e) {
    const size_t mb = (b / v.group) * v.msg_gstride + (b % v.group) * v.msg_bstride;
    const size_t pb = (b / v.group) * v.par_gstride + (b % v.group) * v.par_bstride;
    const uint32_t nch = nchunks ? nchunks : 1;
    uint32_t acc = 0;
#pragma unroll 2
    for (uint32_t ch = 0; ch < nch; ++ch) {
        const uint32_t k = ch * N + (uint32_t)e;
        uint32_t w = 0;
        if (act) {
            if (k < c.message_len)
                w = ld_word(v.msg, v.msg16, mb + (size_t)k * v.msg_estride);
            else if (with_parity && k < c.block_len)
                w = ld_word(v.par, v.par16, pb + (size_t)(k - c.message_len) * v.par_estride);
        }
        w = sub_ct<N>(w, tw, e);
        const uint32_t y = fmul(w, c.pntt_shift[k]);
        acc = ch ? fadd(acc, y) : y;
    }
    return acc;
}

// parity of the 32 / N blocks b0 .. b0 + 32/N - 1 (those below nblocks) on
// the sub-warp transforms
template <int N>
static __device__ __forceinline__ void rsi16_encode_sub_pass(const Rsi16Dev &c, const BlockView &v, size_t b0,
                                                             size_t nblocks, const SubTw<N> &tw, int lane) {
    const int e = lane % N, s = lane / N;
    const size_t b = b0 + s;
    const bool act = b < nblocks;
    uint32_t a = sub_pntt<N>(c, v, act ? b : b0, act, c.pntt_blocks - 1, false, tw, e);
    a = sub_gs<N>(fmul(a, c.ecc_mix[e]), tw, e);
    if (act) {
        const size_t pb = (b / v.group) * v.par_gstride + (b % v.group) * v.par_bstride;
        st_word(v.par, v.par16, pb + (size_t)e * v.par_estride, a);
    }
}

// Syndromes (NTT::pntt over every chunk) of the one block b into
// out[0 .. N) for ecc = N < 32: the warp's 32/N slots take every (32/N)-th
// chunk on the sub-warp transforms and their sums are added (exact mod p, so
// the order does not matter).
template <int N>
static __device__ __forceinline__ void sub_synd_one(const Rsi16Dev &c, const BlockView &v, size_t b, uint32_t *out,
                                                    int lane) {
    constexpr int G = 32 / N;
    const int e = lane % N, s = lane / N;
    SubTw<N> tw;
    sub_twiddles<N>(c, e, tw);
    const size_t mb = (b / v.group) * v.msg_gstride + (b % v.group) * v.msg_bstride;
    const size_t pb = (b / v.group) * v.par_gstride + (b % v.group) * v.par_bstride;
    const uint32_t nch = c.pntt_blocks ? c.pntt_blocks : 1;
    uint32_t acc = 0;
    for (uint32_t base = 0; base < nch; base += G) {
        const uint32_t ch = base + (uint32_t)s;
        const uint32_t k = ch * N + (uint32_t)e;
        uint32_t w = 0;
        if (ch < nch) {
            if (k < c.message_len)
                w = ld_word(v.msg, v.msg16, mb + (size_t)k * v.msg_estride);
            else if (k < c.block_len)
                w = ld_word(v.par, v.par16, pb + (size_t)(k - c.message_len) * v.par_estride);
        }
        w = sub_ct<N>(w, tw, e);
        if (ch < nch) acc = fadd(acc, fmul(w, c.pntt_shift[k]));
    }
#pragma unroll
    for (int o = N; o < 32; o <<= 1) acc = fadd(acc, __shfl_xor_sync(0xffffffffu, acc, o));
    if (lane < N) out[lane] = acc;
    __syncwarp();
}

// Roots of C (degree L) for ecc = N < 32: the inverse partial NTT
// (pintt_ecc, ntt.hpp:206-220) of every chunk on the sub-warp transforms,
// slot s taking chunks s, s + 32/N, ...; the positions i = chunk * N + e with
// a zero go to T in increasing order (at most n1 kept).  Returns their count.
template <int N>
static __device__ __forceinline__ uint32_t sub_roots(const Rsi16Dev &c, const uint32_t *C, uint32_t L, uint32_t *T,
                                                     uint32_t n1, int lane) {
    constexpr int G = 32 / N;
    const int e = lane % N, s = lane / N;
    SubTw<N> tw;
    sub_twiddles<N>(c, e, tw);
    const uint32_t cr = (uint32_t)e <= L ? C[e] : 0u;
    const uint32_t nch = c.block_len / N;
    uint32_t count = 0;
    for (uint32_t base = 0; base < nch; base += G) {
        const uint32_t ch = base + (uint32_t)s;
        uint32_t x = ch < nch ? fmul(cr, c.pintt_shift[ch * N + (uint32_t)e]) : 1u;
        x = sub_gs<N>(x, tw, e);
        const bool hit = ch < nch && x == 0;
        const uint32_t msk = __ballot_sync(0xffffffffu, hit);
        const uint32_t at = count + __popc(msk & ((1u << lane) - 1u));
        if (hit && at < n1) T[at] = ch * N + (uint32_t)e;
        count += __popc(msk);
    }
    return count;
}

// Syndromes of block b into temp[0 .. ecc) on one warp: the sub-warp
// transforms for ecc 2..16, the block gathered into temp and the
// shared-memory transforms otherwise.
static __device__ __forceinline__ void w_synd_block(const Rsi16Dev &c, const BlockView &v, size_t b, uint32_t *temp,
                                                    int lane) {
    switch (c.ecc) {
        case 2: sub_synd_one<2>(c, v, b, temp, lane); return;
        case 4: sub_synd_one<4>(c, v, b, temp, lane); return;
        case 8: sub_synd_one<8>(c, v, b, temp, lane); return;
        case 16: sub_synd_one<16>(c, v, b, temp, lane); return;
        default:
            w_gather(c, v, b, temp, true, lane);
            w_pntt(c, temp, c.pntt_blocks, lane);
            return;
    }
}

// ---------------------------------------------------------------- one block per warp

// parity of block b (ws: block_len words)
static __device__ __forceinline__ void rsi16_encode_block(const Rsi16Dev &c, const BlockView &v, size_t b, uint32_t *ws,
                                                   int lane) {
    w_gather(c, v, b, ws, false, lane);
    w_pntt(c, ws, c.pntt_blocks - 1, lane);
    w_mix(c, ws, lane);
    for (uint32_t k = lane; k < c.ecc; k += 32) st_word(v.par, v.par16, v.poff(b, k), ws[k]);
    __syncwarp();
}

// syndromes of block b (NTT::pntt over every chunk) into out[0 .. ecc)
static __device__ __forceinline__ void rsi16_synd_block(const Rsi16Dev &c, const BlockView &v, size_t b, uint32_t *ws,
                                                        uint32_t *out, int lane) {
    w_gather(c, v, b, ws, true, lane);
    w_pntt(c, ws, c.pntt_blocks, lane);
    for (uint32_t k = lane; k < c.ecc; k += 32) out[k] = ws[k];
    __syncwarp();
}

// RSi16v::_repair, unknown locations (rsi16v_impl.hpp:122-168) with
// _find_roots_ntt (:443-497) and _forney (:500-512); temp: temp_len + 1 words
static __device__ __noinline__ void rsi16_repair_block(const Rsi16Dev &c, const BlockView &v, size_t b, uint32_t *temp,
                                                uint8_t *status, int lane) {
    const uint32_t ecc = c.ecc;
    Scratch s{temp, c.temp_len};

    w_gather(c, v, b, temp, true, lane);
    w_pntt(c, temp, c.pntt_blocks, lane);
    if (w_all_zero(temp, ecc, lane)) {
        if (lane == 0) status[b] = FFGPU_NO_ERRORS;
        return;
    }
    uint32_t *evaluator = temp, *locator = temp + ecc;
    uint32_t loc_len = 0;
    int st = w_sugiyama(c, s, locator, evaluator, temp + 2 * ecc, &loc_len, lane);
    if (st || loc_len > ecc) {
        if (lane == 0) status[b] = FFGPU_STATUS_ASSERT;
        __syncwarp();
        return;
    }
    const uint32_t ev_len = ecc - loc_len + 1;
    uint32_t *deriv = temp + 2 * ecc;
    // _deriv (rsi16v_impl.hpp:608-616)
    for (uint32_t k = lane; k < ecc; k += 32) deriv[k] = (k + 1 < ecc) ? fmul(locator[k + 1], k + 1) : 0u;
    __syncwarp();
    const uint32_t deriv_len = w_poly_len(deriv, ecc, lane);
    uint32_t *roots = temp + 3 * ecc;
    for (uint32_t k = lane; k < c.ntt_len; k += 32) roots[k] = (k < ecc) ? locator[k] : 0u;
    __syncwarp();
    w_pintt(c, roots, lane);
    const bool lanes = loc_len != 0;
    const uint32_t dl = lanes ? deriv_len : 0u, el = lanes ? ev_len : 0u;
    uint32_t count = 0;
    for (uint32_t i0 = 0; i0 < c.block_len; i0 += 32) {
        const uint32_t i = i0 + lane;
        const bool hit = lanes && i < c.block_len && roots[i] == 0;
        count += __popc(__ballot_sync(0xffffffffu, hit));
    }
    // second pass: apply corrections (kept separate so the count is final first)
    for (uint32_t i = lane; i < c.block_len; i += 32) {
        if (!(lanes && roots[i] == 0)) continue;
        uint16_t bb = (uint16_t)i;
        bb = (uint16_t)(((bb >> 1) & 0x5555) | ((bb & 0x5555) << 1));
        bb = (uint16_t)(((bb >> 2) & 0x3333) | ((bb & 0x3333) << 2));
        bb = (uint16_t)(((bb >> 4) & 0x0f0f) | ((bb & 0x0f0f) << 4));
        bb = (uint16_t)((bb >> 8) | (bb << 8));
        const uint32_t x = c.roots_ntt[(uint32_t)(bb >> c.rbo_shift)];
        const uint32_t xi = finv(x);
        const uint32_t num = eval_poly(evaluator, el, xi);
        const uint32_t den = eval_poly(deriv, dl, xi);
        const uint32_t err = fmul(fdiv(num, den), x);
        put_pos(c, v, b, i, fadd(get_pos(c, v, b, i), err));
    }
    __syncwarp();
    if (lane == 0)
        status[b] = count > 0 ? FFGPU_REPAIR_OK : (lanes ? FFGPU_ERROR_LOCATION_FAIL : FFGPU_NO_ERRORS);
}

// When the bounded-distance path may stand in for the reference.  The
// reference's key-equation solver (RSi16v::_sugiyama, rsi16v_impl.hpp:271-440)
// runs the Euclidean algorithm on x^ecc and S(x) = sum_j S_j x^j in the NTT
// domain, and takes every quotient to have degree one: its first step forms
// Q = x^ecc // S(x) from the two top coefficients of S (rsi16v_impl.hpp:
// 313-320), and its later divisions and products (NTT::poly_div_ntt,
// ntt.hpp:471-564) alias in the cyclic NTT domain once a quotient is longer.
// On such a block it returns a wrong locator -- typically with no root at
// all, ErrorLocationFail -- although the errors are within the code's
// capacity, and its bytes and status are only reproduced by the
// step-for-step mirror.  All quotients of that Euclidean run have degree one
// exactly when Berlekamp-Massey on the reversed sequence S_{ecc-1}, ...,
// S_0 is normal: its length grows by one at every even step until it reaches
// its final value (no zero discrepancy at an even step before that).  The
// bounded-distance path accepts a block only then.
//
// Warp-wide Berlekamp-Massey over the syndromes S (forward: S_0 first;
// reverse: S_{ecc-1} first) on the buffers C, B, T of n1 words; returns L,
// C receives the connection polynomial, `normal` the check above (meaningful
// for the reverse run).
static __device__ uint32_t w_bm(const Rsi16Dev &c, const uint32_t *S, uint32_t *&C, uint32_t *&B, uint32_t *&T,
                                uint32_t n1, uint32_t ecc, bool reverse, bool &normal, int lane) {
    for (uint32_t k = lane; k < n1; k += 32) {
        C[k] = k == 0;
        B[k] = k == 0;
    }
    __syncwarp();
    uint32_t L = 0, m = 1, binv = 1;
    bool stalled = false, abnormal = false;
    for (uint32_t n = 0; n < ecc; ++n) {
        // discrepancy d = sum_{i <= L} C_i S_{n-i} (reverse: S_{ecc-1-(n-i)})
        uint32_t acc = 0;
        for (uint32_t i = lane; i <= L && i <= n; i += 32)
            acc += fmul(C[i], reverse ? S[ecc - 1 - (n - i)] : S[n - i]);
        acc = __reduce_add_sync(0xffffffffu, acc) % 0x10001u;
        const uint32_t d = acc;
        if (d == 0) {
            if (!(n & 1) && 2 * L <= n) stalled = true;
            ++m;
            continue;
        }
        const uint32_t coef = fmul(d, binv);
        const bool grow = 2 * L <= n;
        if (grow) {
            abnormal |= stalled;
            for (uint32_t k = lane; k < n1; k += 32) T[k] = C[k];
            __syncwarp();
        }
        for (uint32_t k = lane; k < n1; k += 32)
            if (k >= m) C[k] = fsub(C[k], fmul(coef, B[k - m]));
        __syncwarp();
        if (grow) {
            uint32_t *x = B;
            B = T;
            T = x;
            L = n + 1 - L;
            binv = c.inv_tab[d];
            m = 1;
        } else {
            ++m;
        }
    }
    normal = !abnormal && L > 0 && L <= ecc / 2;
    return L;
}

// Bounded-distance repair of block b by Berlekamp-Massey, for the blocks whose
// error pattern has weight at most t = ecc/2.  The syndromes are the
// reference's (first ecc outputs of the partial NTT: S_j = sum_i r_i X_i^j,
// X_i = w^rbo(i)).  When BM returns a connection polynomial C of length
// L <= t that has exactly L roots X_i^-1 among the block positions, there is
// exactly one error pattern of weight <= t with these syndromes, and every
// correct bounded-distance decoder returns it: the corrections block[i] +=
// X_i Omega(X_i^-1) / C'(X_i^-1) and RepairOk.  The reference's NTT-domain
// Sugiyama is such a decoder only on the blocks w_bm calls normal; the path
// accepts no other block.  Returns false (block untouched) otherwise; the
// caller then runs the reference's algorithm step for step.
// temp: ntt_len + 6 * ecc words.
template <int EPL>
static __device__ __noinline__ bool rsi16_repair_bm_block_t(const Rsi16Dev &c, const BlockView &v, size_t b,
                                                           uint32_t *temp, uint8_t *status,
                                                           const RegTw<EPL ? EPL : 1> &tw, int lane) {
    const uint32_t ecc = c.ecc, t = ecc / 2, n1 = ecc + 1;
    uint32_t *S = temp;
    if constexpr (EPL > 0) {
        uint32_t s[EPL];
        reg_pntt<EPL>(c, v, b, c.pntt_blocks, true, tw, lane, s);
        bool nz = false;
#pragma unroll
        for (int h = 0; h < EPL; ++h) {
            S[lane * EPL + h] = s[h];
            nz |= s[h] != 0;
        }
        __syncwarp();
        if (!__any_sync(0xffffffffu, nz)) {
            if (lane == 0) status[b] = FFGPU_NO_ERRORS;
            return true;
        }
    } else {
        w_synd_block(c, v, b, temp, lane);
        if (w_all_zero(S, ecc, lane)) {
            if (lane == 0) status[b] = FFGPU_NO_ERRORS;
            return true;
        }
    }
    uint32_t *C = temp + ecc, *B = C + n1, *T = B + n1;
    // Berlekamp-Massey on the reversed syndromes: the reference's solver is
    // exact on this block only when that run is normal (w_bm), and its
    // connection polynomial, read backwards, is the locator up to a scalar
    // (the roots and Omega / C' do not depend on the scalar)
    bool normal = false;
    uint32_t L = w_bm(c, S, C, B, T, n1, ecc, true, normal, lane);
    if (!normal || L == 0 || L > t) return false;
    for (uint32_t k = lane; k < n1; k += 32) T[k] = C[k];  // T is free after the run
    __syncwarp();
    for (uint32_t k = lane; k < n1; k += 32) C[k] = k <= L ? T[L - k] : 0u;
    __syncwarp();
    // C must have degree exactly L (checked through the root count below)
    for (uint32_t k = lane; k < n1; k += 32)
        if (k > L && C[k]) L = 0xffffffffu;
    if (__any_sync(0xffffffffu, L == 0xffffffffu)) return false;
    // roots: the inverse partial NTT (pintt_ecc, ntt.hpp:206-220) evaluates C
    // at X_i^-1 for every position; the positions found are compacted into T
    // (free after BM; at most ecc + 1 kept)
    uint32_t count = 0;
    if constexpr (EPL > 0) {
        uint32_t cr[EPL];
#pragma unroll
        for (int h = 0; h < EPL; ++h) cr[h] = (uint32_t)(lane * EPL + h) <= L ? C[lane * EPL + h] : 0u;
        const uint32_t nch = c.block_len / ecc;
        for (uint32_t ch = 0; ch < nch; ++ch) {
            uint32_t x[EPL];
#pragma unroll
            for (int h = 0; h < EPL; ++h) x[h] = fmul(cr[h], c.pintt_shift[ch * ecc + lane * EPL + h]);
            reg_gs<EPL>(x, tw, lane);
#pragma unroll
            for (int h = 0; h < EPL; ++h) {
                const bool hit = x[h] == 0;
                const uint32_t msk = __ballot_sync(0xffffffffu, hit);
                const uint32_t at = count + __popc(msk & ((1u << lane) - 1u));
                if (hit && at < n1) T[at] = ch * ecc + lane * EPL + h;
                count += __popc(msk);
            }
        }
    } else if (ecc == 2 || ecc == 4 || ecc == 8 || ecc == 16) {
        switch (ecc) {
            case 2: count = sub_roots<2>(c, C, L, T, n1, lane); break;
            case 4: count = sub_roots<4>(c, C, L, T, n1, lane); break;
            case 8: count = sub_roots<8>(c, C, L, T, n1, lane); break;
            default: count = sub_roots<16>(c, C, L, T, n1, lane); break;
        }
    } else {
        uint32_t *R = temp + ecc + 3 * n1;  // block_len words, past S, C, B and T
        for (uint32_t k = lane; k < c.block_len; k += 32) R[k] = k <= L ? C[k] : 0u;
        __syncwarp();
        w_pintt(c, R, lane);
        for (uint32_t i0 = 0; i0 < c.block_len; i0 += 32) {
            const uint32_t i = i0 + lane;
            const bool hit = i < c.block_len && R[i] == 0;
            const uint32_t msk = __ballot_sync(0xffffffffu, hit);
            const uint32_t at = count + __popc(msk & ((1u << lane) - 1u));
            if (hit && at < n1) T[at] = i;
            count += __popc(msk);
        }
    }
    __syncwarp();
    if (count != L) return false;
    // evaluator Omega = S * C mod x^L and the derivative C'
    uint32_t *Om = B, *D = B + t + 1;  // B is free now: t + L <= ecc words
    for (uint32_t j = lane; j < L; j += 32) {
        uint32_t s = 0;
        for (uint32_t k = 0; k <= j; ++k) s = fadd(s, fmul(C[k], S[j - k]));
        Om[j] = s;
        D[j] = fmul(C[j + 1], j + 1);
    }
    __syncwarp();
    const uint32_t N = c.ntt_len;
    for (uint32_t r = lane; r < L; r += 32) {
        const uint32_t i = T[r];
        uint16_t bb = (uint16_t)i;
        bb = (uint16_t)(((bb >> 1) & 0x5555) | ((bb & 0x5555) << 1));
        bb = (uint16_t)(((bb >> 2) & 0x3333) | ((bb & 0x3333) << 2));
        bb = (uint16_t)(((bb >> 4) & 0x0f0f) | ((bb & 0x0f0f) << 4));
        bb = (uint16_t)((bb >> 8) | (bb << 8));
        const uint32_t e = (uint32_t)(bb >> c.rbo_shift);
        const uint32_t x = c.roots_ntt[e];
        const uint32_t xi = c.roots_ntt[(N - e) & (N - 1)];
        const uint32_t num = eval_poly(Om, L, xi);
        const uint32_t den = eval_poly(D, L, xi);
        const uint32_t err = fmul(fmul(num, c.inv_tab[den]), x);
        put_pos(c, v, b, i, fadd(get_pos(c, v, b, i), err));
    }
    __syncwarp();
    if (lane == 0) status[b] = FFGPU_REPAIR_OK;
    return true;
}

static __device__ __forceinline__ bool rsi16_repair_bm_block(const Rsi16Dev &c, const BlockView &v, size_t b,
                                                            uint32_t *temp, uint8_t *status, int lane) {
    const RegTw<1> none{};
    return rsi16_repair_bm_block_t<0>(c, v, b, temp, status, none, lane);
}

// ---------------------------------------------------------------- batched repair
//
// The bounded-distance path above, with Berlekamp-Massey run by one lane per
// block over a batch of 32 blocks: the syndromes of the batch are computed
// warp-wide (register transforms) into the columns of a [ecc][32] array, each
// lane then runs the whole iteration for its block on registers, and the
// roots and Forney values are found warp-wide again per block.  The warp-wide
// Berlekamp-Massey spends a shuffle reduction and three passes over the
// coefficients per iteration on one block; here those become per-lane loops.
// Columns are padded to 33 words so that both the row writes of the
// transforms and the column reads of the lanes avoid bank conflicts.
constexpr uint32_t kColStride = 33;

// Berlekamp-Massey of w_bm's reverse run for one block (lane), normalised
// (C <- C - (d / b) x^m B, with x^m B kept pre-shifted), over the reversed
// column S_{ecc-1}, ..., S_0 (stride kColStride), with T + 1 = ecc/2 + 1
// coefficients on registers.  A block the bounded-distance path accepts ends
// with L <= T; while L <= T the connection polynomial has degree <= L and
// every shifted B used has degree <= L, and once L exceeds T it never comes
// back below (the block then goes to the mirror), so the dropped terms never
// change an accepted result.  Returns L, or 0 when the run is not normal or
// L > T; C receives the connection polynomial of the reversed sequence.
template <int T>
static __device__ __forceinline__ uint32_t rsi16_rev_bm_lane(const uint32_t *S, const uint32_t *inv_tab, uint32_t ecc,
                                                             uint32_t (&C)[T + 1]) {
    uint32_t Bs[T + 1];
#pragma unroll
    for (int i = 0; i <= T; ++i) {
        C[i] = i == 0 ? 1u : 0u;
        Bs[i] = i == 1 ? 1u : 0u;
    }
    uint32_t L = 0, binv = 1;
    bool stalled = false, abnormal = false;
#pragma unroll 1
    for (uint32_t n = 0; n < ecc; ++n) {
        uint64_t acc = 0;
#pragma unroll
        for (int i = 0; i <= T; ++i)
            if ((uint32_t)i <= n) acc += (uint64_t)C[i] * S[(ecc - 1 - (n - i)) * kColStride];
        const uint32_t d = (uint32_t)(acc % 0x10001u);
        const uint32_t coef = fmul(d, binv);
        const bool grow = d != 0 && 2 * L <= n;
        if (d == 0 && !(n & 1) && 2 * L <= n) stalled = true;
        abnormal |= grow && stalled;
#pragma unroll
        for (int i = T; i >= 0; --i) {
            const uint32_t bi = Bs[i];
            Bs[i] = i == 0 ? 0u : (grow ? C[i - 1] : Bs[i - 1]);
            C[i] = fsub(C[i], fmul(coef, bi));
        }
        if (grow) {
            L = n + 1 - L;
            binv = inv_tab[d];
        }
    }
    return (abnormal || L > (uint32_t)T) ? 0u : L;
}

// The rest of the bounded-distance path, from a block's syndromes (column S)
// and the lane Berlekamp-Massey's locator (column C, T + 1 words) and length
// L: the degree check, the roots by inverse partial NTT, Omega = S * C mod x^L
// and Forney, exactly as in rsi16_repair_bm_block_t.  The root search runs on
// two blocks at once (twice the independent work per transform stage).

// L in range and C of degree at most L (the root count then checks that it is
// exactly L)
static __device__ __forceinline__ bool rsi16_locator_ok(const Rsi16Dev &c, const uint32_t *C, uint32_t L, int lane) {
    const uint32_t t = c.ecc / 2;
    if (L == 0 || L > t) return false;
    bool high = false;
    for (uint32_t k = L + 1 + lane; k <= t; k += 32) high |= C[k * kColStride] != 0;
    return !__any_sync(0xffffffffu, high);
}

// positions i with C(X_i^-1) = 0 of two locators (columns CA, CB with lengths
// LA, LB), into TA / TB (at most ecc + 1 kept); returns the two root counts
template <int EPL>
static __device__ __forceinline__ void rsi16_roots_pair(const Rsi16Dev &c, const uint32_t *CA, uint32_t LA,
                                                        const uint32_t *CB, uint32_t LB, uint32_t *TA,
                                                        uint32_t *TB, const RegTw<EPL> &tw, int lane,
                                                        uint32_t &countA, uint32_t &countB) {
    const uint32_t ecc = c.ecc, n1 = ecc + 1;
    uint32_t ca[EPL], cb[EPL];
#pragma unroll
    for (int h = 0; h < EPL; ++h) {
        const uint32_t k = (uint32_t)(lane * EPL + h);
        ca[h] = k <= LA ? CA[k * kColStride] : 0u;
        cb[h] = k <= LB ? CB[k * kColStride] : 0u;
    }
    uint32_t na = 0, nb = 0;
    const uint32_t nch = c.block_len / ecc;
    for (uint32_t ch = 0; ch < nch; ++ch) {
        uint32_t x[EPL], y[EPL];
#pragma unroll
        for (int h = 0; h < EPL; ++h) {
            const uint32_t sh = c.pintt_shift[ch * ecc + lane * EPL + h];
            x[h] = fmul(ca[h], sh);
            y[h] = fmul(cb[h], sh);
        }
        reg_gs2<EPL>(x, y, tw, lane);
#pragma unroll
        for (int h = 0; h < EPL; ++h) {
            const uint32_t pos = ch * ecc + lane * EPL + h;
            const uint32_t below = (1u << lane) - 1u;
            const bool ha = x[h] == 0, hb = y[h] == 0;
            const uint32_t ma = __ballot_sync(0xffffffffu, ha), mb = __ballot_sync(0xffffffffu, hb);
            const uint32_t at = na + __popc(ma & below), bt = nb + __popc(mb & below);
            if (ha && at < n1) TA[at] = pos;
            if (hb && bt < n1) TB[bt] = pos;
            na += __popc(ma);
            nb += __popc(mb);
        }
    }
    __syncwarp();
    countA = na;
    countB = nb;
}

// Omega, Forney and the corrections of block b whose L roots are in Tp;
// Om and D are scratch of t + 1 words each
static __device__ __forceinline__ void rsi16_forney_apply(const Rsi16Dev &c, const BlockView &v, size_t b,
                                                          const uint32_t *S, const uint32_t *C, uint32_t L,
                                                          const uint32_t *Tp, uint32_t *Om, uint32_t *D,
                                                          uint8_t *status, int lane) {
    // evaluator Omega = S * C mod x^L and the derivative C'
    for (uint32_t j = lane; j < L; j += 32) {
        uint32_t s = 0;
        for (uint32_t k = 0; k <= j; ++k) s = fadd(s, fmul(C[k * kColStride], S[(j - k) * kColStride]));
        Om[j] = s;
        D[j] = fmul(C[(j + 1) * kColStride], j + 1);
    }
    __syncwarp();
    const uint32_t N = c.ntt_len;
    for (uint32_t r = lane; r < L; r += 32) {
        const uint32_t i = Tp[r];
        uint16_t bb = (uint16_t)i;
        bb = (uint16_t)(((bb >> 1) & 0x5555) | ((bb & 0x5555) << 1));
        bb = (uint16_t)(((bb >> 2) & 0x3333) | ((bb & 0x3333) << 2));
        bb = (uint16_t)(((bb >> 4) & 0x0f0f) | ((bb & 0x0f0f) << 4));
        bb = (uint16_t)((bb >> 8) | (bb << 8));
        const uint32_t e = (uint32_t)(bb >> c.rbo_shift);
        const uint32_t x = c.roots_ntt[e];
        const uint32_t xi = c.roots_ntt[(N - e) & (N - 1)];
        const uint32_t num = eval_poly(Om, L, xi);
        const uint32_t den = eval_poly(D, L, xi);
        const uint32_t err = fmul(fmul(num, c.inv_tab[den]), x);
        put_pos(c, v, b, i, fadd(get_pos(c, v, b, i), err));
    }
    __syncwarp();
    if (lane == 0) status[b] = FFGPU_REPAIR_OK;
}

// RSi16v::_repair with known locations (rsi16v_impl.hpp:171-231),
// _error_locator (:531-542), _error_evaluator (:545-563); positions bp[0 .. count)
static __device__ __noinline__ void rsi16_repair_known_block(const Rsi16Dev &c, const BlockView &v, size_t b,
                                                      const uint32_t *bp, uint32_t count, uint32_t *temp,
                                                      uint8_t *status, int lane) {
    const uint32_t ecc = c.ecc;

    w_synd_block(c, v, b, temp, lane);
    if (w_all_zero(temp, ecc, lane)) {
        if (lane == 0 && status) status[b] = FFGPU_NO_ERRORS;
        return;
    }
    uint32_t *ev = temp, *loc = temp + 2 * ecc, *tmp = temp + 4 * ecc;
    w_fill(loc, 0, ecc, lane);
    for (uint32_t j = 0; j < count; ++j) {
        const uint32_t p = bp[j];
        uint16_t bb = (uint16_t)p;
        bb = (uint16_t)(((bb >> 1) & 0x5555) | ((bb & 0x5555) << 1));
        bb = (uint16_t)(((bb >> 2) & 0x3333) | ((bb & 0x3333) << 2));
        bb = (uint16_t)(((bb >> 4) & 0x0f0f) | ((bb & 0x0f0f) << 4));
        bb = (uint16_t)((bb >> 8) | (bb << 8));
        const uint32_t x = c.roots_ntt[(uint32_t)(bb >> c.rbo_shift)];
        // loc[i] -= loc[i-1] * x for i = count-1 .. 1 (old values), loc[0] -= x
        uint32_t nv[8];
        int n = 0;
        for (uint32_t i = lane; i < count && n < 8; i += 32) nv[n++] = (i == 0) ? fsub(loc[0], x) : fsub(loc[i], fmul(loc[i - 1], x));
        __syncwarp();
        n = 0;
        for (uint32_t i = lane; i < count && n < 8; i += 32) loc[i] = nv[n++];
        __syncwarp();
    }
    for (uint32_t k = ecc + lane; k < 2 * ecc; k += 32) ev[k] = 0;
    __syncwarp();
    w_gs(c.roots_ecc2, ev, 2 * ecc, lane);
    for (uint32_t k = lane; k < 2 * ecc + 1; k += 32) tmp[k] = (k == 0) ? 1u : (k <= count ? loc[k - 1] : 0u);
    __syncwarp();
    w_gs(c.roots_ecc2, tmp, 2 * ecc, lane);
    for (uint32_t k = lane; k < 2 * ecc; k += 32) ev[k] = fmul(ev[k], tmp[k]);
    __syncwarp();
    w_ct(c.roots_i_ecc2, ev, 2 * ecc, lane);
    for (uint32_t k = lane; k < 2 * ecc; k += 32) ev[k] = (k < ecc) ? fmul(ev[k], c.ecc2_len_i) : 0u;
    __syncwarp();
    uint32_t *deriv = temp + ecc;
    for (uint32_t k = lane; k < ecc; k += 32) deriv[k] = fmul(loc[k], k + 1);
    __syncwarp();
    const uint32_t dl = w_poly_len(deriv, ecc, lane);
    __syncwarp();
    // The corrections depend on the syndromes and the positions only: each
    // lane computes those of its listed positions, then lane 0 applies them
    // in list order (positions may repeat, and repeats accumulate).
    for (uint32_t i0 = 0; i0 < count; i0 += 32) {
        const uint32_t i = i0 + lane;
        uint32_t q = 0, err = 0;
        if (i < count) {
            uint16_t bb = (uint16_t)bp[i];
            bb = (uint16_t)(((bb >> 1) & 0x5555) | ((bb & 0x5555) << 1));
            bb = (uint16_t)(((bb >> 2) & 0x3333) | ((bb & 0x3333) << 2));
            bb = (uint16_t)(((bb >> 4) & 0x0f0f) | ((bb & 0x0f0f) << 4));
            bb = (uint16_t)((bb >> 8) | (bb << 8));
            const uint32_t pr = (uint32_t)(bb >> c.rbo_shift);
            const uint32_t x = c.roots_ntt[pr];
            const uint32_t xi = finv(x);
            const uint32_t num = eval_poly(ev, ecc, xi);
            const uint32_t den = eval_poly(deriv, dl, xi);
            err = fmul(fdiv(num, den), x);
            uint16_t cc = (uint16_t)pr;
            cc = (uint16_t)(((cc >> 1) & 0x5555) | ((cc & 0x5555) << 1));
            cc = (uint16_t)(((cc >> 2) & 0x3333) | ((cc & 0x3333) << 2));
            cc = (uint16_t)(((cc >> 4) & 0x0f0f) | ((cc & 0x0f0f) << 4));
            cc = (uint16_t)((cc >> 8) | (cc << 8));
            q = (uint32_t)(cc >> c.rbo_shift);
        }
        const uint32_t nj = count - i0 < 32 ? count - i0 : 32;
        for (uint32_t j = 0; j < nj; ++j) {
            const uint32_t qj = __shfl_sync(0xffffffffu, q, (int)j), ej = __shfl_sync(0xffffffffu, err, (int)j);
            if (lane == 0) put_pos(c, v, b, qj, fadd(get_pos(c, v, b, qj), ej));
        }
    }
    if (lane == 0 && status) status[b] = FFGPU_REPAIR_OK;
    __syncwarp();
}

// One batch of up to 32 blocks (base .. base+nb-1) on one warp: syndromes two
// blocks per pass into the columns of ws, a Berlekamp-Massey per lane, roots
// and Forney per pair; blocks the bounded-distance path does not accept go
// to the step-for-step mirror on mws (which may overlay ws: the columns are
// dead by then).
template <int EPL>
static __device__ __forceinline__ void rsi16_repair32(const Rsi16Dev &c, const BlockView &v, size_t base, int nb, uint8_t *status,
                               const uint8_t *active, const RegTw<EPL> &tw, int lane, uint32_t *ws, uint32_t *mws,
                               unsigned long long &nfast, unsigned long long &nmirror) {
    constexpr int T = 16 * EPL;
    uint32_t *Ssm = ws;
    uint32_t *Csm = Ssm + 32 * EPL * kColStride;
    uint32_t *fin = Csm + (T + 1) * kColStride;
    uint32_t live = 0u, nz = 0u;
    for (int j = 0; j < nb; ++j)
        if (!active || active[base + j]) live |= 1u << j;
    // syndromes two blocks at a time (a lone last block pairs with itself)
    for (uint32_t todo = live; todo;) {
        const int j0 = __ffs(todo) - 1;
        todo &= todo - 1;
        const int j1 = todo ? __ffs(todo) - 1 : j0;
        todo &= todo - 1;
        uint32_t s0[EPL], s1[EPL];
        reg_pntt2<EPL>(c, v, base + j0, base + j1, c.pntt_blocks, true, tw, lane, s0, s1);
        bool any0 = false, any1 = false;
#pragma unroll
        for (int h = 0; h < EPL; ++h) {
            Ssm[(lane * EPL + h) * kColStride + j0] = s0[h];
            Ssm[(lane * EPL + h) * kColStride + j1] = s1[h];
            any0 |= s0[h] != 0;
            any1 |= s1[h] != 0;
        }
        if (__any_sync(0xffffffffu, any0)) nz |= 1u << j0;
        if (__any_sync(0xffffffffu, any1)) nz |= 1u << j1;
    }
    __syncwarp();
    uint32_t L = 0;
    if ((nz >> lane) & 1u) {
        // Berlekamp-Massey on the reversed syndromes: only a normal run is
        // accepted (w_bm; L = 0 sends the block to the mirror), and its
        // connection polynomial read backwards is the locator up to a scalar
        uint32_t C[T + 1];
        L = rsi16_rev_bm_lane<T>(Ssm + lane, c.inv_tab, c.ecc, C);
#pragma unroll
        for (int i = 0; i <= T; ++i) {
            if ((uint32_t)i <= L) Csm[(L - i) * kColStride + lane] = C[i];
            if ((uint32_t)i > L) Csm[i * kColStride + lane] = 0u;
        }
    }
    __syncwarp();
    // blocks whose locator passes the checks get their roots searched in
    // pairs; the others (and those whose root count is not L) go to the
    // mirror
    uint32_t cand = 0u, mirror = 0u;
    for (int j = 0; j < nb; ++j) {
        if (!((live >> j) & 1u)) continue;
        const size_t b = base + j;
        if (!((nz >> j) & 1u)) {
            if (lane == 0) status[b] = FFGPU_NO_ERRORS;
            ++nfast;
            continue;
        }
        const uint32_t Lj = __shfl_sync(0xffffffffu, L, j);
        if (rsi16_locator_ok(c, Csm + j, Lj, lane))
            cand |= 1u << j;
        else
            mirror |= 1u << j;
    }
    uint32_t *TA = fin, *TB = fin + (c.ecc + 1), *Om = TB + (c.ecc + 1), *D = Om + (T + 1);
    for (uint32_t todo = cand; todo;) {
        const int ja = __ffs(todo) - 1;
        todo &= todo - 1;
        const int jb = todo ? __ffs(todo) - 1 : ja;
        todo &= todo - 1;
        const uint32_t La = __shfl_sync(0xffffffffu, L, ja), Lb = __shfl_sync(0xffffffffu, L, jb);
        uint32_t na, nbr;
        rsi16_roots_pair<EPL>(c, Csm + ja, La, Csm + jb, Lb, TA, TB, tw, lane, na, nbr);
        if (na == La) {
            rsi16_forney_apply(c, v, base + ja, Ssm + ja, Csm + ja, La, TA, Om, D, status, lane);
            ++nfast;
        } else {
            mirror |= 1u << ja;
        }
        if (jb != ja) {
            if (nbr == Lb) {
                rsi16_forney_apply(c, v, base + jb, Ssm + jb, Csm + jb, Lb, TB, Om, D, status, lane);
                ++nfast;
            } else {
                mirror |= 1u << jb;
            }
        }
    }
    for (uint32_t todo = mirror; todo; todo &= todo - 1) {
        __syncwarp();
        rsi16_repair_block(c, v, base + (__ffs(todo) - 1), mws, status, lane);
        ++nmirror;
    }
    __syncwarp();  // the batch's columns are read before the next batch writes them
}

}  // namespace ffgpu
