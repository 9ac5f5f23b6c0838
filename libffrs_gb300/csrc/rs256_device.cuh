// RS256 table-path device code shared by the standalone kernels (rs256.cu)
// and the fused batch kernel: GF(2^8) table arithmetic, the byte-serial LFSR,
// and the one-block decoder of rs_decode::decode (reed_solomon.hpp:559-595).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace ffgpu {

// ---------------------------------------------------------------- device

// multiply with a 512-entry exp table (ex[i] = a^(i mod 255), i <= 510)
static __device__ __forceinline__ uint32_t gmul(const uint8_t *ex, const uint8_t *lg, uint32_t a, uint32_t b) {
    return (a && b) ? ex[lg[a] + lg[b]] : 0u;
}
static __device__ __forceinline__ uint32_t gdiv(const uint8_t *ex, const uint8_t *lg, uint32_t a, uint32_t b) {
    return a ? ex[lg[a] + 255u - lg[b]] : 0u;
}
static __device__ __forceinline__ uint32_t ginv(const uint8_t *ex, const uint8_t *lg, uint32_t a) {
    return ex[255u - lg[a]];
}

// Cooperative byte copy global -> shared (coalesced, any alignment).
static __device__ __forceinline__ void stage_bytes(uint8_t *dst, const uint8_t *src, size_t n) {
    for (size_t i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

// One LFSR step: rem <- (rem >> 8) ^ lut[(rem & 0xff) ^ in], rem held as W words.
template <int W>
static __device__ __forceinline__ void lfsr_step(uint32_t (&rem)[W], uint32_t in, const uint32_t *s_lut) {
    const uint32_t fb = (rem[0] & 0xffu) ^ in;
    const uint32_t *row = s_lut + fb * W;
#pragma unroll
    for (int w = 0; w < W - 1; ++w) rem[w] = __funnelshift_r(rem[w], rem[w + 1], 8) ^ row[w];
    rem[W - 1] = (rem[W - 1] >> 8) ^ row[W - 1];
}

template <int W>
static __device__ __forceinline__ uint32_t rem_byte(const uint32_t (&rem)[W], int j) {
    uint32_t v = 0;
#pragma unroll
    for (int w = 0; w < W; ++w)
        if (w == (j >> 2)) v = rem[w];
    return (v >> ((j & 3) * 8)) & 0xffu;
}


// parity of one block: the LFSR over msg_len bytes at my (any alignment)
template <int W>
static __device__ __forceinline__ void rs256_encode_one(const uint8_t *my, int msg_len, const uint32_t *s_lut, uint8_t *out,
                                                 int ecc) {
    uint32_t rem[W];
#pragma unroll
    for (int w = 0; w < W; ++w) rem[w] = 0;
    for (int i = 0; i < msg_len; ++i) lfsr_step<W>(rem, my[i], s_lut);
    for (int j = 0; j < ecc; ++j) out[j] = (uint8_t)rem_byte<W>(rem, j);
}

struct ScratchBytes {
    uint8_t *base;
    size_t stride;
    __device__ __forceinline__ uint8_t &operator[](int k) const { return base[(size_t)k * stride]; }
    __device__ __forceinline__ ScratchBytes operator+(int k) const { return {base + (size_t)k * stride, stride}; }
};
struct DecodeScratchG {
    ScratchBytes S, lam, prev, tmp, pos, mag, ev;
    __device__ DecodeScratchG(uint8_t *g, size_t tid, size_t nthreads) {
        uint8_t *b = g + tid;
        S = {b, nthreads};
        lam = {b + 256 * nthreads, nthreads};
        prev = {b + 512 * nthreads, nthreads};
        tmp = {b + 768 * nthreads, nthreads};
        pos = {b + 1024 * nthreads, nthreads};
        mag = {b + 1280 * nthreads, nthreads};
        ev = {b + 1536 * nthreads, nthreads};
    }
};
constexpr size_t kDecodeScratchBytes = 2048;

// Syndromes from the remainder: S_j = sum_m R[m] a^{-j(m+1)}.
template <int W, typename A>
static __device__ void synds_from_rem(const uint32_t (&rem)[W], int ecc, const uint8_t *ex, const uint8_t *lg, A S) {
    for (int j = 0; j < ecc; ++j) S[j] = 0;
    for (int m = 0; m < ecc; ++m) {
        const uint32_t r = rem_byte<W>(rem, m);
        if (!r) continue;
        const int step = (m + 1) % 255;
        int e = lg[r] % 255;
        for (int j = 0; j < ecc; ++j) {
            S[j] ^= ex[e];
            e -= step;
            if (e < 0) e += 255;
        }
    }
}

// rs_decode::berlekamp_massey (reed_solomon.hpp:655-702); err_poly is
// right-aligned and reversed: err_poly[ecc-1-i] holds Lambda_i.
template <typename A>
static __device__ int rs_bm(A S, int ecc, const uint8_t *ex, const uint8_t *lg, A err_poly, A prev, A temp) {
    for (int i = 0; i < ecc; ++i) {
        prev[i] = 0;
        err_poly[i] = 0;
    }
    prev[ecc - 1] = 1;
    err_poly[ecc - 1] = 1;
    int errors = 0, m = 1;
    uint32_t b = 1;
    for (int n = 0; n < ecc; ++n) {
        uint32_t d = S[n];
        for (int i = 1; i < errors + 1; ++i) d ^= gmul(ex, lg, err_poly[ecc - 1 - i], S[n - i]);
        if (d == 0) {
            m = m + 1;
        } else if (2 * errors <= n) {
            for (int i = 0; i < ecc; ++i) temp[i] = err_poly[i];
            const uint32_t s = gdiv(ex, lg, d, b);
            for (int i = 0; i < ecc; ++i) {
                const uint32_t p = (i < ecc - m) ? prev[i + m] : 0u;
                err_poly[i] ^= gmul(ex, lg, s, p);
            }
            errors = n + 1 - errors;
            for (int i = 0; i < ecc; ++i) prev[i] = temp[i];
            b = d;
            m = 1;
        } else {
            const uint32_t s = gdiv(ex, lg, d, b);
            for (int i = 0; i < ecc; ++i) {
                const uint32_t p = (i < ecc - m) ? prev[i + m] : 0u;
                err_poly[i] ^= gmul(ex, lg, s, p);
            }
            m = m + 1;
        }
    }
    return errors;
}

template <typename A>
static __device__ __forceinline__ uint32_t poly_eval(A p, int n, uint32_t x, const uint8_t *ex, const uint8_t *lg) {
    uint32_t r = 0;
    for (int i = 0; i < n; ++i) r = gmul(ex, lg, r, x) ^ p[i];
    return r;
}

static __device__ void decode_solve(uint8_t *d, uint8_t *p, int msg_len, int ecc, const uint8_t *ex, const uint8_t *lg,
                             const DecodeScratchG &sc, uint8_t *status);

// One block: rs_decode::decode (reed_solomon.hpp:559-595).  Writes the
// status (1/0) or, when synds_out is set, only the syndromes.
template <int W>
static __device__ void decode_one(uint8_t *d, uint8_t *p, int msg_len, int ecc, const uint32_t *s_lut, const uint8_t *ex,
                           const uint8_t *lg, const DecodeScratchG &sc, uint8_t *status, uint8_t *synds_out) {
    uint32_t rem[W];
#pragma unroll
    for (int w = 0; w < W; ++w) rem[w] = 0;
    for (int i = 0; i < msg_len; ++i) lfsr_step<W>(rem, d[i], s_lut);
    for (int i = 0; i < ecc; ++i) lfsr_step<W>(rem, p[i], s_lut);
    uint32_t any = 0;
#pragma unroll
    for (int w = 0; w < W; ++w) any |= rem[w];
    if (synds_out) {
        if (any)
            synds_from_rem<W>(rem, ecc, ex, lg, sc.S);
        else
            for (int j = 0; j < ecc; ++j) sc.S[j] = 0;
        for (int j = 0; j < ecc; ++j) synds_out[j] = sc.S[j];
        return;
    }
    if (!any) {
        *status = 1;
        return;
    }
    synds_from_rem<W>(rem, ecc, ex, lg, sc.S);
    decode_solve(d, p, msg_len, ecc, ex, lg, sc, status);
}

// The part of rs_decode::decode after the syndromes (reed_solomon.hpp:568-594),
// with sc.S holding non-zero syndromes.
static __device__ void decode_solve(uint8_t *d, uint8_t *p, int msg_len, int ecc, const uint8_t *ex, const uint8_t *lg,
                             const DecodeScratchG &sc, uint8_t *status) {
    const int errors = rs_bm(sc.S, ecc, ex, lg, sc.lam, sc.prev, sc.tmp);
    if (errors > ecc / 2) {
        *status = 0;
        return;
    }
    const ScratchBytes loc = sc.lam + (ecc - errors - 1);
    const int size = msg_len + ecc;
    int roots = 0;
    for (int i = 0; i < size && i < 256; ++i) {
        const uint32_t x = ex[(255 - i) % 255];
        if (poly_eval(loc, errors + 1, x, ex, lg) == 0) sc.pos[roots++] = (uint8_t)i;
        if (roots > errors) break;
    }
    if (roots != errors) {
        *status = 0;
        return;
    }
    // Forney: omega = (S reversed * Lambda) mod x^ecc, highest degree first
    const int esize = ecc + errors;
    for (int i = 0; i < esize; ++i) sc.ev[i] = 0;
    for (int i = 0; i < ecc; ++i)
        for (int j = 0; j < errors + 1; ++j) sc.ev[i + j] ^= gmul(ex, lg, sc.S[ecc - 1 - i], loc[j]);
    int begin = errors;
    while (begin < esize && sc.ev[begin] == 0) ++begin;
    if (begin >= esize) {
        *status = 0;
        return;
    }
    // formal derivative in place (gf_poly_deriv_pw2, galois.hpp:725-734)
    const ScratchBytes lp = loc;
    const int psize = errors + 1;
    for (int i = 1; i < psize; ++i) lp[psize - i] = (i & 1) ? lp[psize - i - 1] : 0;
    for (int i = 0; i < errors; ++i) {
        const uint32_t xi = ex[sc.pos[i]];
        const uint32_t xinv = ginv(ex, lg, xi);
        const uint32_t num = poly_eval(sc.ev + begin, esize - begin, xinv, ex, lg);
        const uint32_t den = poly_eval(lp + 1, errors, xinv, ex, lg);
        sc.mag[i] = (uint8_t)gmul(ex, lg, xi, gdiv(ex, lg, num, den));
    }
    for (int i = 0; i < errors; ++i) {
        const int pos = size - 1 - sc.pos[i];
        if (pos < msg_len)
            d[pos] ^= sc.mag[i];
        else
            p[pos - msg_len] ^= sc.mag[i];
    }
    *status = 1;
}


}  // namespace ffgpu
