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
// Rows of four words or more are read 16 bytes at a time (the table is
// 16-byte aligned, in shared or global memory).
template <int W>
static __device__ __forceinline__ void lfsr_step(uint32_t (&rem)[W], uint32_t in, const uint32_t *s_lut) {
    const uint32_t fb = (rem[0] & 0xffu) ^ in;
    const uint32_t *row = s_lut + fb * W;
    uint32_t r[W];
    if constexpr (W >= 4) {
#pragma unroll
        for (int q = 0; q < W / 4; ++q) {
            const uint4 v = reinterpret_cast<const uint4 *>(row)[q];
            r[4 * q] = v.x;
            r[4 * q + 1] = v.y;
            r[4 * q + 2] = v.z;
            r[4 * q + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int w = 0; w < W; ++w) r[w] = row[w];
    }
#pragma unroll
    for (int w = 0; w < W - 1; ++w) rem[w] = __funnelshift_r(rem[w], rem[w + 1], 8) ^ r[w];
    rem[W - 1] = (rem[W - 1] >> 8) ^ r[W - 1];
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

// Per-thread decode scratch: byte columns.  Byte k of a column of thread
// tid sits at column_base[k * nthreads + tid], so that the lock-step accesses
// of a warp fall on consecutive bytes (global memory: one sector; shared
// memory: no bank conflict).
//   S (ecc bytes): syndromes, then the evaluator (written over them);
//   A, B, C (ecc/2 + 2 bytes each, consecutive): the remainder logs while
//   the syndromes are formed (R, spanning all three), then the rotating
//   Berlekamp-Massey polynomials (degree <= L <= ecc/2 while they are live),
//   then Lambda, the root positions and the Chien exponents.
struct DecodeScratchG {
    ScratchBytes S, A, B, C, R;
    // ecc == 0: 256-byte columns; else the compact layout of
    // decode_scratch_bytes(ecc) bytes per thread
    __device__ DecodeScratchG(uint8_t *g, size_t tid, size_t nthreads, int ecc = 0) {
        uint8_t *b = g + tid;
        const size_t s = ecc ? (size_t)ecc : 256, h = ecc ? (size_t)(ecc / 2 + 2) : 256;
        S = {b, nthreads};
        A = {b + s * nthreads, nthreads};
        B = {b + (s + h) * nthreads, nthreads};
        C = {b + (s + 2 * h) * nthreads, nthreads};
        R = A;  // 3h >= ecc bytes from A on
    }
};
constexpr size_t kDecodeScratchBytes = 2048;  // per thread, the 256-byte-column layout
// per thread, the compact layout for ecc
__host__ __device__ constexpr size_t decode_scratch_bytes(int ecc) { return (size_t)ecc + 3 * (size_t)(ecc / 2 + 2); }

// Syndromes from the remainder: S_j = sum_m R[m] a^{-j(m+1)}, j-outer with
// the exponent of each term stepped by j (no multiplications), the remainder
// bytes' logs (mod 255) staged in sc.R (255 marks a zero byte).
template <int W>
static __device__ void synds_from_rem(const uint32_t (&rem)[W], int ecc, const uint8_t *ex, const uint8_t *lg,
                                      const DecodeScratchG &sc) {
    for (int m = 0; m < ecc; ++m) {
        const uint32_t r = rem_byte<W>(rem, m);
        sc.R[m] = r ? lg[r] % 255 : 255;  // logs may be stored as 1..255
    }
    // eight syndromes per pass: one load of each remainder log serves them all
    for (int j0 = 0; j0 < ecc; j0 += 8) {
        uint32_t acc[8];
        int sub[8], step[8];  // sub: j * (m + 1) mod 255
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            acc[q] = 0;
            sub[q] = 0;
            step[q] = j0 + q < ecc ? j0 + q : 0;  // j < 255; past ecc nothing is kept
        }
        for (int m = 0; m < ecc; ++m) {
            const uint32_t lr = sc.R[m];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                sub[q] += step[q];
                if (sub[q] >= 255) sub[q] -= 255;
                const uint32_t v = ex[lr + 255u - (uint32_t)sub[q]];  // lr + 255 - sub <= 510
                acc[q] ^= lr != 255u ? v : 0u;
            }
        }
#pragma unroll
        for (int q = 0; q < 8; ++q)
            if (j0 + q < ecc) sc.S[j0 + q] = (uint8_t)acc[q];
    }
}

// rs_decode::berlekamp_massey (reed_solomon.hpp:655-702) on normal-order
// polynomials (A[k] = Lambda_k, degrees below ecc), with the same updates and
// truncation as the reference's reversed layout.  Loops run over the live
// degrees only, and the three buffers rotate instead of being copied.  The
// locator's degree never exceeds L (every update adds x^m B with
// m + deg B <= the new L), and L never shrinks, so the run stops as soon as
// L passes ecc/2 (the reference's decode then fails whatever follows) and
// the buffers need ecc/2 + 1 coefficients.  Returns L; *lam is left on the
// buffer holding Lambda and *fr, *fr2 on the free ones.
static __device__ int rs_bm(const DecodeScratchG &sc, int ecc, const uint8_t *ex, const uint8_t *lg,
                            ScratchBytes *lam, ScratchBytes *fr, ScratchBytes *fr2) {
    ScratchBytes A = sc.A, P = sc.B, T = sc.C;
    A[0] = 1;
    P[0] = 1;
    int degA = 0, degP = 0, L = 0, m = 1;
    uint32_t b = 1;
    for (int n = 0; n < ecc; ++n) {
        uint32_t d = sc.S[n];
        const int top = L < degA ? L : degA;
        for (int i = 1; i <= top; ++i) d ^= gmul(ex, lg, A[i], sc.S[n - i]);
        if (d == 0) {
            ++m;
            continue;
        }
        const uint32_t s = gdiv(ex, lg, d, b);  // non-zero: d and b are
        const uint32_t lgs = lg[s];
        const int hi = m + degP < ecc - 1 ? m + degP : ecc - 1;
        const int nd = degA > hi ? degA : hi;
        if (2 * L <= n) {
            // L only grows: past ecc/2 the block fails whatever follows
            if (2 * (n + 1 - L) > ecc) return n + 1 - L;
            // T = A + s x^m P; P <- A; A <- T
            for (int k = 0; k <= nd; ++k) {
                uint32_t v = k <= degA ? (uint32_t)A[k] : 0u;
                if (k >= m && k <= hi) {
                    const uint32_t pk = P[k - m];
                    v ^= pk ? (uint32_t)ex[lgs + lg[pk]] : 0u;  // gmul(s, pk)
                }
                T[k] = (uint8_t)v;
            }
            const ScratchBytes oldP = P;
            P = A;
            A = T;
            T = oldP;
            degP = degA;
            degA = nd;
            L = n + 1 - L;
            b = d;
            m = 1;
        } else {
            for (int k = degA + 1; k <= hi; ++k) A[k] = 0;  // stale bytes above the live degree
            for (int k = m; k <= hi; ++k) {
                const uint32_t pk = P[k - m];
                if (pk) A[k] ^= ex[lgs + lg[pk]];  // gmul(s, pk)
            }
            degA = nd;
            ++m;
        }
    }
    // coefficients up to L are read below: clear those above the live degree
    for (int k = degA + 1; k <= L; ++k) A[k] = 0;
    *lam = A;
    *fr = T;
    *fr2 = P;
    return L;
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
        if (any) {
            synds_from_rem<W>(rem, ecc, ex, lg, sc);
            for (int j = 0; j < ecc; ++j) synds_out[j] = sc.S[j];
        } else {
            for (int j = 0; j < ecc; ++j) synds_out[j] = 0;
        }
        return;
    }
    if (!any) {
        *status = 1;
        return;
    }
    synds_from_rem<W>(rem, ecc, ex, lg, sc);
    decode_solve(d, p, msg_len, ecc, ex, lg, sc, status);
}

// The part of rs_decode::decode after the syndromes (reed_solomon.hpp:568-594),
// with sc.S holding non-zero syndromes.  Every decision and every corrected
// byte is the reference's; only the evaluation order of the (exact) field
// sums differs.
static __device__ void decode_solve(uint8_t *d, uint8_t *p, int msg_len, int ecc, const uint8_t *ex, const uint8_t *lg,
                             const DecodeScratchG &sc, uint8_t *status) {
    ScratchBytes lam, pos, xp;
    const int errors = rs_bm(sc, ecc, ex, lg, &lam, &pos, &xp);
    if (errors > ecc / 2) {
        *status = 0;
        return;
    }
    const int size = msg_len + ecc;
    const int npos = size < 256 ? size : 256;
    // Chien search (rs_roots_eval_lut_pw2, reed_solomon.hpp:511-552): the
    // zeros of Lambda at x = a^{-i}, i < size, in increasing i, stopping at
    // errors + 1 roots.  Term k at position i has exponent
    // log(Lambda_k) - i k (mod 255); eight positions per pass, each term's
    // exponent kept in the free buffer xp between passes (255: a zero
    // coefficient).
    for (int k = 0; k <= errors; ++k) {
        const uint32_t c = lam[k];
        xp[k] = c ? lg[c] % 255 : 255;
    }
    int roots = 0;
    for (int i0 = 0; i0 < npos && roots <= errors; i0 += 8) {
        uint32_t acc[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[j] = 0;
        for (int k = 0; k <= errors; ++k) {
            int e = xp[k];
            if (e == 255) continue;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                acc[j] ^= ex[e];
                e -= k;
                if (e < 0) e += 255;
            }
            xp[k] = (uint8_t)e;
        }
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (acc[j] == 0 && i0 + j < npos && roots <= errors) pos[roots++] = (uint8_t)(i0 + j);
    }
    if (roots != errors) {
        *status = 0;
        return;
    }
    // Forney: Omega = (S * Lambda) mod x^ecc, non-zero.  Omega_k needs
    // S_0 .. S_k only, so it is written over S_k from the top down.
    uint32_t anyo = 0;
    for (int k = ecc - 1; k >= 0; --k) {
        uint32_t v = 0;
        const int top = k < errors ? k : errors;
        for (int j = 0; j <= top; ++j) v ^= gmul(ex, lg, lam[j], sc.S[k - j]);
        sc.S[k] = (uint8_t)v;
        anyo |= v;
    }
    if (!anyo) {
        *status = 0;
        return;
    }
    // magnitudes X * Omega(X^-1) / Lambda'(X^-1) (gf_poly_deriv_pw2,
    // galois.hpp:725-734: Lambda'(x) = sum over odd k of Lambda_k x^(k-1)).
    // They depend on the syndromes and Lambda only, and nothing fails from
    // here on, so each is applied as soon as it is known.
    for (int i = 0; i < errors; ++i) {
        const uint32_t xi = ex[pos[i]];
        const uint32_t xinv = ginv(ex, lg, xi);
        const uint32_t lx = lg[xinv], lx2 = lx + lx;  // xinv != 0
        uint32_t num = 0;
        for (int k = ecc - 1; k >= 0; --k) num = (num ? (uint32_t)ex[lg[num] + lx] : 0u) ^ sc.S[k];
        uint32_t den = 0;
        for (int k = errors - ((errors & 1) ? 0 : 1); k >= 1; k -= 2)
            den = (den ? (uint32_t)ex[(lg[den] + lx2) % 255] : 0u) ^ lam[k];  // den xinv^2 + Lambda_k
        const uint8_t mag = (uint8_t)gmul(ex, lg, xi, gdiv(ex, lg, num, den));
        const int q = size - 1 - pos[i];
        if (q < msg_len)
            d[q] ^= mag;
        else
            p[q - msg_len] ^= mag;
    }
    *status = 1;
}


}  // namespace ffgpu
