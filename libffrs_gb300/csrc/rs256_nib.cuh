// RS256 encode (ecc 32, field polynomial 0x11d) by nibble tables: the
// tables, their shared-memory layout and one lane's part of a block, shared
// by rs256_encode_nib_kernel (rs256_bitsliced.cu) and the CPU check of the
// same code (tests/host/rs256_nib_check.cpp).
//
// rs_encode (libffrs/reed_solomon.hpp:225-297) is linear: the parity of a
// message is the XOR over its bytes m_i of m_i * U_e, U_e = x^(32 + e) mod
// g(x) for the byte's degree index e = message_len - 1 - i.  With each byte
// split into nibbles, m * U_e = (m & 15) U_e + (m & 0xf0) U_e, so a degree
// takes two tables of 16 entries of 32 bytes (1 KB); the 223 degrees of the
// longest message fit in one CTA's shared memory.  There is no dependence
// between bytes, which suits batches too small to fill the GPU with the
// bitsliced LFSR (sequential over the message for each 32-block group).
//
// Bank layout: one 128-byte line holds the entries of one nibble value for
// four consecutive degrees 4G .. 4G+3, 32 bytes each.  A quarter warp (the 8
// lanes that one 16-byte shared load serves per wavefront) takes one block:
// lane (r, h) the bytes of degree index e = r (mod 4) and parity half h
// (bytes 16h .. 16h+15).  Its reads land on bank group 2r + h whatever the
// byte values, so a warp's four quarters read their 512 bytes in four
// wavefronts.  The four residues are then XORed (two shuffles in the kernel).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <vector>

namespace ffgpu {

constexpr int kNibDegrees = 224;                // degree indices 0 .. 223 (223 used)
constexpr int kNibLineQ = 8;                    // 16-byte words per line: [r][h]
constexpr int kNibGroupQ = 2 * 16 * kNibLineQ;  // words per group of 4 degrees: [part][v][line]
constexpr int kNibWords = kNibDegrees / 4 * kNibGroupQ;

// GF(2^8) product with the field polynomial 0x11d (gf_mul, libffrs/galois.hpp)
inline uint8_t nib_gmul(uint8_t a, uint8_t b) {
    uint32_t r = 0, x = a;
    for (; b; b >>= 1) {
        if (b & 1) r ^= x;
        x <<= 1;
        if (x & 0x100) x ^= 0x11d;
    }
    return (uint8_t)r;
}

// The tables, as 32-bit words (kNibWords 16-byte words), from g_low[k], the
// coefficient of x^(31 - k) of g(x) = prod_{j < 32} (x - a^j) below its
// leading 1 (so g_low is x^32 mod g).  For degree index e, entry (part, v) is
// val * U_e with val = v (part 0) or v << 4 (part 1), U_e as 32 bytes (byte
// k: the coefficient of x^(31 - k)); half h (bytes 16h .. 16h + 15) of it is
// 16-byte word ((e / 4 * 2 + part) * 16 + v) * 8 + 2 (e % 4) + h.
inline std::vector<uint32_t> nib_tables(const uint8_t *g_low) {
    uint8_t U[32];
    for (int k = 0; k < 32; ++k) U[k] = g_low[k];
    std::vector<uint32_t> t((size_t)kNibWords * 4);
    for (int e = 0; e < kNibDegrees; ++e) {
        for (int part = 0; part < 2; ++part)
            for (int v = 0; v < 16; ++v) {
                const uint8_t val = (uint8_t)(part ? v << 4 : v);
                for (int h = 0; h < 2; ++h) {
                    const size_t word = (((size_t)(e / 4) * 2 + part) * 16 + v) * kNibLineQ + 2 * (e % 4) + h;
                    uint32_t *q = &t[word * 4];
                    for (int k = 0; k < 16; ++k) q[k / 4] |= (uint32_t)nib_gmul(val, U[16 * h + k]) << (8 * (k % 4));
                }
            }
        // U <- x U mod g
        const uint8_t top = U[0];
        for (int k = 0; k < 31; ++k) U[k] = U[k + 1];
        U[31] = 0;
        for (int k = 0; k < 32; ++k) U[k] ^= nib_gmul(top, g_low[k]);
    }
    return t;
}

// the XOR into acc of the entries of the four bytes of w (one per word,
// byte k0 of each) at message indices p0 + 4j + k0, j < 4, whose degree
// indices e0 - 4j lie in line group G0 - j (e0 = ml - 1 - p0 - k0 = r mod 4,
// G0 = e0 >> 2, Tb = T + G0 * kNibGroupQ + 2r + h); MASK: some of the
// indices fall outside [0, ml) and those bytes count as zero
template <bool MASK>
__device__ __forceinline__ void nib_chunk(const uint4 *T, const uint4 *Tb, int ml, int p0, int k0, int rh,
                                          const uint32_t (&w)[4], uint4 &acc) {
    // entry (G, part, v, r, h) at T[((G * 2 + part) * 16 + v) * 8 + 2r + h]
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        uint32_t v = w[j] >> (8 * k0);
        const uint4 *Te = Tb - j * kNibGroupQ;
        if (MASK) {
            const int p = p0 + 4 * j + k0;
            const bool in = p >= 0 && p < ml;
            v = in ? v : 0u;
            Te = in ? Te : T + rh;
        }
        const uint4 lo = Te[(v & 15u) * kNibLineQ], hi = Te[(16 + ((v >> 4) & 15u)) * kNibLineQ];
        acc.x ^= lo.x ^ hi.x;
        acc.y ^= lo.y ^ hi.y;
        acc.z ^= lo.z ^ hi.z;
        acc.w ^= lo.w ^ hi.w;
    }
}

// the 16-byte chunk at address ac as four words; chunks that reach past
// either end of the buffer [d0, d1) (d0 4-byte aligned) are read by 4-byte
// words, the word holding d1 byte by byte, zero outside the buffer
__device__ __forceinline__ void nib_load(uintptr_t ac, uintptr_t d0, uintptr_t d1, uint32_t (&w)[4]) {
    if (ac >= d0 && ac + 16 <= d1) {
        const uint4 q = __ldg(reinterpret_cast<const uint4 *>(ac));
        w[0] = q.x, w[1] = q.y, w[2] = q.z, w[3] = q.w;
    } else {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const uintptr_t aw = ac + 4 * i;
            uint32_t v = 0u;
            if (aw >= d0 && aw + 4 <= d1) {
                v = __ldg(reinterpret_cast<const uint32_t *>(aw));
            } else if (aw >= d0 && aw < d1) {
                for (uintptr_t k = aw; k < d1; ++k)
                    v |= (uint32_t)__ldg(reinterpret_cast<const uint8_t *>(k)) << (8 * (k - aw));
            }
            w[i] = v;
        }
    }
}

// Lane (r, h)'s part of block b's parity half h: the entries of the bytes of
// degree index r (mod 4) of the message at d0 + b * ml (messages back to
// back in [d0, d1)); T holds the line groups of degree indices 0 .. ml - 1.
// The XOR over r = 0 .. 3 is bytes 16h .. 16h + 15 of the parity.
__device__ __forceinline__ uint4 nib_lane(const uint4 *T, uintptr_t d0, uintptr_t d1, size_t b, int ml, int r,
                                          int h) {
    const int rh = 2 * r + h;
    uint4 acc = make_uint4(0u, 0u, 0u, 0u);
    // chunk c: the 16 bytes at a0 + 16c, message indices p00 + 16c ..
    // (p00 in [-15, 0]); this lane's bytes are k0, k0 + 4, .. of each
    const uintptr_t a = d0 + b * (size_t)ml, a0 = a & ~(uintptr_t)15;
    const int p00 = (int)((intptr_t)a0 - (intptr_t)a);
    const int nch = (ml - p00 + 15) >> 4;
    const int k0 = (ml - 1 - p00 - r) & 3;
    const uint4 *Tb = T + (ptrdiff_t)((ml - 1 - p00 - k0) >> 2) * kNibGroupQ + rh;
    uint32_t w[4], wn[4];
    nib_load(a0, d0, d1, w);
    if (nch > 1) nib_load(a0 + 16, d0, d1, wn);
    nib_chunk<true>(T, Tb, ml, p00, k0, rh, w, acc);
    for (int c = 1; c < nch; ++c) {
#pragma unroll
        for (int i = 0; i < 4; ++i) w[i] = wn[i];
        if (c + 1 < nch) nib_load(a0 + 16 * (uintptr_t)(c + 1), d0, d1, wn);
        const int p0 = p00 + 16 * c;
        const uint4 *Tc = Tb - 4 * c * kNibGroupQ;
        if (p0 + 16 <= ml)
            nib_chunk<false>(T, Tc, ml, p0, k0, rh, w, acc);
        else
            nib_chunk<true>(T, Tc, ml, p0, k0, rh, w, acc);
    }
    return acc;
}

}  // namespace ffgpu
