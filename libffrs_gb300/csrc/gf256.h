// GF(2^8) tables and RS256 code construction on the host.
//
// Field: elements are bytes, multiplication modulo x^8 + poly1 (the polynomial
// with its top bit masked off, libffrs/pygf256.hpp:261-263).  exp/log tables
// are built by repeated bit-serial multiplication with the primitive element
// exactly as libffrs/galois.hpp:133-144 builds them, which fixes the
// reference's conventions log[1] == 255, log[0] == 0, inv(0) == 1 and
// div(a, 0) == a (galois.hpp:98-127).
#pragma once

#include <cstdint>
#include <cstring>
#include <vector>

namespace ffgpu {

struct GF256Host {
    uint8_t poly1 = 0x1d;
    uint8_t primitive = 2;
    uint8_t exp[256];
    uint8_t log[256];

    static uint8_t mul_serial(uint8_t poly1, uint8_t a, uint8_t b) {
        uint8_t r = 0;
        for (int i = 7; i >= 0; --i) {
            r = (r & 0x80) ? (uint8_t)((r << 1) ^ poly1) : (uint8_t)(r << 1);
            if (a & (1u << i)) r ^= b;
        }
        return r;
    }

    GF256Host(uint8_t primitive_, uint8_t poly1_) : poly1(poly1_), primitive(primitive_) {
        std::memset(exp, 0, sizeof exp);
        std::memset(log, 0, sizeof log);
        uint8_t x = 1;
        for (int i = 0; i < 256; ++i) {
            exp[i] = x;
            log[x] = (uint8_t)i;
            x = mul_serial(poly1, x, primitive);
        }
    }

    // true when the primitive element generates all 255 non-zero elements,
    // i.e. the tables describe a field and table multiplication is bilinear
    bool is_field() const {
        bool seen[256] = {false};
        for (int i = 0; i < 255; ++i) seen[exp[i]] = true;
        for (int v = 1; v < 256; ++v)
            if (!seen[v]) return false;
        return !seen[0];
    }

    uint8_t mul(uint8_t a, uint8_t b) const {
        if (!a || !b) return 0;
        unsigned r = (unsigned)log[a] + log[b];
        if (r >= 255) r -= 255;
        return exp[r];
    }
    uint8_t inv(uint8_t a) const { return exp[255 - log[a]]; }
};

// g(x) = prod_{i < ecc} (x - a^i), highest degree first, g[0] == 1
// (rs_generator, libffrs/reed_solomon.hpp:65-86)
inline void rs256_generator(const GF256Host &gf, int ecc, uint8_t *gen, uint8_t *roots) {
    uint8_t tmp[257];
    std::memset(gen, 0, (size_t)ecc + 1);
    gen[0] = 1;
    size_t len = 1;
    for (int i = 0; i < ecc; ++i) {
        roots[i] = gf.exp[i];
        std::memset(tmp, 0, len + 1);
        for (size_t a = 0; a < len; ++a) {
            tmp[a] ^= gf.mul(gen[a], 1);
            tmp[a + 1] ^= gf.mul(gen[a], roots[i]);
        }
        ++len;
        std::memcpy(gen, tmp, len);
    }
}

// Row table of the LFSR encoder: lut[v] = (v * x^ecc) mod g as ecc bytes with
// the highest-degree coefficient first; the table the reference's slicing
// encoders are built on (reed_solomon.hpp:204-207, 271-274, via
// gf_poly::poly_mod_x_n, galois.hpp:462-499).
inline void rs256_lut(const GF256Host &gf, int ecc, const uint8_t *gen, std::vector<uint8_t> &lut) {
    lut.assign((size_t)256 * ecc, 0);
    const uint8_t *b = gen + 1;
    std::vector<uint8_t> rem((size_t)ecc);
    for (int v = 0; v < 256; ++v) {
        // a single input coefficient v, i.e. size_a == 1
        if (ecc > 1) {
            std::fill(rem.begin(), rem.end(), 0);
            rem[(size_t)ecc - 1] = (uint8_t)v;
        } else {
            rem[0] = (uint8_t)v;
        }
        for (int i = 0; i < ecc; ++i) {
            uint8_t c = rem[0];
            for (int j = 0; j + 1 < ecc; ++j) rem[(size_t)j] = rem[(size_t)j + 1];
            rem[(size_t)ecc - 1] = 0;
            if (!c) continue;
            for (int j = 0; j < ecc; ++j) rem[(size_t)j] ^= gf.mul(b[j], c);
        }
        std::memcpy(&lut[(size_t)v * ecc], rem.data(), (size_t)ecc);
    }
}

}  // namespace ffgpu
