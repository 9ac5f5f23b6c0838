// The per-thread RS256 decoder of the GPU table path (rs256_device.cuh: the
// LFSR remainder over the table rows, syndromes, Berlekamp-Massey, Chien
// search, Forney), compiled for the host and run block by block against the
// oracle's rs_decode::decode (reed_solomon.hpp:559-595): same status, same
// bytes, both from the oracle's remainder and through decode_one with the
// library's own tables (gf256.h); and the table encoder (rs256_encode_one)
// against the oracle's encoder.  Usage:
// rs256_solve_check <seed> <trials per ecc>; prints "bad N", exits 1 if N > 0.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

#include "gf256.h"
#include "rs256_device.cuh"
extern "C" {
#include "ffrs_oracle.h"
}
using namespace ffgpu;

template <int W>
static int run(int ecc, int trials, std::mt19937 &g) {
    orc_rs256 *rs = orc_rs256_new(ecc, 2, 0x11d);
    uint8_t e256[256], lg[256], ex[512];
    orc_rs256_tables(rs, e256, lg);
    for (int i = 0; i < 512; ++i) ex[i] = e256[i % 255];
    std::vector<uint8_t> scratch(kDecodeScratchBytes);
    // the library's LFSR table (rows of W words) and field tables
    GF256Host gf(2, 0x1d);
    std::vector<uint8_t> gen(ecc + 1), roots(ecc), lutb;
    rs256_generator(gf, ecc, gen.data(), roots.data());
    rs256_lut(gf, ecc, gen.data(), lutb);
    std::vector<uint32_t> lut((size_t)256 * W + 4, 0);
    uint32_t *lut16 = lut.data() + ((16 - ((uintptr_t)lut.data() & 15)) & 15) / 4;  // 16-byte aligned rows
    for (int v = 0; v < 256; ++v)
        for (int j = 0; j < ecc; ++j) lut16[(size_t)v * W + j / 4] |= (uint32_t)lutb[(size_t)v * ecc + j] << (8 * (j % 4));
    uint8_t gex[512];
    for (int i = 0; i < 512; ++i) gex[i] = gf.exp[i % 255];
    int bad = 0;
    for (int t = 0; t < trials; ++t) {
        const int ml = 1 + (int)(g() % (unsigned)(255 - ecc));
        const int n = ml + ecc;
        std::vector<uint8_t> cw(n), par(ecc), rem(ecc);
        for (int i = 0; i < ml; ++i) cw[i] = (uint8_t)g();
        orc_rs256_encode(rs, cw.data(), ml, par.data());
        {
            // the table encoder of the GPU path (rs256_encode_one) on the same message
            std::vector<uint8_t> mine(ecc);
            rs256_encode_one<W>(cw.data(), ml, lut16, mine.data(), ecc);
            if (mine != par) {
                if (bad < 5) std::printf("encode ecc %d msg_len %d: parity differs\n", ecc, ml);
                ++bad;
            }
        }
        std::memcpy(cw.data() + ml, par.data(), ecc);
        // 0 .. ecc/2 + 3 corrupted bytes (some past the capacity)
        const int k = (int)(g() % (unsigned)(ecc / 2 + 4));
        for (int q = 0; q < k; ++q) cw[g() % n] ^= (uint8_t)(1 + g() % 255);
        // the LFSR state after all n bytes: the encoder's remainder of the
        // whole received word
        orc_rs256_encode(rs, cw.data(), n, rem.data());
        uint32_t r[W] = {};
        for (int j = 0; j < ecc; ++j) r[j / 4] |= (uint32_t)rem[j] << (8 * (j % 4));
        std::vector<uint8_t> d(cw.begin(), cw.begin() + ml), p(cw.begin() + ml, cw.end());
        std::vector<uint8_t> dr = d, pr = p;
        const int ok = orc_rs256_decode(rs, dr.data(), ml, pr.data());
        uint32_t any = 0;
        for (int w = 0; w < W; ++w) any |= r[w];
        uint8_t st = 1;
        if (any) {
            std::memset(scratch.data(), 0xA5, scratch.size());  // stale bytes must not matter
            const DecodeScratchG sc(scratch.data(), 0, 1, ecc);
            synds_from_rem<W>(r, ecc, ex, lg, sc);
            decode_solve(d.data(), p.data(), ml, ecc, ex, lg, sc, &st);
        }
        // the whole per-thread decoder from the received bytes
        std::vector<uint8_t> d1(cw.begin(), cw.begin() + ml), p1(cw.begin() + ml, cw.end());
        uint8_t st1 = 9;
        {
            std::memset(scratch.data(), 0x5A, scratch.size());
            const DecodeScratchG sc(scratch.data(), 0, 1, ecc);
            decode_one<W>(d1.data(), p1.data(), ml, ecc, lut16, gex, gf.log, sc, &st1, nullptr);
        }
        if ((int)st1 != (ok ? 1 : 0) || d1 != dr || p1 != pr) {
            if (bad < 5)
                std::printf("decode_one ecc %d msg_len %d corrupted %d: status %d oracle %d\n", ecc, ml, k, st1, ok);
            ++bad;
        }
        if ((int)st != (ok ? 1 : 0) || d != dr || p != pr) {
            if (bad < 5)
                std::printf("ecc %d msg_len %d corrupted %d: status %d oracle %d bytes %s\n", ecc, ml, k, st, ok,
                            d == dr && p == pr ? "same" : "differ");
            ++bad;
        }
    }
    orc_rs256_free(rs);
    return bad;
}

int main(int argc, char **argv) {
    std::mt19937 g(argc > 1 ? (unsigned)std::atoi(argv[1]) : 1u);
    const int n = argc > 2 ? std::atoi(argv[2]) : 2000;
    int bad = 0;
    bad += run<1>(1, n, g);
    bad += run<1>(2, n, g);
    bad += run<1>(4, n, g);
    bad += run<2>(6, n, g);
    bad += run<2>(8, n, g);
    bad += run<4>(13, n, g);
    bad += run<4>(16, n, g);
    bad += run<8>(32, n, g);
    bad += run<16>(64, n, g);
    bad += run<32>(100, n / 4 + 1, g);
    bad += run<64>(254, n / 20 + 1, g);
    std::printf("bad %d\n", bad);
    return bad != 0;
}
