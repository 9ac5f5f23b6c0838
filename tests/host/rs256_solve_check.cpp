// The per-thread RS256 decoder of the GPU table path (remainder -> syndromes,
// Berlekamp-Massey, Chien search, Forney: rs256_device.cuh), compiled for the
// host and run block by block against the oracle's rs_decode::decode
// (reed_solomon.hpp:559-595): same status, same bytes.  Usage:
// rs256_solve_check <seed> <trials per ecc>; prints "bad N", exits 1 if N > 0.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

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
    int bad = 0;
    for (int t = 0; t < trials; ++t) {
        const int ml = 1 + (int)(g() % (unsigned)(255 - ecc));
        const int n = ml + ecc;
        std::vector<uint8_t> cw(n), par(ecc), rem(ecc);
        for (int i = 0; i < ml; ++i) cw[i] = (uint8_t)g();
        orc_rs256_encode(rs, cw.data(), ml, par.data());
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
