// The generated GF(2) networks of the bitsliced RS256 syndrome kernel
// (rs256_synd_gen.cuh: the 32-degree Horner step per bit plane and the
// recombination of the planes into S_j) run on the host over groups of 32
// random codewords, shortened ones included, against the oracle's syndromes
// (rs_synds_lut_pw2::synds, reed_solomon.hpp:412-453).
// Usage: rs256_synd_check <seed> <groups>; prints "bad N", exits 1 if N > 0.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

#include "cuda_runtime.h"
static inline uint32_t xor3(uint32_t a, uint32_t b, uint32_t c) { return a ^ b ^ c; }
#include "rs256_synd_gen.cuh"
extern "C" {
#include "ffrs_oracle.h"
}
using namespace ffgpu::bs;

int main(int argc, char **argv) {
    std::mt19937 g(argc > 1 ? (unsigned)std::atoi(argv[1]) : 1u);
    const int ngroups = argc > 2 ? std::atoi(argv[2]) : 64;
    orc_rs256 *o = orc_rs256_new(32, 2, 0x11d);
    int bad = 0;
    for (int gr = 0; gr < ngroups; ++gr) {
        const int ml = gr % 3 == 0 ? 1 + (int)(g() % 223) : 223;  // shortened blocks too
        const int size = ml + 32;
        std::vector<uint8_t> cw(32 * 256, 0);  // [block][degree], degree 0..255
        for (int j = 0; j < 32; ++j)
            for (int d = 0; d < size; ++d) cw[j * 256 + d] = (uint8_t)g();
        // planes: bit j of P[d][b] = bit b of the degree-d byte of block j
        std::vector<uint32_t> P(256 * 8, 0);
        for (int d = 0; d < 256; ++d)
            for (int b = 0; b < 8; ++b)
                for (int j = 0; j < 32; ++j) P[d * 8 + b] |= (uint32_t)((cw[j * 256 + d] >> b) & 1) << j;
        // rows of every plane, then the two halves of the recombination
        std::vector<uint32_t> rows(8 * kSyndRows);
        for (int b = 0; b < 8; ++b) {
            uint32_t s[kSyndRows] = {};
            for (int w = 0; w < 8; ++w) synd_step32([&](int k) { return P[(255 - 32 * w - k) * 8 + b]; }, s);
            std::memcpy(&rows[b * kSyndRows], s, sizeof s);
        }
        std::vector<uint32_t> X(kSyndRowsB * 8 * 32), out(256 * 32, 0xDEADBEEFu);
        for (int half = 0; half < 2; ++half) {
            const int r0 = half == 0 ? 0 : kSyndRowsA, nr = half == 0 ? kSyndRowsA : kSyndRowsB;
            for (int i = 0; i < nr; ++i)
                for (int b = 0; b < 8; ++b) X[(i * 8 + b) * 32] = rows[b * kSyndRows + r0 + i];
            if (half == 0) {
                synd_combine_A0(X.data(), out.data()); synd_combine_A1(X.data(), out.data());
                synd_combine_A2(X.data(), out.data()); synd_combine_A3(X.data(), out.data());
                synd_combine_A4(X.data(), out.data()); synd_combine_A5(X.data(), out.data());
                synd_combine_A6(X.data(), out.data()); synd_combine_A7(X.data(), out.data());
            } else {
                synd_combine_B0(X.data(), out.data()); synd_combine_B1(X.data(), out.data());
                synd_combine_B2(X.data(), out.data()); synd_combine_B3(X.data(), out.data());
                synd_combine_B4(X.data(), out.data()); synd_combine_B5(X.data(), out.data());
                synd_combine_B6(X.data(), out.data()); synd_combine_B7(X.data(), out.data());
            }
        }
        for (int j = 0; j < 32; ++j) {
            // the block as the reference stores it: data (highest degree first), then parity
            uint8_t data[255], par[32], want[32];
            for (int p = 0; p < size; ++p) (p < ml ? data[p] : par[p - ml]) = cw[j * 256 + (size - 1 - p)];
            orc_rs256_synds(o, data, (size_t)ml, par, want);
            for (int k = 0; k < 32; ++k) {
                uint8_t got = 0;
                for (int b = 0; b < 8; ++b) got |= (uint8_t)(((out[(8 * k + b) * 32] >> j) & 1) << b);
                if (got != want[k]) {
                    if (bad < 5) std::printf("group %d block %d ml %d S_%d: %d oracle %d\n", gr, j, ml, k, got, want[k]);
                    ++bad;
                }
            }
        }
    }
    orc_rs256_free(o);
    std::printf("bad %d\n", bad);
    return bad != 0;
}
