// The RS256 warp solve (rs256_device.cuh: decode_warp_blocks / warp_solve,
// ecc 17..64) run on the host with the warp emulated by 32 threads in lock
// step (stub/warp_emu.h), 32 blocks per pass, each block checked against the
// oracle's rs_decode::decode (reed_solomon.hpp:559-595): same status, same
// bytes.  Usage: rs256_warp_solve_check <seed> <passes per ecc>; prints
// "bad N", exits 1 if N > 0.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <thread>
#include <vector>

#include "warp_emu.h"
#include "gf256.h"
#include "rs256_device.cuh"
extern "C" {
#include "ffrs_oracle.h"
}
using namespace ffgpu;

struct Pass {
    int ecc = 0, ml = 0;
    std::vector<uint8_t> data, par;  // 32 blocks
    std::vector<uint8_t> status;
};

template <int W>
static int run(int ecc, int passes, std::mt19937 &g) {
    orc_rs256 *rs = orc_rs256_new(ecc, 2, 0x11d);
    GF256Host gf(2, 0x1d);
    std::vector<uint8_t> gen(ecc + 1), roots(ecc), lutb;
    rs256_generator(gf, ecc, gen.data(), roots.data());
    rs256_lut(gf, ecc, gen.data(), lutb);
    std::vector<uint32_t> lutv((size_t)256 * W + 4, 0);
    uint32_t *lut = lutv.data() + ((16 - ((uintptr_t)lutv.data() & 15)) & 15) / 4;
    for (int v = 0; v < 256; ++v)
        for (int j = 0; j < ecc; ++j) lut[(size_t)v * W + j / 4] |= (uint32_t)lutb[(size_t)v * ecc + j] << (8 * (j % 4));
    uint8_t ex[512];
    for (int i = 0; i < 512; ++i) ex[i] = gf.exp[i % 255];
    std::vector<uint8_t> srows(32 * warp_solve_row_bytes(ecc)), rcols((size_t)ecc * 32);
    WarpSolveSmem wsm;
    warp_emu::Barrier bar(32);
    warp_emu::bar = &bar;
    Pass P;
    int bad = 0;
    const int nb = 32;
    for (int t = 0; t < passes; ++t) {
        P.ecc = ecc;
        P.ml = 1 + (int)(g() % (unsigned)(255 - ecc));
        const int n = P.ml + ecc;
        P.data.assign((size_t)nb * P.ml, 0);
        P.par.assign((size_t)nb * ecc, 0);
        P.status.assign(nb, 9);
        for (auto &x : P.data) x = (uint8_t)g();
        for (int b = 0; b < nb; ++b) orc_rs256_encode(rs, &P.data[(size_t)b * P.ml], P.ml, &P.par[(size_t)b * ecc]);
        for (int b = 0; b < nb; ++b) {
            const int k = (int)(g() % (unsigned)(ecc / 2 + 4));
            for (int q = 0; q < k; ++q) {
                const int at = (int)(g() % (unsigned)n);
                const uint8_t v = (uint8_t)(1 + g() % 255);
                if (at < P.ml)
                    P.data[(size_t)b * P.ml + at] ^= v;
                else
                    P.par[(size_t)b * ecc + at - P.ml] ^= v;
            }
        }
        std::vector<uint8_t> rd = P.data, rp = P.par;
        std::vector<int> ok(nb);
        for (int b = 0; b < nb; ++b) ok[b] = orc_rs256_decode(rs, &rd[(size_t)b * P.ml], P.ml, &rp[(size_t)b * ecc]);
        const int nact = t % 3 == 2 ? 1 + (int)(g() % 32u) : nb;  // some passes with a partial warp
        std::vector<std::thread> th;
        for (int l = 0; l < 32; ++l)
            th.emplace_back([&, l] {
                warp_emu::lane = l;
                decode_warp_blocks<W>(P.data.data(), P.par.data(), 0, (size_t)nact, P.ml, ecc, lut, ex, gf.log,
                                      srows.data(), rcols.data(), 32, wsm, P.status.data(), l, l);
            });
        for (auto &x : th) x.join();
        for (int b = 0; b < nact; ++b) {
            const bool same = std::memcmp(&P.data[(size_t)b * P.ml], &rd[(size_t)b * P.ml], P.ml) == 0 &&
                              std::memcmp(&P.par[(size_t)b * ecc], &rp[(size_t)b * ecc], ecc) == 0;
            if ((int)P.status[b] != (ok[b] ? 1 : 0) || !same) {
                if (bad < 5)
                    std::printf("ecc %d msg_len %d block %d: status %d oracle %d bytes %s\n", ecc, P.ml, b,
                                P.status[b], ok[b], same ? "same" : "differ");
                ++bad;
            }
        }
    }
    orc_rs256_free(rs);
    return bad;
}

int main(int argc, char **argv) {
    std::mt19937 g(argc > 1 ? (unsigned)std::atoi(argv[1]) : 1u);
    const int n = argc > 2 ? std::atoi(argv[2]) : 20;
    int bad = 0;
    bad += run<8>(17, n, g);
    bad += run<8>(24, n, g);
    bad += run<8>(32, n, g);
    bad += run<16>(33, n, g);
    bad += run<16>(48, n, g);
    bad += run<16>(64, n, g);
    std::printf("bad %d\n", bad);
    return bad != 0;
}
