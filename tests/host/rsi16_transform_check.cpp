// The RSi16 register transforms of the GPU path (rsi16_device.cuh), run on
// the host with the warp emulated by 32 threads in lock step
// (stub/warp_emu.h) on the oracle's own code tables, block by block against
// the oracle:
//   ecc 2..16: sub-warp syndromes of one block (sub_synd_one) and encodes of
//              32/ecc blocks per pass (rsi16_encode_sub_pass);
//   ecc 32, 64: syndromes and encodes two blocks per pass (reg_pntt2,
//              rsi16_encode_pair_reg).
// Usage: rsi16_transform_check <seed> <blocks per code>; prints "bad N",
// exits 1 if N > 0.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <thread>
#include <vector>

#include "warp_emu.h"
#include "rsi16_device.cuh"
extern "C" {
#include "ffrs_oracle.h"
}
using namespace ffgpu;

static const uint32_t *tab(const orc_rsi16 *o, int which) {
    size_t n = 0;
    return orc_rsi16_table(o, which, &n);
}

template <typename F>
static void on_warp(F f) {
    warp_emu::Barrier bar(32);
    warp_emu::bar = &bar;
    std::vector<std::thread> th;
    for (int l = 0; l < 32; ++l)
        th.emplace_back([&, l] {
            warp_emu::lane = l;
            f(l);
        });
    for (auto &t : th) t.join();
}

template <int N>
static int run(size_t block_len, size_t nb, std::mt19937 &g) {
    char err[256];
    orc_rsi16 *o = orc_rsi16_new(block_len, N, 3, err, sizeof err);
    if (!o) {
        std::printf("oracle: %s\n", err);
        return 1;
    }
    const size_t ml = block_len - N;
    Rsi16Dev c{};
    c.roots_ecc = tab(o, 1);
    c.roots_i_ecc = tab(o, 2);
    c.pntt_shift = tab(o, 3);
    c.ecc_mix = tab(o, 5);
    c.block_len = (uint32_t)block_len;
    c.message_len = (uint32_t)ml;
    c.ecc = N;
    c.pntt_blocks = (uint32_t)(block_len / N);
    std::vector<uint16_t> msg(nb * ml), par(nb * N), out(nb * N);
    for (auto &x : msg) x = (uint16_t)g();
    for (auto &x : par) x = (uint16_t)g();
    const BlockView v = contiguous_view(msg.data(), true, ml, par.data(), true, N);
    const BlockView ve = contiguous_view(msg.data(), true, ml, out.data(), true, N);
    std::vector<uint32_t> synd(nb * N);
    on_warp([&](int lane) {
        if constexpr (N < 32) {
            for (size_t b = 0; b < nb; ++b) sub_synd_one<N>(c, v, b, synd.data() + b * N, lane);
            SubTw<N> tw;
            sub_twiddles<N>(c, lane % N, tw);
            for (size_t b0 = 0; b0 < nb; b0 += 32 / N) rsi16_encode_sub_pass<N>(c, ve, b0, nb, tw, lane);
        } else {
            constexpr int EPL = N / 32;
            RegTw<EPL> tw;
            reg_twiddles<EPL>(c, lane, tw);
            for (size_t b = 0; b < nb; b += 2) {
                const size_t b1 = b + 1 < nb ? b + 1 : b;
                uint32_t a0[EPL], a1[EPL];
                reg_pntt2<EPL>(c, v, b, b1, c.pntt_blocks, true, tw, lane, a0, a1);
                for (int h = 0; h < EPL; ++h) {
                    synd[b * N + lane * EPL + h] = a0[h];
                    synd[b1 * N + lane * EPL + h] = a1[h];
                }
                rsi16_encode_pair_reg<EPL>(c, ve, b, b1, tw, lane);
            }
        }
    });
    int bad = 0;
    std::vector<uint32_t> blk(block_len), want(N);
    for (size_t b = 0; b < nb; ++b) {
        for (size_t k = 0; k < ml; ++k) blk[k] = msg[b * ml + k];
        for (size_t k = 0; k < N; ++k) blk[ml + k] = par[b * N + k];
        orc_rsi16_synd(o, blk.data(), want.data());
        if (std::memcmp(want.data(), synd.data() + b * N, N * 4) != 0) {
            if (bad < 3) std::printf("ecc %d block_len %zu block %zu: syndromes differ\n", N, block_len, b);
            ++bad;
        }
    }
    std::vector<uint16_t> pe(nb * N);
    orc_rsi16_encode_blocks(o, msg.data(), nb, pe.data(), 1);
    for (size_t b = 0; b < nb; ++b)
        if (std::memcmp(pe.data() + b * N, out.data() + b * N, N * 2) != 0) {
            if (bad < 6) std::printf("ecc %d block_len %zu block %zu: parity differs\n", N, block_len, b);
            ++bad;
        }
    orc_rsi16_free(o);
    return bad;
}

int main(int argc, char **argv) {
    std::mt19937 g(argc > 1 ? (unsigned)std::atoi(argv[1]) : 1u);
    const size_t nb = argc > 2 ? (size_t)std::atoi(argv[2]) : 40;
    int bad = 0;
    bad += run<2>(130, nb, g);
    bad += run<4>(60, nb, g);
    bad += run<8>(128, nb, g);
    bad += run<8>(32, nb, g);
    bad += run<16>(96, nb, g);
    bad += run<16>(16, nb, g);
    bad += run<32>(256, nb, g);
    bad += run<64>(1024, nb / 2 + 1, g);
    std::printf("bad %d\n", bad);
    return bad != 0;
}
