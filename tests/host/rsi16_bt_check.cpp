// The lazily reduced arithmetic of the one-block-per-thread RSi16 kernels
// (rsi16_bt.cuh), run on the host block by block against the oracle on the
// oracle's own code tables:
//   bt_pntt_chunk over the message chunks, then bt_parity: the parity of a
//     block (CT transform, pntt_shift accumulation, mix, GS transform), as
//     the kernels store it, against the oracle's encode;
//   bt_pntt_chunk over every chunk of a received word: its syndromes, against
//     the oracle's syndromes;
//   bt_rev_bm: the lane Berlekamp-Massey on lazy values, against the
//     canonical one of the warp-batch path (rsi16_rev_bm_lane): same length,
//     same connection polynomial, on the syndromes of the received words and
//     on synthetic syndrome columns.
// ecc 32 and 64, block lengths from two chunks to 65536 words, random words
// and words of all 65535 (the largest lazy sums).  The largest accumulator
// seen is checked against the bound the code assumes (below 2^28 before the
// final reduction).
// Usage: rsi16_bt_check <seed> <blocks per code>; prints "bad N", exits 1 if
// N > 0.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

#include "warp_emu.h"
#include "rsi16_bt.cuh"
extern "C" {
#include "ffrs_oracle.h"
}
using namespace ffgpu;

static const uint32_t *tab(const orc_rsi16 *o, int which) {
    size_t n = 0;
    return orc_rsi16_table(o, which, &n);
}

static uint32_t shoup(uint32_t w) { return (uint32_t)(((uint64_t)w << 32) / 0x10001u); }

static uint32_t acc_max = 0;

// the accumulator of bt_pntt over chunks [0, nch) of one block (words at w)
template <int N>
static void pntt_block(const Rsi16Dev &c, const BtTw<N> &tw, const uint16_t *w, uint32_t nch, uint32_t (&acc)[N]) {
    for (uint32_t ch = 0; ch < nch; ++ch) {
        uint32_t x[N];
        for (int k = 0; k < N; ++k) x[k] = w[(size_t)ch * N + k];
        bt_pntt_chunk<N>(c, tw, x, ch, acc);
    }
    for (int k = 0; k < N; ++k) acc_max = std::max(acc_max, acc[k]);
}

template <int N>
static int run(size_t block_len, size_t nb, std::mt19937 &g) {
    constexpr int T = N / 2;
    char err[256];
    orc_rsi16 *o = orc_rsi16_new(block_len, N, 3, err, sizeof err);
    if (!o) {
        std::printf("oracle: %s\n", err);
        return 1;
    }
    const size_t ml = block_len - N;
    const uint32_t *ex = tab(o, 9), *lg = tab(o, 10);
    std::vector<uint32_t> inv(65537), ps_s(block_len);
    for (uint32_t a = 0; a < 65537; ++a) inv[a] = ex[65536u - lg[a]];
    const uint32_t *ps = tab(o, 3);
    for (size_t i = 0; i < block_len; ++i) ps_s[i] = shoup(ps[i]);
    Rsi16Dev c{};
    c.roots_ecc = tab(o, 1);
    c.roots_i_ecc = tab(o, 2);
    c.pntt_shift = ps;
    c.pntt_shift_s = ps_s.data();
    c.ecc_mix = tab(o, 5);
    c.inv_tab = inv.data();
    c.block_len = (uint32_t)block_len;
    c.message_len = (uint32_t)ml;
    c.ecc = N;
    c.pntt_blocks = (uint32_t)(block_len / N);
    BtTw<N> tw;
    for (int i = 0; i < N / 2; ++i) {
        tw.ct[i] = c.roots_ecc[i];
        tw.gs[i] = c.roots_i_ecc[i];
        tw.ct_s[i] = shoup(tw.ct[i]);
        tw.gs_s[i] = shoup(tw.gs[i]);
    }
    for (int i = 0; i < N; ++i) {
        tw.mix[i] = c.ecc_mix[i];
        tw.mix_s[i] = shoup(tw.mix[i]);
    }

    std::vector<uint16_t> msg(nb * ml), par(nb * N);
    for (size_t b = 0; b < nb; ++b)
        for (size_t i = 0; i < ml; ++i) msg[b * ml + i] = b % 8 == 7 ? 65535u : (uint16_t)g();
    orc_rsi16_encode_blocks(o, msg.data(), nb, par.data(), 1);
    int bad = 0;
    std::vector<uint16_t> cw(block_len);
    std::vector<uint32_t> cw32(block_len), S(N), Scol(N * 33);
    for (size_t b = 0; b < nb; ++b) {
        // encode, as bt_encode_tile stores the parity
        uint32_t acc[N];
        pntt_block<N>(c, tw, &msg[b * ml], c.pntt_blocks - 1, acc);
        bt_parity<N>(tw, acc);
        bool enc_ok = true;
        for (int k = 0; k < N; ++k) enc_ok &= (uint16_t)(ucanon(acc[k]) & 0xffffu) == par[b * N + k];
        if (!enc_ok) {
            if (bad < 3) std::printf("encode: ecc %d block_len %zu block %zu differs\n", N, block_len, b);
            ++bad;
        }
        // a received word: the codeword with 0 .. T + 4 words changed, or all
        // 65535 for one block in eight
        std::memcpy(cw.data(), &msg[b * ml], ml * 2);
        std::memcpy(cw.data() + ml, &par[b * N], N * 2);
        if (b % 8 == 3)
            std::fill(cw.begin(), cw.end(), (uint16_t)65535u);
        else
            for (size_t q = 0, k = g() % (T + 5); q < k; ++q) cw[g() % block_len] = (uint16_t)g();
        for (size_t i = 0; i < block_len; ++i) cw32[i] = cw[i];
        orc_rsi16_synd(o, cw32.data(), S.data());
        pntt_block<N>(c, tw, cw.data(), c.pntt_blocks, acc);
        bool syn_ok = true;
        for (int k = 0; k < N; ++k) {
            const uint32_t s = ucanon(acc[k]);
            syn_ok &= s == S[k];
            Scol[k * 33] = s;
        }
        if (!syn_ok) {
            if (bad < 3) std::printf("syndromes: ecc %d block_len %zu block %zu differ\n", N, block_len, b);
            ++bad;
            continue;
        }
        // Berlekamp-Massey on the reversed syndromes, lazy against canonical
        int32_t Cl[T + 1];
        uint32_t Cc[T + 1];
        const uint32_t Ll = bt_rev_bm<T, N>(Scol.data(), inv.data(), Cl);
        const uint32_t Lc = rsi16_rev_bm_lane<T>(Scol.data(), inv.data(), N, Cc);
        bool bm_ok = Ll == Lc;
        if (bm_ok && Lc)
            for (int i = 0; i <= T; ++i) bm_ok &= (uint32_t)Cl[i] == Cc[i];
        if (!bm_ok) {
            if (bad < 3)
                std::printf("berlekamp-massey: ecc %d block_len %zu block %zu: L %u, canonical %u\n", N, block_len, b,
                            Ll, Lc);
            ++bad;
        }
    }
    orc_rsi16_free(o);
    return bad;
}

// bt_rev_bm against rsi16_rev_bm_lane on synthetic syndrome columns, not
// only those of error patterns: random values, values that are zero with
// probability 1/2 or 7/8, zero runs at either end, one non-zero value, and
// values 0 / 65536 only; these reach the stalled and abnormal branches
template <int N>
static int run_bm_synthetic(size_t count, std::mt19937 &g) {
    constexpr int T = N / 2;
    char err[256];
    orc_rsi16 *o = orc_rsi16_new(N * 4, N, 3, err, sizeof err);
    if (!o) {
        std::printf("oracle: %s\n", err);
        return 1;
    }
    const uint32_t *ex = tab(o, 9), *lg = tab(o, 10);
    std::vector<uint32_t> inv(65537);
    for (uint32_t a = 0; a < 65537; ++a) inv[a] = ex[65536u - lg[a]];
    std::vector<uint32_t> Scol(N * 33);
    int bad = 0, abnormal = 0;
    for (size_t t = 0; t < count; ++t) {
        const int kind = (int)(t % 6);
        for (int k = 0; k < N; ++k) {
            uint32_t v = g() % 65537u;
            if (kind == 1 && (g() & 1)) v = 0;
            if (kind == 2 && (g() & 7)) v = 0;
            if (kind == 3) {
                const int cut = (int)(g() % N);
                if ((t / 6) & 1 ? k < cut : k >= cut) v = 0;
            }
            if (kind == 4) v = k == (int)(t / 6 % N) ? v : 0;
            if (kind == 5) v = (g() & 1) ? 65536u : 0u;
            Scol[k * 33] = v;
        }
        int32_t Cl[T + 1];
        uint32_t Cc[T + 1];
        const uint32_t Ll = bt_rev_bm<T, N>(Scol.data(), inv.data(), Cl);
        const uint32_t Lc = rsi16_rev_bm_lane<T>(Scol.data(), inv.data(), N, Cc);
        abnormal += Lc == 0;
        bool ok = Ll == Lc;
        if (ok && Lc)
            for (int i = 0; i <= T; ++i) ok &= (uint32_t)Cl[i] == Cc[i];
        if (!ok) {
            if (bad < 3) std::printf("synthetic berlekamp-massey: ecc %d case %zu kind %d: L %u, canonical %u\n", N, t,
                                     kind, Ll, Lc);
            ++bad;
        }
    }
    std::printf("ecc %d: %zu synthetic columns, %d declined by both\n", N, count, abnormal);
    orc_rsi16_free(o);
    return bad;
}

int main(int argc, char **argv) {
    std::mt19937 g(argc > 1 ? (unsigned)std::atoi(argv[1]) : 1u);
    const size_t nb = argc > 2 ? (size_t)std::atoi(argv[2]) : 64;
    int bad = 0;
    for (size_t bl : {64, 256, 1024, 4096}) bad += run<32>(bl, nb, g);
    for (size_t bl : {128, 1024, 4096}) bad += run<64>(bl, nb, g);
    bad += run<32>(65536, 8, g);
    bad += run<64>(65536, 8, g);
    bad += run_bm_synthetic<32>(nb * 200, g);
    bad += run_bm_synthetic<64>(nb * 200, g);
    if (acc_max >= (1u << 28)) {
        std::printf("accumulator %u reached 2^28\n", acc_max);
        ++bad;
    }
    std::printf("largest accumulator %u\nbad %d\n", acc_max, bad);
    return bad != 0;
}
