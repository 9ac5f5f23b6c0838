// The RSi16 repair paths of the GPU (rsi16_device.cuh) run on the host with
// the warp emulated by 32 threads in lock step (stub/warp_emu.h), on the
// oracle's own code tables, block by block against the oracle's
// RSi16v::_repair (rsi16v_impl.hpp:122-231): same status, same words.
//   unknown positions, ecc 32/64: 32-block batches with a Berlekamp-Massey
//     per lane (rsi16_repair32), the step-for-step mirror for the rest;
//   unknown positions, other ecc: the per-block bounded-distance path
//     (rsi16_repair_bm_block_t: sub-warp transforms for ecc 2..16, registers
//     for ecc 128), the mirror (rsi16_repair_block) when it declines;
//   known positions: rsi16_repair_known_block.
// Usage: rsi16_repair_check <seed> <batches of 32 blocks per code>; prints
// "bad N", exits 1 if N > 0.
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

struct HostCode {
    orc_rsi16 *o = nullptr;
    std::vector<uint32_t> inv;
    Rsi16Dev c{};
    HostCode(size_t block_len, size_t ecc) {
        char err[256];
        o = orc_rsi16_new(block_len, ecc, 3, err, sizeof err);
        if (!o) {
            std::printf("oracle: %s\n", err);
            std::exit(2);
        }
        const uint32_t *ex = tab(o, 9), *lg = tab(o, 10);
        inv.resize(65537);
        for (uint32_t a = 0; a < 65537; ++a) inv[a] = ex[65536u - lg[a]];  // inv(0) == 1, as the reference's table
        const size_t ntt = orc_rsi16_ntt_len(o);
        c.roots_ntt = tab(o, 0);
        c.roots_ecc = tab(o, 1);
        c.roots_i_ecc = tab(o, 2);
        c.pntt_shift = tab(o, 3);
        c.pintt_shift = tab(o, 4);
        c.ecc_mix = tab(o, 5);
        c.rbo_ecc = tab(o, 6);
        c.roots_ecc2 = tab(o, 7);
        c.roots_i_ecc2 = tab(o, 8);
        c.inv_tab = inv.data();
        c.block_len = (uint32_t)block_len;
        c.message_len = (uint32_t)(block_len - ecc);
        c.ecc = (uint32_t)ecc;
        c.ntt_len = (uint32_t)ntt;
        c.pntt_blocks = (uint32_t)(block_len / ecc);
        c.ecc_mask = (uint32_t)(ecc - 1);
        c.rbo_shift = 16u - (unsigned)__builtin_ctzl(ntt);
        c.ecc_len_i = inv[ecc];
        c.ecc2_len_i = inv[2 * ecc];
        c.temp_len = (uint32_t)(ntt + 6 * ecc);
    }
    ~HostCode() { orc_rsi16_free(o); }
};

// a received word: 0 .. ecc/2 + 3 words changed (uint16 values, as stored)
static void corrupt(std::mt19937 &g, uint16_t *w, size_t n, size_t k) {
    for (size_t q = 0; q < k; ++q) w[g() % n] = (uint16_t)g();
}

static uint32_t pmul(uint32_t a, uint32_t b) { return (uint32_t)((uint64_t)a * b % 65537u); }
static uint32_t ppow(uint32_t a, uint32_t e) {
    uint32_t r = 1;
    for (; e; e >>= 1, a = pmul(a, a))
        if (e & 1) r = pmul(r, a);
    return r;
}

// A received word whose top syndrome S_{ecc-1} = sum_k e_k X_k^{ecc-1} is
// zero (X_i = w^rbo(i), the reference's syndromes): k - 1 random errors and
// a last one that cancels their top syndrome, all within the capacity.  The
// reference's key-equation solver then meets a first quotient of degree two,
// which it does not handle (its result is only reproduced by the mirror).
static void corrupt_top_zero(std::mt19937 &g, const HostCode &h, uint16_t *w, size_t n, size_t ecc) {
    for (int attempt = 0; attempt < 64; ++attempt) {
        const size_t k = 2 + g() % (ecc / 2 - 1);
        std::vector<uint32_t> pos;
        while (pos.size() < k) {
            const uint32_t p = g() % n;
            bool seen = false;
            for (uint32_t q : pos) seen |= q == p;
            if (!seen) pos.push_back(p);
        }
        std::vector<uint32_t> nv(k);
        uint32_t top = 0;
        bool ok = true;
        for (size_t q = 0; q + 1 < k; ++q) {
            const uint32_t e = 1 + g() % 65536u;
            nv[q] = (w[pos[q]] + e) % 65537u;
            ok &= nv[q] != 65536u;
            top = (top + pmul(e, ppow(h.c.roots_ntt[orc_rsi16_rbo(h.o, pos[q])], (uint32_t)ecc - 1))) % 65537u;
        }
        const uint32_t xl = ppow(h.c.roots_ntt[orc_rsi16_rbo(h.o, pos[k - 1])], (uint32_t)ecc - 1);
        const uint32_t el = pmul(65537u - top, ppow(xl, 65535u));
        nv[k - 1] = (w[pos[k - 1]] + el) % 65537u;
        ok &= el != 0 && nv[k - 1] != 65536u;
        if (!ok) continue;
        for (size_t q = 0; q < k; ++q) w[pos[q]] = (uint16_t)nv[q];
        return;
    }
}

template <int EPL>
static int run_unknown(size_t block_len, size_t ecc, size_t nbatch, std::mt19937 &g) {
    HostCode h(block_len, ecc);
    const size_t ml = block_len - ecc, nb = nbatch * 32;
    std::vector<uint16_t> msg(nb * ml), par(nb * ecc);
    for (auto &x : msg) x = (uint16_t)g();
    orc_rsi16_encode_blocks(h.o, msg.data(), nb, par.data(), 1);
    std::vector<uint16_t> cw(block_len);
    for (size_t b = 0; b < nb; ++b) {
        std::memcpy(cw.data(), &msg[b * ml], ml * 2);
        std::memcpy(cw.data() + ml, &par[b * ecc], ecc * 2);
        if (b % 4 == 3 && ecc >= 4)
            corrupt_top_zero(g, h, cw.data(), block_len, ecc);
        else
            corrupt(g, cw.data(), block_len, g() % (ecc / 2 + 4));
        std::memcpy(&msg[b * ml], cw.data(), ml * 2);
        std::memcpy(&par[b * ecc], cw.data() + ml, ecc * 2);
    }
    std::vector<uint16_t> om = msg, op = par;
    std::vector<int8_t> os(nb);
    orc_rsi16_repair_blocks(h.o, om.data(), op.data(), nb, os.data(), 1);
    std::vector<uint8_t> st(nb, 0xEE);
    const BlockView v = contiguous_view(msg.data(), true, ml, par.data(), true, ecc);
    const size_t cols = (ecc + ecc / 2 + 1) * kColStride + 3 * ecc + 4;
    std::vector<uint32_t> ws(cols + h.c.temp_len + 1), mws(h.c.temp_len + 1);
    on_warp([&](int lane) {
        RegTw<EPL ? EPL : 1> tw;
        if constexpr (EPL > 0) reg_twiddles<EPL>(h.c, lane, tw);
        if constexpr (EPL == 1 || EPL == 2) {
            unsigned long long nf = 0, nm = 0;
            for (size_t base = 0; base < nb; base += 32)
                rsi16_repair32<EPL>(h.c, v, base, 32, st.data(), nullptr, tw, lane, ws.data(), mws.data(), nf, nm);
        } else {
            for (size_t b = 0; b < nb; ++b)
                if (!rsi16_repair_bm_block_t<EPL>(h.c, v, b, ws.data(), st.data(), tw, lane))
                    rsi16_repair_block(h.c, v, b, ws.data(), st.data(), lane);
        }
    });
    int bad = 0;
    for (size_t b = 0; b < nb; ++b) {
        const int want = os[b] < 0 ? 255 : os[b];
        const bool same = std::memcmp(&msg[b * ml], &om[b * ml], ml * 2) == 0 &&
                          std::memcmp(&par[b * ecc], &op[b * ecc], ecc * 2) == 0;
        if (st[b] != want || !same) {
            if (bad < 3)
                std::printf("unknown: ecc %zu block_len %zu block %zu: status %d oracle %d words %s\n", ecc, block_len,
                            b, st[b], want, same ? "same" : "differ");
            ++bad;
        }
    }
    return bad;
}

static int run_known(size_t block_len, size_t ecc, size_t nblocks, std::mt19937 &g) {
    HostCode h(block_len, ecc);
    const size_t ml = block_len - ecc;
    std::vector<uint16_t> msg(ml), par(ecc);
    std::vector<uint32_t> blk(block_len), temp(h.c.temp_len + 1), pos, rpos;
    int bad = 0;
    for (size_t t = 0; t < nblocks; ++t) {
        for (auto &x : msg) x = (uint16_t)g();
        orc_rsi16_encode_blocks(h.o, msg.data(), 1, par.data(), 1);
        // count listed positions (distinct), some of them changed
        const size_t count = 1 + g() % ecc;
        pos.clear();
        while (pos.size() < count) {
            const uint32_t p = g() % block_len;
            bool seen = false;
            for (uint32_t q : pos) seen |= q == p;
            if (!seen) pos.push_back(p);
        }
        for (uint32_t p : pos)
            if (g() % 2) (p < ml ? msg[p] : par[p - ml]) = (uint16_t)g();
        // oracle on uint32 words with rbo positions, stored back as uint16
        for (size_t k = 0; k < ml; ++k) blk[k] = msg[k];
        for (size_t k = 0; k < ecc; ++k) blk[ml + k] = par[k];
        rpos.assign(count + 1, 0);
        for (size_t i = 0; i < count; ++i) rpos[i] = orc_rsi16_rbo(h.o, pos[i]);
        const int want = orc_rsi16_repair_known(h.o, blk.data(), rpos.data(), count, temp.data());
        uint8_t st = 0xEE;
        const BlockView v = contiguous_view(msg.data(), true, ml, par.data(), true, ecc);
        std::vector<uint32_t> ws(h.c.temp_len + 1);
        on_warp([&](int lane) { rsi16_repair_known_block(h.c, v, 0, pos.data(), (uint32_t)count, ws.data(), &st, lane); });
        bool same = true;
        for (size_t k = 0; k < ml; ++k) same &= msg[k] == (uint16_t)blk[k];
        for (size_t k = 0; k < ecc; ++k) same &= par[k] == (uint16_t)blk[ml + k];
        if ((int)st != (want < 0 ? 255 : want) || !same) {
            if (bad < 3)
                std::printf("known: ecc %zu block_len %zu count %zu: status %d oracle %d words %s\n", ecc, block_len,
                            count, st, want, same ? "same" : "differ");
            ++bad;
        }
    }
    return bad;
}

int main(int argc, char **argv) {
    std::mt19937 g(argc > 1 ? (unsigned)std::atoi(argv[1]) : 1u);
    const size_t nbatch = argc > 2 ? (size_t)std::atoi(argv[2]) : 2;
    int bad = 0;
    bad += run_unknown<1>(256, 32, nbatch, g);
    bad += run_unknown<2>(1024, 64, nbatch, g);
    bad += run_unknown<0>(128, 8, nbatch, g);
    bad += run_unknown<0>(96, 16, nbatch, g);
    bad += run_unknown<0>(130, 2, nbatch, g);
    bad += run_unknown<4>(512, 128, 1, g);
    bad += run_known(128, 8, 16 * nbatch, g);
    bad += run_known(256, 32, 8 * nbatch, g);
    bad += run_known(96, 16, 8 * nbatch, g);
    std::printf("bad %d\n", bad);
    return bad != 0;
}
