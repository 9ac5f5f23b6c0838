// The nibble-table RS256 encoder (rs256_nib.cuh: the tables, their layout
// and one lane's part of a block, the code rs256_encode_nib_kernel runs) on
// the host, block by block against the oracle's encode.  For every block the
// four lanes r of each parity half h are run and XORed, as the kernel's
// shuffles do.  The staged table is exactly the kernel's shared-memory part
// (the line groups of degree indices 0 .. ml - 1) with poison on both sides,
// and the message buffer starts at 0, 4, 8 or 12 bytes past a 16-byte
// boundary with poison around it (for 4 and 12 and an odd message length it
// also ends inside a 4-byte word), so a read outside either shows up as a
// wrong parity byte.
// Usage: rs256_nib_check <seed> <blocks per case>; prints "bad N", exits 1 if
// N > 0.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

#include "rs256_nib.cuh"
extern "C" {
#include "ffrs_oracle.h"
}
using namespace ffgpu;

static int run(const orc_rs256 *o, const std::vector<uint32_t> &tab, int ml, size_t nb_even, int offset,
               std::mt19937 &g) {
    // an odd block count for offsets 4 and 12: with an odd ml the buffer then
    // ends inside a 4-byte word
    const size_t nb = nb_even - ((offset & 4) ? 1 : 0);
    // staged table: ceil(ml / 4) line groups between poisoned guards
    const size_t groups = (size_t)(ml + 3) / 4, guard = kNibGroupQ;
    std::vector<uint4> stage(guard + groups * kNibGroupQ + guard);
    for (auto &q : stage) q = make_uint4(0xa5a5a5a5u, 0x5a5a5a5au, 0xc3c3c3c3u, 0x3c3c3c3cu);
    std::memcpy(&stage[guard], tab.data(), groups * kNibGroupQ * 16);
    const uint4 *T = &stage[guard];
    // messages back to back, offset bytes past a 16-byte boundary
    std::vector<uint4> raw((nb * ml + offset + 64) / 16 + 2);
    uint8_t *base = reinterpret_cast<uint8_t *>(raw.data());
    std::memset(base, 0x77, raw.size() * 16);
    uint8_t *data = base + 16 + offset;
    for (size_t i = 0; i < nb * (size_t)ml; ++i) data[i] = (uint8_t)g();
    if (nb > 1) std::memset(data, 0xff, ml);  // one all-255 message
    std::vector<uint8_t> want(nb * 32);
    orc_rs256_encode_buffer(o, data, nb * ml, ml, want.data(), 1);
    const uintptr_t d0 = (uintptr_t)data, d1 = d0 + nb * (size_t)ml;
    int bad = 0;
    for (size_t b = 0; b < nb; ++b) {
        uint8_t got[32];
        for (int h = 0; h < 2; ++h) {
            uint4 acc = make_uint4(0u, 0u, 0u, 0u);
            for (int r = 0; r < 4; ++r) {
                const uint4 x = nib_lane(T, d0, d1, b, ml, r, h);
                acc.x ^= x.x, acc.y ^= x.y, acc.z ^= x.z, acc.w ^= x.w;
            }
            std::memcpy(got + 16 * h, &acc, 16);
        }
        if (std::memcmp(got, &want[b * 32], 32) != 0) {
            if (bad < 3) std::printf("ml %d offset %d block %zu: parity differs\n", ml, offset, b);
            ++bad;
        }
    }
    return bad;
}

int main(int argc, char **argv) {
    std::mt19937 g(argc > 1 ? (unsigned)std::atoi(argv[1]) : 1u);
    const size_t nb = argc > 2 ? (size_t)std::atoi(argv[2]) : 64;
    orc_rs256 *o = orc_rs256_new(32, 2, 0x11d);
    uint8_t gen[33], roots[32];
    orc_rs256_generator(o, gen, roots);
    const std::vector<uint32_t> tab = nib_tables(gen + 1);  // x^32 mod g
    int bad = 0;
    for (int ml : {223, 222, 221, 220, 200, 161, 100, 33, 17, 16, 15, 4, 3, 1})
        for (int offset : {0, 4, 8, 12}) bad += run(o, tab, ml, nb, offset, g);
    orc_rs256_free(o);
    std::printf("bad %d\n", bad);
    return bad != 0;
}
