/* Host emulation of the warp intrinsics used by the device headers: 32
 * std::threads run one warp in lock step and meet at a barrier at every
 * shuffle, vote, reduction and __syncwarp (the code under test calls them at
 * warp-uniform points only).  Test infrastructure, not product code. */
#pragma once
#include <atomic>
#include <cstdint>
#include <thread>

namespace warp_emu {
// a yielding spin barrier (the lanes meet thousands of times per block)
struct Barrier {
    std::atomic<int> count{0}, gen{0};
    int n;
    explicit Barrier(int n_) : n(n_) {}
    void arrive_and_wait() {
        const int g = gen.load(std::memory_order_acquire);
        if (count.fetch_add(1, std::memory_order_acq_rel) == n - 1) {
            count.store(0, std::memory_order_relaxed);
            gen.fetch_add(1, std::memory_order_release);
        } else {
            while (gen.load(std::memory_order_acquire) == g) std::this_thread::yield();
        }
    }
};
inline thread_local int lane = 0;
inline Barrier *bar = nullptr;
inline uint32_t xchg[32];
}  // namespace warp_emu

inline void __syncwarp(unsigned = 0xffffffffu) { warp_emu::bar->arrive_and_wait(); }
inline uint32_t __shfl_sync(unsigned, uint32_t v, int src) {
    warp_emu::xchg[warp_emu::lane] = v;
    warp_emu::bar->arrive_and_wait();
    const uint32_t r = warp_emu::xchg[src & 31];
    warp_emu::bar->arrive_and_wait();
    return r;
}
inline uint32_t __shfl_xor_sync(unsigned m, uint32_t v, int o) { return __shfl_sync(m, v, warp_emu::lane ^ o); }
inline unsigned __ballot_sync(unsigned, int p) {
    warp_emu::xchg[warp_emu::lane] = p != 0;
    warp_emu::bar->arrive_and_wait();
    unsigned m = 0;
    for (int i = 0; i < 32; ++i) m |= warp_emu::xchg[i] << i;
    warp_emu::bar->arrive_and_wait();
    return m;
}
inline int __any_sync(unsigned m, int p) { return __ballot_sync(m, p) != 0; }
inline unsigned __reduce_add_sync(unsigned, unsigned v) {
    warp_emu::xchg[warp_emu::lane] = v;
    warp_emu::bar->arrive_and_wait();
    unsigned s = 0;
    for (int i = 0; i < 32; ++i) s += warp_emu::xchg[i];
    warp_emu::bar->arrive_and_wait();
    return s;
}
inline unsigned __reduce_max_sync(unsigned, unsigned v) {
    warp_emu::xchg[warp_emu::lane] = v;
    warp_emu::bar->arrive_and_wait();
    unsigned s = 0;
    for (int i = 0; i < 32; ++i) s = s > warp_emu::xchg[i] ? s : warp_emu::xchg[i];
    warp_emu::bar->arrive_and_wait();
    return s;
}
inline int __popc(unsigned x) { return __builtin_popcount(x); }
inline int __ffs(unsigned x) { return __builtin_ffs((int)x); }
