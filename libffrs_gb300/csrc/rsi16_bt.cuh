// RSi16 with one block per thread: the ecc-point NTTs of a block run in one
// thread's registers, 32 blocks per warp, so that every butterfly is a
// register operation (no shuffles, no selects, no duplicated multiplies) and
// the field values are reduced lazily.
//
// Lazy GF(65537) values, p = 2^16 + 1.  Every operation keeps the value's
// residue mod p, so the results are the exact field values that the
// reference's canonical arithmetic (libffrs/galois.hpp:258-346) gives; only
// outputs are brought to [0, p).  Two forms:
//
// * The transforms (bt_ct_u, bt_gs_u) keep uint32 values below a bound known
//   at compile time for each stage.  A product by a table constant w uses
//   Shoup's method with w' = floor(w 2^32 / p): for any x < 2^32,
//   x w - floor(x w' / 2^32) p lies in [0, 2p), and the 32-bit wraparound
//   gives it exactly (smul: three multiply instructions).  A butterfly's
//   difference adds K, a multiple of p at least the stage's input bound, so
//   it stays non-negative.  For 64-point transforms the bounds stay below
//   2^25 (the stage-by-stage counts are at bt_ct_u and bt_gs_u).
// * The other steps (Berlekamp-Massey, Horner, Forney) keep signed int32
//   values within (-2^30, 2^30).  A product x = a w (|a| < 2^31,
//   0 <= w <= 65536, taken to 64 bits) written as x = h 2^32 + l1 2^16 + l0
//   (l0, l1 in [0, 65535], h the signed high word) is congruent to
//   l0 - l1 + h, since 2^16 = -1 and 2^32 = 1 (mod p) (lmul: one wide
//   multiply and three integer operations).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "rsi16.cuh"
#include "rsi16_device.cuh"

namespace ffgpu {

static __device__ __forceinline__ int32_t lmul(int32_t a, uint32_t w) {
    const long long x = (long long)a * (long long)(int32_t)w;
    const uint32_t lo = (uint32_t)x;
    return (int32_t)(lo & 0xffffu) - (int32_t)(lo >> 16) + (int32_t)(x >> 32);
}

// [0, p) from a lazy value with |v| < 2^30: v = (v >> 16) 2^16 + (v & 0xffff)
// with an arithmetic shift, so v = (v & 0xffff) - (v >> 16), which lies in
// [-2^14, 65535 + 2^14]; one conditional add and one conditional subtract.
static __device__ __forceinline__ uint32_t lcanon(int32_t v) {
    int32_t r = (v & 0xffff) - (v >> 16);
    r = r < 0 ? r + 0x10001 : r;
    r = r >= 0x10001 ? r - 0x10001 : r;
    return (uint32_t)r;
}

// x w mod p into [0, 2p) for any x < 2^32 and w < p, w' = floor(w 2^32 / p)
static __device__ __forceinline__ uint32_t smul(uint32_t x, uint32_t w, uint32_t ws) {
    return x * w - __umulhi(x, ws) * 0x10001u;
}

// [0, p) from an unsigned lazy value v < 2^31
static __device__ __forceinline__ uint32_t ucanon(uint32_t v) {
    const int32_t r = (int32_t)(v & 0xffffu) - (int32_t)(v >> 16);
    return (uint32_t)(r < 0 ? r + 0x10001 : r);
}

// the least multiple of p that is at least b
__host__ __device__ constexpr uint32_t pmul_ceil(uint32_t b) { return (b + 0x10000u) / 0x10001u * 0x10001u; }

// Twiddles of one code, passed as a kernel parameter: with every index a
// compile-time constant they are read as constant-bank operands.  Each has
// its Shoup companion.
//   ct[ef * i]: roots_ecc (the CT stages, index < N / 2)
//   gs[i << ef]: roots_i_ecc (the GS stages, index < N / 2)
//   mix: ecc_mix (RSi16v::_mix_ecc, libffrs/rsi16v_impl.hpp:100-119)
template <int N>
struct BtTw {
    uint32_t ct[N / 2];
    uint32_t gs[N / 2];
    uint32_t mix[N];
    uint32_t ct_s[N / 2], gs_s[N / 2], mix_s[N];  // the Shoup companions floor(w 2^32 / p)
    // the accessors the transforms use (a twiddle source; BtTwShared is the other)
    __device__ __forceinline__ uint32_t get_ct(int i) const { return ct[i]; }
    __device__ __forceinline__ uint32_t get_cts(int i) const { return ct_s[i]; }
    __device__ __forceinline__ uint32_t get_gs(int i) const { return gs[i]; }
    __device__ __forceinline__ uint32_t get_gss(int i) const { return gs_s[i]; }
    __device__ __forceinline__ uint32_t get_mix(int i) const { return mix[i]; }
    __device__ __forceinline__ uint32_t get_mixs(int i) const { return mix_s[i]; }
};

// A BtTw in shared memory, read at every use.  The kernels that take the
// twiddles as a parameter read them as constant-bank operands; from shared
// memory the compiler would hoist all 4N of them into registers ahead of the
// transforms and spill, so each read here is a volatile load.
template <int N>
struct BtTwShared {
    uint32_t base;  // shared-window address of the BtTw<N>
    __device__ __forceinline__ uint32_t ld(int w) const {
        uint32_t v;
        asm volatile("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(base + 4u * (uint32_t)w));
        return v;
    }
    __device__ __forceinline__ uint32_t get_ct(int i) const { return ld(i); }
    __device__ __forceinline__ uint32_t get_gs(int i) const { return ld(N / 2 + i); }
    __device__ __forceinline__ uint32_t get_mix(int i) const { return ld(N + i); }
    __device__ __forceinline__ uint32_t get_cts(int i) const { return ld(2 * N + i); }
    __device__ __forceinline__ uint32_t get_gss(int i) const { return ld(2 * N + N / 2 + i); }
    __device__ __forceinline__ uint32_t get_mixs(int i) const { return ld(3 * N + i); }
};

template <int N>
constexpr int bt_log() {
    return N == 32 ? 5 : (N == 64 ? 6 : 7);
}

// ct_butterfly (libffrs/ntt.hpp:225-249) on one thread's vector: RBO input,
// normal order output, inputs below 2^16 (message words).  Butterflies with
// twiddle index 0 (a factor of 1) take no product.  With inputs below B, a
// stage's outputs are below B + K, K = the least multiple of p at least
// max(B, 2p): a + m < B + 2p, a - m + K < B + K (m < 2p after a product, m < B
// without).  From B = 2^16 the six stages of 64 points end below 6.3 * 10^6.
template <int N, class TW>
static __device__ __forceinline__ void bt_ct_u(uint32_t (&x)[N], const TW &tw) {
    uint32_t B = 0x10000u;
#pragma unroll
    for (int st = 0; st < bt_log<N>(); ++st) {
        const int stride = 1 << st, ef = (N >> 1) >> st;
        const uint32_t K = pmul_ceil(B > 0x20002u ? B : 0x20002u);
#pragma unroll
        for (int j = 0; j < N; ++j) {
            if (j & stride) continue;
            const int i = j & (stride - 1);
            const uint32_t a = x[j];
            const uint32_t m = i ? smul(x[j + stride], tw.get_ct(ef * i), tw.get_cts(ef * i)) : x[j + stride];
            x[j] = a + m;
            x[j + stride] = a - m + K;
        }
        B += K;
    }
}

// gs_butterfly (libffrs/ntt.hpp:280-302) on one thread's vector: normal order
// input, RBO output, inputs below 2p (products).  With inputs below B a stage's
// outputs are below B + K, K = the least multiple of p at least B: a + b < 2B,
// a - b + K < B + K, a product < 2p.  From B = 2p the six stages of 64 points
// end below 2^6 * 2p < 2^24.
template <int N, class TW>
static __device__ __forceinline__ void bt_gs_u(uint32_t (&x)[N], const TW &tw) {
    uint32_t B = 0x20002u;
#pragma unroll
    for (int st = 0; st < bt_log<N>(); ++st) {
        const int stride = (N >> 1) >> st, ef = st;
        const uint32_t K = pmul_ceil(B);
#pragma unroll
        for (int j = 0; j < N; ++j) {
            if (j & stride) continue;
            const int i = j & (stride - 1);
            const uint32_t a = x[j], b = x[j + stride];
            x[j] = a + b;
            const uint32_t d = a - b + K;
            x[j + stride] = i ? smul(d, tw.get_gs(i << ef), tw.get_gss(i << ef)) : d;
        }
        B += K;
    }
}

// ---------------------------------------------------------------- warp tile staging
//
// A warp's 32 blocks are staged chunk by chunk: chunk ch of block r (N uint16
// words, 2N bytes) lands in row r of a warp-private shared buffer.  The copy
// is coalesced (each 16-byte cp.async of a warp instruction covers whole
// rows: for N = 64, 4 rows of 128 bytes) and the 16-byte segments of row r
// are stored at segment s ^ (r & 7), so that the row reads below (one row
// per thread, 16 bytes at a time) hit distinct banks within each quarter
// warp.  Rows of blocks past the end are zero-filled.

template <int N>
struct BtTile {
    static constexpr int kRowBytes = 2 * N;
    static constexpr int kSegs = kRowBytes / 16;      // 16-byte segments per row
    static constexpr int kRowsPerIssue = 32 / kSegs;  // rows one warp instruction covers
    static constexpr int kBufBytes = 32 * kRowBytes;  // one chunk of 32 blocks
    static_assert(kSegs == 8 || kSegs == 4, "rows of 128 or 64 bytes");
    // the slot of segment s of row r.  A quarter warp reads one segment of 8
    // consecutive rows; they must hit the 8 distinct 16-byte bank groups of a
    // 128-byte bank cycle.  128-byte rows: s ^ (r & 7).  64-byte rows, two per
    // cycle: the even rows take groups 0-3 and the odd rows 4-7, so
    // s ^ ((r >> 1) & 3).
    static __device__ __forceinline__ int swz(int s, int r) { return kSegs == 8 ? s ^ (r & 7) : s ^ ((r >> 1) & 3); }
};

static __device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// cp.async of chunk `ch` of the warp's blocks [blk0, blk0 + 32) into buf.
// Block r's words start at words + (blk0 + r) * row_stride (uint16 units).
template <int N>
static __device__ __forceinline__ void bt_issue(uint8_t *buf, const uint16_t *words, size_t row_stride, size_t blk0,
                                                size_t nblocks, uint32_t ch, int lane) {
    using T = BtTile<N>;
    const int seg = lane % T::kSegs;
#pragma unroll
    for (int it = 0; it < 32 / T::kRowsPerIssue; ++it) {
        const int r = it * T::kRowsPerIssue + lane / T::kSegs;
        const bool in = blk0 + r < nblocks;
        const uint16_t *src = in ? words + (blk0 + r) * row_stride + (size_t)ch * N + seg * 8 : words;
        const uint32_t dst = smem_addr(buf + r * T::kRowBytes + (T::swz(seg, r) << 4));
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(in ? 16 : 0)
                     : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

// row `lane` of buf as N values
template <int N>
static __device__ __forceinline__ void bt_read_row(const uint8_t *buf, int lane, uint32_t (&x)[N]) {
    using T = BtTile<N>;
#pragma unroll
    for (int s = 0; s < T::kSegs; ++s) {
        const uint4 q = *reinterpret_cast<const uint4 *>(buf + lane * T::kRowBytes + (T::swz(s, lane) << 4));
        const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            x[8 * s + 2 * i] = w[i] & 0xffffu;
            x[8 * s + 2 * i + 1] = w[i] >> 16;
        }
    }
}

// One chunk of NTT::pntt (libffrs/ntt.hpp:133-152) on one thread: x (chunk
// ch of a block, words below 2^16) is transformed and added to acc times
// pntt_shift of the chunk; chunk 0 initialises acc.
template <int N, class TW>
static __device__ __forceinline__ void bt_pntt_chunk(const Rsi16Dev &c, const TW &tw, uint32_t (&x)[N], uint32_t ch,
                                                     uint32_t (&acc)[N]) {
    bt_ct_u<N>(x, tw);
    if (ch == 0) {
        // pntt_shift of chunk 0 is root^(j * rbo(0)) = 1
#pragma unroll
        for (int k = 0; k < N; ++k) acc[k] = x[k];
    } else {
        const uint4 *sh = reinterpret_cast<const uint4 *>(c.pntt_shift + (size_t)ch * N);
        const uint4 *shs = reinterpret_cast<const uint4 *>(c.pntt_shift_s + (size_t)ch * N);
#pragma unroll
        for (int q = 0; q < N / 4; ++q) {
            const uint4 s = __ldg(sh + q), ss = __ldg(shs + q);
            acc[4 * q] += smul(x[4 * q], s.x, ss.x);
            acc[4 * q + 1] += smul(x[4 * q + 1], s.y, ss.y);
            acc[4 * q + 2] += smul(x[4 * q + 2], s.z, ss.z);
            acc[4 * q + 3] += smul(x[4 * q + 3], s.w, ss.w);
        }
    }
}

// the parity of a block from its pntt_message accumulator: RSi16v::_mix_ecc
// (libffrs/rsi16v_impl.hpp:100-119), then gs_butterfly; acc ends lazily
// reduced (below 2^24), in storage order
template <int N, class TW>
static __device__ __forceinline__ void bt_parity(const TW &tw, uint32_t (&acc)[N]) {
#pragma unroll
    for (int k = 0; k < N; ++k) acc[k] = smul(acc[k], tw.get_mix(k), tw.get_mixs(k));
    bt_gs_u<N>(acc, tw);
}

// NTT::pntt (libffrs/ntt.hpp:133-152) of the warp's 32 blocks over chunks
// [0, nch), one block per lane: acc = sum_ch ct(chunk_ch) * pntt_shift_ch,
// lazily reduced: below 6.3 * 10^6 + (nch - 1) 2p < 2^28 for nch <= 1024.
// `words` / `row_stride` give chunk ch of block b at
// words + b * row_stride + ch * N; when `par` is given, chunk nch - 1 is read
// from par + b * N instead (the parity chunk of a codeword).
template <int N, class TW>
static __device__ __forceinline__ void bt_pntt(const Rsi16Dev &c, const TW &tw, uint8_t *bufs,
                                               const uint16_t *words, size_t row_stride, const uint16_t *par,
                                               size_t blk0, size_t nblocks, uint32_t nch, int lane,
                                               uint32_t (&acc)[N]) {
    using T = BtTile<N>;
    auto issue = [&](uint32_t ch) {
        uint8_t *buf = bufs + (ch & 1) * T::kBufBytes;
        if (par && ch == nch - 1)
            bt_issue<N>(buf, par, N, blk0, nblocks, 0, lane);
        else
            bt_issue<N>(buf, words, row_stride, blk0, nblocks, ch, lane);
    };
    issue(0);
    for (uint32_t ch = 0; ch < nch; ++ch) {
        if (ch + 1 < nch) {
            issue(ch + 1);
            asm volatile("cp.async.wait_group 1;" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;" ::: "memory");
        }
        __syncwarp();
        uint32_t x[N];
        bt_read_row<N>(bufs + (ch & 1) * T::kBufBytes, lane, x);
        __syncwarp();  // every lane has read the buffer before the next issue refills it
        bt_pntt_chunk<N>(c, tw, x, ch, acc);
    }
}

// v == 0 (mod p) for any int32 v.  p is odd, so multiplication by its
// inverse mod 2^32 (0xffff0001: 65537 * 0xffff0001 = 2^48 + 1) permutes the
// 32-bit words and sends the multiple k p to k; the multiples of p in the
// int32 range are k p with |k| <= 32767, so v is one of them exactly when
// v * p^-1 + 32767 (mod 2^32) is at most 65534.
static __device__ __forceinline__ bool lzero(int32_t v) {
    return (uint32_t)v * 0xffff0001u + 32767u <= 65534u;
}

// [0, p) from a lazy 64-bit value with |x| < 2^62: x = h 2^32 + l1 2^16 + l0
static __device__ __forceinline__ uint32_t lcanon64(long long x) {
    const uint32_t lo = (uint32_t)x;
    return lcanon((int32_t)(lo & 0xffffu) - (int32_t)(lo >> 16) + (int32_t)(x >> 32));
}

// ---------------------------------------------------------------- one-block-per-thread repair
//
// RSi16v::_repair, unknown locations (libffrs/rsi16v_impl.hpp:122-168), on
// the bounded-distance path of the warp kernels: syndromes by bt_pntt over
// every chunk (the parity chunk last), Berlekamp-Massey on the reversed
// syndromes per lane (bt_rev_bm: a normal run's connection polynomial read
// backwards is the locator), the roots by inverse partial NTT per lane
// (_find_roots_ntt, :443-497) and Forney (_forney, :500-512) block by block
// across the warp, one root per lane.  A block the path does not accept
// (abnormal run, L out of range, root count not L) is repaired by the
// step-for-step mirror on the warp.
//
// Shared memory of one warp, in words: the syndrome columns S[N][33] (lane j
// owns column j; Omega later replaces S in place), then a region that first
// holds the two staging buffers of bt_pntt and afterwards the locator
// columns Loc[N/2 + 1][33] (the derivative later replaces them in place) and
// the root lists Rts[N/2 + 1][33].

template <int N>
struct BtRepairSmem {
    static constexpr int kCol = 33;
    static constexpr int kS = N * kCol;
    static constexpr int kLoc = (N / 2 + 1) * kCol;
    static constexpr int kStage = 2 * BtTile<N>::kBufBytes / 4;
    static constexpr int kR = kStage > 2 * kLoc ? kStage : 2 * kLoc;
    // rounded to 16 bytes: every warp's staging buffers start on a 16-byte
    // boundary (cp.async of 16 bytes)
    static constexpr int kWords = (kS + kR + 3) / 4 * 4;
    static_assert(kS % 4 == 0, "the staging buffers start on a 16-byte boundary");
};

// Berlekamp-Massey on the reversed syndrome column S_{E-1}, ..., S_0 (stride
// 33): the same steps and the same normality and length checks as
// rsi16_rev_bm_lane, with the connection polynomial C and the shifted
// previous one (Bs) kept lazily reduced (|C_i| < 2^23 after E <= 64 steps)
// and each discrepancy summed exactly in 64 bits.  Before step n, C has
// degree at most n and Bs at most n + 1, so the discrepancy takes the terms
// i <= n and the update the coefficients i <= n + 2; groups of four
// coefficients beyond that are skipped by branches on n (uniform across the
// warp).  Returns L, or 0 when the run is not normal or L > T; C is left in
// [0, p).
template <int T, int E>
static __device__ __forceinline__ uint32_t bt_rev_bm(const uint32_t *S, const uint32_t *inv_tab,
                                                     int32_t (&C)[T + 1]) {
    int32_t Bs[T + 1];
#pragma unroll
    for (int i = 0; i <= T; ++i) {
        C[i] = i == 0 ? 1 : 0;
        Bs[i] = i == 1 ? 1 : 0;
    }
    uint32_t L = 0, binv = 1;
    bool stalled = false, abnormal = false;
#pragma unroll 1
    for (int n = 0; n < E; ++n) {
        // four independent partial sums: a dependent chain of T + 1 wide
        // multiply-adds would leave the lane waiting on each one
        long long acc[4] = {0, 0, 0, 0};
#pragma unroll
        for (int g = 0; g <= T / 4; ++g) {
            if (4 * g > n) break;
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int i = 4 * g + u;
                if (i <= T && i <= n) acc[u] += (long long)C[i] * (int32_t)S[(E - 1 - (n - i)) * 33];
            }
        }
        const uint32_t d = lcanon64((acc[0] + acc[1]) + (acc[2] + acc[3]));
        const uint32_t coef = fmul(d, binv);
        const bool grow = d != 0 && 2 * L <= (uint32_t)n;
        if (d == 0 && !(n & 1) && 2 * L <= (uint32_t)n) stalled = true;
        abnormal |= grow && stalled;
#pragma unroll
        for (int g = T / 4; g >= 0; --g) {
            if (4 * g > n + 2) continue;
#pragma unroll
            for (int u = 3; u >= 0; --u) {
                const int i = 4 * g + u;
                if (i > T) continue;
                const int32_t bi = Bs[i];
                Bs[i] = i == 0 ? 0 : (grow ? C[i - 1] : Bs[i - 1]);
                C[i] -= lmul(bi, coef);
            }
        }
        if (grow) {
            L = n + 1 - L;
            binv = inv_tab[d];
        }
    }
#pragma unroll
    for (int i = 0; i <= T; ++i) C[i] = (int32_t)lcanon(C[i]);
    return (abnormal || L > (uint32_t)T) ? 0u : L;
}

// position i of block b (message words, then parity words)
static __device__ __forceinline__ uint16_t *bt_word(uint16_t *msg, uint16_t *par, uint32_t ml, uint32_t ecc,
                                                    size_t b, uint32_t i) {
    return i < ml ? msg + b * ml + i : par + b * ecc + (i - ml);
}

// The repair of the warp's tile [blk0, blk0 + 32), lane = block.  Returns the
// lanes whose block goes to the mirror; adds the accepted blocks (and the
// clean ones) to nfast.
template <int N, class TW>
static __device__ __forceinline__ uint32_t bt_repair_tile(const Rsi16Dev &c, const TW &tw, uint16_t *msg,
                                                          uint16_t *par, size_t blk0, size_t nblocks,
                                                          uint8_t *status, const uint8_t *active, uint32_t *ws,
                                                          int lane, unsigned long long &nfast) {
    using M = BtRepairSmem<N>;
    constexpr int T = N / 2;
    constexpr int K = M::kCol;
    uint32_t *Ssm = ws, *R = ws + M::kS;
    uint32_t *Lsm = R, *Rts = R + M::kLoc;
    const size_t b = blk0 + lane;
    const bool in = b < nblocks && (!active || active[b]);

    // syndromes: S_k = pntt(codeword)_k
    bool nz = false;
    {
        uint32_t acc[N];
        bt_pntt<N>(c, tw, reinterpret_cast<uint8_t *>(R), msg, c.message_len, par, blk0, nblocks, c.pntt_blocks,
                   lane, acc);
#pragma unroll
        for (int k = 0; k < N; ++k) {
            const uint32_t s = ucanon(acc[k]);
            Ssm[k * K + lane] = s;
            nz |= s != 0;
        }
    }
    __syncwarp();
    // 0: nothing to do, 1: bounded-distance path, 2: mirror
    int path = 0;
    uint32_t L = 0;
    if (in && !nz) {
        status[b] = FFGPU_NO_ERRORS;
        ++nfast;
    } else if (in) {
        int32_t C[T + 1];
        L = bt_rev_bm<T, N>(Ssm + lane, c.inv_tab, C);
#pragma unroll
        for (int i = 0; i <= T; ++i) {
            if ((uint32_t)i <= L) Lsm[(L - i) * K + lane] = (uint32_t)C[i];
            if ((uint32_t)i > L) Lsm[i * K + lane] = 0u;
        }
        path = L ? 1 : 2;
    }
    // roots: positions ch * N + k with Loc(X^-1) = 0, by inverse partial NTT
    // of the locator (pintt_shift, then gs_butterfly) chunk by chunk
    if (path == 1) {
        int32_t loc[T + 1];
#pragma unroll
        for (int k = 0; k <= T; ++k) loc[k] = (int32_t)Lsm[k * K + lane];
        uint32_t cnt = 0;
        for (uint32_t ch = 0; ch < c.pntt_blocks; ++ch) {
            uint32_t x[N];
            // pintt_shift of chunk ch, 16 bytes at a time (the last load also
            // reads the chunk's entries T + 1 .. T + 3, unused)
            const uint4 *sh = reinterpret_cast<const uint4 *>(c.pintt_shift + (size_t)ch * N);
            const uint4 *shs = reinterpret_cast<const uint4 *>(c.pintt_shift_s + (size_t)ch * N);
#pragma unroll
            for (int q = 0; q <= T / 4; ++q) {
                const uint4 s4 = __ldg(sh + q), ss4 = __ldg(shs + q);
                const uint32_t sv[4] = {s4.x, s4.y, s4.z, s4.w}, svs[4] = {ss4.x, ss4.y, ss4.z, ss4.w};
#pragma unroll
                for (int i = 0; i < 4; ++i)
                    if (4 * q + i <= T) x[4 * q + i] = smul((uint32_t)loc[4 * q + i], sv[i], svs[i]);
            }
#pragma unroll
            for (int k = T + 1; k < N; ++k) x[k] = 0;
            bt_gs_u<N>(x, tw);
            uint32_t z[N / 32];
#pragma unroll
            for (int h = 0; h < N / 32; ++h) {
                z[h] = 0;
#pragma unroll
                for (int k = 0; k < 32; ++k) z[h] |= (uint32_t)lzero((int32_t)x[32 * h + k]) << k;
            }
#pragma unroll
            for (int h = 0; h < N / 32; ++h) {
                for (uint32_t m = z[h]; m; m &= m - 1) {
                    if (cnt <= (uint32_t)T) Rts[cnt * K + lane] = ch * N + 32 * h + (__ffs(m) - 1);
                    ++cnt;
                }
            }
        }
        if (cnt != L) path = 2;
    }
    if (path == 1) {
        // Omega = S * Loc mod x^L, in place over S (high degrees first, so
        // that S_0 .. S_j are still there for Omega_j)
        for (uint32_t j = L; j-- > 0;) {
            uint64_t s0 = 0, s1 = 0;
            uint32_t k = 0;
            for (; k + 1 <= j; k += 2) {
                s0 += (uint64_t)Lsm[k * K + lane] * Ssm[(j - k) * K + lane];
                s1 += (uint64_t)Lsm[(k + 1) * K + lane] * Ssm[(j - k - 1) * K + lane];
            }
            if (k == j) s0 += (uint64_t)Lsm[k * K + lane] * Ssm[0 * K + lane];
            Ssm[j * K + lane] = lcanon64((long long)(s0 + s1));
        }
        // the derivative Loc'_j = (j + 1) Loc_{j+1}, in place over Loc
        for (uint32_t j = 0; j < L; ++j) Lsm[j * K + lane] = fmul(Lsm[(j + 1) * K + lane], j + 1);
        status[b] = FFGPU_REPAIR_OK;
        ++nfast;
    }
    __syncwarp();
    // Forney, e_i = X_i Omega(X_i^-1) / Loc'(X_i^-1), in two passes.  First
    // block by block, lane r on root r: Omega(X^-1) into row T + r of the
    // block's syndrome column (rows T .. N - 1 are free once Omega is built)
    // and Loc'(X^-1) into row r of its locator column (the derivative is dead
    // once the block's evaluations are done).  Then every lane finishes its
    // own block's roots four at a time: the inverse, the product and the
    // read-modify-write of the word, with the loads of four roots in flight.
    const uint32_t NN = c.ntt_len;
    for (uint32_t todo = __ballot_sync(0xffffffffu, path == 1); todo; todo &= todo - 1) {
        const int j = __ffs(todo) - 1;
        const uint32_t Lj = __shfl_sync(0xffffffffu, L, j);
        uint32_t den = 0;
        if ((uint32_t)lane < Lj) {
            const uint32_t i = Rts[lane * K + j];
            const uint32_t e = (__brev(i) >> 16) >> c.rbo_shift;
            const uint32_t xi = c.roots_ntt[(NN - e) & (NN - 1)];
            int32_t num = 0, dn = 0;
            for (uint32_t k = Lj; k-- > 0;) {
                num = lmul(num, xi) + (int32_t)Ssm[k * K + j];
                dn = lmul(dn, xi) + (int32_t)Lsm[k * K + j];
            }
            Ssm[(T + lane) * K + j] = lcanon(num);
            den = lcanon(dn);
        }
        __syncwarp();  // every lane has read the derivative before it is overwritten
        if ((uint32_t)lane < Lj) Lsm[lane * K + j] = den;
    }
    __syncwarp();
    if (path == 1) {
        for (uint32_t r0 = 0; r0 < L; r0 += 4) {
            uint32_t pos[4], x[4], inv[4], num[4], old[4];
            uint16_t *w[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint32_t r = r0 + q < L ? r0 + q : r0;
                pos[q] = Rts[r * K + lane];
                num[q] = Ssm[(T + r) * K + lane];
                const uint32_t e = (__brev(pos[q]) >> 16) >> c.rbo_shift;
                x[q] = c.roots_ntt[e];
                inv[q] = c.inv_tab[Lsm[r * K + lane]];
                w[q] = bt_word(msg, par, c.message_len, N, b, pos[q]);
                old[q] = *w[q];
            }
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (r0 + q < L) *w[q] = (uint16_t)fadd(old[q], fmul(fmul(num[q], inv[q]), x[q]));
        }
    }
    __syncwarp();  // the columns are read before the next tile's staging overwrites them
    return __ballot_sync(0xffffffffu, path == 2);
}

// Parity of the warp's tile [blk0, blk0 + 32), one block per lane:
// NTT::pntt_message (libffrs/ntt.hpp:160-180) over the message chunks,
// RSi16v::_mix_ecc and the GS transform; msg / par are contiguous blocks.
template <int N, class TW>
static __device__ __forceinline__ void bt_encode_tile(const Rsi16Dev &c, const TW &tw, uint8_t *bufs,
                                                      const uint16_t *msg, uint16_t *par, size_t blk0,
                                                      size_t nblocks, int lane) {
    uint32_t acc[N];
    bt_pntt<N>(c, tw, bufs, msg, c.message_len, nullptr, blk0, nblocks, c.pntt_blocks - 1, lane, acc);
    bt_parity<N>(tw, acc);
    const size_t b = blk0 + lane;
    if (b < nblocks) {
        uint4 *o = reinterpret_cast<uint4 *>(par + b * N);
#pragma unroll
        for (int q = 0; q < N / 8; ++q) {
            uint32_t w[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) w[i] = ucanon(acc[8 * q + 2 * i]) & 0xffffu | ucanon(acc[8 * q + 2 * i + 1]) << 16;
            o[q] = make_uint4(w[0], w[1], w[2], w[3]);
        }
    }
}

// Shared memory of one warp of the bt kernels: two chunk buffers.
template <int N>
constexpr int bt_warp_smem() {
    return 2 * BtTile<N>::kBufBytes;
}

}  // namespace ffgpu
