// Bitsliced RS256 kernels for the default field (primitive 2, polynomial
// 0x11d) with ecc_len in {2, 4, 8, 16, 32}.
//
// Layout: a "group" is 32 consecutive blocks; bit j of a 32-bit plane word
// belongs to block j.  Byte position i of the group is 8 planes (one per bit).
// A GF(2^8) multiplication by a constant is then a fixed XOR network over the
// 8 planes, computed for all 32 blocks at once with LOP3.
//
// The generator g(x) = prod_{j<ecc}(x - a^j) is split into factors
// g_t(x) = prod_{16t <= j < 16t+d}(x - a^j) of degree d <= 16; one thread per
// (group, factor) runs the byte-serial LFSR of the reference's encoder
// (rem <- (rem >> 8) ^ lut[rem0 ^ in], reed_solomon.hpp:194-195) modulo g_t.
// Its update needs the products g_t[m] * fb for every coefficient m; the
// "four Russians" trick forms the 15 XOR combinations of each nibble of fb once
// and every output plane is then old_plane ^ lo[c1] ^ hi[c2], one LOP3.
//
// Encode recovers the parity (data * x^ecc mod g) from the factor remainders
// with a fixed GF(2)-linear map (Chinese remainders); decode turns each factor
// remainder R = r * x^d mod g_t into its syndromes S_j = r(a^j) = R(a^j) a^{-jd}.
// All selector tables are computed at compile time and reach the code as
// template constants, so every plane index is resolved to a register.
//
// Encode batches too small to fill the GPU with that LFSR (ecc 32) take the
// byte-parallel nibble-table kernel instead (rs256_encode_nib_kernel).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <utility>

#include "common.cuh"
#include "rs256.cuh"
#include "rs256_nib.cuh"
#include "rs256_synd_gen.cuh"

namespace ffgpu {
namespace bs {

// ---------------------------------------------------------------- compile-time field

struct Field {
    uint8_t exp[512];
    uint8_t log[256];
};

constexpr uint8_t mul_serial(uint8_t a, uint8_t b) {
    uint8_t r = 0;
    for (int i = 7; i >= 0; --i) {
        r = (r & 0x80) ? (uint8_t)((r << 1) ^ 0x1d) : (uint8_t)(r << 1);
        if (a & (1 << i)) r ^= b;
    }
    return r;
}

constexpr Field make_field() {
    Field f{};
    uint8_t x = 1;
    for (int i = 0; i < 255; ++i) {
        f.exp[i] = x;
        f.log[x] = (uint8_t)i;
        x = mul_serial(x, 2);
    }
    for (int i = 255; i < 512; ++i) f.exp[i] = f.exp[i - 255];
    return f;
}

constexpr Field F = make_field();

constexpr uint8_t gm(uint8_t a, uint8_t b) { return (a && b) ? F.exp[F.log[a] + F.log[b]] : 0; }
constexpr uint8_t apow(int e) {
    e %= 255;
    if (e < 0) e += 255;
    return F.exp[e];
}
// input-bit mask of output bit o of the multiplication by c: bit b set when
// bit o of c * 2^b is set
constexpr uint8_t sel_of(uint8_t c, int o) {
    uint8_t s = 0;
    for (int b = 0; b < 8; ++b)
        if ((gm(c, (uint8_t)(1 << b)) >> o) & 1) s |= (uint8_t)(1 << b);
    return s;
}

// g_t = prod_{j=J0}^{J0+D-1} (x - a^j), highest degree first
template <int D>
struct Poly {
    uint8_t c[D + 1];
};
template <int D>
constexpr Poly<D> factor_poly(int J0) {
    Poly<D> g{};
    g.c[0] = 1;
    int len = 1;
    for (int j = J0; j < J0 + D; ++j) {
        uint8_t r = apow(j);
        uint8_t ng[D + 1] = {};
        for (int a = 0; a < len; ++a) {
            ng[a] ^= g.c[a];
            ng[a + 1] ^= gm(g.c[a], r);
        }
        ++len;
        for (int a = 0; a < len; ++a) g.c[a] = ng[a];
    }
    return g;
}

// LFSR selectors: new R[m][o] = R[m+1][o] ^ (g[m+1] * fb)[o]
template <int D>
struct LfsrSel {
    uint8_t s[D][8];
};
template <int D>
constexpr LfsrSel<D> make_lfsr_sel(int J0) {
    LfsrSel<D> L{};
    const Poly<D> g = factor_poly<D>(J0);
    for (int m = 0; m < D; ++m)
        for (int o = 0; o < 8; ++o) L.s[m][o] = sel_of(g.c[m + 1], o);
    return L;
}

// remainder -> syndromes: S_{J0+j} = sum_m R[m] a^{-(J0+j)(m+1)}
template <int D>
struct SyndSel {
    uint8_t s[D][D][8];  // [m][j][o]
};
template <int D>
constexpr SyndSel<D> make_synd_sel(int J0) {
    SyndSel<D> S{};
    for (int m = 0; m < D; ++m)
        for (int j = 0; j < D; ++j)
            for (int o = 0; o < 8; ++o) S.s[m][j][o] = sel_of(apow(-(J0 + j) * (m + 1)), o);
    return S;
}

// ---- polynomial helpers over GF(2^8) (compile time), highest degree first
template <int N>
struct P {
    int n;  // number of coefficients
    uint8_t c[N];
};

// a mod b, b monic of degree db (db + 1 coefficients)
template <int N, int M>
constexpr P<N> pmod(P<N> a, const P<M> &b) {
    const int db = b.n - 1;
    for (int i = 0; i + db < a.n; ++i) {
        uint8_t q = a.c[i];
        if (!q) continue;
        for (int k = 0; k <= db; ++k) a.c[i + k] ^= gm(q, b.c[k]);
    }
    // keep the low db coefficients
    P<N> r{};
    r.n = db;
    for (int k = 0; k < db; ++k) r.c[k] = a.c[a.n - db + k];
    return r;
}

template <int N>
constexpr P<N> pmul(const P<N> &a, const P<N> &b) {
    P<N> r{};
    r.n = a.n + b.n - 1;
    for (int i = 0; i < a.n; ++i)
        for (int j = 0; j < b.n; ++j) r.c[i + j] ^= gm(a.c[i], b.c[j]);
    return r;
}

// Chinese-remainder map for ecc = 32 (two degree-16 factors): the parity
// coefficient vector P (32 bytes, highest first) is linear in the two factor
// remainders R0 = data * x^16 mod g0, R1 = data * x^16 mod g1:
//   P = data * x^32 mod g = sum_t [x^16 * R_t * E_t mod g_t] * G_t
// with G_t = g / g_t and E_t = G_t^{-1} mod g_t.  The selector table gives,
// for every input byte (t, m) and output bit (p, o), the input-bit mask.
struct CrtSel {
    uint8_t s[2][16][32][8];  // [t][m][p][o]
};

template <int N>
constexpr P<N> pinv_mod(const P<N> &a, const P<N> &m) {
    // inverse of a modulo m by exhaustive linear solve over the remainders:
    // a * e = 1 mod m with deg e < deg m; solved by Gaussian elimination on
    // the 16x16 GF(2^8) system
    const int d = m.n - 1;
    uint8_t A[16][17] = {};
    for (int k = 0; k < d; ++k) {
        // column k: a * x^(d-1-k) mod m
        P<N> xk{};
        xk.n = d - k;
        xk.c[0] = 1;
        P<N> prod = pmul(a, xk);
        P<N> r = pmod(prod, m);
        // r has d coefficients, highest first
        for (int row = 0; row < d; ++row) A[row][k] = r.c[row];
    }
    for (int row = 0; row < d; ++row) A[row][d] = (row == d - 1) ? 1 : 0;  // target polynomial 1
    for (int col = 0; col < d; ++col) {
        int piv = col;
        while (piv < d && A[piv][col] == 0) ++piv;
        for (int k = 0; k <= d; ++k) {
            uint8_t t = A[col][k];
            A[col][k] = A[piv][k];
            A[piv][k] = t;
        }
        uint8_t inv = F.exp[255 - F.log[A[col][col]]];
        for (int k = 0; k <= d; ++k) A[col][k] = gm(A[col][k], inv);
        for (int row = 0; row < d; ++row)
            if (row != col && A[row][col]) {
                uint8_t f = A[row][col];
                for (int k = 0; k <= d; ++k) A[row][k] ^= gm(f, A[col][k]);
            }
    }
    P<N> e{};
    e.n = d;
    for (int k = 0; k < d; ++k) e.c[k] = A[k][d];
    return e;
}

constexpr CrtSel make_crt_sel() {
    CrtSel C{};
    using Q = P<80>;
    Q g[2] = {};
    for (int t = 0; t < 2; ++t) {
        Poly<16> f = factor_poly<16>(16 * t);
        g[t].n = 17;
        for (int k = 0; k < 17; ++k) g[t].c[k] = f.c[k];
    }
    Q G[2] = {g[1], g[0]};  // g / g_t
    Q E[2] = {pinv_mod(pmod(G[0], g[0]), g[0]), pinv_mod(pmod(G[1], g[1]), g[1])};
    for (int t = 0; t < 2; ++t) {
        for (int m = 0; m < 16; ++m) {
            for (int b = 0; b < 8; ++b) {
                // basis input: R_t = 2^b at coefficient m (x^(15-m))
                Q r{};
                r.n = 16;
                r.c[m] = (uint8_t)(1 << b);
                Q x16{};
                x16.n = 17;
                x16.c[0] = 1;
                Q u = pmod(pmul(pmul(r, x16), E[t]), g[t]);  // 16 coefficients
                Q p = pmul(u, G[t]);                            // degree <= 31: up to 32 coefficients
                // align to 32 coefficients, highest first
                uint8_t out[32] = {};
                for (int k = 0; k < p.n; ++k) out[32 - p.n + k] = p.c[k];
                for (int pp = 0; pp < 32; ++pp)
                    for (int o = 0; o < 8; ++o)
                        if ((out[pp] >> o) & 1) C.s[t][m][pp][o] |= (uint8_t)(1 << b);
            }
        }
    }
    return C;
}

// Selector tables of the T = E / D factors of degree D.
template <int D, int T>
struct LfsrSet {
    LfsrSel<D> f[T];
};
template <int D, int T>
constexpr LfsrSet<D, T> make_lfsr_set() {
    LfsrSet<D, T> s{};
    for (int t = 0; t < T; ++t) s.f[t] = make_lfsr_sel<D>(D * t);
    return s;
}
template <int D, int T>
struct SyndSet {
    SyndSel<D> f[T];
};
template <int D, int T>
constexpr SyndSet<D, T> make_synd_set() {
    SyndSet<D, T> s{};
    for (int t = 0; t < T; ++t) s.f[t] = make_synd_sel<D>(D * t);
    return s;
}

// g split into T = E / D factors of degree D, one thread per factor and group.
// The encoder needs D = 16 (its CRT map is built for two factors).  For the
// syndromes D = 8 halves the remainder state per thread but doubles the
// nibble-combination work per byte; measured on GB300 it was slower
// (0.52 ms against 0.38 ms per 1,048,576 blocks), so both use D = 16.
template <int E_, int DD = (E_ > 16 ? 16 : E_)>
struct Code {
    static constexpr int E = E_;
    static constexpr int D = DD;      // factor degree
    static constexpr int T = E / D;   // factors (threads per group)
    static constexpr LfsrSet<D, T> lfsrs = make_lfsr_set<D, T>();
    static constexpr SyndSet<D, T> synds = make_synd_set<D, T>();
    template <int t>
    static constexpr const LfsrSel<D> &lfsr() {
        return lfsrs.f[t];
    }
    template <int t>
    static constexpr const SyndSel<D> &synd() {
        return synds.f[t];
    }
};
template <int E>
using SyndCode = Code<E>;

struct CrtHolder {
    static constexpr CrtSel crt = make_crt_sel();
};

// ---------------------------------------------------------------- device helpers

// three-input logic in one LOP3 (PTX lop3.b32; the immediate is the truth
// table over the operand masks 0xF0, 0xCC, 0xAA)
__device__ __forceinline__ uint32_t xor3(uint32_t a, uint32_t b, uint32_t c) {
    uint32_t d;
    asm("lop3.b32 %0, %1, %2, %3, 0x96;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}
// (a & b) ^ c
__device__ __forceinline__ uint32_t andxor(uint32_t a, uint32_t b, uint32_t c) {
    uint32_t d;
    asm("lop3.b32 %0, %1, %2, %3, 0x6A;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}
// (m & a) | (~m & b)
__device__ __forceinline__ uint32_t bitsel(uint32_t m, uint32_t a, uint32_t b) {
    uint32_t d;
    asm("lop3.b32 %0, %1, %2, %3, 0xCA;" : "=r"(d) : "r"(m), "r"(a), "r"(b));
    return d;
}

// 32x32 bit transpose in registers: afterwards a[c] bit r == old a[r] bit c
__device__ __forceinline__ void transpose32(uint32_t (&a)[32]) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        const uint32_t x = a[k], y = a[k + 16];
        a[k] = __byte_perm(x, y, 0x5410);
        a[k + 16] = __byte_perm(x, y, 0x7632);
    }
#pragma unroll
    for (int k0 = 0; k0 < 32; k0 += 16)
#pragma unroll
        for (int k = k0; k < k0 + 8; ++k) {
            const uint32_t x = a[k], y = a[k + 8];
            a[k] = __byte_perm(x, y, 0x6240);
            a[k + 8] = __byte_perm(x, y, 0x7351);
        }
#pragma unroll
    for (int j = 4, sh = 0; j >= 1; j >>= 1, ++sh) {
        const uint32_t m = j == 4 ? 0x0F0F0F0Fu : (j == 2 ? 0x33333333u : 0x55555555u);
#pragma unroll
        for (int k = 0; k < 32; ++k) {
            if (k & j) continue;
            const uint32_t t = ((a[k] >> j) ^ a[k + j]) & m;
            a[k + j] ^= t;
            a[k] ^= t << j;
        }
    }
}

// nibble combinations of 8 planes: lo[c] = XOR of f[b] for bits b of c (b < 4),
// hi[c] the same over f[4..7]
__device__ __forceinline__ void combos(const uint32_t (&f)[8], uint32_t (&lo)[16], uint32_t (&hi)[16]) {
    lo[0] = 0u;
    hi[0] = 0u;
#pragma unroll
    for (int c = 1; c < 16; ++c) {
        const int low = c & -c;
        const int bit = low == 1 ? 0 : (low == 2 ? 1 : (low == 4 ? 2 : 3));
        lo[c] = (c == low) ? f[bit] : (lo[c ^ low] ^ f[bit]);
        hi[c] = (c == low) ? f[bit + 4] : (hi[c ^ low] ^ f[bit + 4]);
    }
}

// base ^ (the combination selected by S), in one LOP3 when both nibbles are used
template <uint8_t S>
__device__ __forceinline__ uint32_t pickx(uint32_t base, const uint32_t (&lo)[16], const uint32_t (&hi)[16]) {
    constexpr int a = S & 15, h = S >> 4;
    if constexpr (a && h)
        return xor3(base, lo[a], hi[h]);
    else if constexpr (a)
        return base ^ lo[a];
    else if constexpr (h)
        return base ^ hi[h];
    else
        return base;
}

template <uint8_t S>
__device__ __forceinline__ uint32_t pick(const uint32_t (&lo)[16], const uint32_t (&hi)[16]) {
    constexpr int a = S & 15, h = S >> 4;
    if constexpr (a && h)
        return lo[a] ^ hi[h];
    else if constexpr (a)
        return lo[a];
    else if constexpr (h)
        return hi[h];
    else
        return 0u;
}

// one LFSR step of factor t: R[m] <- R[m+1] ^ g[m+1] * (R[0] ^ in)
template <typename CD, int t, int... K>
__device__ __forceinline__ void lfsr_apply(uint32_t (&R)[CD::D][8], const uint32_t (&lo)[16],
                                           const uint32_t (&hi)[16], std::integer_sequence<int, K...>) {
    constexpr int D = CD::D;
    ((R[K / 8][K % 8] = pickx<CD::template lfsr<t>().s[K / 8][K % 8]>(
          (K / 8 + 1 < D) ? R[(K / 8 + 1 < D) ? K / 8 + 1 : 0][K % 8] : 0u, lo, hi)),
     ...);
}

template <typename CD, int t>
__device__ __forceinline__ void lfsr_step(uint32_t (&R)[CD::D][8], const uint32_t (&in)[8]) {
    constexpr int D = CD::D;
    uint32_t f[8];
#pragma unroll
    for (int b = 0; b < 8; ++b) f[b] = R[0][b] ^ in[b];
    uint32_t lo[16], hi[16];
    combos(f, lo, hi);
    lfsr_apply<CD, t>(R, lo, hi, std::make_integer_sequence<int, D * 8>{});
}

// S[j][o] ^= (c_{m,j} * r)[o] for one remainder byte m
template <typename CD, int t, int M, int... K>
__device__ __forceinline__ void synd_accum(uint32_t (&S)[CD::D][8], const uint32_t (&lo)[16],
                                           const uint32_t (&hi)[16], std::integer_sequence<int, K...>) {
    ((S[K / 8][K % 8] = pickx<CD::template synd<t>().s[M][K / 8][K % 8]>(S[K / 8][K % 8], lo, hi)), ...);
}

template <typename CD, int t, int... M>
__device__ __forceinline__ void rem_to_synd(const uint32_t *rs, int stride, uint32_t (&S)[CD::D][8],
                                            std::integer_sequence<int, M...>) {
    constexpr int D = CD::D;
    auto one = [&](auto mc) {
        constexpr int m = decltype(mc)::value;
        uint32_t r[8];
#pragma unroll
        for (int b = 0; b < 8; ++b) r[b] = rs[(m * 8 + b) * stride];
        uint32_t lo[16], hi[16];
        combos(r, lo, hi);
        synd_accum<CD, t, m>(S, lo, hi, std::make_integer_sequence<int, D * 8>{});
    };
    (one(std::integral_constant<int, M>{}), ...);
}

// parity half p0 .. p0+15 (ecc 32): P[pp][o] ^= crt(t, m)[pp][o] over all (t, m)
template <int T, int M, int P0, int... K>
__device__ __forceinline__ void crt_accum(uint32_t (&Pp)[16][8], const uint32_t (&lo)[16], const uint32_t (&hi)[16],
                                          std::integer_sequence<int, K...>) {
    ((Pp[K / 8][K % 8] = pickx<CrtHolder::crt.s[T][M][P0 + K / 8][K % 8]>(Pp[K / 8][K % 8], lo, hi)), ...);
}

template <int P0, int... TM>
__device__ __forceinline__ void crt_map(const uint32_t *rs, int stride, uint32_t (&Pp)[16][8],
                                        std::integer_sequence<int, TM...>) {
    auto one = [&](auto tc) {
        constexpr int tm = decltype(tc)::value;
        constexpr int t = tm / 16, m = tm % 16;
        uint32_t r[8];
#pragma unroll
        for (int b = 0; b < 8; ++b) r[b] = rs[((t * 16 + m) * 8 + b) * stride];
        uint32_t lo[16], hi[16];
        combos(r, lo, hi);
        crt_accum<t, m, P0>(Pp, lo, hi, std::make_integer_sequence<int, 128>{});
    };
    (one(std::integral_constant<int, TM>{}), ...);
}

// Decode scratch of one tile (32 groups = 1024 blocks): kTileWords<E> words,
// word w of group g at w * 32 + g.  It first holds the bitsliced syndromes
// (w = 8j + b: bit b of S_j), then the record the Berlekamp-Massey kernel
// leaves for the Chien kernel (RecLayout).
template <int E>
constexpr int kTileWords = E * 9 * 32;

// The record of one group after Berlekamp-Massey: C_0..C_t (w = 8k + b),
// Omega_0..Omega_{t-1}, the 6 planes of L, the mask of live blocks (non-zero
// syndromes and inside the call).
template <int E>
struct RecLayout {
    static constexpr int t = E / 2;
    static constexpr int kC = 0;
    static constexpr int kOm = 8 * (t + 1);
    static constexpr int kL = kOm + 8 * t;
    static constexpr int kLive = kL + 6;
    static_assert(kLive < E * 9, "record larger than the tile scratch");
};

// ---------------------------------------------------------------- window loader

// Tile geometry: G groups of 32 blocks per CTA.  A window is 32 consecutive
// codeword positions of every block of the tile, held as 8 words per block.
// Column q (bytes 4q .. 4q+3 of the window) of group g lives in words
// [g*256 + q*32, +32), with word j (block j) stored at j ^ (g & 31): a warp
// always works on 32 consecutive groups (or 32 blocks of one group), so every
// shared-memory access below touches 32 different banks.
__device__ __forceinline__ int swz(int g) { return g & 31; }

// the n < 4 bytes at p (the last of an array) as the low bytes of a word,
// the rest zero; out of line, so that the loads around it keep their
// registers
static __device__ __noinline__ uint32_t ldg_tail(const uint8_t *p, size_t n) {
    uint32_t v = 0u;
    for (size_t q = 0; q < n; ++q) v |= (uint32_t)__ldg(p + q) << (8 * q);
    return v;
}

// Load window bytes [p0, p0 + 32) of every block of the tile from the segment
// `base` (block b at base + b * seg_len; total bytes of the segment array in
// `total`).  Positions at or beyond seg_len are never consumed.
__device__ __forceinline__ void load_window(uint32_t *buf, const uint8_t *__restrict__ base, size_t seg_len,
                                            size_t total, size_t first_block, int nblocks_tile, int p0, int G) {
    // four blocks per round: their 36 loads are issued before any is used
    constexpr int R = 4;
    for (int b0 = threadIdx.x; b0 < G * 32; b0 += R * blockDim.x) {
        uint32_t w[R][9];
        uint32_t sh[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int b = b0 + r * blockDim.x;
            sh[r] = 0;
            if (b < G * 32 && b < nblocks_tile) {
                const size_t start = (first_block + b) * seg_len + p0;
                const size_t a0 = start & ~(size_t)3;
                sh[r] = (uint32_t)(start & 3) * 8;
#pragma unroll
                for (int i = 0; i < 9; ++i) {
                    const size_t aw = a0 + 4 * i;
                    w[r][i] = aw + 4 <= total ? __ldg(reinterpret_cast<const uint32_t *>(base + aw))
                                              : (aw < total ? ldg_tail(base + aw, total - aw) : 0u);
                }
            } else {
#pragma unroll
                for (int i = 0; i < 9; ++i) w[r][i] = 0u;
            }
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int b = b0 + r * blockDim.x;
            if (b < G * 32) {
                const int g = b >> 5, j = b & 31;
                uint32_t *dst = buf + g * 256 + (j ^ swz(g));
#pragma unroll
                for (int k = 0; k < 8; ++k) dst[k * 32] = __funnelshift_r(w[r][k], w[r][k + 1], sh[r]);
            }
        }
    }
}

// transpose the columns this thread owns (q = t, t + T, ...) in place
template <int T>
__device__ __forceinline__ void transpose_window(uint32_t *buf, int g, int t) {
    const int s = swz(g);
#pragma unroll 1
    for (int q = t; q < 8; q += T) {
        uint32_t *col = buf + g * 256 + q * 32;
        uint32_t a[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) a[j] = col[j ^ s];
        transpose32(a);
#pragma unroll
        for (int c = 0; c < 32; ++c) col[c ^ s] = a[c];
    }
}

// planes of window position i (0..31) of group g
template <int T>
__device__ __forceinline__ void read_planes(const uint32_t *buf, int g, int i, uint32_t (&in)[8]) {
    const int q = i >> 2, qb = i & 3;
    const int s = swz(g);
    const uint32_t *col = buf + g * 256 + q * 32;
#pragma unroll
    for (int b = 0; b < 8; ++b) in[b] = col[(qb * 8 + b) ^ s];
}

// ---------------------------------------------------------------- kernels

constexpr int kGroups = 64;      // groups per CTA tile of the encoder (2048 blocks)
// groups per CTA tile of the syndrome kernel (2048 blocks; 32-group tiles of
// two warps measured 0.44 ms against 0.38 ms per 1,048,576 blocks on GB300)
constexpr int kSyndGroups = 64;

template <typename CD, int t>
__device__ __forceinline__ void run_lfsr_window(const uint32_t *buf, int g, int npos, uint32_t (&R)[CD::D][8]) {
    constexpr int T = CD::T;
#pragma unroll 2
    for (int i = 0; i < npos; ++i) {
        uint32_t in[8];
        read_planes<T>(buf, g, i, in);
        lfsr_step<CD, t>(R, in);
    }
}

// Factor remainders R_t = (codeword segment) * x^d mod g_t over the segments
// (data, message_len bytes per block) then optionally (parity, E bytes).
template <int E>
__device__ __forceinline__ size_t total_bytes_e(int seg, size_t nblocks, int msg_len) {
    return seg == 0 ? nblocks * (size_t)msg_len : nblocks * (size_t)E;
}

template <typename CD, int t, int G = kGroups>
__device__ __forceinline__ void factor_remainder(uint32_t *buf, const uint8_t *data, int msg_len,
                                                 const uint8_t *parity, size_t first, int nb_tile, int g,
                                                 size_t nblocks_total, uint32_t (&R)[CD::D][8]) {
    constexpr int E = CD::E;
    auto total_bytes = [](int seg, size_t nb, int ml) { return total_bytes_e<E>(seg, nb, ml); };
    constexpr int T = CD::T;
#pragma unroll
    for (int m = 0; m < CD::D; ++m)
#pragma unroll
        for (int b = 0; b < 8; ++b) R[m][b] = 0u;
    for (int seg = 0; seg < (parity ? 2 : 1); ++seg) {
        const uint8_t *base = seg == 0 ? data : parity;
        const int len = seg == 0 ? msg_len : E;
        for (int p0 = 0; p0 < len; p0 += 32) {
            __syncthreads();
            load_window(buf, base, (size_t)len, total_bytes(seg, nblocks_total, msg_len), first, nb_tile, p0, G);
            __syncthreads();
            transpose_window<T>(buf, g, t);
            __syncthreads();
            run_lfsr_window<CD, t>(buf, g, min(32, len - p0), R);
        }
    }
}

// factor_remainder / rem_to_synd for the runtime factor index t
template <typename CD, int G, int... I>
__device__ __forceinline__ void factor_remainder_t(int t, uint32_t *buf, const uint8_t *data, int msg_len,
                                                   const uint8_t *parity, size_t first, int nb_tile, int g,
                                                   size_t nblocks_total, uint32_t (&R)[CD::D][8],
                                                   std::integer_sequence<int, I...>) {
    ((t == I ? factor_remainder<CD, I, G>(buf, data, msg_len, parity, first, nb_tile, g, nblocks_total, R)
             : void()),
     ...);
}
template <typename CD, int... I>
__device__ __forceinline__ void rem_to_synd_t(int t, const uint32_t *rs, int stride, uint32_t (&S)[CD::D][8],
                                              std::integer_sequence<int, I...>) {
    ((t == I ? rem_to_synd<CD, I>(rs, stride, S, std::make_integer_sequence<int, CD::D>{}) : void()), ...);
}

// Syndromes of every block.  PLANES = false: E bytes per block, S_0 first.
// PLANES = true: bitsliced, for the solve kernel: group G (blocks 32G ..
// 32G+31) keeps plane word k = 8j + b (bit b of S_j) at
// planes[(G / 32) * kTileWords<E> + k * 32 + G % 32], so that 32 consecutive
// groups read or write one plane word with one coalesced access.
template <int E, bool PLANES, int G = kSyndGroups>
__global__ void __launch_bounds__(G * SyndCode<E>::T) bs_synd_kernel(const uint8_t *__restrict__ data,
                                                                         const uint8_t *__restrict__ parity,
                                                                         size_t nblocks, int msg_len,
                                                                         uint8_t *__restrict__ synds) {
    using CD = SyndCode<E>;
    constexpr int T = CD::T, D = CD::D;
    __shared__ uint32_t buf[G * 256];
    const int tid = threadIdx.x;
    // one factor per warp: warps T w .. T w + T - 1 share the 32 groups 32w .. 32w+31
    const int warp = tid >> 5, lane = tid & 31;
    const int t = warp % T, g = (warp / T) * 32 + lane;
    const size_t ntiles = (nblocks + G * 32 - 1) / (G * 32);
    for (size_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const size_t first = tile * G * 32;
        const int nb_tile = (int)min((size_t)G * 32, nblocks - first);
        uint32_t R[D][8];
        uint32_t S[D][8];
        factor_remainder_t<CD, G>(t, buf, data, msg_len, parity, first, nb_tile, g, nblocks, R,
                               std::make_integer_sequence<int, T>{});
        // stash remainders, interleaved by thread
        __syncthreads();
        const int stride = G * T;
#pragma unroll
        for (int m = 0; m < D; ++m)
#pragma unroll
            for (int b = 0; b < 8; ++b) buf[(m * 8 + b) * stride + tid] = R[m][b];
#pragma unroll
        for (int m = 0; m < D; ++m)
#pragma unroll
            for (int b = 0; b < 8; ++b) S[m][b] = 0u;
        rem_to_synd_t<CD>(t, buf + tid, stride, S, std::make_integer_sequence<int, T>{});
        if constexpr (PLANES) {
            const size_t G = first / 32 + g;
            if ((int)(g * 32) < nb_tile) {
                uint32_t *o = reinterpret_cast<uint32_t *>(synds) + (G / 32) * (size_t)kTileWords<E> + G % 32;
#pragma unroll
                for (int m = 0; m < D; ++m)
#pragma unroll
                    for (int b = 0; b < 8; ++b) o[((t * D + m) * 8 + b) * 32] = S[m][b];
            }
        } else {
            // S planes -> per-block syndrome bytes: 4 syndromes per transpose
#pragma unroll
            for (int q = 0; q < (D + 3) / 4; ++q) {
                uint32_t a[32];
#pragma unroll
                for (int k = 0; k < 32; ++k) a[k] = (q * 4 + k / 8 < D) ? S[(q * 4 + k / 8 < D) ? q * 4 + k / 8 : 0][k % 8] : 0u;
                transpose32(a);
                const int jb = t * D + q * 4;  // first syndrome index of this word
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    const size_t blk = first + (size_t)g * 32 + j;
                    if ((int)(g * 32 + j) < nb_tile) {
                        uint8_t *o = synds + blk * E + jb;
                        if (D >= 4) {
                            *reinterpret_cast<uint32_t *>(o) = a[j];
                        } else {
                            for (int k = 0; k < D; ++k) o[k] = (uint8_t)(a[j] >> (8 * k));
                        }
                    }
                }
            }
        }
    }
}

// encode, ecc 32 only (two factors): parity = CRT(R0, R1)
__global__ void __launch_bounds__(kGroups * 2) bs_encode32_kernel(const uint8_t *__restrict__ data, size_t nblocks,
                                                                  int msg_len, uint8_t *__restrict__ parity) {
    constexpr int E = 32, T = 2, D = 16;
    __shared__ uint32_t buf[kGroups * 256];
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int t = warp % T, g = (warp / T) * 32 + lane;
    const size_t ntiles = (nblocks + kGroups * 32 - 1) / (kGroups * 32);
    for (size_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const size_t first = tile * kGroups * 32;
        const int nb_tile = (int)min((size_t)kGroups * 32, nblocks - first);
        uint32_t R[D][8];
        if (t == 0)
            factor_remainder<Code<E>, 0>(buf, data, msg_len, nullptr, first, nb_tile, g, nblocks, R);
        else
            factor_remainder<Code<E>, 1>(buf, data, msg_len, nullptr, first, nb_tile, g, nblocks, R);
        __syncthreads();
        // stash: group g's two factor remainders, [(t*16+m)*8+b] * stride + g
        const int stride = kGroups;
#pragma unroll
        for (int m = 0; m < D; ++m)
#pragma unroll
            for (int b = 0; b < 8; ++b) buf[((t * 16 + m) * 8 + b) * stride + g] = R[m][b];
        __syncthreads();
        // thread t computes parity bytes 16t .. 16t+15 from all 32 remainder bytes
        uint32_t Pp[16][8];
#pragma unroll
        for (int p = 0; p < 16; ++p)
#pragma unroll
            for (int o = 0; o < 8; ++o) Pp[p][o] = 0u;
        if (t == 0)
            crt_map<0>(buf + g, stride, Pp, std::make_integer_sequence<int, 32>{});
        else
            crt_map<16>(buf + g, stride, Pp, std::make_integer_sequence<int, 32>{});
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            uint32_t a[32];
#pragma unroll
            for (int k = 0; k < 32; ++k) a[k] = Pp[q * 4 + k / 8][k % 8];
            transpose32(a);
            const int pb = t * 16 + q * 4;
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                if ((int)(g * 32 + j) < nb_tile)
                    *reinterpret_cast<uint32_t *>(parity + (first + (size_t)g * 32 + j) * E + pb) = a[j];
            }
        }
        __syncthreads();
    }
}


// ---------------------------------------------------------------- bitsliced solve
//
// Decoding from the bitsliced syndromes, 32 blocks per plane word, following
// rs_decode::decode (reed_solomon.hpp:559-595) step by step:
//   * Berlekamp-Massey (berlekamp_massey, reed_solomon.hpp:655-702) in its
//     inversion-free form C <- b C - d x^m B, with x^m B kept pre-shifted;
//     the length L is a 6-plane bitsliced counter;
//   * error evaluator Omega = S * C mod x^t (its degree is below L whenever
//     the decoder succeeds, so t coefficients are exact);
//   * Chien search over the positions 0 .. size-1 with x = a^{-i}, as the
//     reference scans them, counting the roots of every block;
//   * Forney: e = Omega(x) / Lodd(x) with Lodd the odd-degree part of C, which
//     equals X * Omega(X^-1) / C'(X^-1) of the reference in characteristic 2.
// A block is repaired when its syndromes are non-zero, L <= ecc/2 and the
// number of roots equals L; this is exactly when the reference returns true
// (with roots == L, C has L distinct roots and Omega != 0).
//
// bs_bm_kernel runs Berlekamp-Massey and the evaluator, bs_chien_kernel the
// Chien search, Forney and the corrections; one CTA = one tile of 32 groups
// (1024 blocks) in both.

__device__ __forceinline__ void reduce15(uint32_t (&p)[15], uint32_t (&r)[8]) {
#pragma unroll
    for (int k = 14; k >= 8; --k) {  // x^8 = x^4 + x^3 + x^2 + 1
        p[k - 8] ^= p[k];
        p[k - 6] ^= p[k];
        p[k - 5] ^= p[k];
        p[k - 4] ^= p[k];
    }
#pragma unroll
    for (int o = 0; o < 8; ++o) r[o] = p[o];
}

// r = a * b (r may alias a or b)
__device__ __forceinline__ void vmul(const uint32_t (&a)[8], const uint32_t (&b)[8], uint32_t (&r)[8]) {
    uint32_t p[15];
#pragma unroll
    for (int k = 0; k < 15; ++k) p[k] = 0u;
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) p[i + j] = andxor(a[i], b[j], p[i + j]);
    reduce15(p, r);
}

// p += a * b without the reduction (15 planes); several products can share
// one reduce15
__device__ __forceinline__ void vmul_acc15(const uint32_t (&a)[8], const uint32_t (&b)[8], uint32_t (&p)[15]) {
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) p[i + j] = andxor(a[i], b[j], p[i + j]);
}

__device__ __forceinline__ void vsqr(const uint32_t (&a)[8], uint32_t (&r)[8]) {
    uint32_t p[15];
#pragma unroll
    for (int k = 0; k < 15; ++k) p[k] = (k & 1) ? 0u : a[k >> 1];
    reduce15(p, r);
}

// r = x^254 = 1 / x (0 for x = 0): x^240 * x^14 with x^240 = (x^15)^16
__device__ __forceinline__ void vinv(const uint32_t (&x)[8], uint32_t (&r)[8]) {
    uint32_t x2[8], x3[8], x12[8], x14[8], y[8];
    vsqr(x, x2);
    vmul(x2, x, x3);
    vsqr(x3, y);
    vsqr(y, x12);
    vmul(x12, x2, x14);
    vmul(x12, x3, y);  // x^15
#pragma unroll
    for (int k = 0; k < 4; ++k) vsqr(y, y);
    vmul(y, x14, r);
}

constexpr int next_bit(int s, int from) {
    while (from < 8 && !((s >> from) & 1)) ++from;
    return from;
}

// acc ^ XOR of in[b] over the set bits b >= B of S, two inputs per LOP3
template <uint8_t S, int B>
__device__ __forceinline__ uint32_t xsel_acc(uint32_t acc, const uint32_t (&in)[8]) {
    constexpr int f = next_bit(S, B);
    if constexpr (f >= 8) {
        return acc;
    } else {
        constexpr int g = next_bit(S, f + 1);
        if constexpr (g >= 8)
            return acc ^ in[f];
        else
            return xsel_acc<S, g + 1>(xor3(acc, in[f], in[g]), in);
    }
}

// XOR of in[b] over the set bits b of S
template <uint8_t S>
__device__ __forceinline__ uint32_t xsel(const uint32_t (&in)[8]) {
    constexpr int f = next_bit(S, 0);
    if constexpr (f >= 8)
        return 0u;
    else
        return xsel_acc<S, f + 1>(in[f], in);
}

template <uint8_t C, int... O>
__device__ __forceinline__ void cmul_(const uint32_t (&in)[8], uint32_t (&out)[8], std::integer_sequence<int, O...>) {
    ((out[O] = xsel<sel_of(C, O)>(in)), ...);
}

// x <- C * x, C a compile-time constant
template <uint8_t C>
__device__ __forceinline__ void cmul_inplace(uint32_t (&x)[8]) {
    uint32_t o[8];
    cmul_<C>(x, o, std::make_integer_sequence<int, 8>{});
#pragma unroll
    for (int b = 0; b < 8; ++b) x[b] = o[b];
}

// per-block L <= c for a warp-uniform constant c
__device__ __forceinline__ uint32_t le_const(const uint32_t (&L)[6], int c) {
    uint32_t gt = 0u, eq = ~0u;
#pragma unroll
    for (int b = 5; b >= 0; --b) {
        const uint32_t cb = ((c >> b) & 1) ? ~0u : 0u;
        gt |= eq & L[b] & ~cb;
        eq &= ~(L[b] ^ cb);
    }
    return ~gt;
}

// L <- cond ? a - L : L (6 bits, a warp-uniform constant)
__device__ __forceinline__ void l_update(uint32_t (&L)[6], int a, uint32_t cond) {
    uint32_t carry = ~0u;  // a + ~L + 1
#pragma unroll
    for (int b = 0; b < 6; ++b) {
        const uint32_t ab = ((a >> b) & 1) ? ~0u : 0u;
        const uint32_t x = ~L[b];
        const uint32_t s = ab ^ x ^ carry;
        carry = (ab & x) | (carry & (ab ^ x));
        L[b] = bitsel(cond, s, L[b]);
    }
}

// the largest L of the 32 x 32 blocks of a warp (bit-serial per lane, then
// across the lanes): warp-uniform
__device__ __forceinline__ int max_len(const uint32_t (&L)[6]) {
    uint32_t cand = ~0u;
    int res = 0;
#pragma unroll
    for (int b = 5; b >= 0; --b) {
        const uint32_t t = cand & L[b];
        const bool nz = t != 0u;
        res |= (int)nz << b;
        cand = nz ? t : cand;
    }
    return (int)__reduce_max_sync(0xffffffffu, (unsigned)res);
}

template <int E>
struct SolveGeom {
    static constexpr int P = 4;              // warps per tile
    static constexpr int t = E / 2;
    static constexpr int K = t / P;          // C coefficients and Omega terms per warp
    static constexpr int kS = E * 8 * 32;    // words: syndrome planes of 32 groups
    // BM exchange rows: the d partials of every warp, then the top C and Bs
    // of every warp but the last (the next warp's lower neighbours)
    static constexpr int kXrows = P * 8 + (P - 1) * 16;
    static constexpr int kX = 2 * kXrows * 32;     // double-buffered
    static constexpr int kCp = (t + 1) * 8 * 32;   // C_0..C_t planes (Omega)
    static constexpr int kWords = kS + (kX > kCp ? kX : kCp);
    static constexpr size_t smem = (size_t)kWords * 4;
    static_assert(K % 2 == 0, "K must be even");
};

// Berlekamp-Massey and the error evaluator of a tile.  One CTA = 32 groups
// (1024 blocks) and P = 4 warps: warp h keeps the coefficients C_i, i = hK+1
// .. hK+K (K = t/P), and computes the evaluator terms Omega_k, k = Pv+h; warp
// 0 also keeps C_0.  The warps meet through shared memory once per BM
// iteration.  The result goes to the tile's record (RecLayout) for
// bs_chien_kernel.
//
// Berlekamp-Massey runs inversion-free: C <- b C + d x^m B, B <- C and b <- d
// on a length change.  Every C it produces is a non-zero multiple (per block)
// of the normalised algorithm's C <- C - (d / b) x^m B, its discrepancies are
// the same multiples of the normalised ones (so the same length changes
// happen), and Omega = S C mod x^t carries the same factor: the roots, the
// root count, L and the Forney values Omega(x) / Lodd(x) are the normalised
// algorithm's.
template <int E>
__global__ void __launch_bounds__(128, 4) bs_bm_kernel(size_t nblocks, uint32_t *__restrict__ planes) {
    using G = SolveGeom<E>;
    constexpr int t = G::t, K = G::K, P = G::P;
    extern __shared__ __align__(16) uint32_t sm[];
    uint32_t *Ssm = sm;           // [E*8][32] syndrome planes
    uint32_t *Xb = sm + G::kS;    // BM exchange, then the C planes
    uint32_t *Csm = Xb;

    const int lane = threadIdx.x & 31, h = threadIdx.x >> 5;
    const size_t ngroups = (nblocks + 31) / 32;
    const size_t tile = blockIdx.x;
    const size_t grp = tile * 32 + lane;
    const bool valid = grp < ngroups;
    uint32_t *tplanes = planes + tile * (size_t)kTileWords<E>;

    // phase 0: syndrome planes of the 32 groups, one contiguous region of
    // E * 1024 bytes, copied asynchronously 16 bytes per thread and round
    // (groups past the end hold stale words; their blocks are never touched)
    {
        const char *src = reinterpret_cast<const char *>(tplanes);
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(Ssm);
#pragma unroll 4
        for (int off = threadIdx.x * 16; off < E * 1024; off += 128 * 16)
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst + off), "l"(src + off) : "memory");
        asm volatile("cp.async.commit_group;" ::: "memory");
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    __syncthreads();
    uint32_t anyS = 0u;
    for (int k = 0; k < E * 8; ++k) anyS |= Ssm[k * 32 + lane];
    const size_t blk0 = grp * 32;
    const uint32_t vmask = !valid ? 0u : (nblocks - blk0 >= 32 ? ~0u : ((1u << (nblocks - blk0)) - 1u));

    // phase 1: Berlekamp-Massey
    uint32_t C[K][8], Bs[K][8], C0[8], bb[8], L[6];
#pragma unroll
    for (int u = 0; u < K; ++u)
#pragma unroll
        for (int b = 0; b < 8; ++b) {
            C[u][b] = 0u;
            Bs[u][b] = (h == 0 && u == 0 && b == 0) ? ~0u : 0u;  // x^1 * B, B = 1
        }
#pragma unroll
    for (int b = 0; b < 8; ++b) C0[b] = bb[b] = b == 0 ? ~0u : 0u;  // C_0 = 1, b = 1
#pragma unroll
    for (int b = 0; b < 6; ++b) L[b] = 0u;
    constexpr int kTop = P * 8;  // first exchange row of the warp tops
    int lmax = 0;                // the tile's largest L (every warp holds the same L planes)
#pragma unroll 1
    for (int n = 0; n < E; ++n) {
        // partial discrepancy, one reduction for all products; at the start
        // of iteration n, C_i = 0 for i > n
        uint32_t p15[15];
#pragma unroll
        for (int k = 0; k < 15; ++k) p15[k] = 0u;
        if (h == 0) {
            uint32_t sn[8];
#pragma unroll
            for (int b = 0; b < 8; ++b) sn[b] = Ssm[(n * 8 + b) * 32 + lane];
            vmul_acc15(C0, sn, p15);
        }
#pragma unroll
        for (int u = 0; u < K; ++u) {
            const int j = n - (h * K + 1 + u);
            if (j >= 0 && h * K + 1 + u <= lmax) {
                uint32_t sj[8];
#pragma unroll
                for (int b = 0; b < 8; ++b) sj[b] = Ssm[(j * 8 + b) * 32 + lane];
                vmul_acc15(C[u], sj, p15);
            }
        }
        uint32_t dp[8];
        reduce15(p15, dp);
        uint32_t *X = Xb + (n & 1) * (G::kXrows * 32);
#pragma unroll
        for (int b = 0; b < 8; ++b) X[(h * 8 + b) * 32 + lane] = dp[b];
        if (h < P - 1) {
#pragma unroll
            for (int b = 0; b < 8; ++b) {
                X[(kTop + h * 16 + b) * 32 + lane] = C[K - 1][b];
                X[(kTop + h * 16 + 8 + b) * 32 + lane] = Bs[K - 1][b];
            }
        }
        __syncthreads();
        uint32_t d[8], nzd = 0u;
#pragma unroll
        for (int b = 0; b < 8; ++b) {
            uint32_t s = X[b * 32 + lane];
#pragma unroll
            for (int w = 1; w < P; ++w) s ^= X[(w * 8 + b) * 32 + lane];
            d[b] = s;
            nzd |= s;
        }
        const uint32_t cond = nzd & le_const(L, n >> 1);
        // the new lengths first: every block's new C has degree at most its
        // new L, so the products above the tile's largest new L are zero
        l_update(L, n + 1, cond);
        lmax = max_len(L);
        // C_i <- b C_i + d Bs_i and Bs_i <- cond ? C_{i-1} : Bs_{i-1}, from
        // the top down; C_i = Bs_i = 0 for i > n+1, so those products are
        // skipped, and so are those above lmax
#pragma unroll
        for (int u = K - 1; u >= 0; --u) {
            uint32_t lc[8], lb[8];
#pragma unroll
            for (int b = 0; b < 8; ++b) {
                if (u > 0) {
                    lc[b] = C[u - 1][b];
                    lb[b] = Bs[u - 1][b];
                } else if (h == 0) {
                    lc[b] = C0[b];  // Bs_0 = 0
                    lb[b] = 0u;
                } else {
                    lc[b] = X[(kTop + (h - 1) * 16 + b) * 32 + lane];
                    lb[b] = X[(kTop + (h - 1) * 16 + 8 + b) * 32 + lane];
                }
            }
            if (h * K + 1 + u <= n + 1 && h * K + 1 + u <= lmax) {
                uint32_t pr[15];
#pragma unroll
                for (int k = 0; k < 15; ++k) pr[k] = 0u;
                vmul_acc15(bb, C[u], pr);
                vmul_acc15(d, Bs[u], pr);
                reduce15(pr, C[u]);
            }
#pragma unroll
            for (int b = 0; b < 8; ++b) Bs[u][b] = bitsel(cond, lc[b], lb[b]);
        }
        if (h == 0) vmul(bb, C0, C0);
#pragma unroll
        for (int b = 0; b < 8; ++b) bb[b] = bitsel(cond, d[b], bb[b]);
    }
    __syncthreads();  // BM exchange reads done before the C planes overwrite it

    // phase 2: Omega_k = sum_{i=0}^{k} C_i S_{k-i}, k = Pv + h
    if (h == 0) {
#pragma unroll
        for (int b = 0; b < 8; ++b) Csm[b * 32 + lane] = C0[b];
    }
#pragma unroll
    for (int u = 0; u < K; ++u)
#pragma unroll
        for (int b = 0; b < 8; ++b) Csm[((h * K + u + 1) * 8 + b) * 32 + lane] = C[u][b];
    __syncthreads();
    uint32_t Ot[K][8];
#pragma unroll
    for (int v = 0; v < K; ++v) {
        const int k = P * v + h;
        uint32_t p15[15];
#pragma unroll
        for (int q = 0; q < 15; ++q) p15[q] = 0u;
        for (int i = 0; i <= k; ++i) {
            uint32_t ci[8], sj[8];
#pragma unroll
            for (int b = 0; b < 8; ++b) {
                ci[b] = Csm[(i * 8 + b) * 32 + lane];
                sj[b] = Ssm[((k - i) * 8 + b) * 32 + lane];
            }
            vmul_acc15(ci, sj, p15);
        }
        reduce15(p15, Ot[v]);
    }
    // the record (RecLayout) over this tile's syndromes: every syndrome of the
    // tile was read into shared memory in phase 0, by this CTA only
    using R = RecLayout<E>;
    uint32_t *rec = tplanes + lane;
    if (h == 0) {
#pragma unroll
        for (int b = 0; b < 8; ++b) rec[(R::kC + b) * 32] = C0[b];
#pragma unroll
        for (int b = 0; b < 6; ++b) rec[(R::kL + b) * 32] = L[b];
        rec[R::kLive * 32] = anyS & vmask;
    }
#pragma unroll
    for (int u = 0; u < K; ++u)
#pragma unroll
        for (int b = 0; b < 8; ++b) rec[(R::kC + 8 * (h * K + 1 + u) + b) * 32] = C[u][b];
#pragma unroll
    for (int v = 0; v < K; ++v)
#pragma unroll
        for (int b = 0; b < 8; ++b) rec[(R::kOm + 8 * (P * v + h) + b) * 32] = Ot[v][b];
}

// ---------------------------------------------------------------- syndromes by bit plane (ecc 32)
//
// bs_synd32_kernel: the bitsliced syndromes of ecc_len 32 through the
// generated networks of rs256_synd_gen.cuh (split by bit plane, odd j and
// j = 0 evaluated per plane, Horner in steps of 32 degrees).  One CTA per
// tile (32 groups, 1024 blocks), eight warps: warp w evaluates bit plane w
// of every group, lane = group.  Per window of 32 degrees (255 .. 0):
//   * load: the window's bytes of every block as 4-byte words (cp.async, one
//     window ahead of the arithmetic; zeros before the block's first degree);
//   * transpose: thread (w, group) turns column w (window bytes 4w .. 4w+3)
//     of the group's 32 blocks into 8 planes x 4 degrees;
//   * Horner step: warp w reads plane w of the window's 32 degrees.
// The rows of the eight planes are then combined into S_0 .. S_31 (two
// halves through shared memory) and stored as the tile's syndrome planes.
struct Synd32Geom {
    static constexpr int kRawStride = 32 * 9 + 1;   // words per group: 32 blocks x 9 words, + 1 against conflicts
    static constexpr int kRaw = 32 * kRawStride;    // one window of the tile
    static constexpr int kP = 8 * 32 * 32;          // planes [bit][degree][group]
    static constexpr int kWords = 2 * kRaw + kP;
    static_assert(kSyndRowsB * 8 * 32 <= 2 * kRaw && kSyndRowsA <= kSyndRowsB, "exchange does not fit");
    static constexpr size_t smem = (size_t)kWords * 4;
};

// cp.async of window w's words of the tile into raw: block b's word k at
// raw[(b / 32) * kRawStride + (b % 32) * 9 + k].  Bytes outside the array
// are zero-filled (not read).
__device__ __forceinline__ void synd32_load(uint32_t *raw, const uint8_t *__restrict__ data,
                                            const uint8_t *__restrict__ parity, size_t nblocks, int msg_len,
                                            size_t first, int w) {
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(raw);
    const int t = threadIdx.x;
    if (w < 7) {
        // offsets relative to the tile's first data byte fit in 32 bits;
        // word q = 9 b + k of the window goes to thread q % 256, so that a
        // warp reads whole consecutive stretches of the tile
        // bytes from tile0 to the end of the array, clamped: a window's
        // offsets stay below 2^18.  Offsets precede the array only in the
        // first tile (elsewhere tile0 >= 1024 > 224 bytes back).
        const long long tile0 = (long long)first * msg_len;
        const long long left = (long long)(nblocks * (size_t)msg_len) - tile0;
        const int total = left < (1 << 30) ? (int)left : (1 << 30);
        const int lo = first == 0 ? 0 : -(1 << 30);
        const int c = msg_len - 224 + 32 * w;
        const uint8_t *tb = data + tile0;
        int b = t / 9, k = t - 9 * (t / 9);
#pragma unroll 4
        for (int i = 0; i < 36; ++i) {
            const int ak = ((b * msg_len + c) & ~3) + 4 * k;  // may precede the array
            const bool in = ak >= lo && ak < total;
            // the word holding the array's last byte is read only up to it
            const int nbytes = in ? min(4, total - ak) : 0;
            const uint32_t dst = sbase + (uint32_t)(((b >> 5) * Synd32Geom::kRawStride + (b & 31) * 9 + k) * 4);
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(dst), "l"(in ? tb + ak : data),
                         "r"(nbytes)
                         : "memory");
            // q += 256 = 9 * 28 + 4
            b += 28;
            k += 4;
            if (k >= 9) {
                k -= 9;
                ++b;
            }
        }
    } else {
        // the parity bytes of the tile are one contiguous stretch: word q of it
        // (block q / 8, word q % 8) goes to thread q % 256
        const long long total = (long long)(nblocks * 32) - (long long)first * 32;
        const uint8_t *tb = parity + first * 32;
#pragma unroll 4
        for (int i = 0; i < 32; ++i) {
            const int q = t + 256 * i, b = q >> 3, k = q & 7;
            const bool in = (long long)q * 4 < total;
            const uint32_t dst = sbase + (uint32_t)(((b >> 5) * Synd32Geom::kRawStride + (b & 31) * 9 + k) * 4);
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(dst), "l"(in ? tb + 4 * q : parity),
                         "r"(in ? 4 : 0)
                         : "memory");
        }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

// Thread (w, lane) of a tile's CTA: column w (window bytes 4w .. 4w+3) of the
// 32 blocks of group `lane`, staged in raw by synd32_load, into the bit
// planes P[(b * 32 + k) * 32 + lane] (bit b of window byte k, bit j = block
// j).  Message windows (win < 7) are realigned from the staged words and
// cleared before the block's first byte.
__device__ __forceinline__ void synd32_transpose(const uint32_t *raw, uint32_t *P, int win, size_t first,
                                                 int msg_len, int lane, int w) {
    using G = Synd32Geom;
    uint32_t a[32];
    const uint32_t *rg = raw + lane * G::kRawStride + w;
    if (win < 7) {
        const long long p0 = (long long)msg_len - 224;  // first data byte of window 0
        const long long c0 = p0 + 32 * win + 4 * w;     // position of the column's first byte
        const uint32_t keep = c0 >= 0 ? ~0u : (c0 <= -4 ? 0u : (~0u << (8 * (int)(-c0))));
        // byte offset (mod 4) of block j's window: (first + 32 lane + j) * msg_len + p0
        uint32_t off = (uint32_t)((((long long)first * msg_len + p0) & 3) + (uint32_t)(lane * 32 * msg_len));
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            a[j] = __funnelshift_r(rg[j * 9], rg[j * 9 + 1], (off & 3) * 8) & keep;
            off += (uint32_t)msg_len;
        }
    } else {
#pragma unroll
        for (int j = 0; j < 32; ++j) a[j] = rg[j * 9];
    }
    transpose32(a);  // a[8r + b]: bit b of window byte 4w + r, bit j = block j
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int b = 0; b < 8; ++b) P[(b * 32 + 4 * w + r) * 32 + lane] = a[8 * r + b];
}

// The rows s of the eight planes (thread (w, lane) holds plane w of group
// lane) into the syndrome planes out[(8j + b) * 32] (bit b of S_j; out is
// offset by lane), in two halves through X (offset by lane).  Starts and ends
// with a barrier.
__device__ __forceinline__ void synd32_combine(const uint32_t (&s)[kSyndRows], uint32_t *X, uint32_t *out, int w) {
    __syncthreads();
#pragma unroll
    for (int i = 0; i < kSyndRowsA; ++i) X[(i * 8 + w) * 32] = s[i];
    __syncthreads();
    switch (w) {
        case 0: synd_combine_A0(X, out); break;
        case 1: synd_combine_A1(X, out); break;
        case 2: synd_combine_A2(X, out); break;
        case 3: synd_combine_A3(X, out); break;
        case 4: synd_combine_A4(X, out); break;
        case 5: synd_combine_A5(X, out); break;
        case 6: synd_combine_A6(X, out); break;
        default: synd_combine_A7(X, out); break;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < kSyndRowsB; ++i) X[(i * 8 + w) * 32] = s[kSyndRowsA + i];
    __syncthreads();
    switch (w) {
        case 0: synd_combine_B0(X, out); break;
        case 1: synd_combine_B1(X, out); break;
        case 2: synd_combine_B2(X, out); break;
        case 3: synd_combine_B3(X, out); break;
        case 4: synd_combine_B4(X, out); break;
        case 5: synd_combine_B5(X, out); break;
        case 6: synd_combine_B6(X, out); break;
        default: synd_combine_B7(X, out); break;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(256, 1) bs_synd32_kernel(const uint8_t *__restrict__ data,
                                                           const uint8_t *__restrict__ parity, size_t nblocks,
                                                           int msg_len, uint32_t *__restrict__ planes) {
    using G = Synd32Geom;
    extern __shared__ __align__(16) uint32_t sm[];
    uint32_t *raw0 = sm, *P = sm + 2 * G::kRaw;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const size_t tile = blockIdx.x, first = tile * 1024;
    uint32_t s[kSyndRows];
#pragma unroll
    for (int i = 0; i < kSyndRows; ++i) s[i] = 0u;
    synd32_load(raw0, data, parity, nblocks, msg_len, first, 0);
#pragma unroll 1
    for (int win = 0; win < 8; ++win) {
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        __syncthreads();
        synd32_transpose(raw0 + (win & 1) * G::kRaw, P, win, first, msg_len, lane, w);
        __syncthreads();
        if (win < 7) synd32_load(raw0 + ((win + 1) & 1) * G::kRaw, data, parity, nblocks, msg_len, first, win + 1);
        const uint32_t *Pw = P + w * 32 * 32 + lane;
        synd_step32([&](int k) { return Pw[k * 32]; }, s);
    }
    // the rows of all planes into S_j
    synd32_combine(s, raw0 + lane, planes + tile * (size_t)kTileWords<32> + lane, w);
}

// ---------------------------------------------------------------- encode by nibble tables (ecc 32)
//
// The tables, their layout and one lane's part of a block are in
// rs256_nib.cuh; the kernel stages the tables and gives each quarter warp a
// block.

// tab: kNibWords words (all degree groups); dynamic shared memory holds the
// groups of degree indices 0 .. ml - 1.  Each warp takes four blocks at a
// time, one per quarter.
__global__ void __launch_bounds__(1024, 1) rs256_encode_nib_kernel(const uint8_t *__restrict__ data, size_t nblocks,
                                                                    int ml, const uint4 *__restrict__ tab,
                                                                    uint8_t *__restrict__ parity) {
    extern __shared__ __align__(16) uint4 T[];
    {
        const uint32_t tb = (uint32_t)__cvta_generic_to_shared(T);
        const int nq = (ml + 3) / 4 * kNibGroupQ;
        for (int q = threadIdx.x; q < nq; q += blockDim.x)
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(tb + 16u * q), "l"(tab + q) : "memory");
        asm volatile("cp.async.commit_group;" ::: "memory");
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        __syncthreads();
    }
    const int lane = threadIdx.x & 31, quarter = lane >> 3, rh = lane & 7, r = rh >> 1, h = rh & 1;
    const uintptr_t d0 = (uintptr_t)data, d1 = d0 + nblocks * (size_t)ml;
    const bool out16 = ((uintptr_t)parity & 15) == 0;
    const size_t nwarps = (size_t)gridDim.x * (blockDim.x >> 5);
    for (size_t base = ((size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 4; base < nblocks;
         base += nwarps * 4) {
        const size_t b = base + quarter;
        uint4 acc = make_uint4(0u, 0u, 0u, 0u);
        if (b < nblocks) acc = nib_lane(T, d0, d1, b, ml, r, h);
        // XOR of the four residues r (lane bits 1 and 2)
#pragma unroll
        for (int m = 2; m <= 4; m <<= 1) {
            acc.x ^= __shfl_xor_sync(0xffffffffu, acc.x, m);
            acc.y ^= __shfl_xor_sync(0xffffffffu, acc.y, m);
            acc.z ^= __shfl_xor_sync(0xffffffffu, acc.z, m);
            acc.w ^= __shfl_xor_sync(0xffffffffu, acc.w, m);
        }
        if (b < nblocks && r == 0) {
            uint8_t *o = parity + b * 32 + 16 * h;
            if (out16) {
                *reinterpret_cast<uint4 *>(o) = acc;
            } else {
                uint32_t *o4 = reinterpret_cast<uint32_t *>(o);
                o4[0] = acc.x, o4[1] = acc.y, o4[2] = acc.z, o4[3] = acc.w;
            }
        }
    }
}

// ---------------------------------------------------------------- Chien search and Forney
//
// bs_chien_kernel: one CTA per tile (32 groups, 1024 blocks) and four warps;
// lane = group.  From the Berlekamp-Massey record of every group:
//   1. Chien search over the scan indices i = 0 .. size-1 (x = a^{-i}, the
//      error degree; byte position size-1-i, as the reference scans them):
//      warp h takes i = 64h .. 64h+63 and holds all t + 1 terms C_k x^k, so a
//      position needs no exchange between warps; the blocks whose locator
//      vanishes there form one root-mask word.
//   2. The 256 root masks of a group become 8 words per block (32 x 32 bit
//      transposes).
//   3. Per block: the root count and the roots in scan order, one slot each.
//   4. Forney per slot, bitsliced over the 32 blocks of a group: x of the
//      slot's root, e = Omega(x) / Lodd(x) (Horner on both, one inversion).
//   5. Status and corrections, as rs_decode::decode (reed_solomon.hpp:
//      559-595): a block with non-zero syndromes is repaired exactly when
//      L <= t and it has L roots; otherwise it is left untouched.
template <int E>
struct ChienGeom {
    static constexpr int t = E / 2;
    static constexpr int R = t / 4;                 // slots per thread (phase 4)
    static constexpr int kA = 256 * 33;             // root masks, then their transposes, then coefficients
    static constexpr int kCoef = (t + t / 2) * 8;   // Omega_0..t-1, C_1, C_3, .., C_{t-1}: planes per group
    static_assert(kCoef * 32 <= kA, "coefficients do not fit");
    static constexpr int kX = 32 * 4 * 32;          // packed x (then e) bytes [block][4][group]
    static constexpr int kDeg = t * 32 * 32 / 4;    // root scan indices, bytes [slot][block][group]
    static constexpr int kCnt = 32 * 32 / 4;        // root counts, bytes [block][group]
    static constexpr int kExp = 256 / 4;            // a^0 .. a^254 (bytes)
    static constexpr int kWords = kA + kX + kDeg + kCnt + kExp;
    static constexpr size_t smem = (size_t)kWords * 4;
};

template <int E, int H, int... K>
__device__ __forceinline__ void chien_start(uint32_t (&T)[E / 2 + 1][8], std::integer_sequence<int, K...>) {
    // T_k <- C_k a^{-64 H k}, k = 1..t
    (cmul_inplace<apow(-(64 * H * (K + 1)))>(T[K + 1]), ...);
}

template <int E, int... K>
__device__ __forceinline__ void chien_next(uint32_t (&T)[E / 2 + 1][8], std::integer_sequence<int, K...>) {
    // T_k <- T_k a^{-k}, k = 1..t
    (cmul_inplace<apow(-(K + 1))>(T[K + 1]), ...);
}

// positions 64H .. 64H+63 of one group: root-mask words into rm[i * 32]
template <int E, int H>
__device__ __forceinline__ void chien_scan(uint32_t (&T)[E / 2 + 1][8], int size, uint32_t live, uint32_t *rm) {
    constexpr int t = E / 2;
    chien_start<E, H>(T, std::make_integer_sequence<int, t>{});
#pragma unroll 1
    for (int p = 0; p < 64; ++p) {
        const int i = 64 * H + p;
        uint32_t nz = 0u;
#pragma unroll
        for (int b = 0; b < 8; ++b) {
            uint32_t v = T[0][b];
#pragma unroll
            for (int k = 1; k <= t; k += 2) v = (k + 1 <= t) ? xor3(v, T[k][b], T[k + 1][b]) : (v ^ T[k][b]);
            nz |= v;
        }
        rm[i * 32] = i < size ? (~nz & live) : 0u;
        chien_next<E>(T, std::make_integer_sequence<int, t>{});
    }
}

template <int E>
__global__ void __launch_bounds__(128, 3) bs_chien_kernel(uint8_t *__restrict__ data, uint8_t *__restrict__ parity,
                                                          size_t nblocks, int msg_len,
                                                          const uint32_t *__restrict__ planes,
                                                          uint8_t *__restrict__ status,
                                                          const uint8_t *__restrict__ exp512) {
    using G = ChienGeom<E>;
    using Rl = RecLayout<E>;
    constexpr int t = G::t, RS = G::R;
    extern __shared__ __align__(16) uint32_t sm[];
    uint32_t *A = sm;                   // [256][32] masks; [32 blocks * 8][33] transposed; coefficients
    uint32_t *Xv = sm + G::kA;          // [block][4][group] packed x, then e
    uint8_t *deg = reinterpret_cast<uint8_t *>(Xv + G::kX);         // [slot][block][group]
    uint8_t *cnt = deg + G::kDeg * 4;                                // [block][group]
    uint8_t *ex = cnt + G::kCnt * 4;                                 // a^0 .. a^254

    const int lane = threadIdx.x & 31, h = threadIdx.x >> 5;
    const size_t tile = blockIdx.x;
    const uint32_t *rec = planes + tile * (size_t)kTileWords<E> + lane;
    const int size = msg_len + E;
    for (int i = threadIdx.x; i < 255; i += 128) ex[i] = exp512[i];
    const uint32_t live = rec[Rl::kLive * 32];

    // phase 1: Chien search
    {
        uint32_t T[t + 1][8];
#pragma unroll
        for (int k = 0; k <= t; ++k)
#pragma unroll
            for (int b = 0; b < 8; ++b) T[k][b] = rec[(Rl::kC + 8 * k + b) * 32];
        switch (h) {
            case 0: chien_scan<E, 0>(T, size, live, A + lane); break;
            case 1: chien_scan<E, 1>(T, size, live, A + lane); break;
            case 2: chien_scan<E, 2>(T, size, live, A + lane); break;
            default: chien_scan<E, 3>(T, size, live, A + lane); break;
        }
    }
    __syncthreads();

    // phase 2: masks of positions 32q .. 32q+31 (q = 2h, 2h+1) to one word per
    // block (bit r: a root at position 32q + r), stored at [(j * 8 + q)][33]
    {
        uint32_t a[2][32];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
#pragma unroll
            for (int r = 0; r < 32; ++r) a[u][r] = A[((2 * h + u) * 32 + r) * 32 + lane];
            transpose32(a[u]);
        }
        __syncthreads();
#pragma unroll
        for (int u = 0; u < 2; ++u)
#pragma unroll
            for (int j = 0; j < 32; ++j) A[(j * 8 + 2 * h + u) * 33 + lane] = a[u][j];
    }
    __syncthreads();

    // phase 3: per block (j = 8h .. 8h+7) the root count and the roots in scan
    // order; slot s keeps the scan index and x = a^{-i} (packed: word
    // [j][s % 4], byte s / 4)
#pragma unroll 1
    for (int j = 8 * h; j < 8 * h + 8; ++j) {
        int c = 0;
#pragma unroll 1
        for (int q = 0; q < 8; ++q) {
            uint32_t w = A[(j * 8 + q) * 33 + lane];
            while (w) {
                const int r = __ffs(w) - 1;
                w &= w - 1;
                if (c < t) {
                    const int i = 32 * q + r;
                    deg[(c * 32 + j) * 32 + lane] = (uint8_t)i;
                    reinterpret_cast<uint8_t *>(Xv + (j * 4 + (c & 3)) * 32 + lane)[c >> 2] = ex[(255 - i) % 255];
                }
                ++c;
            }
        }
        cnt[j * 32 + lane] = (uint8_t)(c < 255 ? c : 255);
    }
    __syncthreads();

    // The corrections of phase 5 change a few bytes in most lines of the
    // tile's data, which the syndrome kernel read long before (evicted from
    // L2 by then).  The tile's data and parity are two contiguous stretches:
    // prefetch them into L2 now, so that phase 4 hides the DRAM reads and the
    // final XORs hit L2 (issued at the kernel's start, the prefetches of all
    // resident tiles held about as much as L2 and were partly evicted again).  Bulk prefetches need 16-byte aligned
    // addresses and sizes: each stretch is trimmed inwards to that, in pieces
    // of at most 2 KiB.
    {
        const size_t first = tile * 1024;
        const size_t nb = nblocks - first < 1024 ? nblocks - first : 1024;
        const uintptr_t d0 = reinterpret_cast<uintptr_t>(data + first * (size_t)msg_len);
        const uintptr_t p0 = reinterpret_cast<uintptr_t>(parity + first * E);
        const uintptr_t db = (d0 + 15) & ~(uintptr_t)15, de = (d0 + nb * (size_t)msg_len) & ~(uintptr_t)15;
        const uintptr_t pb = (p0 + 15) & ~(uintptr_t)15, pe = (p0 + nb * E) & ~(uintptr_t)15;
        const size_t dn = de > db ? de - db : 0, pn = pe > pb ? pe - pb : 0;
        const size_t dpieces = (dn + 2047) / 2048, ppieces = (pn + 2047) / 2048;
        for (size_t q = threadIdx.x; q < dpieces + ppieces; q += 128) {
            const bool isd = q < dpieces;
            const size_t off = (isd ? q : q - dpieces) * 2048, len = isd ? dn : pn;
            const uint32_t n = (uint32_t)(len - off < 2048 ? len - off : 2048);  // a multiple of 16
            asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"((isd ? db : pb) + off), "r"(n) : "memory");
        }
    }
    // phase 4: Forney.  The coefficient planes go to shared memory first
    // (Omega_0..t-1, then C_1, C_3, ..., C_{t-1}); thread h evaluates the
    // slots 4r + h (r < t/4) of all 32 blocks of its group.
    for (int w = h; w < G::kCoef; w += 4)
        A[w * 32 + lane] = w < 8 * t ? rec[(Rl::kOm + w) * 32] : rec[(Rl::kC + 8 * (2 * ((w - 8 * t) / 8) + 1) + (w & 7)) * 32];
    __syncthreads();
    {
        uint32_t a[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) a[j] = Xv[(j * 4 + h) * 32 + lane];
        transpose32(a);  // a[8r + b]: bit b of x, slot 4r + h, bit j = block j
        // Horner for all RS slots at once: each coefficient is read once and
        // feeds RS independent products
        uint32_t om[RS][8], y[RS][8], lo[RS][8];
#pragma unroll
        for (int r = 0; r < RS; ++r)
#pragma unroll
            for (int b = 0; b < 8; ++b) om[r][b] = A[(8 * (t - 1) + b) * 32 + lane];
#pragma unroll 1
        for (int k = t - 2; k >= 0; --k) {
            uint32_t cf[8];
#pragma unroll
            for (int b = 0; b < 8; ++b) cf[b] = A[(8 * k + b) * 32 + lane];
#pragma unroll
            for (int r = 0; r < RS; ++r) {
                uint32_t x[8];
#pragma unroll
                for (int b = 0; b < 8; ++b) x[b] = a[8 * r + b];
                vmul(om[r], x, om[r]);
#pragma unroll
                for (int b = 0; b < 8; ++b) om[r][b] ^= cf[b];
            }
        }
        // Lodd(x) = x * sum_m C_{2m+1} (x^2)^m
#pragma unroll
        for (int r = 0; r < RS; ++r) {
            uint32_t x[8];
#pragma unroll
            for (int b = 0; b < 8; ++b) x[b] = a[8 * r + b];
            vsqr(x, y[r]);
#pragma unroll
            for (int b = 0; b < 8; ++b) lo[r][b] = A[(8 * t + 8 * (t / 2 - 1) + b) * 32 + lane];
        }
#pragma unroll 1
        for (int m = t / 2 - 2; m >= 0; --m) {
            uint32_t cf[8];
#pragma unroll
            for (int b = 0; b < 8; ++b) cf[b] = A[(8 * t + 8 * m + b) * 32 + lane];
#pragma unroll
            for (int r = 0; r < RS; ++r) {
                vmul(lo[r], y[r], lo[r]);
#pragma unroll
                for (int b = 0; b < 8; ++b) lo[r][b] ^= cf[b];
            }
        }
#pragma unroll
        for (int r = 0; r < RS; ++r) {
            uint32_t x[8], inv[8];
#pragma unroll
            for (int b = 0; b < 8; ++b) x[b] = a[8 * r + b];
            vmul(lo[r], x, lo[r]);
            vinv(lo[r], inv);
            vmul(om[r], inv, om[r]);
#pragma unroll
            for (int b = 0; b < 8; ++b) a[8 * r + b] = om[r][b];
        }
        transpose32(a);  // byte r of word j: e of block j, slot 4r + h
#pragma unroll
        for (int j = 0; j < 32; ++j) Xv[(j * 4 + h) * 32 + lane] = a[j];
    }
    __syncthreads();

    // phase 5: statuses and corrections of blocks j = 8h .. 8h+7, two blocks
    // per pass.  Every corrected byte belongs to one block alone, so plain byte
    // loads and stores do (neighbouring blocks share words, not bytes); all
    // loads of a pass are issued before its stores.
    const size_t grp = tile * 32 + lane;
    uint32_t Lp[6];
#pragma unroll
    for (int b = 0; b < 6; ++b) Lp[b] = rec[(Rl::kL + b) * 32];
#pragma unroll 1
    for (int j0 = 8 * h; j0 < 8 * h + 8; j0 += 2) {
        int c[2];
        uint8_t *ad[2][t];
        uint8_t v[2][t];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int j = j0 + u;
            const size_t blk = grp * 32 + j;
            c[u] = 0;
            if (blk >= nblocks) continue;
            if (!((live >> j) & 1u)) {
                status[blk] = 1;
                continue;
            }
            int l = 0;
#pragma unroll
            for (int b = 0; b < 6; ++b) l |= (int)((Lp[b] >> j) & 1u) << b;
            const int cj = cnt[j * 32 + lane];
            if (l > t || cj != l) {
                status[blk] = 0;
                continue;
            }
            status[blk] = 1;
            c[u] = cj;
#pragma unroll
            for (int sl = 0; sl < t; ++sl) {
                if (sl < cj) {
                    const int p = size - 1 - deg[(sl * 32 + j) * 32 + lane];
                    ad[u][sl] = p < msg_len ? data + blk * (size_t)msg_len + p
                                            : parity + blk * (size_t)E + (p - msg_len);
                    v[u][sl] = *ad[u][sl];
                }
            }
        }
#pragma unroll
        for (int u = 0; u < 2; ++u)
#pragma unroll
            for (int sl = 0; sl < t; ++sl)
                if (sl < c[u])
                    *ad[u][sl] =
                        v[u][sl] ^ reinterpret_cast<const uint8_t *>(Xv + ((j0 + u) * 4 + (sl & 3)) * 32 + lane)[sl >> 2];
    }
}

}  // namespace bs

// ---------------------------------------------------------------- dispatch

struct FastState {
    int ecc;
    std::once_flag nib_once;
    uint4 *nib_tab = nullptr;  // the encoder's nibble tables (ecc 32), built at first use
};

bool rs256_fast_init(Rs256Code &c) {
    if (c.primitive != 2 || (c.polynomial & 0xff) != 0x1d) return false;
    if (c.ecc != 32 && c.ecc != 16 && c.ecc != 8 && c.ecc != 4 && c.ecc != 2) return false;
    c.fast_state = new FastState{c.ecc};
    return true;
}

void rs256_fast_free(Rs256Code &c) {
    auto *fs = static_cast<FastState *>(c.fast_state);
    if (fs && fs->nib_tab) cudaFree(fs->nib_tab);
    delete fs;
    c.fast_state = nullptr;
}

static int sm_count() {
    static const int n = [] {  // once per process (a thread-safe static initialiser)
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        return v > 0 ? v : 132;
    }();
    return n;
}

static unsigned tiles_grid(size_t nblocks) {
    const size_t tiles = (nblocks + bs::kGroups * 32 - 1) / (bs::kGroups * 32);
    return (unsigned)std::max<size_t>(1, std::min<size_t>(tiles, (size_t)sm_count() * 4));
}

// CTAs of the syndrome kernel: one per tile, at most twice the resident
// count (2T warps of 255 registers per CTA)
static unsigned synd_grid(size_t nblocks, int T) {
    const size_t tiles = (nblocks + bs::kSyndGroups * 32 - 1) / (bs::kSyndGroups * 32);
    return (unsigned)std::max<size_t>(1, std::min<size_t>(tiles, (size_t)sm_count() * (8 / T)));
}

static bool aligned4(const void *p) { return ((uintptr_t)p & 3) == 0; }

bool rs256_fast_encode(const Rs256Code &c, const uint8_t *data, size_t nblocks, int msg_len, uint8_t *parity,
                       cudaStream_t st) {
    if (!c.fast || c.table_only || c.ecc != 32 || !aligned4(data) || !aligned4(parity)) return false;
    if (!nblocks) return true;
    const size_t ntiles = (nblocks + 1023) / 1024;
    if (3 * ntiles < 4 * (size_t)sm_count() && msg_len >= 1 && msg_len <= 223) {
        // the LFSR kernel takes one wave (about 0.12 ms on 152 SMs) for any
        // batch up to 2048 blocks per SM; the nibble tables take time in
        // proportion to the blocks and are faster below about 1,365 per SM
        auto *fs = static_cast<FastState *>(c.fast_state);
        std::call_once(fs->nib_once, [&] {
            constexpr bs::Poly<32> g = bs::factor_poly<32>(0);
            const std::vector<uint32_t> t = nib_tables(g.c + 1);  // x^32 mod g
            FFGPU_CHECK_CUDA(cudaMalloc(&fs->nib_tab, t.size() * 4));
            FFGPU_CHECK_CUDA(cudaMemcpy(fs->nib_tab, t.data(), t.size() * 4, cudaMemcpyHostToDevice));
            FFGPU_CHECK_CUDA(cudaFuncSetAttribute(bs::rs256_encode_nib_kernel,
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  kNibWords * 16));
        });
        // four blocks per warp, one CTA per SM
        const size_t warps = (nblocks + 3) / 4, sms = (size_t)sm_count();
        const unsigned threads = (unsigned)std::min<size_t>(1024, (warps + sms - 1) / sms * 32);
        const unsigned grid = (unsigned)std::min(sms, (warps * 32 + threads - 1) / threads);
        KernelTimer kt_timer("rs256_encode_nib_kernel", st);
        bs::rs256_encode_nib_kernel<<<grid, threads, (size_t)(msg_len + 3) / 4 * kNibGroupQ * 16, st>>>(
            data, nblocks, msg_len, fs->nib_tab, parity);
        check_launch("rs256_encode_nib_kernel");
        return true;
    }
    KernelTimer kt_timer("bs_encode32_kernel", st);
    bs::bs_encode32_kernel<<<tiles_grid(nblocks), bs::kGroups * 2, 0, st>>>(data, nblocks, msg_len, parity);
    check_launch("bs_encode32_kernel");
    return true;
}

// syndromes of nblocks blocks, ecc bytes each
bool rs256_fast_synds(const Rs256Code &c, const uint8_t *data, const uint8_t *parity, size_t nblocks, int msg_len,
                      uint8_t *synds, cudaStream_t st) {
    if (!c.fast || c.table_only || (c.ecc != 32 && c.ecc != 16)) return false;
    if (!aligned4(data) || !aligned4(parity) || !aligned4(synds)) return false;
    if (!nblocks) return true;
    KernelTimer kt_timer("bs_synd_kernel", st);
    if (c.ecc == 32)
        bs::bs_synd_kernel<32, false><<<synd_grid(nblocks, bs::SyndCode<32>::T), bs::kSyndGroups * bs::SyndCode<32>::T, 0, st>>>(data, parity, nblocks, msg_len, synds);
    else
        bs::bs_synd_kernel<16, false><<<synd_grid(nblocks, bs::SyndCode<16>::T), bs::kSyndGroups * bs::SyndCode<16>::T, 0, st>>>(data, parity, nblocks, msg_len, synds);
    check_launch("bs_synd_kernel");
    return true;
}

// bytes of the bitsliced syndrome planes (and, later, the corrections) of
// nblocks blocks: whole tiles of 32 groups
size_t rs256_fast_scratch_bytes(int ecc, size_t nblocks) {
    const size_t ngroups = (nblocks + 31) / 32, ntiles = (ngroups + 31) / 32;
    return ntiles * (size_t)(ecc == 32 ? bs::kTileWords<32> : bs::kTileWords<16>) * 4;
}

// the decode kernels' shared-memory attributes, set once per process (a
// thread-safe static initialiser)
template <int E>
static void bs_decode_attrs() {
    static const bool attrs = [] {
        if constexpr (E == 32)
            cudaFuncSetAttribute(bs::bs_synd32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)bs::Synd32Geom::smem);
        cudaFuncSetAttribute(bs::bs_bm_kernel<E>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)bs::SolveGeom<E>::smem);
        cudaFuncSetAttribute(bs::bs_chien_kernel<E>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)bs::ChienGeom<E>::smem);
        // several CTAs of 128 threads per SM need the largest shared-memory carveout
        cudaFuncSetAttribute(bs::bs_bm_kernel<E>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        cudaFuncSetAttribute(bs::bs_chien_kernel<E>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        return true;
    }();
    (void)attrs;
}

template <int E>
static void launch_bs_decode(const Rs256Code &c, uint8_t *data, uint8_t *parity, size_t nblocks, int msg_len,
                             uint8_t *status, uint32_t *planes, cudaStream_t st) {
    constexpr int T = bs::SyndCode<E>::T;
    const size_t ntiles = ((nblocks + 31) / 32 + 31) / 32;
    bs_decode_attrs<E>();
    if constexpr (E == 32) {
        KernelTimer kt_timer("bs_synd32_kernel", st);
        bs::bs_synd32_kernel<<<(unsigned)ntiles, 256, bs::Synd32Geom::smem, st>>>(data, parity, nblocks, msg_len,
                                                                                  planes);
        check_launch("bs_synd32_kernel");
    } else {
        KernelTimer kt_timer("bs_synd_kernel", st);
        bs::bs_synd_kernel<E, true><<<synd_grid(nblocks, T), bs::kSyndGroups * T, 0, st>>>(
            data, parity, nblocks, msg_len, reinterpret_cast<uint8_t *>(planes));
        check_launch("bs_synd_kernel");
    }
    {
        KernelTimer kt_timer("bs_bm_kernel", st);
        bs::bs_bm_kernel<E><<<(unsigned)ntiles, 128, bs::SolveGeom<E>::smem, st>>>(nblocks, planes);
        check_launch("bs_bm_kernel");
    }
    KernelTimer kt_timer("bs_chien_kernel", st);
    bs::bs_chien_kernel<E><<<(unsigned)ntiles, 128, bs::ChienGeom<E>::smem, st>>>(data, parity, nblocks, msg_len,
                                                                                    planes, status, c.d_exp512);
    check_launch("bs_chien_kernel");
}

// decode with caller-provided scratch of rs256_fast_scratch_bytes(ecc, nblocks)
bool rs256_fast_decode_with(const Rs256Code &c, uint8_t *data, uint8_t *parity, size_t nblocks, int msg_len,
                            uint8_t *status, void *scratch, cudaStream_t st) {
    if (!c.fast || c.table_only || (c.ecc != 32 && c.ecc != 16)) return false;
    if (!aligned4(data) || !aligned4(parity) || !aligned4(scratch)) return false;
    if (!nblocks) return true;
    if (c.ecc == 32)
        launch_bs_decode<32>(c, data, parity, nblocks, msg_len, status, (uint32_t *)scratch, st);
    else
        launch_bs_decode<16>(c, data, parity, nblocks, msg_len, status, (uint32_t *)scratch, st);
    return true;
}

bool rs256_fast_decode(const Rs256Code &c, uint8_t *data, uint8_t *parity, size_t nblocks, int msg_len,
                       uint8_t *status, cudaStream_t st) {
    if (!c.fast || c.table_only || (c.ecc != 32 && c.ecc != 16)) return false;
    if (!aligned4(data) || !aligned4(parity)) return false;
    if (!nblocks) return true;
    void *scratch = nullptr;
    FFGPU_CHECK_CUDA(cudaMallocAsync(&scratch, rs256_fast_scratch_bytes(c.ecc, nblocks), st));
    try {
        rs256_fast_decode_with(c, data, parity, nblocks, msg_len, status, scratch, st);
    } catch (...) {
        cudaFreeAsync(scratch, st);
        throw;
    }
    FFGPU_CHECK_CUDA(cudaFreeAsync(scratch, st));
    return true;
}

}  // namespace ffgpu
