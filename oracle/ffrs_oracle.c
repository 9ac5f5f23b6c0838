/*
 * ffrs_oracle.c -- CPU restatement of the libffrs block-coding hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see ffrs_oracle.h).  Each function cites the
 * reference code it restates; paths are relative to the zydd/libffrs project.
 * Parity is pinned by tests/golden/ fixtures made with the reference's own
 * pybind11 module (tests/golden/make_golden.py).
 */
#include "ffrs_oracle.h"

#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ======================================================================
 * GF(2^8): exp/log tables built with the bit-serial multiplication
 * (libffrs/galois.hpp:93-146, 624-651), table multiplication (:653-667).
 * ====================================================================== */
typedef struct {
    uint8_t exp[256];
    uint8_t log[256];
    uint8_t poly1;
    uint8_t primitive;
} gf256;

static uint8_t gf256_mul_serial(uint8_t poly1, uint8_t a, uint8_t b) {
    uint8_t r = 0;
    for (int i = 7; i >= 0; --i) {
        if (r & 0x80)
            r = (uint8_t)((r << 1) ^ poly1);
        else
            r = (uint8_t)(r << 1);
        if (a & (1u << i)) r ^= b;
    }
    return r;
}

static void gf256_init(gf256 *g, uint8_t primitive, uint8_t poly1) {
    memset(g, 0, sizeof *g);
    g->poly1 = poly1;
    g->primitive = primitive;
    uint8_t x = 1;
    for (int i = 0; i < 256; ++i) {
        g->exp[i] = x;
        g->log[x] = (uint8_t)i;
        x = gf256_mul_serial(poly1, x, primitive);
    }
}

static inline uint8_t gf256_mul(const gf256 *g, uint8_t a, uint8_t b) {
    if (a == 0 || b == 0) return 0;
    unsigned r = (unsigned)g->log[a] + g->log[b];
    if (r >= 255) r -= 255;
    return g->exp[r];
}

static inline uint8_t gf256_inv(const gf256 *g, uint8_t a) { return g->exp[255 - g->log[a]]; }

static inline uint8_t gf256_div(const gf256 *g, uint8_t a, uint8_t b) {
    if (a == 0) return 0;
    unsigned r = (unsigned)g->log[a] + 255 - g->log[b];
    if (r >= 255) r -= 255;
    return g->exp[r];
}

/* galois.hpp:502-507 */
static uint8_t gf256_poly_eval(const gf256 *g, const uint8_t *p, size_t n, uint8_t x, uint8_t r) {
    for (size_t i = 0; i < n; ++i) r = gf256_mul(g, r, x) ^ p[i];
    return r;
}

/* galois.hpp:462-499, poly_mod_x_n: remainder of a(x) * x^n mod (x^n + b(x)) */
static void gf256_poly_mod_x_n(const gf256 *g, const uint8_t *a, size_t size_a, const uint8_t *b, size_t size_b,
                               uint8_t *rem) {
    uint8_t tmp[256];
    if (size_a >= size_b) {
        memcpy(tmp, a, size_b);
        for (size_t i = 0; i < size_a - size_b; ++i) {
            uint8_t c = tmp[0];
            memmove(tmp, tmp + 1, size_b - 1);
            tmp[size_b - 1] = a[size_b + i];
            if (!c) continue;
            for (size_t j = 0; j < size_b; ++j) tmp[j] ^= gf256_mul(g, b[j], c);
        }
    } else {
        memset(tmp, 0, size_b - size_a);
        memcpy(tmp + (size_b - size_a), a, size_a);
    }
    for (size_t i = 0; i < size_b; ++i) {
        uint8_t c = tmp[0];
        memmove(tmp, tmp + 1, size_b - 1);
        tmp[size_b - 1] = 0;
        if (!c) continue;
        for (size_t j = 0; j < size_b; ++j) tmp[j] ^= gf256_mul(g, b[j], c);
    }
    memcpy(rem, tmp, size_b);
}

/* ======================================================================
 * RS256 (libffrs/reed_solomon.hpp, libffrs/pyrs256.hpp)
 * ====================================================================== */
struct orc_rs256 {
    gf256 gf;
    int ecc;
    uint8_t generator[256];
    uint8_t roots[256];
    uint8_t err_roots[256];
    uint8_t lut[256][256]; /* lut[v] = v * x^ecc mod g, ecc bytes (slicing table row 0) */
};

orc_rs256 *orc_rs256_new(int ecc_len, int primitive, int polynomial) {
    if (ecc_len < 1 || ecc_len > 254) return NULL;
    orc_rs256 *rs = (orc_rs256 *)calloc(1, sizeof *rs);
    gf256_init(&rs->gf, (uint8_t)primitive, (uint8_t)(polynomial & 0xff)); /* pygf256.hpp:261-263 */
    rs->ecc = ecc_len;

    /* rs_generator (reed_solomon.hpp:65-86): g(x) = prod_{i<ecc} (x - a^i), highest degree first */
    uint8_t tmp[256];
    memset(rs->generator, 0, sizeof rs->generator);
    rs->generator[0] = 1;
    size_t len = 1;
    for (int i = 0; i < ecc_len; ++i) {
        rs->roots[i] = rs->gf.exp[i];
        uint8_t factor[2] = {1, rs->roots[i]};
        memset(tmp, 0, len + 1);
        for (size_t a = 0; a < len; ++a)
            for (size_t b = 0; b < 2; ++b) tmp[a + b] ^= gf256_mul(&rs->gf, rs->generator[a], factor[b]);
        len += 1;
        memcpy(rs->generator, tmp, len);
    }

    /* rs_encode_slice_*::init (reed_solomon.hpp:201-217, 268-292): row 0 of the slicing table */
    for (int v = 0; v < 256; ++v) {
        uint8_t in = (uint8_t)v;
        gf256_poly_mod_x_n(&rs->gf, &in, 1, &rs->generator[1], (size_t)ecc_len, rs->lut[v]);
    }
    /* rs_roots_eval_lut_pw2 ctor (reed_solomon.hpp:540-544) */
    for (int i = 0; i < 256; ++i) rs->err_roots[i] = gf256_inv(&rs->gf, rs->gf.exp[i]);
    return rs;
}

void orc_rs256_free(orc_rs256 *rs) { free(rs); }
int orc_rs256_ecc_len(const orc_rs256 *rs) { return rs->ecc; }

void orc_rs256_generator(const orc_rs256 *rs, uint8_t *generator, uint8_t *roots) {
    memcpy(generator, rs->generator, (size_t)rs->ecc + 1);
    memcpy(roots, rs->roots, (size_t)rs->ecc);
}

void orc_rs256_tables(const orc_rs256 *rs, uint8_t *exp256, uint8_t *log256) {
    memcpy(exp256, rs->gf.exp, 256);
    memcpy(log256, rs->gf.log, 256);
}

/* Byte-at-a-time LFSR with the slicing table's row 0.  The reference's
 * slicing-by-N loops (reed_solomon.hpp:171-198, 230-265) combine N rows of the
 * same linear table and finish their tail with exactly this recurrence
 * (:194-195, :256-262), so for a field the results are identical. */
void orc_rs256_encode(const orc_rs256 *rs, const uint8_t *msg, size_t len, uint8_t *parity) {
    const int ecc = rs->ecc;
    uint8_t rem[256];
    memset(rem, 0, sizeof rem);
    for (size_t i = 0; i < len; ++i) {
        uint8_t fb = rem[0] ^ msg[i];
        const uint8_t *row = rs->lut[fb];
        for (int j = 0; j < ecc - 1; ++j) rem[j] = rem[j + 1] ^ row[j];
        rem[ecc - 1] = row[ecc - 1];
    }
    memcpy(parity, rem, (size_t)ecc);
}

typedef struct {
    void (*fn)(void *ctx, size_t begin, size_t end);
    void *ctx;
    size_t begin, end;
} orc_job;

static void *orc_job_run(void *p) {
    orc_job *j = (orc_job *)p;
    j->fn(j->ctx, j->begin, j->end);
    return NULL;
}

static void orc_parallel_for(size_t n, int threads, void (*fn)(void *, size_t, size_t), void *ctx) {
    if (threads <= 1 || n < 2) {
        fn(ctx, 0, n);
        return;
    }
    if ((size_t)threads > n) threads = (int)n;
    pthread_t *tid = (pthread_t *)calloc((size_t)threads, sizeof(pthread_t));
    orc_job *jobs = (orc_job *)calloc((size_t)threads, sizeof(orc_job));
    for (int t = 0; t < threads; ++t) {
        jobs[t].fn = fn;
        jobs[t].ctx = ctx;
        jobs[t].begin = n * (size_t)t / (size_t)threads;
        jobs[t].end = n * (size_t)(t + 1) / (size_t)threads;
        pthread_create(&tid[t], NULL, orc_job_run, &jobs[t]);
    }
    for (int t = 0; t < threads; ++t) pthread_join(tid[t], NULL);
    free(tid);
    free(jobs);
}

typedef struct {
    const orc_rs256 *rs;
    const uint8_t *buf;
    uint8_t *out;
    size_t message_len;
} rs_enc_ctx;

static void rs_enc_range(void *p, size_t b, size_t e) {
    rs_enc_ctx *c = (rs_enc_ctx *)p;
    for (size_t i = b; i < e; ++i)
        orc_rs256_encode(c->rs, c->buf + i * c->message_len, c->message_len, c->out + i * (size_t)c->rs->ecc);
}

/* PyRS256::py_encode (pyrs256.hpp:99-127) */
size_t orc_rs256_encode_buffer(const orc_rs256 *rs, const uint8_t *buf, size_t len, size_t message_len, uint8_t *out,
                               int threads) {
    if (len == 0 || message_len == 0) return 0;
    size_t full = len / message_len;
    size_t rem = len - full * message_len;
    rs_enc_ctx c = {rs, buf, out, message_len};
    orc_parallel_for(full, threads, rs_enc_range, &c);
    if (rem) orc_rs256_encode(rs, buf + len - rem, rem, out + full * (size_t)rs->ecc);
    return (full + (rem ? 1 : 0)) * (size_t)rs->ecc;
}

/* rs_synds_lut_pw2::synds (reed_solomon.hpp:424-431): S_j = r(a^j), data then remainder */
void orc_rs256_synds(const orc_rs256 *rs, const uint8_t *data, size_t size, const uint8_t *rem, uint8_t *synds) {
    for (int j = 0; j < rs->ecc; ++j) {
        uint8_t t = gf256_poly_eval(&rs->gf, data, size, rs->roots[j], 0);
        synds[j] = gf256_poly_eval(&rs->gf, rem, (size_t)rs->ecc, rs->roots[j], t);
    }
}

/* rs_decode::berlekamp_massey (reed_solomon.hpp:655-702); err_poly right-aligned, reversed */
static size_t rs_berlekamp_massey(const orc_rs256 *rs, const uint8_t *synds, uint8_t *err_poly) {
    const size_t ecc = (size_t)rs->ecc;
    uint8_t prev[256], temp[256];
    memset(prev, 0, ecc);
    memset(err_poly, 0, ecc);
    prev[ecc - 1] = 1;
    err_poly[ecc - 1] = 1;
    size_t errors = 0, m = 1;
    uint8_t b = 1;
    for (size_t n = 0; n < ecc; ++n) {
        uint8_t d = synds[n];
        for (size_t i = 1; i < errors + 1; ++i) d ^= gf256_mul(&rs->gf, err_poly[ecc - 1 - i], synds[n - i]);
        if (d == 0) {
            m = m + 1;
        } else if (2 * errors <= n) {
            memcpy(temp, err_poly, ecc);
            /* poly_shift(prev, ecc, m) (galois.hpp:509-516) */
            size_t i = 0;
            for (; i < ecc - m; ++i) prev[i] = prev[i + m];
            for (; i < ecc; ++i) prev[i] = 0;
            uint8_t s = gf256_div(&rs->gf, d, b);
            for (i = 0; i < ecc; ++i) err_poly[i] ^= gf256_mul(&rs->gf, s, prev[i]);
            errors = n + 1 - errors;
            memcpy(prev, temp, ecc);
            b = d;
            m = 1;
        } else {
            size_t i = 0;
            for (; i < ecc - m; ++i) temp[i] = prev[i + m];
            for (; i < ecc; ++i) temp[i] = 0;
            uint8_t s = gf256_div(&rs->gf, d, b);
            for (i = 0; i < ecc; ++i) err_poly[i] ^= gf256_mul(&rs->gf, s, temp[i]);
            m = m + 1;
        }
    }
    return errors;
}

/* rs_roots_eval_lut_pw2::roots (reed_solomon.hpp:516-537): zeros of the locator at a^-i, i < max */
static size_t rs_roots(const orc_rs256 *rs, const uint8_t *poly, size_t poly_size, size_t max_pos, uint8_t *roots) {
    size_t count = 0;
    for (size_t i = 0; i < max_pos && i < 256; ++i)
        if (gf256_poly_eval(&rs->gf, poly, poly_size, rs->err_roots[i], 0) == 0) roots[count++] = (uint8_t)i;
    return count;
}

/* rs_decode::forney (reed_solomon.hpp:704-743) */
static int rs_forney(const orc_rs256 *rs, const uint8_t *synds, uint8_t *err_poly, const uint8_t *err_pos,
                     size_t err_count, uint8_t *err_mag) {
    const size_t ecc = (size_t)rs->ecc;
    uint8_t err_eval[512], synds_rev[256];
    for (size_t i = 0; i < ecc; ++i) synds_rev[i] = synds[ecc - 1 - i];
    size_t size = ecc + err_count + 1 - 1;
    memset(err_eval, 0, size);
    for (size_t i = 0; i < ecc; ++i)
        for (size_t j = 0; j < err_count + 1; ++j) err_eval[i + j] ^= gf256_mul(&rs->gf, synds_rev[i], err_poly[j]);
    /* ex_synth_div by x^ecc leaves the quotient in the first err_count entries */
    size_t begin = size - (ecc + 1) + 1;
    while (begin < size && err_eval[begin] == 0) begin++;
    if (begin >= size) return 0; /* the reference would read past its buffer here */
    size_t eval_size = size - begin;
    /* gf_poly_deriv_pw2 (galois.hpp:725-734) */
    size_t psize = err_count + 1;
    for (size_t i = 1; i < psize; ++i) err_poly[psize - i] = (i & 1) ? err_poly[psize - i - 1] : 0;
    const uint8_t *deriv = err_poly + 1;
    for (size_t i = 0; i < err_count; ++i) {
        uint8_t xi = rs->gf.exp[err_pos[i]];
        uint8_t xi_inv = gf256_inv(&rs->gf, xi);
        uint8_t n = gf256_poly_eval(&rs->gf, &err_eval[begin], eval_size, xi_inv, 0);
        uint8_t d = gf256_poly_eval(&rs->gf, deriv, err_count, xi_inv, 0);
        err_mag[i] = gf256_mul(&rs->gf, xi, gf256_div(&rs->gf, n, d));
    }
    return 1;
}

/* rs_decode::decode (reed_solomon.hpp:559-595) */
int orc_rs256_decode(const orc_rs256 *rs, uint8_t *data, size_t size, uint8_t *rem) {
    const size_t ecc = (size_t)rs->ecc;
    uint8_t synds[256];
    orc_rs256_synds(rs, data, size, rem, synds);
    int all_zero = 1;
    for (size_t i = 0; i < ecc; ++i)
        if (synds[i]) all_zero = 0;
    if (all_zero) return 1;

    uint8_t err_poly[256];
    size_t errors = rs_berlekamp_massey(rs, synds, err_poly);
    if (errors > ecc / 2) return 0;

    uint8_t err_pos[256], err_mag[256];
    uint8_t *loc = &err_poly[ecc - errors - 1];
    size_t roots = rs_roots(rs, loc, errors + 1, size + ecc, err_pos);
    if (errors != roots) return 0;
    if (!rs_forney(rs, synds, loc, err_pos, errors, err_mag)) return 0;
    for (size_t i = 0; i < errors; ++i) {
        size_t pos = size + ecc - 1 - err_pos[i];
        if (pos >= size + ecc) return 0;
        if (pos < size)
            data[pos] ^= err_mag[i];
        else
            rem[pos - size] ^= err_mag[i];
    }
    return 1;
}

typedef struct {
    const orc_rs256 *rs;
    uint8_t *data, *parity, *status;
    size_t message_len;
} rs_dec_ctx;

static void rs_dec_range(void *p, size_t b, size_t e) {
    rs_dec_ctx *c = (rs_dec_ctx *)p;
    const size_t ecc = (size_t)c->rs->ecc;
    for (size_t i = b; i < e; ++i)
        c->status[i] =
            (uint8_t)orc_rs256_decode(c->rs, c->data + i * c->message_len, c->message_len, c->parity + i * ecc);
}

void orc_rs256_decode_blocks(const orc_rs256 *rs, uint8_t *data, uint8_t *parity, size_t nblocks, size_t message_len,
                             uint8_t *status, int threads) {
    rs_dec_ctx c = {rs, data, parity, status, message_len};
    orc_parallel_for(nblocks, threads, rs_dec_range, &c);
}

/* ======================================================================
 * GF(65537) (libffrs/galois.hpp:168-216, 258-395; libffrs/pygfi16.hpp)
 * ====================================================================== */
uint32_t orc_gfi16_mul(uint32_t a, uint32_t b) {
    uint32_t r = a * b;
    if (r == 0 && a && b) return 1;
    r = (r & 0xffffu) - (r >> 16);
    if (r >= 0x80000000u) r += 0x10001u;
    return r;
}
uint32_t orc_gfi16_add(uint32_t a, uint32_t b) {
    uint32_t r = a + b;
    if (r >= 0x10001u) r -= 0x10001u;
    return r;
}
uint32_t orc_gfi16_sub(uint32_t a, uint32_t b) {
    uint32_t r = a - b;
    if (r >= 0x80000000u) r += 0x10001u;
    return r;
}
static inline uint32_t gfi_neg(uint32_t a) { return a == 0 ? 0 : 0x10001u - a; }
#define MUL orc_gfi16_mul
#define ADD orc_gfi16_add
#define SUB orc_gfi16_sub

struct orc_rsi16 {
    uint32_t *exp, *log; /* 65537 entries each */
    uint32_t primitive;
    size_t block_len, message_len, ecc, ntt_len, pntt_blocks;
    uint32_t ecc_mask;
    unsigned rbo_shift;
    uint32_t root, ntt_len_i, ecc_len_i, ecc2_len_i;
    uint32_t *roots_ntt, *roots_i_ntt, *roots_ecc, *roots_i_ecc, *roots_ecc2, *roots_i_ecc2;
    uint32_t *pntt_shift, *pintt_shift, *rbo_ecc, *ecc_mix, *ecc_mix_i;
};

uint32_t orc_gfi16_inv(const orc_rsi16 *rs, uint32_t a) { return rs->exp[65536u - rs->log[a]]; }
uint32_t orc_gfi16_div(const orc_rsi16 *rs, uint32_t a, uint32_t b) {
    if (a == 0) return 0;
    uint32_t r = rs->log[a] + 65536u - rs->log[b];
    if (r >= 65536u) r -= 65536u;
    return rs->exp[r];
}
uint32_t orc_gfi16_pow(const orc_rsi16 *rs, uint32_t a, uint32_t e) {
    uint32_t p = rs->log[a] * e; /* uint32 wrap, as GFT arithmetic */
    return rs->exp[p % 65536u];
}
#define INV(a) orc_gfi16_inv(rs, (a))
#define DIV(a, b) orc_gfi16_div(rs, (a), (b))
#define POW(a, e) orc_gfi16_pow(rs, (a), (e))

static uint16_t rbo16(uint16_t b) {
    b = (uint16_t)(((b >> 1) & 0x5555) | ((b & 0x5555) << 1));
    b = (uint16_t)(((b >> 2) & 0x3333) | ((b & 0x3333) << 2));
    b = (uint16_t)(((b >> 4) & 0x0f0f) | ((b & 0x0f0f) << 4));
    b = (uint16_t)((b >> 8) | (b << 8));
    return b;
}
uint32_t orc_rsi16_rbo(const orc_rsi16 *rs, uint32_t i) { return (uint32_t)(rbo16((uint16_t)i) >> rs->rbo_shift); }

static void seterr(char *err, size_t errlen, const char *msg) {
    if (err && errlen) snprintf(err, errlen, "%s", msg);
}

void orc_rsi16_free(orc_rsi16 *rs) {
    if (!rs) return;
    free(rs->exp);
    free(rs->log);
    free(rs->roots_ntt);
    free(rs->roots_i_ntt);
    free(rs->roots_ecc);
    free(rs->roots_i_ecc);
    free(rs->roots_ecc2);
    free(rs->roots_i_ecc2);
    free(rs->pntt_shift);
    free(rs->pintt_shift);
    free(rs->rbo_ecc);
    free(rs->ecc_mix);
    free(rs->ecc_mix_i);
    free(rs);
}

/* PyGFi16 ctor (pygfi16.hpp:43-50), NTT ctor (ntt.hpp:55-123), RSi16v ctor
 * (rsi16v_impl.hpp:68-86), PyRSi16 ctor checks (pyrsi16.hpp:76-84). */
orc_rsi16 *orc_rsi16_new(size_t block_len, size_t ecc_len, uint32_t primitive, char *err, size_t errlen) {
    if (ecc_len < 2 || (ecc_len & (ecc_len - 1)) || block_len < ecc_len || block_len % ecc_len || block_len > 65536) {
        seterr(err, errlen, "invalid RSi16 geometry");
        return NULL;
    }
    orc_rsi16 *rs = (orc_rsi16 *)calloc(1, sizeof *rs);
    rs->exp = (uint32_t *)calloc(65537, sizeof(uint32_t));
    rs->log = (uint32_t *)calloc(65537, sizeof(uint32_t));
    rs->primitive = primitive;
    /* gf_exp_log_lut with gf_mul_mod (galois.hpp:133-144, 239-250) */
    uint32_t x = 1;
    for (uint32_t i = 0; i < 65537; ++i) {
        rs->exp[i] = x;
        rs->log[x] = i;
        uint64_t prod = (uint64_t)x * primitive;
        uint32_t res = prod > 0xffffffffull ? 1u : (uint32_t)prod;
        x = res % 0x10001u;
    }
    if (!(POW(primitive, 32768) == 65536 && POW(primitive, 65536) == 1)) {
        seterr(err, errlen, "not a primitive element of GF(65537)");
        orc_rsi16_free(rs);
        return NULL;
    }
    rs->block_len = block_len;
    rs->ecc = ecc_len;
    rs->message_len = block_len - ecc_len;
    rs->ecc_mask = (uint32_t)(ecc_len - 1);
    rs->pntt_blocks = block_len / ecc_len;
    size_t lg = 0;
    while (((size_t)1 << lg) < block_len) ++lg;
    if (lg == 0) lg = 1;
    rs->ntt_len = (size_t)1 << lg;
    rs->rbo_shift = 16u - (unsigned)__builtin_ctzl(rs->ntt_len);
    rs->ntt_len_i = INV((uint32_t)rs->ntt_len);
    rs->ecc_len_i = INV((uint32_t)ecc_len);
    rs->ecc2_len_i = INV((uint32_t)(ecc_len * 2));
    rs->root = POW(primitive, (uint32_t)(65536 / rs->ntt_len));
    if (POW(rs->root, (uint32_t)rs->ntt_len) != 1 || POW(rs->root, (uint32_t)(rs->ntt_len / 2)) != 65536) {
        seterr(err, errlen, "ntt root of unity sanity check failed");
        orc_rsi16_free(rs);
        return NULL;
    }
    const size_t n = rs->ntt_len;
    uint32_t root_i = INV(rs->root);
    rs->roots_ntt = (uint32_t *)calloc(n, 4);
    rs->roots_i_ntt = (uint32_t *)calloc(n, 4);
    for (size_t i = 0; i < n; ++i) {
        rs->roots_ntt[i] = POW(rs->root, (uint32_t)i);
        rs->roots_i_ntt[i] = POW(root_i, (uint32_t)i);
    }
    rs->rbo_ecc = (uint32_t *)calloc(ecc_len, 4);
    for (size_t i = 0; i < ecc_len; ++i) rs->rbo_ecc[i] = orc_rsi16_rbo(rs, (uint32_t)(i * (n / ecc_len)));
    uint32_t ecc_root = POW(primitive, (uint32_t)(65536 / ecc_len));
    if (POW(ecc_root, (uint32_t)ecc_len) != 1 || POW(ecc_root, (uint32_t)(ecc_len / 2)) != 65536) {
        seterr(err, errlen, "ntt root of unity sanity check failed");
        orc_rsi16_free(rs);
        return NULL;
    }
    uint32_t ecc_root_i = INV(ecc_root);
    rs->roots_ecc = (uint32_t *)calloc(ecc_len, 4);
    rs->roots_i_ecc = (uint32_t *)calloc(ecc_len, 4);
    for (size_t i = 0; i < ecc_len; ++i) {
        rs->roots_ecc[i] = POW(ecc_root, (uint32_t)i);
        rs->roots_i_ecc[i] = POW(ecc_root_i, (uint32_t)i);
    }
    uint32_t ecc2_root = POW(primitive, (uint32_t)(65536 / (ecc_len * 2)));
    if (POW(ecc2_root, (uint32_t)(ecc_len * 2)) != 1 || POW(ecc2_root, (uint32_t)ecc_len) != 65536) {
        seterr(err, errlen, "ntt root of unity sanity check failed");
        orc_rsi16_free(rs);
        return NULL;
    }
    uint32_t ecc2_root_i = INV(ecc2_root);
    rs->roots_ecc2 = (uint32_t *)calloc(ecc_len * 2, 4);
    rs->roots_i_ecc2 = (uint32_t *)calloc(ecc_len * 2, 4);
    for (size_t i = 0; i < ecc_len * 2; ++i) {
        rs->roots_ecc2[i] = POW(ecc2_root, (uint32_t)i);
        rs->roots_i_ecc2[i] = POW(ecc2_root_i, (uint32_t)i);
    }
    rs->pntt_shift = (uint32_t *)calloc(block_len, 4);
    for (size_t i = 0; i < block_len; ++i) {
        size_t blk = (i / ecc_len) * ecc_len, j = i - blk;
        rs->pntt_shift[i] = POW(rs->root, (uint32_t)(j * orc_rsi16_rbo(rs, (uint32_t)blk)));
    }
    rs->pintt_shift = (uint32_t *)calloc(n, 4);
    for (size_t i = 0; i < n; ++i) {
        size_t blk = (i / ecc_len) * ecc_len, j = i - blk;
        rs->pintt_shift[i] = DIV(POW(root_i, (uint32_t)(j * orc_rsi16_rbo(rs, (uint32_t)blk))), (uint32_t)n);
    }
    rs->ecc_mix = (uint32_t *)calloc(ecc_len, 4);
    rs->ecc_mix_i = (uint32_t *)calloc(ecc_len, 4);
    uint32_t w = rs->roots_ntt[orc_rsi16_rbo(rs, (uint32_t)(block_len - ecc_len))];
    uint32_t w_i = INV(w);
    for (size_t i = 0; i < ecc_len; ++i) {
        rs->ecc_mix[i] = gfi_neg(DIV(POW(w_i, (uint32_t)i), (uint32_t)ecc_len));
        rs->ecc_mix_i[i] = gfi_neg(POW(w, (uint32_t)i));
    }
    return rs;
}

size_t orc_rsi16_ntt_len(const orc_rsi16 *rs) { return rs->ntt_len; }
uint32_t orc_rsi16_root(const orc_rsi16 *rs) { return rs->root; }

const uint32_t *orc_rsi16_table(const orc_rsi16 *rs, int which, size_t *len) {
    switch (which) {
        case 0: *len = rs->ntt_len; return rs->roots_ntt;
        case 1: *len = rs->ecc; return rs->roots_ecc;
        case 2: *len = rs->ecc; return rs->roots_i_ecc;
        case 3: *len = rs->block_len; return rs->pntt_shift;
        case 4: *len = rs->ntt_len; return rs->pintt_shift;
        case 5: *len = rs->ecc; return rs->ecc_mix;
        case 6: *len = rs->ecc; return rs->rbo_ecc;
        case 7: *len = 2 * rs->ecc; return rs->roots_ecc2;
        case 8: *len = 2 * rs->ecc; return rs->roots_i_ecc2;
        case 9: *len = 65537; return rs->exp;
        case 10: *len = 65537; return rs->log;
        default: *len = 0; return NULL;
    }
}

/* ct_butterfly (ntt.hpp:225-249): RBO input, normal order output */
static void ct_butterfly(const uint32_t *roots, uint32_t *block, size_t n) {
    for (size_t stride = 1, exp_f = n >> 1; stride < n; stride *= 2, exp_f >>= 1) {
        for (size_t start = 0; start < n; start += stride * 2) {
            uint32_t a = block[start], b = block[start + stride];
            block[start] = ADD(a, b);
            block[start + stride] = SUB(a, b);
            for (size_t i = start + 1; i < start + stride; ++i) {
                uint32_t w = roots[exp_f * (i - start)];
                a = block[i];
                b = block[i + stride];
                uint32_t m = MUL(b, w);
                block[i] = ADD(a, m);
                block[i + stride] = SUB(a, m);
            }
        }
    }
}

/* gs_butterfly (ntt.hpp:280-302): normal order input, RBO output */
static void gs_butterfly(const uint32_t *roots, uint32_t *block, size_t n, size_t end) {
    for (size_t stride = n / 2, exp_f = 0; stride > 0; stride /= 2, exp_f += 1) {
        for (size_t start = 0; start < end; start += stride * 2) {
            uint32_t a = block[start], b = block[start + stride];
            block[start] = ADD(a, b);
            block[start + stride] = SUB(a, b);
            for (size_t i = start + 1; i < start + stride; ++i) {
                uint32_t w = roots[(i - start) << exp_f];
                a = block[i];
                b = block[i + stride];
                block[i] = ADD(a, b);
                block[i + stride] = MUL(SUB(a, b), w);
            }
        }
    }
}

static void nttr(const orc_rsi16 *rs, uint32_t *b) { gs_butterfly(rs->roots_ecc, b, rs->ecc, rs->ecc); }
static void inttr(const orc_rsi16 *rs, uint32_t *b) {
    ct_butterfly(rs->roots_i_ecc, b, rs->ecc);
    for (size_t i = 0; i < rs->ecc; ++i) b[i] = MUL(b[i], rs->ecc_len_i);
}
static void nttr2(const orc_rsi16 *rs, uint32_t *b) { gs_butterfly(rs->roots_ecc2, b, rs->ecc * 2, rs->ecc * 2); }
static void inttr2(const orc_rsi16 *rs, uint32_t *b) {
    ct_butterfly(rs->roots_i_ecc2, b, rs->ecc * 2);
    for (size_t i = 0; i < rs->ecc * 2; ++i) b[i] = MUL(b[i], rs->ecc2_len_i);
}

/* NTT::pntt (ntt.hpp:133-152): first ecc outputs of the partial NTT, in place */
static void pntt(const orc_rsi16 *rs, uint32_t *block, size_t nchunks) {
    const size_t ecc = rs->ecc;
    ct_butterfly(rs->roots_ecc, block, ecc);
    for (size_t j = 0; j < ecc; ++j) block[j] = MUL(block[j], rs->pntt_shift[j]);
    for (size_t i = 1; i < nchunks; ++i) {
        uint32_t *p = &block[i * ecc];
        ct_butterfly(rs->roots_ecc, p, ecc);
        for (size_t j = 0; j < ecc; ++j) p[j] = MUL(p[j], rs->pntt_shift[i * ecc + j]);
        for (size_t j = 0; j < ecc; ++j) block[j] = ADD(block[j], p[j]);
    }
}

void orc_rsi16_synd(const orc_rsi16 *rs, const uint32_t *block, uint32_t *synds) {
    uint32_t *tmp = (uint32_t *)malloc(rs->block_len * 4);
    memcpy(tmp, block, rs->block_len * 4);
    pntt(rs, tmp, rs->pntt_blocks);
    memcpy(synds, tmp, rs->ecc * 4);
    free(tmp);
}

/* RSi16v::_mix_ecc (rsi16v_impl.hpp:100-106) */
void orc_rsi16_mix_ecc(const orc_rsi16 *rs, uint32_t *ecc) {
    for (size_t j = 0; j < rs->ecc; ++j) ecc[j] = MUL(ecc[j], rs->ecc_mix[j]);
    gs_butterfly(rs->roots_i_ecc, ecc, rs->ecc, rs->ecc);
}

/* RSi16v::_encode = pntt_message_residue + _mix_ecc_residue (rsi16v_impl.hpp:93-119,
 * ntt.hpp:180-199).  The residue forms are exact, so the canonical pntt_message
 * (ntt.hpp:160-178) and _mix_ecc give the same parity. */
void orc_rsi16_encode_u32(const orc_rsi16 *rs, const uint32_t *msg, uint32_t *parity) {
    uint32_t *tmp = (uint32_t *)malloc(rs->block_len * 4);
    memcpy(tmp, msg, rs->message_len * 4);
    memset(tmp + rs->message_len, 0, rs->ecc * 4);
    pntt(rs, tmp, rs->pntt_blocks - 1);
    orc_rsi16_mix_ecc(rs, tmp);
    memcpy(parity, tmp, rs->ecc * 4);
    free(tmp);
}

typedef struct {
    const orc_rsi16 *rs;
    const uint16_t *msg;
    uint16_t *parity;
} rsi_enc_ctx;

static void rsi_enc_range(void *p, size_t b, size_t e) {
    rsi_enc_ctx *c = (rsi_enc_ctx *)p;
    const orc_rsi16 *rs = c->rs;
    uint32_t *m = (uint32_t *)malloc(rs->block_len * 4), *par = (uint32_t *)malloc(rs->ecc * 4);
    for (size_t i = b; i < e; ++i) {
        for (size_t k = 0; k < rs->message_len; ++k) m[k] = c->msg[i * rs->message_len + k];
        orc_rsi16_encode_u32(rs, m, par);
        for (size_t k = 0; k < rs->ecc; ++k) c->parity[i * rs->ecc + k] = (uint16_t)par[k];
    }
    free(m);
    free(par);
}

/* PyRSi16::encode_blocks (pyrsi16.hpp:127-140), interleave == 1 */
void orc_rsi16_encode_blocks(const orc_rsi16 *rs, const uint16_t *msg, size_t nblocks, uint16_t *parity, int threads) {
    rsi_enc_ctx c = {rs, msg, parity};
    orc_parallel_for(nblocks, threads, rsi_enc_range, &c);
}

/* PyRSi16::_encode_interleaved (pyrsi16.hpp:323-361), column by column */
void orc_rsi16_encode_interleaved_u32(const orc_rsi16 *rs, const uint32_t *msg, size_t interleave, uint32_t *parity) {
    uint32_t *m = (uint32_t *)malloc(rs->block_len * 4), *par = (uint32_t *)malloc(rs->ecc * 4);
    for (size_t c = 0; c < interleave; ++c) {
        for (size_t k = 0; k < rs->message_len; ++k) m[k] = msg[c + k * interleave];
        orc_rsi16_encode_u32(rs, m, par);
        for (size_t k = 0; k < rs->ecc; ++k) parity[c + k * interleave] = par[k];
    }
    free(m);
    free(par);
}

/* NTT::pintt_ecc (ntt.hpp:206-220) */
void orc_rsi16_pintt_ecc(const orc_rsi16 *rs, uint32_t *b) {
    const size_t ecc = rs->ecc;
    for (size_t i = 1; i < rs->block_len / ecc; ++i) {
        memcpy(&b[i * ecc], &b[0], ecc * 4);
        for (size_t j = 0; j < ecc; ++j) b[i * ecc + j] = MUL(b[i * ecc + j], rs->pintt_shift[i * ecc + j]);
        gs_butterfly(rs->roots_i_ecc, &b[i * ecc], ecc, ecc);
    }
    for (size_t j = 0; j < ecc; ++j) b[j] = MUL(b[j], rs->pintt_shift[j]);
    gs_butterfly(rs->roots_i_ecc, &b[0], ecc, ecc);
}

static uint32_t poly_len(const uint32_t *r, uint32_t n) {
    while (n > 0 && r[n - 1] == 0) --n;
    return n;
}

/* NTT::_reverse_ntt_vec (ntt.hpp:343-354) */
static void reverse_ntt_vec(const orc_rsi16 *rs, uint32_t *v, uint32_t shift) {
    const size_t ecc = rs->ecc;
    for (size_t i = 1; i < ecc; ++i) {
        uint32_t j = rs->rbo_ecc[i];
        uint32_t k = rs->rbo_ecc[ecc - j];
        if (i < k) {
            uint32_t t = v[i];
            v[i] = v[k];
            v[k] = t;
        }
        v[i] = MUL(v[i], rs->roots_i_ecc[j]);
        v[i] = MUL(v[i], rs->roots_ecc[(shift * j) & rs->ecc_mask]);
    }
}

/* The scratch layouts below mirror the reference's temp_ntt1_ecc6 buffer, so a
 * length that runs past one polynomial reads the same neighbour the reference
 * reads.  `lim` is the end of that buffer. */
typedef struct {
    uint32_t *base;
    size_t size;
} scratch;

static int in_scratch(const scratch *s, const uint32_t *p, size_t n) {
    return p >= s->base && (size_t)(p - s->base) + n <= s->size;
}

/* NTT::poly_inv_mod_xn_rev (ntt.hpp:363-469), W = 1 */
static int poly_inv_mod_xn_rev(const orc_rsi16 *rs, const scratch *s, uint32_t *g, uint32_t g_len, uint32_t g0,
                               uint32_t a_len, uint32_t *a) {
    const uint32_t ecc = (uint32_t)rs->ecc;
    uint32_t a0 = INV(g0);
    for (uint32_t i = 0; i < ecc; ++i) a[i] = a0;
    uint32_t l = 2;
    uint32_t a_max = a_len;
    while (l < a_len) {
        if (g_len + l - 2 > ecc) return ORC_ASSERT_FAIL; /* py_assert at ntt.hpp:388-391 */
        for (uint32_t i = 0; i < ecc; ++i) {
            uint32_t a_i = a[i];
            uint32_t ag = MUL(a_i, g[i]);
            a[i] = MUL(a_i, SUB(2, ag));
        }
        inttr(rs, a);
        if (l > ecc) return ORC_ASSERT_FAIL; /* the reference would overrun its buffer */
        for (uint32_t i = l; i < ecc; ++i) a[i] = 0;
        nttr(rs, a);
        l *= 2;
    }
    for (uint32_t i = 0; i < ecc; ++i) {
        uint32_t ag = MUL(a[i], g[i]);
        g[i] = SUB(2, ag);
    }
    for (uint32_t i = 0; i < ecc; ++i) g[i] = MUL(a[i], g[i]);
    inttr(rs, a);
    inttr(rs, g);
    memcpy(a, g, ecc * 4);
    if (l > ecc) return ORC_ASSERT_FAIL;
    for (uint32_t i = l; i < ecc; ++i) a[i] = 0;
    if (!in_scratch(s, a, a_max)) return ORC_ASSERT_FAIL;
    for (uint32_t i = 0, j = a_max; i + 1 < j; ++i, --j) { /* std::reverse(&a[0], &a[a_max]) */
        uint32_t t = a[i];
        a[i] = a[j - 1];
        a[j - 1] = t;
    }
    /* vec::copy_n(&a[0], a_max - a_len, a_len, &a[0], 0) is a no-op for W = 1 */
    if (a_len < ecc)
        for (uint32_t i = a_len; i < ecc; ++i) a[i] = 0;
    else if (a_len > ecc)
        return ORC_ASSERT_FAIL;
    nttr(rs, a);
    return 0;
}

/* NTT::poly_div_ntt (ntt.hpp:471-564), W = 1 */
static int poly_div_ntt(const orc_rsi16 *rs, const scratch *s, const uint32_t *f, uint32_t f_len, const uint32_t *g,
                        uint32_t g_len, uint32_t f0, uint32_t g0, uint32_t *t, uint32_t *q, uint32_t *q_len_out) {
    const uint32_t ecc = (uint32_t)rs->ecc;
    uint32_t q_len = f_len - g_len + 1;
    if (!(g_len > 0)) return ORC_ASSERT_FAIL; /* py_assert(g_len > 0) */
    if (f_len < g_len) {
        for (uint32_t i = 0; i < ecc; ++i) q[i] = 0;
        *q_len_out = 0;
        return 0;
    }
    memcpy(t, g, ecc * 4);
    reverse_ntt_vec(rs, t, g_len);
    int st = poly_inv_mod_xn_rev(rs, s, t, g_len, g0, q_len, q);
    if (st) return st;
    memcpy(t, f, ecc * 4);
    for (uint32_t j = 0; j < ecc; ++j) t[j] = SUB(t[j], f0);
    for (uint32_t i = 0; i < ecc; ++i) t[i] = MUL(t[i], q[i]);
    inttr(rs, t);
    uint32_t right_n = q_len < ecc - g_len ? q_len : ecc - g_len;
    if (!in_scratch(s, t + g_len, right_n) || !in_scratch(s, q, right_n)) return ORC_ASSERT_FAIL;
    memmove(q, t + g_len, (size_t)right_n * 4);
    if (!in_scratch(s, t, q_len - right_n) || !in_scratch(s, q + right_n, q_len - right_n)) return ORC_ASSERT_FAIL;
    memmove(q + right_n, t, (size_t)(q_len - right_n) * 4);
    if (q_len < ecc)
        for (uint32_t i = q_len; i < ecc; ++i) q[i] = 0;
    else if (q_len > ecc && !in_scratch(s, q, q_len))
        return ORC_ASSERT_FAIL;
    nttr(rs, q);
    *q_len_out = q_len;
    return 0;
}

/* RSi16v::_sugiyama (rsi16v_impl.hpp:271-440), W = 1.  a1 and temp4 must sit
 * inside the scratch buffer `s` with the reference's layout. */
static int sugiyama(const orc_rsi16 *rs, const scratch *s, uint32_t *a1, uint32_t *r1, uint32_t *temp4,
                    uint32_t *a1_len_out) {
    const uint32_t ecc = (uint32_t)rs->ecc, mask = rs->ecc_mask;
    memset(temp4, 0, (size_t)ecc * 4 * 4);
    memset(a1, 0, (size_t)ecc * 4);
    uint32_t a1_len;
    uint32_t q_len = 0, t_len = 0;
    uint32_t *q = &temp4[0], *t = &temp4[ecc], *a2 = &temp4[2 * ecc], *r2 = &temp4[3 * ecc];
    uint32_t a2_len = 1;
    for (uint32_t i = 0; i < ecc; ++i) a2[i] = 1;
    uint32_t r1_len = poly_len(r1, ecc);
    memcpy(r2, r1, (size_t)ecc * 4);
    uint32_t r2_len = r1_len;
    uint32_t r2l = r2[0];
    uint32_t lanes = (uint32_t)(-(int32_t)(r1_len != 0));
    {
        uint32_t r1h = r1[(r1_len - 1) & mask];
        uint32_t r1h2 = r1[(uint32_t)(r1_len - 2) & mask];
        a1[1] = gfi_neg(INV(r1h));
        a1[0] = MUL(r1h2, MUL(a1[1], a1[1]));
        a1_len = 2 & lanes;
        for (uint32_t i = 0; i < ecc; ++i) r1[i] = MUL(a1[0], r1[i]);
        for (uint32_t i = 1; i < ecc; ++i) r1[i] = ADD(r1[i], MUL(a1[1], r2[i - 1]));
        r1_len = poly_len(r1, ecc - 1) & lanes;
        for (uint32_t i = r1_len; i < ecc; ++i) r1[i] = 0;
        nttr(rs, a1);
        nttr(rs, r2);
    }
    uint32_t cond = (uint32_t)(-(int32_t)(r1_len >= ecc / 2));
    if (cond) {
        for (uint32_t it = 1; it < ecc / 2; ++it) {
            uint32_t r1h = r1[(r1_len - 1) & mask];
            uint32_t r1l = r1[0];
            nttr(rs, r1);
            int st = poly_div_ntt(rs, s, r2, r2_len & cond, r1, r1_len, r2l, r1h, t, q, &q_len);
            if (st) return st;
            for (uint32_t i = 0; i < ecc; ++i) t[i] = MUL(q[i], a1[i]);
            t_len = q_len + a1_len - 1;
            for (uint32_t i = 0; i < ecc; ++i) q[i] = MUL(q[i], r1[i]);
            q_len = q_len + r1_len - 1;
            for (uint32_t i = 0; i < ecc; ++i) t[i] = SUB(a2[i], t[i]);
            t_len = a2_len > t_len ? a2_len : t_len;
            for (uint32_t i = 0; i < ecc; ++i) q[i] = SUB(r2[i], q[i]);
            q_len = r2_len > q_len ? r2_len : q_len;
            memcpy(a2, a1, (size_t)ecc * 4);
            a2_len = a1_len;
            memcpy(r2, r1, (size_t)ecc * 4);
            r2_len = r1_len;
            r2l = r1l;
            cond = (uint32_t)(-(int32_t)(r1_len >= ecc / 2));
            if (!cond) {
                inttr(rs, r1);
                break;
            }
            memcpy(a1, t, (size_t)ecc * 4);
            memcpy(r1, q, (size_t)ecc * 4);
            a1_len = t_len;
            r1_len = q_len;
            inttr(rs, r1);
            if (!in_scratch(s, r1, r1_len & cond)) return ORC_ASSERT_FAIL;
            r1_len = poly_len(r1, r1_len & cond);
        }
    }
    inttr(rs, a1);
    if (!in_scratch(s, a1, a1_len & lanes)) return ORC_ASSERT_FAIL;
    a1_len = poly_len(a1, a1_len & lanes);
    uint32_t a10i = INV(a1[0]);
    for (uint32_t i = 0; i < ecc; ++i) a1[i] = MUL(a1[i], a10i);
    for (uint32_t i = 0; i < ecc; ++i) r1[i] = MUL(r1[i], a10i);
    *a1_len_out = a1_len & lanes;
    return 0;
}

int orc_rsi16_sugiyama(const orc_rsi16 *rs, uint32_t *a1, uint32_t *r1, uint32_t *temp4, uint32_t *a1_len) {
    /* py_sugiyama (pyrsi16.hpp:653-674): a1 | r1 | temp4 laid out back to back */
    (void)temp4;
    const size_t ecc = rs->ecc;
    size_t tl = rs->ntt_len + 6 * ecc;
    uint32_t *buf = (uint32_t *)calloc(tl, 4);
    memcpy(buf + ecc, r1, ecc * 4);
    scratch s = {buf, tl};
    int st = sugiyama(rs, &s, buf, buf + ecc, buf + 2 * ecc, a1_len);
    memcpy(a1, buf, ecc * 4);
    memcpy(r1, buf + ecc, ecc * 4);
    free(buf);
    return st;
}

static uint32_t eval_poly(const uint32_t *r, uint32_t r_len, uint32_t x) {
    uint32_t sum = 0;
    for (uint32_t i = r_len; i-- > 0;) sum = ADD(MUL(sum, x), r[i]);
    return sum;
}

/* RSi16v::_forney (rsi16v_impl.hpp:500-512) */
static uint32_t forney(const orc_rsi16 *rs, const uint32_t *deriv, uint32_t deriv_len, const uint32_t *ev,
                       uint32_t ev_len, uint32_t x) {
    uint32_t x_inv = INV(x);
    uint32_t num = eval_poly(ev, ev_len, x_inv);
    uint32_t den = eval_poly(deriv, deriv_len, x_inv);
    return MUL(DIV(num, den), x);
}

size_t orc_rsi16_temp_len(const orc_rsi16 *rs) { return rs->ntt_len + 6 * rs->ecc; }

/* RSi16v::_repair, unknown locations (rsi16v_impl.hpp:122-168) */
int orc_rsi16_repair(const orc_rsi16 *rs, uint32_t *block, uint32_t *temp) {
    const uint32_t ecc = (uint32_t)rs->ecc;
    scratch s = {temp, orc_rsi16_temp_len(rs)};
    uint32_t *synds = temp;
    memcpy(synds, block, rs->block_len * 4);
    pntt(rs, synds, rs->pntt_blocks);
    int nz = 0;
    for (uint32_t i = 0; i < ecc; ++i)
        if (synds[i]) nz = 1;
    if (!nz) return ORC_NO_ERRORS;
    uint32_t *evaluator = synds, *locator = temp + ecc;
    uint32_t locator_len;
    int st = sugiyama(rs, &s, locator, evaluator, temp + 2 * ecc, &locator_len);
    if (st) return st;
    uint32_t evaluator_len = ecc - locator_len + 1;
    uint32_t *deriv = temp + 2 * ecc;
    memcpy(deriv, locator, (size_t)ecc * 4);
    /* _deriv (rsi16v_impl.hpp:608-616) */
    for (uint32_t i = 0; i < ecc - 1; ++i) deriv[i] = MUL(deriv[i + 1], i + 1);
    deriv[ecc - 1] = 0;
    uint32_t deriv_len = poly_len(deriv, ecc);
    /* _find_roots_ntt (rsi16v_impl.hpp:443-497) */
    uint32_t *roots = temp + 3 * ecc;
    memset(roots, 0, rs->ntt_len * 4);
    memcpy(roots, locator, (size_t)ecc * 4);
    if (locator_len > ecc) return ORC_ASSERT_FAIL; /* py_assert at :454 */
    orc_rsi16_pintt_ecc(rs, roots);
    uint32_t lanes = (uint32_t)(-(int32_t)(locator_len != 0));
    uint32_t dl = deriv_len & lanes, el = evaluator_len & lanes;
    uint32_t root_count = 0;
    for (uint32_t i = 0; i < rs->block_len; ++i) {
        uint32_t x = rs->roots_ntt[orc_rsi16_rbo(rs, i)];
        uint32_t loc = (uint32_t)(roots[i] == 0) & lanes;
        root_count += 1 & loc;
        if (loc) {
            uint32_t e = forney(rs, deriv, dl, evaluator, el, x);
            block[i] = ADD(block[i], e);
        }
    }
    if (root_count > 0) return ORC_REPAIR_OK;
    return lanes ? ORC_ERROR_LOCATION_FAIL : ORC_NO_ERRORS;
}

/* RSi16v::_repair, known locations (rsi16v_impl.hpp:171-231) with
 * _error_locator (:531-542) and _error_evaluator (:545-563).  `pos` holds
 * positions in RBO form (ntt.rbo of the block position). */
int orc_rsi16_repair_known(const orc_rsi16 *rs, uint32_t *block, const uint32_t *pos_rbo, size_t count,
                           uint32_t *temp) {
    const uint32_t ecc = (uint32_t)rs->ecc;
    uint32_t *synds = temp;
    memcpy(synds, block, rs->block_len * 4);
    pntt(rs, synds, rs->pntt_blocks);
    int nz = 0;
    for (uint32_t i = 0; i < ecc; ++i)
        if (synds[i]) nz = 1;
    if (!nz) return ORC_NO_ERRORS;
    uint32_t *ev = temp, *loc = temp + 2 * ecc, *tmp = temp + 4 * ecc;
    memset(loc, 0, (size_t)ecc * 4);
    for (size_t j = 0; j < count; ++j) {
        uint32_t x = rs->roots_ntt[pos_rbo[j]];
        for (size_t i = count - 1; i > 0; --i) loc[i] = SUB(loc[i], MUL(loc[i - 1], x));
        loc[0] = SUB(loc[0], x);
    }
    memset(ev + ecc, 0, (size_t)ecc * 4);
    nttr2(rs, ev);
    memcpy(tmp + 1, loc, count * 4);
    tmp[0] = 1;
    for (size_t i = count + 1; i < 2 * (size_t)ecc + 1; ++i) tmp[i] = 0;
    nttr2(rs, tmp);
    for (uint32_t i = 0; i < 2 * ecc; ++i) ev[i] = MUL(ev[i], tmp[i]);
    inttr2(rs, ev);
    memset(ev + ecc, 0, (size_t)ecc * 4);
    uint32_t *deriv = temp + ecc;
    memcpy(deriv, loc, (size_t)ecc * 4);
    for (uint32_t i = 0; i < ecc; ++i) deriv[i] = MUL(deriv[i], i + 1); /* _deriv_shifted */
    uint32_t deriv_len = poly_len(deriv, ecc);
    for (size_t i = 0; i < count; ++i) {
        uint32_t p = orc_rsi16_rbo(rs, pos_rbo[i]);
        uint32_t x = rs->roots_ntt[pos_rbo[i]];
        uint32_t e = forney(rs, deriv, deriv_len, ev, ecc, x);
        block[p] = ADD(block[p], e);
    }
    return ORC_REPAIR_OK;
}

typedef struct {
    const orc_rsi16 *rs;
    uint16_t *msg, *parity;
    int8_t *status;
} rsi_rep_ctx;

static void rsi_rep_range(void *p, size_t b, size_t e) {
    rsi_rep_ctx *c = (rsi_rep_ctx *)p;
    const orc_rsi16 *rs = c->rs;
    uint32_t *blk = (uint32_t *)malloc(rs->block_len * 4), *tmp = (uint32_t *)calloc(orc_rsi16_temp_len(rs), 4);
    for (size_t i = b; i < e; ++i) {
        uint16_t *m = c->msg + i * rs->message_len, *q = c->parity + i * rs->ecc;
        for (size_t k = 0; k < rs->message_len; ++k) blk[k] = m[k];
        for (size_t k = 0; k < rs->ecc; ++k) blk[rs->message_len + k] = q[k];
        int st = orc_rsi16_repair(rs, blk, tmp);
        c->status[i] = (int8_t)st;
        if (st < 0) continue; /* RuntimeError: the reference never copies back */
        for (size_t k = 0; k < rs->message_len; ++k) m[k] = (uint16_t)blk[k];
        for (size_t k = 0; k < rs->ecc; ++k) q[k] = (uint16_t)blk[rs->message_len + k];
    }
    free(blk);
    free(tmp);
}

/* PyRSi16::py_repair (pyrsi16.hpp:588-631), interleave == 1, unknown locations */
void orc_rsi16_repair_blocks(const orc_rsi16 *rs, uint16_t *msg, uint16_t *parity, size_t nblocks, int8_t *status,
                             int threads) {
    rsi_rep_ctx c = {rs, msg, parity, status};
    orc_parallel_for(nblocks, threads, rsi_rep_range, &c);
}

/* PyRSi16::_repair_interleaved with SIMD_W = 1 (pyrsi16.hpp:390-522).  count < 0
 * selects unknown locations.  pos holds block positions (not RBO). */
int orc_rsi16_repair_interleaved_u32(const orc_rsi16 *rs, uint32_t *msg, uint32_t *ecc, size_t interleave,
                                     size_t col_start, size_t col_count, const uint32_t *pos, long count) {
    uint32_t *blk = (uint32_t *)malloc(rs->block_len * 4), *tmp = (uint32_t *)calloc(orc_rsi16_temp_len(rs), 4);
    uint32_t *prbo = NULL;
    if (count >= 0) {
        prbo = (uint32_t *)malloc(((size_t)count + 1) * 4);
        for (long i = 0; i < count; ++i) prbo[i] = orc_rsi16_rbo(rs, pos[i]);
    }
    int res = ORC_NO_ERRORS;
    for (size_t c = col_start; c < col_start + col_count; ++c) {
        for (size_t k = 0; k < rs->message_len; ++k) blk[k] = msg[c + k * interleave];
        for (size_t k = 0; k < rs->ecc; ++k) blk[rs->message_len + k] = ecc[c + k * interleave];
        int st = count >= 0 ? orc_rsi16_repair_known(rs, blk, prbo, (size_t)count, tmp) : orc_rsi16_repair(rs, blk, tmp);
        if (st < 0) {
            res = st;
            break;
        }
        if (st > res) res = st;
        for (size_t k = 0; k < rs->message_len; ++k) msg[c + k * interleave] = blk[k];
        for (size_t k = 0; k < rs->ecc; ++k) ecc[c + k * interleave] = blk[rs->message_len + k];
    }
    free(blk);
    free(tmp);
    free(prbo);
    return res;
}

/* ======================================================================
 * CIRC16 (libffrs/pycirc16.hpp)
 * ====================================================================== */
struct orc_circ16 {
    orc_rsi16 *rsi, *rso;
    size_t interleave, rso_interleave;
    size_t block_len, message_len, rsi_interleaved_ecc_len, rsio_ecc_len, ecc_len, rso_interleaved_ecc_len;
};

orc_circ16 *orc_circ16_new(size_t ib, size_t ie, size_t ob, size_t oe, size_t interleave, uint32_t primitive, char *err,
                           size_t errlen) {
    if (interleave == 0) {
        seterr(err, errlen, "interleave must be positive");
        return NULL;
    }
    orc_rsi16 *rsi = orc_rsi16_new(ib, ie, primitive, err, errlen);
    if (!rsi) return NULL;
    orc_rsi16 *rso = orc_rsi16_new(ob, oe, primitive, err, errlen);
    if (!rso) {
        orc_rsi16_free(rsi);
        return NULL;
    }
    orc_circ16 *c = (orc_circ16 *)calloc(1, sizeof *c);
    c->rsi = rsi;
    c->rso = rso;
    c->interleave = interleave;
    c->rso_interleave = rsi->message_len * interleave;
    c->block_len = ib * ob * interleave;
    c->message_len = rso->message_len * c->rso_interleave;
    c->rso_interleaved_ecc_len = rso->ecc * c->rso_interleave;
    c->rsi_interleaved_ecc_len = rsi->ecc * rso->message_len * interleave;
    c->rsio_ecc_len = rsi->ecc * rso->ecc * interleave;
    c->ecc_len = c->rso_interleaved_ecc_len + c->rsi_interleaved_ecc_len + c->rsio_ecc_len;
    return c;
}

void orc_circ16_free(orc_circ16 *c) {
    if (!c) return;
    orc_rsi16_free(c->rsi);
    orc_rsi16_free(c->rso);
    free(c);
}
size_t orc_circ16_message_len(const orc_circ16 *c) { return c->message_len; }
size_t orc_circ16_ecc_len(const orc_circ16 *c) { return c->ecc_len; }

/* PyCIRC16::encode_block (pycirc16.hpp:352-363): [rso_ecc | rsi_ecc | rsio_ecc] */
void orc_circ16_encode(const orc_circ16 *c, const uint16_t *msg, uint16_t *ecc) {
    const orc_rsi16 *rsi = c->rsi, *rso = c->rso;
    uint32_t *m = (uint32_t *)malloc(c->message_len * 4);
    uint32_t *po = (uint32_t *)malloc(c->rso_interleaved_ecc_len * 4);
    uint32_t *bi = (uint32_t *)malloc(rsi->block_len * 4), *pi = (uint32_t *)malloc(rsi->ecc * 4);
    for (size_t i = 0; i < c->message_len; ++i) m[i] = msg[i];
    orc_rsi16_encode_interleaved_u32(rso, m, c->rso_interleave, po);
    for (size_t i = 0; i < c->rso_interleaved_ecc_len; ++i) ecc[i] = (uint16_t)po[i];
    uint16_t *rsi_ecc = ecc + c->rso_interleaved_ecc_len;
    size_t nrows = rso->message_len * c->interleave;
    for (size_t b = 0; b < nrows; ++b) {
        orc_rsi16_encode_u32(rsi, m + b * rsi->message_len, pi);
        for (size_t k = 0; k < rsi->ecc; ++k) rsi_ecc[b * rsi->ecc + k] = (uint16_t)pi[k];
    }
    uint16_t *rsio = rsi_ecc + c->rsi_interleaved_ecc_len;
    size_t orows = rso->ecc * c->interleave;
    for (size_t b = 0; b < orows; ++b) { /* encoded from the untruncated outer parity */
        orc_rsi16_encode_u32(rsi, po + b * rsi->message_len, pi);
        for (size_t k = 0; k < rsi->ecc; ++k) rsio[b * rsi->ecc + k] = (uint16_t)pi[k];
    }
    (void)bi;
    free(m);
    free(po);
    free(bi);
    free(pi);
}

typedef struct {
    const orc_circ16 *c;
    const uint16_t *msg;
    uint16_t *ecc;
} circ_enc_ctx;

static void circ_enc_range(void *p, size_t b, size_t e) {
    circ_enc_ctx *x = (circ_enc_ctx *)p;
    for (size_t i = b; i < e; ++i)
        orc_circ16_encode(x->c, x->msg + i * x->c->message_len, x->ecc + i * x->c->ecc_len);
}

void orc_circ16_encode_blocks(const orc_circ16 *c, const uint16_t *msg, size_t nblocks, uint16_t *ecc, int threads) {
    circ_enc_ctx x = {c, msg, ecc};
    orc_parallel_for(nblocks, threads, circ_enc_range, &x);
}

typedef struct {
    const orc_circ16 *c;
    uint32_t *rsi_temp, *rsi_repair_temp, *rsi_synd, *rso_ecc, *rsi_ecc, *rsio_ecc;
} circ_rep;

static size_t rso_ecc_offset(const orc_circ16 *c, size_t k, size_t row) {
    return c->rso_interleave * row + k * c->rsi->message_len;
}
static size_t rsi_ecc_offset(const orc_circ16 *c, size_t k, size_t row) {
    return (row * c->interleave + k) * c->rsi->ecc;
}
static int any_synd(const circ_rep *r, const uint32_t *s) {
    for (size_t i = 0; i < r->c->rsi->ecc; ++i)
        if (s[i]) return 1;
    return 0;
}

static void circ_rep_init(circ_rep *r, const orc_circ16 *c, const uint16_t *msg, const uint16_t *ecc) {
    const orc_rsi16 *rsi = c->rsi, *rso = c->rso;
    r->c = c;
    r->rsi_temp = (uint32_t *)calloc(rsi->block_len, 4);
    r->rsi_repair_temp = (uint32_t *)calloc(orc_rsi16_temp_len(rsi), 4);
    r->rsi_synd = (uint32_t *)calloc(rso->block_len * rsi->ecc * c->interleave, 4);
    r->rso_ecc = (uint32_t *)calloc(c->rso_interleaved_ecc_len, 4);
    r->rsi_ecc = (uint32_t *)calloc(rsi->ecc * rso->block_len * c->interleave, 4);
    r->rsio_ecc = r->rsi_ecc + c->rsi_interleaved_ecc_len;
    /* load_ecc (pycirc16.hpp:159-163) */
    for (size_t i = 0; i < c->rso_interleaved_ecc_len; ++i) r->rso_ecc[i] = ecc[i];
    for (size_t i = 0; i < rsi->ecc * rso->block_len * c->interleave; ++i)
        r->rsi_ecc[i] = ecc[c->rso_interleaved_ecc_len + i];
    /* compute_rsi_synd (pycirc16.hpp:165-181) via synd_blocks (pyrsi16.hpp:190-200) */
    size_t nrows = rso->message_len * c->interleave;
    for (size_t b = 0; b < nrows; ++b) {
        for (size_t k = 0; k < rsi->message_len; ++k) r->rsi_temp[k] = msg[b * rsi->message_len + k];
        for (size_t k = 0; k < rsi->ecc; ++k) r->rsi_temp[rsi->message_len + k] = r->rsi_ecc[b * rsi->ecc + k];
        pntt(rsi, r->rsi_temp, rsi->pntt_blocks);
        memcpy(&r->rsi_synd[b * rsi->ecc], r->rsi_temp, rsi->ecc * 4);
    }
    size_t orows = rso->ecc * c->interleave;
    for (size_t b = 0; b < orows; ++b) {
        for (size_t k = 0; k < rsi->message_len; ++k) r->rsi_temp[k] = r->rso_ecc[b * rsi->message_len + k];
        for (size_t k = 0; k < rsi->ecc; ++k) r->rsi_temp[rsi->message_len + k] = r->rsio_ecc[b * rsi->ecc + k];
        pntt(rsi, r->rsi_temp, rsi->pntt_blocks);
        memcpy(&r->rsi_synd[c->rsi_interleaved_ecc_len + b * rsi->ecc], r->rsi_temp, rsi->ecc * 4);
    }
}

static void circ_rep_free(circ_rep *r) {
    free(r->rsi_temp);
    free(r->rsi_repair_temp);
    free(r->rsi_synd);
    free(r->rso_ecc);
    free(r->rsi_ecc);
}

/* CircRepair::repair_outer_zeros (pycirc16.hpp:183-240) */
static void circ_repair_outer_zeros(circ_rep *r, size_t k) {
    const orc_circ16 *c = r->c;
    const orc_rsi16 *rsi = c->rsi, *rso = c->rso;
    size_t *zeros = (size_t *)malloc((rsi->block_len + 1) * sizeof(size_t));
    uint32_t *zrbo = (uint32_t *)malloc((rsi->block_len + 1) * 4);
    for (size_t i = rso->message_len; i < rso->block_len; ++i) {
        size_t nz = 0;
        size_t ro = rso_ecc_offset(c, k, i - rso->message_len);
        size_t io = rsi_ecc_offset(c, k, i);
        if (!any_synd(r, &r->rsi_synd[io])) continue;
        for (size_t j = 0; j < rsi->message_len; ++j)
            if (r->rso_ecc[ro + j] == 0) zeros[nz++] = j;
        for (size_t j = 0; j < rsi->ecc; ++j)
            if (r->rsi_ecc[io + j] == 0) zeros[nz++] = rsi->message_len + j;
        if (nz == 0) continue;
        if (nz > rsi->ecc) continue;
        memcpy(r->rsi_temp, &r->rso_ecc[ro], rsi->message_len * 4);
        memcpy(r->rsi_temp + rsi->message_len, &r->rsi_ecc[io], rsi->ecc * 4);
        for (size_t z = 0; z < nz; ++z) zrbo[z] = orc_rsi16_rbo(rsi, (uint32_t)zeros[z]);
        orc_rsi16_repair_known(rsi, r->rsi_temp, zrbo, nz, r->rsi_repair_temp);
        int ok = 1;
        for (size_t z = 0; z < nz; ++z)
            if ((r->rsi_temp[zeros[z]] & 0xffff) != 0) ok = 0;
        if (ok) {
            memcpy(&r->rso_ecc[ro], r->rsi_temp, rsi->message_len * 4);
            memcpy(&r->rsi_ecc[io], r->rsi_temp + rsi->message_len, rsi->ecc * 4);
            pntt(rsi, r->rsi_temp, rsi->pntt_blocks);
            memcpy(&r->rsi_synd[io], r->rsi_temp, rsi->ecc * 4);
        }
    }
    free(zeros);
    free(zrbo);
}

/* CircRepair::repair_inner_zeros (pycirc16.hpp:242-281) */
static void circ_repair_inner_zeros(circ_rep *r, size_t k) {
    const orc_circ16 *c = r->c;
    const orc_rsi16 *rsi = c->rsi, *rso = c->rso;
    for (size_t i = 0; i < rso->block_len; ++i) {
        size_t io = rsi_ecc_offset(c, k, i);
        if (!any_synd(r, &r->rsi_synd[io])) continue;
        int has_zero = 0;
        for (size_t j = 0; j < rsi->ecc; ++j)
            if (r->rsi_ecc[io + j] == 0) has_zero = 1;
        if (!has_zero) continue;
        memcpy(r->rsi_temp, &r->rsi_synd[io], rsi->ecc * 4);
        orc_rsi16_mix_ecc(rsi, r->rsi_temp);
        int all0 = 1;
        for (size_t j = 0; j < rsi->ecc; ++j)
            if ((r->rsi_temp[j] & 0xffff) != 0) all0 = 0;
        if (all0) {
            memcpy(&r->rsi_ecc[io], r->rsi_temp, rsi->ecc * 4);
            memset(&r->rsi_synd[io], 0, rsi->ecc * 4);
        }
    }
}

static size_t circ_find_error_locations(circ_rep *r, size_t k, size_t *loc) {
    size_t n = 0;
    for (size_t i = 0; i < r->c->rso->block_len; ++i)
        if (any_synd(r, &r->rsi_synd[rsi_ecc_offset(r->c, k, i)])) loc[n++] = i;
    return n;
}

/* PyCIRC16::py_repair via CircRepair (pycirc16.hpp:307-330, 365-384) */
int orc_circ16_repair(const orc_circ16 *c, uint16_t *msg, uint16_t *ecc) {
    const orc_rsi16 *rsi = c->rsi, *rso = c->rso;
    circ_rep r;
    circ_rep_init(&r, c, msg, ecc);
    size_t *loc = (size_t *)malloc((rso->block_len + 1) * sizeof(size_t));
    uint32_t *loc32 = (uint32_t *)malloc((rso->block_len + 1) * 4);
    /* rso.repair_interleaved works on message words widened to uint32 and
     * writes them back truncated, which is what a uint32 copy does here. */
    uint32_t *m32 = (uint32_t *)malloc(c->message_len * 4);
    for (size_t i = 0; i < c->message_len; ++i) m32[i] = msg[i];
    int rc = 0;
    for (size_t k = 0; k < c->interleave && rc == 0; ++k) {
        circ_repair_outer_zeros(&r, k);
        circ_repair_inner_zeros(&r, k);
        size_t n = circ_find_error_locations(&r, k, loc);
        if (n == 0) continue;
        for (size_t i = 0; i < n; ++i) loc32[i] = (uint32_t)loc[i];
        int st;
        if (n <= rso->ecc)
            st = orc_rsi16_repair_interleaved_u32(rso, m32, r.rso_ecc, c->rso_interleave, k * rsi->message_len,
                                                  rsi->message_len, loc32, (long)n);
        else
            st = orc_rsi16_repair_interleaved_u32(rso, m32, r.rso_ecc, c->rso_interleave, k * rsi->message_len,
                                                  rsi->message_len, NULL, -1);
        for (size_t i = 0; i < c->message_len; ++i) m32[i] &= 0xffff;
        if (st < 0) rc = st;
    }
    for (size_t i = 0; i < c->message_len; ++i) msg[i] = (uint16_t)m32[i];
    if (rc == 0) {
        /* recompute_inner_ecc (pycirc16.hpp:320-324) + dump_ecc (:326-330) */
        size_t nrows = rso->message_len * c->interleave;
        for (size_t b = 0; b < nrows; ++b) orc_rsi16_encode_u32(rsi, m32 + b * rsi->message_len, r.rsi_ecc + b * rsi->ecc);
        size_t orows = rso->ecc * c->interleave;
        for (size_t b = 0; b < orows; ++b)
            orc_rsi16_encode_u32(rsi, r.rso_ecc + b * rsi->message_len, r.rsio_ecc + b * rsi->ecc);
        for (size_t i = 0; i < c->rso_interleaved_ecc_len; ++i) ecc[i] = (uint16_t)r.rso_ecc[i];
        for (size_t i = 0; i < rsi->ecc * rso->block_len * c->interleave; ++i)
            ecc[c->rso_interleaved_ecc_len + i] = (uint16_t)r.rsi_ecc[i];
    }
    free(m32);
    free(loc);
    free(loc32);
    circ_rep_free(&r);
    return rc;
}

/* PyCIRC16::py_find_outer_error_locations (pycirc16.hpp:386-405) */
long orc_circ16_find_outer_error_locations(const orc_circ16 *c, const uint16_t *msg, const uint16_t *ecc, size_t k,
                                           size_t *out, size_t out_cap) {
    circ_rep r;
    circ_rep_init(&r, c, msg, ecc);
    circ_repair_outer_zeros(&r, k);
    circ_repair_inner_zeros(&r, k);
    size_t *loc = (size_t *)malloc((c->rso->block_len + 1) * sizeof(size_t));
    size_t n = circ_find_error_locations(&r, k, loc);
    for (size_t i = 0; i < n && i < out_cap; ++i) out[i] = loc[i];
    free(loc);
    circ_rep_free(&r);
    return (long)n;
}
