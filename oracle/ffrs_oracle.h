/*
 * ffrs_oracle.h -- CPU restatement of the libffrs block-coding algorithms.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path in
 * libffrs_gb300: only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it.  The product path never calls it.
 *
 * Every function restates the reference algorithm it names (file:line inside
 * the zydd/libffrs project) in plain C, including the reference's control-flow
 * quirks (lengths kept as uint32 with wrap-around, inv(0) == 1, div(a, 0) == a,
 * the NTT-domain Sugiyama termination rule).  Parity is pinned against the
 * reference itself: tests/golden/ holds fixtures produced by the reference's
 * own pybind11 module and the oracle must reproduce them byte for byte.
 */
#ifndef FFRS_ORACLE_H
#define FFRS_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes of the RSi16 repair (libffrs/rsi16v.hpp:32-38) */
enum { ORC_NO_ERRORS = 0, ORC_NO_ERRORS_ZERO = 1, ORC_REPAIR_OK = 2, ORC_REPAIR_FAIL = 3, ORC_ERROR_LOCATION_FAIL = 4 };
/* a reference py_assert that would raise RuntimeError */
#define ORC_ASSERT_FAIL (-1)

/* ---------------------------------------------------------------- RS256 */
typedef struct orc_rs256 orc_rs256;

orc_rs256 *orc_rs256_new(int ecc_len, int primitive, int polynomial);
void orc_rs256_free(orc_rs256 *rs);
int orc_rs256_ecc_len(const orc_rs256 *rs);
void orc_rs256_generator(const orc_rs256 *rs, uint8_t *generator, uint8_t *roots);
void orc_rs256_tables(const orc_rs256 *rs, uint8_t *exp256, uint8_t *log256);
/* parity of one (possibly shortened) message, ecc_len bytes */
void orc_rs256_encode(const orc_rs256 *rs, const uint8_t *msg, size_t len, uint8_t *parity);
/* RS256.encode(buffer): full message_len chunks then a shortened tail */
size_t orc_rs256_encode_buffer(const orc_rs256 *rs, const uint8_t *buf, size_t len, size_t message_len, uint8_t *out,
                               int threads);
void orc_rs256_synds(const orc_rs256 *rs, const uint8_t *data, size_t size, const uint8_t *rem, uint8_t *synds);
/* RS256.repair(data, ecc): returns 1 (true) or 0 (false), in place */
int orc_rs256_decode(const orc_rs256 *rs, uint8_t *data, size_t size, uint8_t *rem);
/* nblocks independent repairs: data is nblocks x message_len, parity nblocks x ecc_len */
void orc_rs256_decode_blocks(const orc_rs256 *rs, uint8_t *data, uint8_t *parity, size_t nblocks, size_t message_len,
                             uint8_t *status, int threads);

/* ---------------------------------------------------------------- GF(65537) / RSi16 */
typedef struct orc_rsi16 orc_rsi16;

/* returns NULL and fills err on a reference py_assert failure */
orc_rsi16 *orc_rsi16_new(size_t block_len, size_t ecc_len, uint32_t primitive, char *err, size_t errlen);
void orc_rsi16_free(orc_rsi16 *rs);
size_t orc_rsi16_ntt_len(const orc_rsi16 *rs);
uint32_t orc_rsi16_root(const orc_rsi16 *rs);
uint32_t orc_rsi16_rbo(const orc_rsi16 *rs, uint32_t i);
/* read-only views of the code tables (for kernel table checks) */
const uint32_t *orc_rsi16_table(const orc_rsi16 *rs, int which, size_t *len);

/* GF(65537) scalar ops (libffrs/galois.hpp:258-395, 168-216) */
uint32_t orc_gfi16_mul(uint32_t a, uint32_t b);
uint32_t orc_gfi16_add(uint32_t a, uint32_t b);
uint32_t orc_gfi16_sub(uint32_t a, uint32_t b);
uint32_t orc_gfi16_inv(const orc_rsi16 *rs, uint32_t a);
uint32_t orc_gfi16_div(const orc_rsi16 *rs, uint32_t a, uint32_t b);
uint32_t orc_gfi16_pow(const orc_rsi16 *rs, uint32_t a, uint32_t e);

/* parity of one block from message_len words (values may be 65536) */
void orc_rsi16_encode_u32(const orc_rsi16 *rs, const uint32_t *msg, uint32_t *parity);
/* nblocks blocks, uint16 message words -> uint16 parity words (truncating) */
void orc_rsi16_encode_blocks(const orc_rsi16 *rs, const uint16_t *msg, size_t nblocks, uint16_t *parity, int threads);
/* interleaved encode of one interleaved block (pyrsi16.hpp:323-361) */
void orc_rsi16_encode_interleaved_u32(const orc_rsi16 *rs, const uint32_t *msg, size_t interleave, uint32_t *parity);
void orc_rsi16_synd(const orc_rsi16 *rs, const uint32_t *block, uint32_t *synds);
/* temp must hold orc_rsi16_temp_len() words */
size_t orc_rsi16_temp_len(const orc_rsi16 *rs);
int orc_rsi16_repair(const orc_rsi16 *rs, uint32_t *block, uint32_t *temp);
int orc_rsi16_repair_known(const orc_rsi16 *rs, uint32_t *block, const uint32_t *pos, size_t count, uint32_t *temp);
/* RSi16.repair for nblocks single blocks (uint16 in/out), status per block (negative = assert) */
void orc_rsi16_repair_blocks(const orc_rsi16 *rs, uint16_t *msg, uint16_t *parity, size_t nblocks, int8_t *status,
                             int threads);
/* repair_interleaved W=1 semantics; message and ecc hold uint32 words */
int orc_rsi16_repair_interleaved_u32(const orc_rsi16 *rs, uint32_t *msg, uint32_t *ecc, size_t interleave,
                                     size_t col_start, size_t col_count, const uint32_t *pos, long count);
int orc_rsi16_sugiyama(const orc_rsi16 *rs, uint32_t *a1, uint32_t *r1, uint32_t *temp4, uint32_t *a1_len);
void orc_rsi16_pintt_ecc(const orc_rsi16 *rs, uint32_t *block);
void orc_rsi16_mix_ecc(const orc_rsi16 *rs, uint32_t *ecc);

/* ---------------------------------------------------------------- CIRC16 */
typedef struct orc_circ16 orc_circ16;
orc_circ16 *orc_circ16_new(size_t inner_block_len, size_t inner_ecc_len, size_t outer_block_len, size_t outer_ecc_len,
                           size_t interleave, uint32_t primitive, char *err, size_t errlen);
void orc_circ16_free(orc_circ16 *c);
size_t orc_circ16_message_len(const orc_circ16 *c);
size_t orc_circ16_ecc_len(const orc_circ16 *c);
void orc_circ16_encode(const orc_circ16 *c, const uint16_t *msg, uint16_t *ecc);
void orc_circ16_encode_blocks(const orc_circ16 *c, const uint16_t *msg, size_t nblocks, uint16_t *ecc, int threads);
int orc_circ16_repair(const orc_circ16 *c, uint16_t *msg, uint16_t *ecc);
long orc_circ16_find_outer_error_locations(const orc_circ16 *c, const uint16_t *msg, const uint16_t *ecc, size_t k,
                                           size_t *out, size_t out_cap);

#ifdef __cplusplus
}
#endif
#endif
