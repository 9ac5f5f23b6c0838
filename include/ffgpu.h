/*
 * ffgpu.h -- C ABI of the GB300 block-coding library (libffgpu.so).
 *
 * Plain pointers, sizes and status codes; no C++ or torch types.  Every
 * function returns FFGPU_OK (0) or a negative FFGPU_E* code; the message of
 * the last failure on the calling thread is ffgpu_last_error().
 *
 * "Device" entry points take device pointers and a cudaStream_t passed as
 * void*, enqueue work and return without synchronising.  "Host" entry points
 * take host buffers, stage them through pinned memory, run on the library's
 * stream and return after the results are back in the caller's buffers.
 *
 * Each declaration names the reference interface it replaces; paths are
 * relative to the zydd/libffrs project.
 */
#ifndef FFGPU_H
#define FFGPU_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define FFGPU_API __attribute__((visibility("default")))
#else
#define FFGPU_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define FFGPU_OK 0
#define FFGPU_EINVAL (-1)   /* bad argument: ValueError in the reference binding */
#define FFGPU_ECUDA (-2)    /* CUDA runtime failure */
#define FFGPU_ENOMEM (-3)   /* device or pinned allocation failed */
#define FFGPU_EASSERT (-4)  /* a reference py_assert would fire: RuntimeError */
#define FFGPU_ETIMEOUT (-5) /* a bounded device wait gave up */
#define FFGPU_ECANCELLED (-6) /* a served request was withdrawn by ffgpu_server_cancel */

/* RSi16 repair status (libffrs/rsi16v.hpp:32-38) */
#define FFGPU_NO_ERRORS 0
#define FFGPU_NO_ERRORS_ZERO 1
#define FFGPU_REPAIR_OK 2
#define FFGPU_REPAIR_FAIL 3
#define FFGPU_ERROR_LOCATION_FAIL 4
/* per-block status value meaning "the reference raises RuntimeError here" */
#define FFGPU_STATUS_ASSERT 0xFF

typedef struct ffgpu_rs256 ffgpu_rs256;
typedef struct ffgpu_rsi16 ffgpu_rsi16;
typedef struct ffgpu_circ16 ffgpu_circ16;

/* ---------------------------------------------------------------- runtime */
FFGPU_API const char *ffgpu_last_error(void);
FFGPU_API const char *ffgpu_version(void);
/* select the device used by later calls on this process (default 0) */
FFGPU_API int ffgpu_init(int device);
/* number of kernels this library has launched since load (for accounting) */
FFGPU_API uint64_t ffgpu_kernel_launches(void);
/* No reference counterpart (measurement support).  While enabled, every
 * kernel launch is bracketed by a CUDA event pair on its stream;
 * ffgpu_timing_collect waits for the recorded launches and writes one line
 * "<kernel> <total ms> <launches>" per kernel into out (NUL-terminated,
 * truncated to cap), the full length into *len, and forgets them. */
FFGPU_API int ffgpu_timing_enable(int on);
FFGPU_API int ffgpu_timing_collect(char *out, size_t cap, size_t *len);
/* No reference counterpart (tuning).  The host-buffer decode entry points
 * copy, decode and copy back in chunks of blocks on three streams so that
 * transfers overlap decoding; 0 (the default) chooses the chunk from the
 * request size, any other value fixes the blocks per chunk. */
FFGPU_API int ffgpu_set_host_chunk_blocks(size_t blocks);
/* the library's own stream (cudaStream_t) */
FFGPU_API void *ffgpu_default_stream(void);
FFGPU_API int ffgpu_synchronize(void *stream);

/* create_buffer (libffrs/pyffrs.cpp:41-98): zeroed, page-locked host memory */
FFGPU_API int ffgpu_host_alloc(size_t bytes, void **out);
FFGPU_API int ffgpu_host_free(void *ptr);

/* ---------------------------------------------------------------- RS256 */
/* PyRS256 ctor (libffrs/pyrs256.hpp:63-97): GF(2^8) tables, generator and the
 * encoder's table, resident on the device.  ecc_len in [1, 254]. */
FFGPU_API int ffgpu_rs256_create(int ecc_len, int primitive, int polynomial, ffgpu_rs256 **out);
FFGPU_API int ffgpu_rs256_destroy(ffgpu_rs256 *code);
/* generator (ecc_len + 1 bytes) and generator_roots (ecc_len bytes),
 * pyrs256.hpp:165-169 */
FFGPU_API int ffgpu_rs256_generator(const ffgpu_rs256 *code, uint8_t *generator, uint8_t *roots);

/* nblocks messages of message_len bytes, back to back, -> nblocks x ecc_len
 * parity bytes (rs_encode_slice_pw2_dispatch::encode, reed_solomon.hpp:335-337,
 * looped as in PyRS256::py_encode, pyrs256.hpp:118-120) */
FFGPU_API int ffgpu_rs256_encode(const ffgpu_rs256 *code, const uint8_t *data, size_t nblocks, size_t message_len,
                       uint8_t *parity, void *stream);
/* in-place repair of nblocks (data, parity) pairs; status[i] = 1 (true) or 0
 * (false) exactly as rs_decode::decode (reed_solomon.hpp:559-595) called by
 * PyRS256::py_repair (pyrs256.hpp:129-131) once per block */
FFGPU_API int ffgpu_rs256_decode(const ffgpu_rs256 *code, uint8_t *data, uint8_t *parity, size_t nblocks, size_t message_len,
                       uint8_t *status, void *stream);
/* syndromes of nblocks blocks, ecc_len bytes each (PyRS256::py_synds, pyrs256.hpp:133-140) */
FFGPU_API int ffgpu_rs256_synds(const ffgpu_rs256 *code, const uint8_t *data, const uint8_t *parity, size_t nblocks,
                      size_t message_len, uint8_t *synds, void *stream);

/* host-buffer forms: RS256.encode(buffer) including the shortened tail block
 * (pyrs256.hpp:99-127); out must hold ceil(len / message_len) * ecc_len bytes */
FFGPU_API int ffgpu_rs256_encode_host(const ffgpu_rs256 *code, const uint8_t *buf, size_t len, size_t message_len, uint8_t *out);
FFGPU_API int ffgpu_rs256_decode_host(const ffgpu_rs256 *code, uint8_t *data, uint8_t *parity, size_t nblocks,
                            size_t message_len, uint8_t *status);
FFGPU_API int ffgpu_rs256_synds_host(const ffgpu_rs256 *code, const uint8_t *data, const uint8_t *parity, size_t nblocks,
                           size_t message_len, uint8_t *synds);
/* No reference counterpart.  ffgpu_rs256_decode without any allocation: the
 * same kernels and results, on a fixed 18 MiB scratch array compiled into the
 * library, for callers that cannot allocate device memory on their hot path.
 * Covers ecc_len 16/32 with primitive 2 and polynomial 0x11d and 4-byte
 * aligned buffers; at most 524,288 blocks per call at ecc_len 32 (1,048,576
 * at 16), else FFGPU_EINVAL.  One scratch per device: calls that may overlap
 * on the device (other streams or threads) race and must be ordered by the
 * caller.  Make the first call on a device outside stream capture.  The
 * scratch is the current device's, so the stream must belong to it
 * (checked); a code set to the table decoder (ffgpu_rs256_set_table_only)
 * is rejected with FFGPU_EINVAL. */
FFGPU_API int ffgpu_rs256_decode_noalloc(const ffgpu_rs256 *code, uint8_t *data, uint8_t *parity, size_t nblocks,
                                         size_t message_len, uint8_t *status, void *stream);
/* No reference counterpart.  table_only != 0 makes this code use the
 * byte-table kernels only (the bitsliced kernels are otherwise chosen for
 * ecc_len 16/32 with primitive 2 and 4-byte aligned buffers); results are
 * identical either way, the switch exists to cross-check the two kernel
 * families. */
FFGPU_API int ffgpu_rs256_set_table_only(ffgpu_rs256 *code, int table_only);

/* ---------------------------------------------------------------- RSi16 */
/* PyRSi16 ctor (libffrs/pyrsi16.hpp:41-125), NTT ctor (libffrs/ntt.hpp:55-123),
 * RSi16v ctor (libffrs/rsi16v_impl.hpp:68-86). */
FFGPU_API int ffgpu_rsi16_create(size_t block_len, size_t ecc_len, uint32_t primitive, ffgpu_rsi16 **out);
FFGPU_API int ffgpu_rsi16_destroy(ffgpu_rsi16 *code);
/* No reference counterpart (observability).  Blocks that the unknown-location
 * repair served with the bounded-distance (Berlekamp-Massey) path and with the
 * step-for-step mirror of the reference's algorithm, since load or the last
 * reset; synchronises the device. */
FFGPU_API int ffgpu_rsi16_repair_counters(uint64_t *fast_blocks, uint64_t *mirror_blocks, int reset);
/* root, ntt_len */
FFGPU_API int ffgpu_rsi16_info(const ffgpu_rsi16 *code, uint32_t *root, size_t *ntt_len);

/* nblocks x message_len uint16 words -> nblocks x ecc_len uint16 parity words
 * (RSi16v::_encode, rsi16v_impl.hpp:93-119, via PyRSi16::encode_blocks,
 * pyrsi16.hpp:127-140; parity truncated to 16 bits as pyrsi16.hpp:370) */
FFGPU_API int ffgpu_rsi16_encode(const ffgpu_rsi16 *code, const uint16_t *msg, size_t nblocks, uint16_t *parity, void *stream);
/* interleaved encode of nblocks interleaved blocks (PyRSi16::_encode_interleaved,
 * pyrsi16.hpp:323-361): msg is message_len x interleave words per block,
 * parity ecc_len x interleave words per block */
FFGPU_API int ffgpu_rsi16_encode_interleaved(const ffgpu_rsi16 *code, const uint16_t *msg, size_t nblocks, size_t interleave,
                                   uint16_t *parity, void *stream);
/* unknown-location repair of nblocks blocks in place, W = 1 semantics
 * (RSi16v::_repair, rsi16v_impl.hpp:122-168, as PyRSi16::py_repair,
 * pyrsi16.hpp:588-631); status[i] is a RepairStatus or FFGPU_STATUS_ASSERT */
FFGPU_API int ffgpu_rsi16_repair(const ffgpu_rsi16 *code, uint16_t *msg, uint16_t *parity, size_t nblocks, uint8_t *status,
                       void *stream);
/* interleaved repair (PyRSi16::repair_interleaved, pyrsi16.hpp:160-176, with
 * W = 1 semantics): one interleaved block; error_pos == NULL selects unknown
 * locations.  *status receives the max over columns. */
FFGPU_API int ffgpu_rsi16_repair_interleaved(const ffgpu_rsi16 *code, uint16_t *msg, uint16_t *parity, size_t interleave,
                                   const uint32_t *error_pos, size_t error_count, uint8_t *status, void *stream);
/* known-location repair of nblocks blocks sharing one error position list
 * (RSi16v::_repair with positions, rsi16v_impl.hpp:171-231) */
FFGPU_API int ffgpu_rsi16_repair_known(const ffgpu_rsi16 *code, uint16_t *msg, uint16_t *parity, size_t nblocks,
                             const uint32_t *error_pos, size_t error_count, uint8_t *status, void *stream);
/* syndromes, ecc_len uint32 words per block (PyRSi16::py_synd, pyrsi16.hpp:633-651) */
FFGPU_API int ffgpu_rsi16_synd(const ffgpu_rsi16 *code, const uint16_t *msg, const uint16_t *parity, size_t nblocks,
                     uint32_t *synds, void *stream);
/* Sugiyama on nblocks syndrome vectors (PyRSi16::py_sugiyama<1>, pyrsi16.hpp:653-674) */
FFGPU_API int ffgpu_rsi16_sugiyama(const ffgpu_rsi16 *code, const uint32_t *synds, size_t nblocks, uint32_t *locator,
                         uint32_t *evaluator, uint8_t *status, void *stream);
/* zeros of pintt_ecc(poly) (PyRSi16::py_roots, pyrsi16.hpp:676-691): out
 * receives block_len flags (1 = zero) */
FFGPU_API int ffgpu_rsi16_roots(const ffgpu_rsi16 *code, const uint32_t *poly, uint8_t *is_zero, void *stream);

FFGPU_API int ffgpu_rsi16_encode_host(const ffgpu_rsi16 *code, const uint16_t *msg, size_t nblocks, size_t interleave,
                            uint16_t *parity);
FFGPU_API int ffgpu_rsi16_synd_host(const ffgpu_rsi16 *code, const uint16_t *msg, const uint16_t *parity,
                                    size_t nblocks, uint32_t *synds);
FFGPU_API int ffgpu_rsi16_sugiyama_host(const ffgpu_rsi16 *code, const uint32_t *synds, size_t nblocks,
                                       uint32_t *locator, uint32_t *evaluator, uint8_t *status);
FFGPU_API int ffgpu_rsi16_roots_host(const ffgpu_rsi16 *code, const uint32_t *poly, uint8_t *is_zero);
FFGPU_API int ffgpu_rsi16_repair_host(const ffgpu_rsi16 *code, uint16_t *msg, uint16_t *parity, size_t nblocks,
                            size_t interleave, const uint32_t *error_pos, long error_count, uint8_t *status);

/* ---------------------------------------------------------------- CIRC16 */
/* PyCIRC16 ctor (libffrs/pycirc16.hpp:46-65) */
FFGPU_API int ffgpu_circ16_create(size_t inner_block_len, size_t inner_ecc_len, size_t outer_block_len, size_t outer_ecc_len,
                        size_t interleave, uint32_t primitive, ffgpu_circ16 **out);
FFGPU_API int ffgpu_circ16_destroy(ffgpu_circ16 *code);
/* message_len, ecc_len of one CIRC16 block in uint16 words */
FFGPU_API int ffgpu_circ16_info(const ffgpu_circ16 *code, size_t *message_len, size_t *ecc_len);
/* nblocks CIRC16 blocks: [rso_ecc | rsi_ecc | rsio_ecc] per block
 * (PyCIRC16::py_encode / encode_block, pycirc16.hpp:337-363) */
FFGPU_API int ffgpu_circ16_encode(const ffgpu_circ16 *code, const uint16_t *msg, size_t nblocks, uint16_t *ecc, void *stream);
/* in-place repair of one CIRC16 block (CircRepair, pycirc16.hpp:135-335,
 * PyCIRC16::py_repair :365-384); *assert_fail is set when the reference
 * would raise RuntimeError */
FFGPU_API int ffgpu_circ16_repair(const ffgpu_circ16 *code, uint16_t *msg, uint16_t *ecc, size_t nblocks, uint8_t *status,
                        void *stream);
/* outer error rows of interleave k after the zero heuristics
 * (PyCIRC16::py_find_outer_error_locations, pycirc16.hpp:386-405); flags has
 * outer_block_len entries */
FFGPU_API int ffgpu_circ16_find_outer_error_locations(const ffgpu_circ16 *code, const uint16_t *msg, const uint16_t *ecc,
                                            size_t k, uint8_t *flags, void *stream);

FFGPU_API int ffgpu_circ16_encode_host(const ffgpu_circ16 *code, const uint16_t *msg, size_t nblocks, uint16_t *ecc);
/* rows (outer_block_len capacity) receives the outer error rows of group k */
FFGPU_API int ffgpu_circ16_find_outer_error_locations_host(const ffgpu_circ16 *code, const uint16_t *msg,
                                                           const uint16_t *ecc, size_t k, uint32_t *rows,
                                                           size_t *count);
FFGPU_API int ffgpu_circ16_repair_host(const ffgpu_circ16 *code, uint16_t *msg, uint16_t *ecc, size_t nblocks, uint8_t *status);

/* ---------------------------------------------------------------- batch */
/* No reference counterpart.  A batch collects requests of any mix of codes,
 * geometries and directions (device buffers, laid out as for the per-code
 * entry points above) and serves all of them in one launch sequence: the
 * CIRC16 requests gathered per code and direction through the staged
 * encode / repair on a high-priority stream, beside one persistent kernel per
 * item class (RS256 by remainder width, RSi16) on forked streams.  The sequence can
 * be captured into a CUDA graph and replayed.  Results are byte-identical to
 * calling the per-code entry point once per request.  A batch holds pointers:
 * the buffers must stay valid while it is planned, captured and launched. */
typedef struct ffgpu_batch ffgpu_batch;
#define FFGPU_OP_ENCODE 0
#define FFGPU_OP_DECODE 1
FFGPU_API int ffgpu_batch_create(ffgpu_batch **out);
FFGPU_API int ffgpu_batch_destroy(ffgpu_batch *batch);
FFGPU_API int ffgpu_batch_clear(ffgpu_batch *batch);
/* RS256: ENCODE writes parity (ffgpu_rs256_encode); DECODE repairs in place
 * and writes one status byte per block (ffgpu_rs256_decode) */
FFGPU_API int ffgpu_batch_add_rs256(ffgpu_batch *batch, const ffgpu_rs256 *code, int op, uint8_t *data,
                                    uint8_t *parity, size_t nblocks, size_t message_len, uint8_t *status);
/* RSi16: as ffgpu_rsi16_encode / ffgpu_rsi16_repair */
FFGPU_API int ffgpu_batch_add_rsi16(ffgpu_batch *batch, const ffgpu_rsi16 *code, int op, uint16_t *msg,
                                    uint16_t *parity, size_t nblocks, uint8_t *status);
/* CIRC16: as ffgpu_circ16_encode / ffgpu_circ16_repair (status 0 or 0xFF
 * per codeword) */
FFGPU_API int ffgpu_batch_add_circ16(ffgpu_batch *batch, const ffgpu_circ16 *code, int op, uint16_t *msg,
                                     uint16_t *ecc, size_t nblocks, uint8_t *status);
/* cut the requests into work items (longest first) and upload them; with
 * autotune != 0, candidate schedules (RS256 blocks per item, RSi16 blocks per
 * item, CTAs per SM) are timed on the batch itself -- decode buffers are saved
 * and restored around every trial -- and the fastest is kept */
FFGPU_API int ffgpu_batch_plan(ffgpu_batch *batch, int autotune, void *stream);
/* capture the launch sequence into a CUDA graph (later launches replay it) */
FFGPU_API int ffgpu_batch_capture(ffgpu_batch *batch, void *stream);
/* serve every request: the launch sequence, or one graph replay */
FFGPU_API int ffgpu_batch_launch(ffgpu_batch *batch, void *stream);
FFGPU_API int ffgpu_batch_info(const ffgpu_batch *batch, int *tile_rs256, int *tile_rsi16, int *ctas_per_sm,
                               size_t *items, unsigned *grid);

/* ---------------------------------------------------------------- serving */
/* No reference counterpart.  A server accepts requests on HOST buffers from
 * any thread (same layouts and in-place semantics as the *_host entry
 * points; page-locked memory from ffgpu_host_alloc copies fastest) and
 * completes them asynchronously: a scheduler thread admits queued requests
 * into one of `slots` CUDA streams while their device buffers fit in the HBM
 * budget (0: 80% of the free memory), serves every request admitted together
 * with one fused batch launch between its copies, and retires slots as they
 * finish, so requests that arrive while others run overlap with them.  Results
 * are byte-identical to serving each request alone. */
typedef struct ffgpu_server ffgpu_server;
FFGPU_API int ffgpu_server_create(size_t hbm_budget, int slots, int max_batch, ffgpu_server **out);
/* waits for every submitted request, then frees the server */
FFGPU_API int ffgpu_server_destroy(ffgpu_server *server);
FFGPU_API int ffgpu_server_submit_rs256(ffgpu_server *server, const ffgpu_rs256 *code, int op, uint8_t *data,
                                        uint8_t *parity, size_t nblocks, size_t message_len, uint8_t *status,
                                        uint64_t *ticket);
FFGPU_API int ffgpu_server_submit_rsi16(ffgpu_server *server, const ffgpu_rsi16 *code, int op, uint16_t *msg,
                                        uint16_t *parity, size_t nblocks, uint8_t *status, uint64_t *ticket);
FFGPU_API int ffgpu_server_submit_circ16(ffgpu_server *server, const ffgpu_circ16 *code, int op, uint16_t *msg,
                                         uint16_t *ecc, size_t nblocks, uint8_t *status, uint64_t *ticket);
/* state: 0 queued, 1 running, 2 done, 3 failed, 4 cancelled; times are
 * seconds since the server was created (submitted, admitted into a slot,
 * completion seen) */
FFGPU_API int ffgpu_server_poll(ffgpu_server *server, uint64_t ticket, int *state, double *t_submit,
                                double *t_start, double *t_done);
/* block until the request is done; timeout_s < 0 waits without limit.  A
 * failed request returns its error (FFGPU_ENOMEM when its device buffers
 * could not be allocated), a cancelled one FFGPU_ECANCELLED. */
FFGPU_API int ffgpu_server_wait(ffgpu_server *server, uint64_t ticket, double timeout_s);
/* forget a finished (done, failed or cancelled) request */
FFGPU_API int ffgpu_server_release(ffgpu_server *server, uint64_t ticket);
/* withdraw a request that is still queued (state 0): it becomes state 4 and
 * its buffers are never touched; ffgpu_server_wait on it returns
 * FFGPU_ECANCELLED.  A request already admitted (state >= 1) is not
 * withdrawn: FFGPU_EINVAL. */
FFGPU_API int ffgpu_server_cancel(ffgpu_server *server, uint64_t ticket);
/* Test hook for the failure path, no device involved: the next n slot
 * allocations of any server report out-of-memory (FFGPU_ENOMEM) as a failed
 * cudaMallocAsync would; their requests fail, the server keeps serving. */
FFGPU_API int ffgpu_server_debug_fail_allocs(int n);

#ifdef __cplusplus
}
#endif
#endif
