// C ABI: RSi16 entry points.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "handles.h"
#include "rsi16.cuh"

using namespace ffgpu;


// NULL is the CUDA default stream, as everywhere in the CUDA runtime
static cudaStream_t pick(void *stream) { return (cudaStream_t)stream; }

static void check_positions(const Rsi16Code &c, const uint32_t *pos, size_t count) {
    // py_repair asserts error_pos.size() <= ecc_len (pyrsi16.hpp:605, 623); a
    // position must address a word of the block
    if (count > c.ecc) throw Error(FFGPU_EASSERT, "Assertion failed: error_pos->size() <= ecc_len");
    for (size_t i = 0; i < count; ++i)
        FFGPU_REQUIRE(pos[i] < c.block_len, "error position out of range: " + std::to_string(pos[i]));
}

extern "C" {

int ffgpu_rsi16_create(size_t block_len, size_t ecc_len, uint32_t primitive, ffgpu_rsi16 **out) {
    return guarded([&] {
        FFGPU_REQUIRE(out, "out is NULL");
        lib_stream();
        auto h = std::make_unique<ffgpu_rsi16>();
        h->code = std::make_unique<Rsi16Code>(block_len, ecc_len, primitive);
        *out = h.release();
    });
}

int ffgpu_rsi16_destroy(ffgpu_rsi16 *code) {
    return guarded([&] { delete code; });
}

int ffgpu_rsi16_info(const ffgpu_rsi16 *code, uint32_t *root, size_t *ntt_len) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        if (root) *root = code->code->root;
        if (ntt_len) *ntt_len = code->code->ntt_len;
    });
}

int ffgpu_rsi16_repair_counters(uint64_t *fast_blocks, uint64_t *mirror_blocks, int reset) {
    return guarded([&] { rsi16_repair_counters(fast_blocks, mirror_blocks, reset != 0); });
}

int ffgpu_rsi16_encode(const ffgpu_rsi16 *code, const uint16_t *msg, size_t nblocks, uint16_t *parity, void *stream) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        const Rsi16Code &c = *code->code;
        rsi16_encode(c, contiguous_view((void *)msg, true, c.message_len, parity, true, c.ecc), nblocks, pick(stream));
    });
}

int ffgpu_rsi16_encode_interleaved(const ffgpu_rsi16 *code, const uint16_t *msg, size_t nblocks, size_t interleave,
                                   uint16_t *parity, void *stream) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        FFGPU_REQUIRE(interleave >= 1, "interleave must be positive");
        const Rsi16Code &c = *code->code;
        rsi16_encode(c, interleaved_view((void *)msg, true, c.message_len, parity, true, c.ecc, interleave),
                     nblocks * interleave, pick(stream));
    });
}

int ffgpu_rsi16_repair(const ffgpu_rsi16 *code, uint16_t *msg, uint16_t *parity, size_t nblocks, uint8_t *status,
                       void *stream) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        const Rsi16Code &c = *code->code;
        rsi16_repair(c, contiguous_view(msg, true, c.message_len, parity, true, c.ecc), nblocks, status, pick(stream));
    });
}

int ffgpu_rsi16_repair_known(const ffgpu_rsi16 *code, uint16_t *msg, uint16_t *parity, size_t nblocks,
                             const uint32_t *error_pos, size_t error_count, uint8_t *status, void *stream) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        const Rsi16Code &c = *code->code;
        rsi16_repair_known(c, contiguous_view(msg, true, c.message_len, parity, true, c.ecc), nblocks, error_pos,
                           nullptr, nullptr, (uint32_t)error_count, nullptr, status, pick(stream));
    });
}

int ffgpu_rsi16_repair_interleaved(const ffgpu_rsi16 *code, uint16_t *msg, uint16_t *parity, size_t interleave,
                                   const uint32_t *error_pos, size_t error_count, uint8_t *status, void *stream) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        const Rsi16Code &c = *code->code;
        BlockView v = interleaved_view(msg, true, c.message_len, parity, true, c.ecc, interleave);
        if (error_pos)
            rsi16_repair_known(c, v, interleave, error_pos, nullptr, nullptr, (uint32_t)error_count, nullptr, status,
                               pick(stream));
        else
            rsi16_repair(c, v, interleave, status, pick(stream));
    });
}

int ffgpu_rsi16_synd(const ffgpu_rsi16 *code, const uint16_t *msg, const uint16_t *parity, size_t nblocks,
                     uint32_t *synds, void *stream) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        const Rsi16Code &c = *code->code;
        rsi16_synd(c, contiguous_view((void *)msg, true, c.message_len, (void *)parity, true, c.ecc), nblocks, synds,
                   pick(stream));
    });
}

int ffgpu_rsi16_sugiyama(const ffgpu_rsi16 *code, const uint32_t *synds, size_t nblocks, uint32_t *locator,
                         uint32_t *evaluator, uint8_t *status, void *stream) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        rsi16_sugiyama(*code->code, synds, nblocks, locator, evaluator, status, pick(stream));
    });
}

int ffgpu_rsi16_roots(const ffgpu_rsi16 *code, const uint32_t *poly, uint8_t *is_zero, void *stream) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        rsi16_roots(*code->code, poly, is_zero, pick(stream));
    });
}

// RSi16.encode(buffer) (pyrsi16.hpp:568-586): nblocks interleaved blocks of
// message_len * interleave words -> nblocks * ecc_len * interleave words.
int ffgpu_rsi16_encode_host(const ffgpu_rsi16 *code, const uint16_t *msg, size_t nblocks, size_t interleave,
                            uint16_t *parity) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        FFGPU_REQUIRE(interleave >= 1, "interleave must be positive");
        ffgpu_rsi16 *h = const_cast<ffgpu_rsi16 *>(code);
        const Rsi16Code &c = *h->code;
        if (!nblocks) return;
        std::lock_guard<std::mutex> lk(h->mu);
        cudaStream_t st = lib_stream();
        const size_t nm = nblocks * interleave * c.message_len, np = nblocks * interleave * c.ecc;
        uint16_t *dm = (uint16_t *)h->d_msg.get(nm * 2);
        uint16_t *dp = (uint16_t *)h->d_par.get(np * 2);
        if (interleave == 1) {
            // chunks of blocks on the pipeline streams: copies in, encodes and
            // copies out of different chunks overlap
            const size_t chunk = host_chunk_blocks(nblocks, 8192, 16);
            uint16_t *hp = pipeline_out(parity, chunk < nblocks, h->h_par, np * 2);
            OutputDrain drain;
            HostPipeline pl;
            size_t k = 0;
            for (size_t b0 = 0; b0 < nblocks; b0 += chunk, ++k) {
                const size_t n = std::min(chunk, nblocks - b0);
                uint16_t *cm = dm + b0 * c.message_len, *cp = dp + b0 * c.ecc;
                const size_t om = b0 * c.message_len;
                FFGPU_CHECK_CUDA(
                    cudaMemcpyAsync(cm, msg + om, n * c.message_len * 2, cudaMemcpyHostToDevice, pl.up()));
                cudaStream_t ps = pl.compute(k);
                rsi16_encode(c, contiguous_view(cm, true, c.message_len, cp, true, c.ecc), n, ps);
                ps = pl.to_down(k);
                FFGPU_CHECK_CUDA(cudaMemcpyAsync(hp + b0 * c.ecc, cp, n * c.ecc * 2, cudaMemcpyDeviceToHost, ps));
                drain.copy(parity + b0 * c.ecc, hp + b0 * c.ecc, n * c.ecc * 2);
                drain.chunk(ps);
            }
            drain.finish();
            pl.sync();
            return;
        }
        FFGPU_CHECK_CUDA(cudaMemcpyAsync(dm, msg, nm * 2, cudaMemcpyHostToDevice, st));
        if (interleave == 1)
            rsi16_encode(c, contiguous_view(dm, true, c.message_len, dp, true, c.ecc), nblocks, st);
        else
            rsi16_encode(c, interleaved_view(dm, true, c.message_len, dp, true, c.ecc, interleave),
                         nblocks * interleave, st);
        FFGPU_CHECK_CUDA(cudaMemcpyAsync(parity, dp, np * 2, cudaMemcpyDeviceToHost, st));
        FFGPU_CHECK_CUDA(cudaStreamSynchronize(st));
    });
}

// RSi16.repair (pyrsi16.hpp:588-631) for nblocks blocks (interleave == 1) or
// one interleaved block; error_count < 0 selects unknown locations.  status
// receives one value per block (interleave == 1) or the maximum over the
// columns (interleave > 1), as RepairStatus; FFGPU_STATUS_ASSERT marks a
// block for which the reference raises RuntimeError.
int ffgpu_rsi16_repair_host(const ffgpu_rsi16 *code, uint16_t *msg, uint16_t *parity, size_t nblocks,
                            size_t interleave, const uint32_t *error_pos, long error_count, uint8_t *status) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        FFGPU_REQUIRE(interleave >= 1, "interleave must be positive");
        FFGPU_REQUIRE(interleave == 1 || nblocks == 1, "interleaved repair takes one interleaved block");
        ffgpu_rsi16 *h = const_cast<ffgpu_rsi16 *>(code);
        const Rsi16Code &c = *h->code;
        if (!nblocks) return;
        if (error_count >= 0) check_positions(c, error_pos, (size_t)error_count);
        std::lock_guard<std::mutex> lk(h->mu);
        cudaStream_t st = lib_stream();
        const size_t ncol = nblocks * interleave;
        const size_t nm = ncol * c.message_len, np = ncol * c.ecc;
        uint16_t *dm = (uint16_t *)h->d_msg.get(nm * 2);
        uint16_t *dp = (uint16_t *)h->d_par.get(np * 2);
        uint8_t *ds = (uint8_t *)h->d_status.get(ncol);
        if (interleave == 1 && error_count < 0) {
            // contiguous blocks, unknown locations: every block is written back
            // whatever its status, so chunks of blocks pipeline their copies and
            // repairs over the pipeline streams
            const size_t chunk = host_chunk_blocks(nblocks, 32768, 8);
            // outputs in pageable memory come back through page-locked staging
            const bool chunked = chunk < nblocks;
            uint16_t *h_m = pipeline_out(msg, chunked, h->h_msg, nm * 2);
            uint16_t *h_p = pipeline_out(parity, chunked, h->h_par, np * 2);
            uint8_t *h_s = pipeline_out(status, chunked, h->h_status, nblocks);
            OutputDrain drain;
            HostPipeline pl;
            size_t k = 0;
            for (size_t b0 = 0; b0 < nblocks; b0 += chunk, ++k) {
                const size_t n = std::min(chunk, nblocks - b0);
                const size_t om = b0 * c.message_len, op = b0 * c.ecc;
                uint16_t *cm = dm + om, *cp = dp + op;
                FFGPU_CHECK_CUDA(
                    cudaMemcpyAsync(cm, msg + om, n * c.message_len * 2, cudaMemcpyHostToDevice, pl.up()));
                FFGPU_CHECK_CUDA(cudaMemcpyAsync(cp, parity + op, n * c.ecc * 2, cudaMemcpyHostToDevice, pl.up()));
                cudaStream_t ps = pl.compute(k);
                rsi16_repair(c, contiguous_view(cm, true, c.message_len, cp, true, c.ecc), n, ds + b0, ps);
                ps = pl.to_down(k);
                FFGPU_CHECK_CUDA(cudaMemcpyAsync(h_m + om, cm, n * c.message_len * 2, cudaMemcpyDeviceToHost, ps));
                FFGPU_CHECK_CUDA(cudaMemcpyAsync(h_p + op, cp, n * c.ecc * 2, cudaMemcpyDeviceToHost, ps));
                FFGPU_CHECK_CUDA(cudaMemcpyAsync(h_s + b0, ds + b0, n, cudaMemcpyDeviceToHost, ps));
                drain.copy(msg + om, h_m + om, n * c.message_len * 2);
                drain.copy(parity + op, h_p + op, n * c.ecc * 2);
                drain.copy(status + b0, h_s + b0, n);
                drain.chunk(ps);
            }
            drain.finish();
            pl.sync();
            return;
        }
        FFGPU_CHECK_CUDA(cudaMemcpyAsync(dm, msg, nm * 2, cudaMemcpyHostToDevice, st));
        FFGPU_CHECK_CUDA(cudaMemcpyAsync(dp, parity, np * 2, cudaMemcpyHostToDevice, st));
        BlockView v = interleave == 1 ? contiguous_view(dm, true, c.message_len, dp, true, c.ecc)
                                      : interleaved_view(dm, true, c.message_len, dp, true, c.ecc, interleave);
        if (error_count >= 0) {
            uint32_t *dpos = (uint32_t *)h->d_pos.get((size_t)error_count * 4 + 4);
            if (error_count)
                FFGPU_CHECK_CUDA(cudaMemcpyAsync(dpos, error_pos, (size_t)error_count * 4, cudaMemcpyHostToDevice, st));
            rsi16_repair_known(c, v, ncol, dpos, nullptr, nullptr, (uint32_t)error_count, nullptr, ds, st);
        } else {
            rsi16_repair(c, v, ncol, ds, st);
        }
        std::vector<uint8_t> s(ncol);
        FFGPU_CHECK_CUDA(cudaMemcpyAsync(s.data(), ds, ncol, cudaMemcpyDeviceToHost, st));
        FFGPU_CHECK_CUDA(cudaStreamSynchronize(st));
        size_t first_assert = ncol;
        if (interleave > 1)
            for (size_t j = 0; j < ncol; ++j)
                if (s[j] == FFGPU_STATUS_ASSERT) {
                    first_assert = j;
                    break;
                }
        if (first_assert == ncol) {
            FFGPU_CHECK_CUDA(cudaMemcpyAsync(msg, dm, nm * 2, cudaMemcpyDeviceToHost, st));
            FFGPU_CHECK_CUDA(cudaMemcpyAsync(parity, dp, np * 2, cudaMemcpyDeviceToHost, st));
            FFGPU_CHECK_CUDA(cudaStreamSynchronize(st));
        } else {
            // the reference's column loop (pyrsi16.hpp:410-429) stops at the
            // raising column: only the columns before it are written back
            std::vector<uint16_t> hm(nm), hp(np);
            FFGPU_CHECK_CUDA(cudaMemcpyAsync(hm.data(), dm, nm * 2, cudaMemcpyDeviceToHost, st));
            FFGPU_CHECK_CUDA(cudaMemcpyAsync(hp.data(), dp, np * 2, cudaMemcpyDeviceToHost, st));
            FFGPU_CHECK_CUDA(cudaStreamSynchronize(st));
            for (size_t k = 0; k < c.message_len; ++k)
                for (size_t j = 0; j < first_assert; ++j) msg[k * interleave + j] = hm[k * interleave + j];
            for (size_t k = 0; k < c.ecc; ++k)
                for (size_t j = 0; j < first_assert; ++j) parity[k * interleave + j] = hp[k * interleave + j];
        }
        if (interleave == 1) {
            std::memcpy(status, s.data(), ncol);
        } else {
            uint8_t m = 0;
            for (uint8_t x : s) {
                if (x == FFGPU_STATUS_ASSERT) {
                    m = FFGPU_STATUS_ASSERT;
                    break;
                }
                m = std::max(m, x);
            }
            status[0] = m;
        }
    });
}

int ffgpu_rsi16_synd_host(const ffgpu_rsi16 *code, const uint16_t *msg, const uint16_t *parity, size_t nblocks,
                          uint32_t *synds) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        ffgpu_rsi16 *h = const_cast<ffgpu_rsi16 *>(code);
        const Rsi16Code &c = *h->code;
        if (!nblocks) return;
        std::lock_guard<std::mutex> lk(h->mu);
        cudaStream_t st = lib_stream();
        const size_t nm = nblocks * c.message_len, np = nblocks * c.ecc;
        uint16_t *dm = (uint16_t *)h->d_msg.get(nm * 2);
        uint16_t *dp = (uint16_t *)h->d_par.get(np * 2);
        uint32_t *ds = (uint32_t *)h->d_pos.get(np * 4);
        FFGPU_CHECK_CUDA(cudaMemcpyAsync(dm, msg, nm * 2, cudaMemcpyHostToDevice, st));
        FFGPU_CHECK_CUDA(cudaMemcpyAsync(dp, parity, np * 2, cudaMemcpyHostToDevice, st));
        rsi16_synd(c, contiguous_view(dm, true, c.message_len, dp, true, c.ecc), nblocks, ds, st);
        FFGPU_CHECK_CUDA(cudaMemcpyAsync(synds, ds, np * 4, cudaMemcpyDeviceToHost, st));
        FFGPU_CHECK_CUDA(cudaStreamSynchronize(st));
    });
}

int ffgpu_rsi16_sugiyama_host(const ffgpu_rsi16 *code, const uint32_t *synds, size_t nblocks, uint32_t *locator,
                              uint32_t *evaluator, uint8_t *status) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        ffgpu_rsi16 *h = const_cast<ffgpu_rsi16 *>(code);
        const Rsi16Code &c = *h->code;
        if (!nblocks) return;
        std::lock_guard<std::mutex> lk(h->mu);
        cudaStream_t st = lib_stream();
        const size_t n = nblocks * c.ecc;
        uint32_t *buf = (uint32_t *)h->d_pos.get(n * 12 + nblocks);
        FFGPU_CHECK_CUDA(cudaMemcpyAsync(buf, synds, n * 4, cudaMemcpyHostToDevice, st));
        uint8_t *ds = (uint8_t *)(buf + 3 * n);
        rsi16_sugiyama(c, buf, nblocks, buf + n, buf + 2 * n, ds, st);
        FFGPU_CHECK_CUDA(cudaMemcpyAsync(locator, buf + n, n * 4, cudaMemcpyDeviceToHost, st));
        FFGPU_CHECK_CUDA(cudaMemcpyAsync(evaluator, buf + 2 * n, n * 4, cudaMemcpyDeviceToHost, st));
        FFGPU_CHECK_CUDA(cudaMemcpyAsync(status, ds, nblocks, cudaMemcpyDeviceToHost, st));
        FFGPU_CHECK_CUDA(cudaStreamSynchronize(st));
    });
}

int ffgpu_rsi16_roots_host(const ffgpu_rsi16 *code, const uint32_t *poly, uint8_t *is_zero) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        ffgpu_rsi16 *h = const_cast<ffgpu_rsi16 *>(code);
        const Rsi16Code &c = *h->code;
        std::lock_guard<std::mutex> lk(h->mu);
        cudaStream_t st = lib_stream();
        uint32_t *dp = (uint32_t *)h->d_pos.get(c.ecc * 4 + c.block_len + 64);
        uint8_t *dz = (uint8_t *)(dp + c.ecc);
        FFGPU_CHECK_CUDA(cudaMemcpyAsync(dp, poly, c.ecc * 4, cudaMemcpyHostToDevice, st));
        rsi16_roots(c, dp, dz, st);
        FFGPU_CHECK_CUDA(cudaMemcpyAsync(is_zero, dz, c.block_len, cudaMemcpyDeviceToHost, st));
        FFGPU_CHECK_CUDA(cudaStreamSynchronize(st));
    });
}

}  // extern "C"
