// C ABI: CIRC16 entry points.
#include <cuda_runtime.h>

#include <cstring>
#include <memory>
#include <mutex>
#include <vector>

#include "circ16.cuh"
#include "common.cuh"
#include "handles.h"

using namespace ffgpu;


// NULL is the CUDA default stream, as everywhere in the CUDA runtime
static cudaStream_t pick(void *stream) { return (cudaStream_t)stream; }

extern "C" {

int ffgpu_circ16_create(size_t inner_block_len, size_t inner_ecc_len, size_t outer_block_len, size_t outer_ecc_len,
                        size_t interleave, uint32_t primitive, ffgpu_circ16 **out) {
    return guarded([&] {
        FFGPU_REQUIRE(out, "out is NULL");
        lib_stream();
        auto h = std::make_unique<ffgpu_circ16>();
        h->code = std::make_unique<Circ16Code>(inner_block_len, inner_ecc_len, outer_block_len, outer_ecc_len,
                                               interleave, primitive);
        *out = h.release();
    });
}

int ffgpu_circ16_destroy(ffgpu_circ16 *code) {
    return guarded([&] { delete code; });
}

int ffgpu_circ16_info(const ffgpu_circ16 *code, size_t *message_len, size_t *ecc_len) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        if (message_len) *message_len = code->code->message_len;
        if (ecc_len) *ecc_len = code->code->ecc_len;
    });
}

int ffgpu_circ16_encode(const ffgpu_circ16 *code, const uint16_t *msg, size_t nblocks, uint16_t *ecc, void *stream) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        ffgpu_circ16 *h = const_cast<ffgpu_circ16 *>(code);
        std::lock_guard<std::mutex> lk(h->mu);
        circ16_encode(*h->code, msg, nblocks, ecc, pick(stream));
    });
}

// status[i]: 0 when block i was repaired as the reference does (which always
// returns False), FFGPU_STATUS_ASSERT when the reference raises RuntimeError
// for it (its message is then left as the reference leaves it and its ecc is
// not written back).
int ffgpu_circ16_repair(const ffgpu_circ16 *code, uint16_t *msg, uint16_t *ecc, size_t nblocks, uint8_t *status,
                        void *stream) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        ffgpu_circ16 *h = const_cast<ffgpu_circ16 *>(code);
        std::lock_guard<std::mutex> lk(h->mu);
        // every repair stage as one launch over all codewords
        circ16_repair_many(*h->code, msg, ecc, nblocks, status, pick(stream));
    });
}

int ffgpu_circ16_find_outer_error_locations(const ffgpu_circ16 *code, const uint16_t *msg, const uint16_t *ecc,
                                            size_t k, uint8_t *flags, void *stream) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        ffgpu_circ16 *h = const_cast<ffgpu_circ16 *>(code);
        std::lock_guard<std::mutex> lk(h->mu);
        Circ16Code &c = *h->code;
        FFGPU_REQUIRE(k < c.interleave, "interleave index out of range");
        cudaStream_t st = pick(stream);
        std::vector<uint32_t> locs(c.rso->block_len);
        uint32_t n = 0;
        circ16_repair_one(c, const_cast<uint16_t *>(msg), const_cast<uint16_t *>(ecc), st, true, k, locs.data(), &n,
                          nullptr);
        FFGPU_CHECK_CUDA(cudaStreamSynchronize(st));
        std::vector<uint8_t> f(c.rso->block_len, 0);
        for (uint32_t i = 0; i < n; ++i) f[locs[i]] = 1;
        FFGPU_CHECK_CUDA(cudaMemcpy(flags, f.data(), f.size(), cudaMemcpyHostToDevice));
    });
}

int ffgpu_circ16_encode_host(const ffgpu_circ16 *code, const uint16_t *msg, size_t nblocks, uint16_t *ecc) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        ffgpu_circ16 *h = const_cast<ffgpu_circ16 *>(code);
        std::lock_guard<std::mutex> lk(h->mu);
        Circ16Code &c = *h->code;
        if (!nblocks) return;
        cudaStream_t st = lib_stream();
        uint16_t *dm = (uint16_t *)h->d_msg.get(nblocks * c.message_len * 2);
        uint16_t *de = (uint16_t *)h->d_ecc.get(nblocks * c.ecc_len * 2);
        FFGPU_CHECK_CUDA(cudaMemcpyAsync(dm, msg, nblocks * c.message_len * 2, cudaMemcpyHostToDevice, st));
        circ16_encode(c, dm, nblocks, de, st);
        FFGPU_CHECK_CUDA(cudaMemcpyAsync(ecc, de, nblocks * c.ecc_len * 2, cudaMemcpyDeviceToHost, st));
        FFGPU_CHECK_CUDA(cudaStreamSynchronize(st));
    });
}

int ffgpu_circ16_find_outer_error_locations_host(const ffgpu_circ16 *code, const uint16_t *msg, const uint16_t *ecc,
                                                 size_t k, uint32_t *rows, size_t *count) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        ffgpu_circ16 *h = const_cast<ffgpu_circ16 *>(code);
        std::lock_guard<std::mutex> lk(h->mu);
        Circ16Code &c = *h->code;
        if (k >= c.interleave) throw Error(FFGPU_EASSERT, "Assertion failed: interleave < this->interleave");
        cudaStream_t st = lib_stream();
        uint16_t *dm = (uint16_t *)h->d_msg.get(c.message_len * 2 * 2);
        uint16_t *de = (uint16_t *)h->d_ecc.get(c.ecc_len * 2);
        FFGPU_CHECK_CUDA(cudaMemcpyAsync(dm, msg, c.message_len * 2, cudaMemcpyHostToDevice, st));
        FFGPU_CHECK_CUDA(cudaMemcpyAsync(de, ecc, c.ecc_len * 2, cudaMemcpyHostToDevice, st));
        uint32_t n = 0;
        circ16_repair_one(c, dm, de, st, true, k, rows, &n, nullptr);
        FFGPU_CHECK_CUDA(cudaStreamSynchronize(st));
        *count = n;
    });
}

int ffgpu_circ16_repair_host(const ffgpu_circ16 *code, uint16_t *msg, uint16_t *ecc, size_t nblocks,
                             uint8_t *status) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        ffgpu_circ16 *h = const_cast<ffgpu_circ16 *>(code);
        std::lock_guard<std::mutex> lk(h->mu);
        Circ16Code &c = *h->code;
        if (!nblocks) return;
        cudaStream_t st = lib_stream();
        const size_t nm = nblocks * c.message_len * 2, ne = nblocks * c.ecc_len * 2;
        uint16_t *dm = (uint16_t *)h->d_msg.get(nm);
        uint16_t *de = (uint16_t *)h->d_ecc.get(ne);
        uint8_t *ds = (uint8_t *)h->d_status.get(nblocks);
        FFGPU_CHECK_CUDA(cudaMemcpyAsync(dm, msg, nm, cudaMemcpyHostToDevice, st));
        FFGPU_CHECK_CUDA(cudaMemcpyAsync(de, ecc, ne, cudaMemcpyHostToDevice, st));
        circ16_repair_many(c, dm, de, nblocks, ds, st);
        FFGPU_CHECK_CUDA(cudaMemcpyAsync(msg, dm, nm, cudaMemcpyDeviceToHost, st));
        FFGPU_CHECK_CUDA(cudaMemcpyAsync(ecc, de, ne, cudaMemcpyDeviceToHost, st));
        if (status) FFGPU_CHECK_CUDA(cudaMemcpyAsync(status, ds, nblocks, cudaMemcpyDeviceToHost, st));
        FFGPU_CHECK_CUDA(cudaStreamSynchronize(st));
    });
}

}  // extern "C"
