// C ABI: runtime helpers and the RS256 entry points.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <functional>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <sys/mman.h>
#include <unistd.h>

#include <cerrno>

#include "common.cuh"
#include "handles.h"
#include "rs256.cuh"

namespace ffgpu {

std::atomic<uint64_t> g_launches{0};
static thread_local std::string t_last_error;
void set_error(const std::string &msg) { t_last_error = msg; }

static std::mutex g_stream_mu;
static cudaStream_t g_stream = nullptr;
static int g_device = 0;

static std::atomic<size_t> g_chunk_blocks{0};

size_t host_chunk_blocks(size_t nblocks, size_t min_chunk, size_t max_chunks) {
    const size_t fixed = g_chunk_blocks.load();
    if (fixed) return fixed;
    return std::max<size_t>(min_chunk, (nblocks + max_chunks - 1) / max_chunks);
}

// ---- parallel host copies
namespace {
struct CopyPool {
    std::mutex mu;
    std::condition_variable cv;
    std::deque<std::function<void()>> q;
    unsigned workers = 0;
    explicit CopyPool(unsigned n) : workers(n) {
        for (unsigned i = 0; i < n; ++i)
            std::thread([this] {
                for (;;) {
                    std::function<void()> job;
                    {
                        std::unique_lock<std::mutex> lk(mu);
                        cv.wait(lk, [this] { return !q.empty(); });
                        job = std::move(q.front());
                        q.pop_front();
                    }
                    job();
                }
            }).detach();
    }
    void push(std::function<void()> f) {
        {
            std::lock_guard<std::mutex> lk(mu);
            q.push_back(std::move(f));
        }
        cv.notify_one();
    }
};

CopyPool &copy_pool() {
    // created on first use and never destroyed: its detached workers sleep
    // on the queue until the process exits
    static CopyPool *p = new CopyPool(std::max(1u, std::min(8u, std::thread::hardware_concurrency() / 2)));
    return *p;
}
}  // namespace

// Runs job(off, len) over [0, n) split into parts of at least min_part bytes
// (page multiples): the calling thread takes the first part, the copy pool
// the others; returns when every part is done.
static void split_run(size_t n, size_t min_part, const std::function<void(size_t, size_t)> &job) {
    CopyPool &pool = copy_pool();
    const size_t parts = std::max<size_t>(1, std::min<size_t>(n / min_part, pool.workers + 1));
    if (parts == 1) {
        job(0, n);
        return;
    }
    const size_t each = ((n + parts - 1) / parts + 4095) & ~(size_t)4095;
    std::mutex m;
    std::condition_variable done;
    size_t left = 0;
    for (size_t p = 1; p < parts && p * each < n; ++p) ++left;
    const size_t helpers = left;
    for (size_t p = 1; p <= helpers; ++p) {
        const size_t off = p * each, len = std::min(each, n - off);
        pool.push([&, off, len] {
            job(off, len);
            std::lock_guard<std::mutex> lk(m);
            if (--left == 0) done.notify_one();
        });
    }
    job(0, std::min(each, n));
    std::unique_lock<std::mutex> lk(m);
    done.wait(lk, [&] { return left == 0; });
}

void host_copy(void *dst, const void *src, size_t n) {
    split_run(n, 1u << 20, [&](size_t off, size_t len) { std::memcpy((char *)dst + off, (const char *)src + off, len); });
}

// Maps in the pages of [p, p + n) ahead of the copies into them: a fresh
// pageable output (a new bytearray) otherwise takes its page faults, and the
// kernel's zeroing of every page, inside the copies at the end of a host
// pipeline.  madvise(MADV_POPULATE_WRITE) faults the pages in writable
// without changing their contents (so outputs that alias inputs are safe), a
// part per pool thread; kernels without it (before Linux 5.14) skip this.
#ifndef MADV_POPULATE_WRITE
#define MADV_POPULATE_WRITE 23
#endif
static void host_prefault(void *p, size_t n) {
    static const size_t page = [] {
        const long v = sysconf(_SC_PAGESIZE);
        return v > 0 ? (size_t)v : (size_t)4096;
    }();
    static std::atomic<bool> unsupported{false};
    if (unsupported.load(std::memory_order_relaxed)) return;
    split_run(n, 2u << 20, [&](size_t off, size_t len) {
        const uintptr_t a = ((uintptr_t)p + off + page - 1) & ~(uintptr_t)(page - 1);
        const uintptr_t b = ((uintptr_t)p + off + len) & ~(uintptr_t)(page - 1);
        if (b > a && madvise((void *)a, b - a, MADV_POPULATE_WRITE) != 0 && errno == EINVAL)
            unsupported.store(true, std::memory_order_relaxed);
    });
}

// Ordering events of the host pipelines, reused across calls (creating and
// destroying a few dozen events per call costs more than the reuse)
namespace {
std::mutex g_sync_ev_mu;
std::vector<cudaEvent_t> g_sync_ev;
}  // namespace

static cudaEvent_t sync_event_get() {
    {
        std::lock_guard<std::mutex> lk(g_sync_ev_mu);
        if (!g_sync_ev.empty()) {
            cudaEvent_t e = g_sync_ev.back();
            g_sync_ev.pop_back();
            return e;
        }
    }
    cudaEvent_t e = nullptr;
    FFGPU_CHECK_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return e;
}

static void sync_event_put(cudaEvent_t e) {
    std::lock_guard<std::mutex> lk(g_sync_ev_mu);
    g_sync_ev.push_back(e);
}

OutputDrain::~OutputDrain() {
    for (auto &c : chunks_) sync_event_put(c.ev);
}

void OutputDrain::copy(void *dst, const void *src, size_t n) {
    if (dst != src && n) parts_.push_back({dst, src, n});
}

void OutputDrain::chunk(cudaStream_t st) {
    if (parts_.size() == open_) return;
    cudaEvent_t ev = sync_event_get();
    chunks_.push_back({ev, open_, parts_.size() - open_});
    FFGPU_CHECK_CUDA(cudaEventRecord(ev, st));
    open_ = parts_.size();
}

void OutputDrain::finish() {
    // the outputs' pages are mapped in (in parallel) while the GPU still
    // works on the chunks, before any chunk is copied out
    // (adjacent parts, such as one output's chunks, are merged first, so that
    // each output is one parallel pass)
    std::vector<std::pair<char *, size_t>> runs;
    for (auto &pt : parts_) runs.push_back({(char *)pt.dst, pt.n});
    std::sort(runs.begin(), runs.end());
    size_t w = 0;
    for (size_t i = 0; i < runs.size(); ++i) {
        if (w && runs[w - 1].first + runs[w - 1].second == runs[i].first)
            runs[w - 1].second += runs[i].second;
        else
            runs[w++] = runs[i];
    }
    runs.resize(w);
    for (auto &r : runs)
        if (r.second >= (1u << 20)) host_prefault(r.first, r.second);
    for (auto &c : chunks_) {
        FFGPU_CHECK_CUDA(cudaEventSynchronize(c.ev));
        for (size_t i = c.first; i < c.first + c.count; ++i) host_copy(parts_[i].dst, parts_[i].src, parts_[i].n);
    }
}

// streams of the host-buffer pipelines (created on first use): the compute
// streams, then the upload and the download stream
static cudaStream_t pipe_slot(size_t i) {
    static std::mutex mu;
    static cudaStream_t s[kPipeStreams + 2] = {};
    std::lock_guard<std::mutex> lk(mu);
    cudaStream_t &x = s[i];
    if (!x) FFGPU_CHECK_CUDA(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
    return x;
}
cudaStream_t pipe_stream(size_t k) { return pipe_slot(k % kPipeStreams); }
cudaStream_t pipe_up() { return pipe_slot(kPipeStreams); }
cudaStream_t pipe_down() { return pipe_slot(kPipeStreams + 1); }

HostPipeline::~HostPipeline() {
    for (cudaEvent_t e : evs_) sync_event_put(e);
}

cudaEvent_t HostPipeline::record(cudaStream_t s) {
    cudaEvent_t e = sync_event_get();
    evs_.push_back(e);
    FFGPU_CHECK_CUDA(cudaEventRecord(e, s));
    return e;
}

cudaStream_t HostPipeline::compute(size_t k) {
    cudaStream_t cs = pipe_stream(k);
    FFGPU_CHECK_CUDA(cudaStreamWaitEvent(cs, record(up()), 0));
    return cs;
}

cudaStream_t HostPipeline::to_down(size_t k) {
    FFGPU_CHECK_CUDA(cudaStreamWaitEvent(down(), record(pipe_stream(k)), 0));
    return down();
}

void HostPipeline::sync() { FFGPU_CHECK_CUDA(cudaStreamSynchronize(down())); }

// The library is bound to one device, the one ffgpu_init names (default 0):
// its stream, the pipeline streams and the code tables live there.  The
// caller's current device is left as it was.
cudaStream_t lib_stream() {
    std::lock_guard<std::mutex> lk(g_stream_mu);
    if (!g_stream) {
        int prev = 0;
        FFGPU_CHECK_CUDA(cudaGetDevice(&prev));
        FFGPU_CHECK_CUDA(cudaSetDevice(g_device));
        const cudaError_t e = cudaStreamCreateWithFlags(&g_stream, cudaStreamNonBlocking);
        cudaSetDevice(prev);
        FFGPU_CHECK_CUDA(e);
        // the per-call scratch comes from the stream-ordered pool; keep freed
        // blocks in the pool across synchronisations instead of unmapping them
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, g_device) == cudaSuccess) {
            uint64_t keep = ~0ull;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
    }
    return g_stream;
}

// ---- per-kernel timing
static std::atomic<bool> g_timing{false};
static std::mutex g_timing_mu;
static std::vector<cudaEvent_t> g_event_pool;
struct Timed {
    std::string name;
    cudaEvent_t start, stop;
};
static std::vector<Timed> g_timed;

bool timing_on() { return g_timing.load(std::memory_order_relaxed); }

cudaEvent_t timing_event() {
    std::lock_guard<std::mutex> lk(g_timing_mu);
    if (!g_event_pool.empty()) {
        cudaEvent_t e = g_event_pool.back();
        g_event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    FFGPU_CHECK_CUDA(cudaEventCreate(&e));
    return e;
}

void timing_push(const char *name, cudaEvent_t start, cudaEvent_t stop) {
    std::lock_guard<std::mutex> lk(g_timing_mu);
    g_timed.push_back({name, start, stop});
}

}  // namespace ffgpu

using namespace ffgpu;


extern "C" {

const char *ffgpu_last_error(void) { return t_last_error.c_str(); }
const char *ffgpu_version(void) { return "libffrs-gb300 0.1.0 (sm_103a)"; }
uint64_t ffgpu_kernel_launches(void) { return g_launches.load(); }

int ffgpu_set_host_chunk_blocks(size_t blocks) {
    return guarded([&] { g_chunk_blocks.store(blocks); });
}

int ffgpu_timing_enable(int on) {
    return guarded([&] { g_timing.store(on != 0); });
}

int ffgpu_timing_collect(char *out, size_t cap, size_t *len) {
    return guarded([&] {
        std::vector<Timed> done;
        {
            std::lock_guard<std::mutex> lk(g_timing_mu);
            done.swap(g_timed);
        }
        std::vector<std::pair<std::string, std::pair<double, long>>> acc;
        for (auto &t : done) {
            FFGPU_CHECK_CUDA(cudaEventSynchronize(t.stop));
            float ms = 0.f;
            FFGPU_CHECK_CUDA(cudaEventElapsedTime(&ms, t.start, t.stop));
            bool found = false;
            for (auto &a : acc)
                if (a.first == t.name) {
                    a.second.first += ms;
                    a.second.second += 1;
                    found = true;
                }
            if (!found) acc.push_back({t.name, {ms, 1}});
        }
        {
            std::lock_guard<std::mutex> lk(g_timing_mu);
            for (auto &t : done) {
                g_event_pool.push_back(t.start);
                g_event_pool.push_back(t.stop);
            }
        }
        std::string text;
        for (auto &a : acc)
            text += a.first + " " + std::to_string(a.second.first) + " " + std::to_string(a.second.second) + "\n";
        if (len) *len = text.size();
        if (out && cap) {
            const size_t n = std::min(cap - 1, text.size());
            std::memcpy(out, text.data(), n);
            out[n] = 0;
        }
    });
}

int ffgpu_init(int device) {
    return guarded([&] {
        int n = 0;
        FFGPU_CHECK_CUDA(cudaGetDeviceCount(&n));
        FFGPU_REQUIRE(device >= 0 && device < n, "no such CUDA device");
        g_device = device;
        FFGPU_CHECK_CUDA(cudaSetDevice(device));
    });
}

void *ffgpu_default_stream(void) {
    void *s = nullptr;
    guarded([&] { s = (void *)lib_stream(); });
    return s;
}

int ffgpu_synchronize(void *stream) {
    return guarded([&] { FFGPU_CHECK_CUDA(cudaStreamSynchronize((cudaStream_t)stream)); });
}

int ffgpu_host_alloc(size_t bytes, void **out) {
    return guarded([&] {
        FFGPU_REQUIRE(out, "out is NULL");
        void *p = nullptr;
        if (cudaHostAlloc(&p, bytes ? bytes : 1, cudaHostAllocPortable) != cudaSuccess)
            throw Error(FFGPU_ENOMEM, "cudaHostAlloc failed");
        std::memset(p, 0, bytes);
        *out = p;
    });
}

int ffgpu_host_free(void *ptr) {
    return guarded([&] {
        if (ptr) FFGPU_CHECK_CUDA(cudaFreeHost(ptr));
    });
}

int ffgpu_rs256_create(int ecc_len, int primitive, int polynomial, ffgpu_rs256 **out) {
    return guarded([&] {
        FFGPU_REQUIRE(out, "out is NULL");
        lib_stream();
        auto h = std::make_unique<ffgpu_rs256>();
        h->code = std::make_unique<Rs256Code>(ecc_len, primitive, polynomial);
        *out = h.release();
    });
}

int ffgpu_rs256_destroy(ffgpu_rs256 *code) {
    return guarded([&] { delete code; });
}

int ffgpu_rs256_generator(const ffgpu_rs256 *code, uint8_t *generator, uint8_t *roots) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        const Rs256Code &c = *code->code;
        if (generator) std::memcpy(generator, c.generator, (size_t)c.ecc + 1);
        if (roots) std::memcpy(roots, c.roots, (size_t)c.ecc);
    });
}

static void check_rs_geometry(const Rs256Code &c, size_t message_len) {
    FFGPU_REQUIRE(message_len >= 1 && message_len + (size_t)c.ecc <= 255, "block_len must be <= 255");
}

int ffgpu_rs256_encode(const ffgpu_rs256 *code, const uint8_t *data, size_t nblocks, size_t message_len,
                       uint8_t *parity, void *stream) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        check_rs_geometry(*code->code, message_len);
        rs256_encode(*code->code, data, nblocks, (int)message_len, parity,
                     (cudaStream_t)stream);
    });
}

int ffgpu_rs256_decode(const ffgpu_rs256 *code, uint8_t *data, uint8_t *parity, size_t nblocks, size_t message_len,
                       uint8_t *status, void *stream) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        check_rs_geometry(*code->code, message_len);
        rs256_decode(*code->code, data, parity, nblocks, (int)message_len, status,
                     (cudaStream_t)stream);
    });
}

int ffgpu_rs256_synds(const ffgpu_rs256 *code, const uint8_t *data, const uint8_t *parity, size_t nblocks,
                      size_t message_len, uint8_t *synds, void *stream) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        check_rs_geometry(*code->code, message_len);
        rs256_synds(*code->code, data, parity, nblocks, (int)message_len, synds, (cudaStream_t)stream);
    });
}

int ffgpu_rs256_encode_host(const ffgpu_rs256 *code, const uint8_t *buf, size_t len, size_t message_len,
                            uint8_t *out) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        ffgpu_rs256 *h = const_cast<ffgpu_rs256 *>(code);
        const Rs256Code &c = *h->code;
        check_rs_geometry(c, message_len);
        if (len == 0) return;
        std::lock_guard<std::mutex> lk(h->mu);
        cudaStream_t st = lib_stream();
        const size_t full = len / message_len, tail = len - full * message_len;
        const size_t nout = (full + (tail ? 1 : 0)) * (size_t)c.ecc;
        uint8_t *d_in = (uint8_t *)h->d_data.get(len);
        uint8_t *d_out = (uint8_t *)h->d_parity.get(nout);
        // chunks of full blocks on the pipeline streams (copy in, encode and
        // copy out of different chunks overlap); the ragged tail block goes
        // with the last chunk.  Each chunk costs fixed host work (events, the
        // staged output copy); below about a quarter million blocks that
        // costs more than the overlap gains (65,536 blocks: 109 GB/s whole,
        // 75 GB/s in four chunks), so smaller calls stay whole.
        const size_t chunk = std::max<size_t>(1, host_chunk_blocks(full, 262144, 4));
        uint8_t *h_out = pipeline_out(out, chunk < full, h->h_parity, nout);
        OutputDrain drain;
        HostPipeline pl;
        size_t k = 0;
        for (size_t b0 = 0; b0 < full || (k == 0 && tail); b0 += chunk, ++k) {
            const size_t n = std::min(chunk, full - b0);
            const bool last = b0 + n >= full;
            const size_t out_bytes = (n + (last && tail ? 1 : 0)) * (size_t)c.ecc;
            const size_t i0 = b0 * message_len, o0 = b0 * (size_t)c.ecc;
            // within a chunk of 32 K blocks or more, the upload goes in four
            // pieces and each piece's encode waits only for its own copy (the
            // encode takes time in proportion to its blocks); the output
            // stays one copy
            const size_t nsub = n >= 32768 ? 4 : 1;
            for (size_t q = 0; q < nsub; ++q) {
                const size_t s0 = n * q / nsub, s1 = n * (q + 1) / nsub;
                const size_t bytes = (s1 - s0) * message_len + (q + 1 == nsub && last ? tail : 0);
                FFGPU_CHECK_CUDA(cudaMemcpyAsync(d_in + i0 + s0 * message_len, buf + i0 + s0 * message_len, bytes,
                                                 cudaMemcpyHostToDevice, pl.up()));
                st = pl.compute(k);  // waits for the copies issued so far
                if (s1 > s0)
                    rs256_encode(c, d_in + i0 + s0 * message_len, s1 - s0, (int)message_len,
                                 d_out + o0 + s0 * (size_t)c.ecc, st);
            }
            if (last && tail)
                rs256_encode(c, d_in + full * message_len, 1, (int)tail, d_out + full * (size_t)c.ecc, st);
            st = pl.to_down(k);
            FFGPU_CHECK_CUDA(cudaMemcpyAsync(h_out + o0, d_out + o0, out_bytes, cudaMemcpyDeviceToHost, st));
            drain.copy(out + o0, h_out + o0, out_bytes);
            drain.chunk(st);
        }
        drain.finish();
        pl.sync();
    });
}

int ffgpu_rs256_decode_host(const ffgpu_rs256 *code, uint8_t *data, uint8_t *parity, size_t nblocks,
                            size_t message_len, uint8_t *status) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        ffgpu_rs256 *h = const_cast<ffgpu_rs256 *>(code);
        const Rs256Code &c = *h->code;
        check_rs_geometry(c, message_len);
        if (nblocks == 0) return;
        std::lock_guard<std::mutex> lk(h->mu);
        const size_t nd = nblocks * message_len, np = nblocks * (size_t)c.ecc;
        uint8_t *d_d = (uint8_t *)h->d_data.get(nd);
        uint8_t *d_p = (uint8_t *)h->d_parity.get(np);
        uint8_t *d_s = (uint8_t *)h->d_status.get(nblocks);
        // chunks of blocks: the upload of one chunk, the decode of another and
        // the download of a third overlap; outputs in pageable memory come
        // back through page-locked staging
        const size_t chunk = host_chunk_blocks(nblocks, 131072, 8);
        const bool chunked = chunk < nblocks;
        uint8_t *h_d = pipeline_out(data, chunked, h->h_data, nd);
        uint8_t *h_p = pipeline_out(parity, chunked, h->h_parity, np);
        uint8_t *h_s = pipeline_out(status, chunked, h->h_status, nblocks);
        OutputDrain drain;
        HostPipeline pl;
        size_t k = 0;
        for (size_t b0 = 0; b0 < nblocks; b0 += chunk, ++k) {
            const size_t n = std::min(chunk, nblocks - b0);
            const size_t od = b0 * message_len, op = b0 * (size_t)c.ecc;
            uint8_t *dd = d_d + od, *dp = d_p + op, *ds = d_s + b0;
            FFGPU_CHECK_CUDA(cudaMemcpyAsync(dd, data + od, n * message_len, cudaMemcpyHostToDevice, pl.up()));
            FFGPU_CHECK_CUDA(cudaMemcpyAsync(dp, parity + op, n * (size_t)c.ecc, cudaMemcpyHostToDevice, pl.up()));
            cudaStream_t st = pl.compute(k);
            rs256_decode(c, dd, dp, n, (int)message_len, ds, st);
            st = pl.to_down(k);
            FFGPU_CHECK_CUDA(cudaMemcpyAsync(h_d + od, dd, n * message_len, cudaMemcpyDeviceToHost, st));
            FFGPU_CHECK_CUDA(cudaMemcpyAsync(h_p + op, dp, n * (size_t)c.ecc, cudaMemcpyDeviceToHost, st));
            FFGPU_CHECK_CUDA(cudaMemcpyAsync(h_s + b0, ds, n, cudaMemcpyDeviceToHost, st));
            drain.copy(data + od, h_d + od, n * message_len);
            drain.copy(parity + op, h_p + op, n * (size_t)c.ecc);
            drain.copy(status + b0, h_s + b0, n);
            drain.chunk(st);
        }
        drain.finish();
        pl.sync();
    });
}

int ffgpu_rs256_synds_host(const ffgpu_rs256 *code, const uint8_t *data, const uint8_t *parity, size_t nblocks,
                           size_t message_len, uint8_t *synds) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        ffgpu_rs256 *h = const_cast<ffgpu_rs256 *>(code);
        const Rs256Code &c = *h->code;
        check_rs_geometry(c, message_len);
        if (nblocks == 0) return;
        std::lock_guard<std::mutex> lk(h->mu);
        cudaStream_t st = lib_stream();
        const size_t nd = nblocks * message_len, np = nblocks * (size_t)c.ecc;
        uint8_t *d_d = (uint8_t *)h->d_data.get(nd);
        uint8_t *d_p = (uint8_t *)h->d_parity.get(np);
        uint8_t *d_s = (uint8_t *)h->d_status.get(np);
        FFGPU_CHECK_CUDA(cudaMemcpyAsync(d_d, data, nd, cudaMemcpyHostToDevice, st));
        FFGPU_CHECK_CUDA(cudaMemcpyAsync(d_p, parity, np, cudaMemcpyHostToDevice, st));
        rs256_synds(c, d_d, d_p, nblocks, (int)message_len, d_s, st);
        FFGPU_CHECK_CUDA(cudaMemcpyAsync(synds, d_s, np, cudaMemcpyDeviceToHost, st));
        FFGPU_CHECK_CUDA(cudaStreamSynchronize(st));
    });
}

int ffgpu_rs256_set_table_only(ffgpu_rs256 *code, int table_only) {
    return guarded([&] {
        FFGPU_REQUIRE(code, "code is NULL");
        std::lock_guard<std::mutex> lk(code->mu);
        code->code->table_only = table_only != 0;
    });
}

}  // extern "C"
