// Serving engine: requests on host buffers arrive at any time from any thread;
// a scheduler thread admits them into GPU "slots" (one CUDA stream each) while
// the HBM budget and the slot count allow, gathers every request queued at that
// moment into one micro-batch (one fused persistent launch through the batch
// path, between its host-to-device and device-to-host copies), and retires
// slots as their completion events fire.  Requests that arrive while others
// run are admitted as soon as a slot and memory free up, so copies and kernels
// of different micro-batches overlap on the device (continuous batching).
// Code tables stay resident in the code objects the requests name.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <string>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "common.cuh"
#include "handles.h"

namespace {

using clk = std::chrono::steady_clock;

enum : int { SK_RS256 = 0, SK_RSI16 = 1, SK_CIRC16 = 2 };

struct SrvReq {
    uint64_t id = 0;
    int kind = 0, op = 0;
    const void *code = nullptr;
    uint8_t *a = nullptr, *b = nullptr;  // host: data / message, parity / ecc (in place)
    uint8_t *status = nullptr;           // host, decode only
    size_t nblocks = 0, msg_len = 0;
    size_t a_bytes = 0, b_bytes = 0, s_bytes = 0;
    double t_submit = 0, t_start = 0, t_done = 0;
    int state = 0;  // 0 queued, 1 running, 2 done, 3 failed, 4 cancelled
    std::string error;
    int error_code = FFGPU_ECUDA;
};

struct Slot {
    cudaStream_t st = nullptr;
    cudaEvent_t done = nullptr;
    ffgpu_batch *batch = nullptr;
    std::vector<SrvReq *> reqs;
    void *dev = nullptr;
    size_t dev_bytes = 0;
    bool busy = false;
};

}  // namespace

extern "C" {
int ffgpu_batch_create(ffgpu_batch **out);
int ffgpu_batch_destroy(ffgpu_batch *b);
int ffgpu_batch_clear(ffgpu_batch *b);
int ffgpu_batch_add_rs256(ffgpu_batch *b, const ffgpu_rs256 *code, int op, uint8_t *data, uint8_t *parity,
                          size_t nblocks, size_t message_len, uint8_t *status);
int ffgpu_batch_add_rsi16(ffgpu_batch *b, const ffgpu_rsi16 *code, int op, uint16_t *msg, uint16_t *parity,
                          size_t nblocks, uint8_t *status);
int ffgpu_batch_add_circ16(ffgpu_batch *b, const ffgpu_circ16 *code, int op, uint16_t *msg, uint16_t *ecc,
                           size_t nblocks, uint8_t *status);
int ffgpu_batch_plan(ffgpu_batch *b, int autotune, void *stream);
int ffgpu_batch_launch(ffgpu_batch *b, void *stream);
}

struct ffgpu_server {
    std::mutex mu;
    std::condition_variable cv, done_cv;
    std::deque<SrvReq *> queue;
    std::unordered_map<uint64_t, std::unique_ptr<SrvReq>> reqs;
    std::vector<Slot> slots;
    size_t budget = 0, in_use = 0;
    size_t max_batch = 64;
    uint64_t next_id = 1;
    bool stop = false;
    int device = 0;
    clk::time_point t0 = clk::now();
    std::thread worker;

    double now() const { return std::chrono::duration<double>(clk::now() - t0).count(); }
};

namespace {

size_t round16(size_t n) { return (n + 255) & ~(size_t)255; }

// device bytes of one request (its buffers, 256-byte aligned)
size_t dev_need(const SrvReq &r) { return round16(r.a_bytes) + round16(r.b_bytes) + round16(r.s_bytes); }

void fail_slot_requests(ffgpu_server &S, Slot &sl, const std::string &msg, int code) {
    for (SrvReq *r : sl.reqs) {
        r->state = 3;
        r->error = msg;
        r->error_code = code;
        r->t_done = S.now();
    }
}

// Allocation failures injected by ffgpu_server_debug_fail_allocs: the next n
// slot allocations report out-of-memory without calling CUDA, so that tests
// exercise the failure path on the host.
std::atomic<int> g_fail_allocs{0};

bool take_injected_failure() {
    int n = g_fail_allocs.load();
    while (n > 0)
        if (g_fail_allocs.compare_exchange_weak(n, n - 1)) return true;
    return false;
}

// issue one micro-batch on a free slot (called with the lock released): the
// device buffers, the batch's work list (planned while the slot's stream is
// idle, its tables uploaded on that stream), then copies in, the batch
// launch, copies out, the stream-ordered free and the completion event.
void issue(ffgpu_server &S, Slot &sl) {
    size_t total = 0;
    for (SrvReq *r : sl.reqs) total += dev_need(*r);
    sl.dev_bytes = total;
    if (take_injected_failure())
        throw ffgpu::Error(FFGPU_ENOMEM, "cudaMallocAsync: out of memory (injected)");
    FFGPU_CHECK_CUDA(cudaMallocAsync(&sl.dev, total, sl.st));
    uint8_t *base = static_cast<uint8_t *>(sl.dev);
    ffgpu_batch_clear(sl.batch);
    std::vector<std::array<uint8_t *, 3>> dptr;
    size_t off = 0;
    for (SrvReq *r : sl.reqs) {
        uint8_t *da = base + off;
        off += round16(r->a_bytes);
        uint8_t *db = base + off;
        off += round16(r->b_bytes);
        uint8_t *ds = base + off;
        off += round16(r->s_bytes);
        dptr.push_back({da, db, ds});
        int rc = 0;
        if (r->kind == SK_RS256)
            rc = ffgpu_batch_add_rs256(sl.batch, static_cast<const ffgpu_rs256 *>(r->code), r->op, da, db, r->nblocks,
                                       r->msg_len, r->op == FFGPU_OP_DECODE ? ds : nullptr);
        else if (r->kind == SK_RSI16)
            rc = ffgpu_batch_add_rsi16(sl.batch, static_cast<const ffgpu_rsi16 *>(r->code), r->op,
                                       reinterpret_cast<uint16_t *>(da), reinterpret_cast<uint16_t *>(db),
                                       r->nblocks, r->op == FFGPU_OP_DECODE ? ds : nullptr);
        else
            rc = ffgpu_batch_add_circ16(sl.batch, static_cast<const ffgpu_circ16 *>(r->code), r->op,
                                        reinterpret_cast<uint16_t *>(da), reinterpret_cast<uint16_t *>(db),
                                        r->nblocks, r->op == FFGPU_OP_DECODE ? ds : nullptr);
        if (rc) throw ffgpu::Error(rc, ffgpu_last_error());
    }
    // the plan needs only the device pointers; the slot's stream holds
    // nothing but the allocation yet, so its synchronisation returns at once
    if (int rc = ffgpu_batch_plan(sl.batch, 0, sl.st)) throw ffgpu::Error(rc, ffgpu_last_error());
    for (size_t i = 0; i < sl.reqs.size(); ++i) {
        SrvReq *r = sl.reqs[i];
        FFGPU_CHECK_CUDA(cudaMemcpyAsync(dptr[i][0], r->a, r->a_bytes, cudaMemcpyHostToDevice, sl.st));
        if (r->op == FFGPU_OP_DECODE)
            FFGPU_CHECK_CUDA(cudaMemcpyAsync(dptr[i][1], r->b, r->b_bytes, cudaMemcpyHostToDevice, sl.st));
    }
    if (int rc = ffgpu_batch_launch(sl.batch, sl.st)) throw ffgpu::Error(rc, ffgpu_last_error());
    for (size_t i = 0; i < sl.reqs.size(); ++i) {
        SrvReq *r = sl.reqs[i];
        if (r->op == FFGPU_OP_DECODE) {
            FFGPU_CHECK_CUDA(cudaMemcpyAsync(r->a, dptr[i][0], r->a_bytes, cudaMemcpyDeviceToHost, sl.st));
            FFGPU_CHECK_CUDA(cudaMemcpyAsync(r->status, dptr[i][2], r->s_bytes, cudaMemcpyDeviceToHost, sl.st));
        }
        FFGPU_CHECK_CUDA(cudaMemcpyAsync(r->b, dptr[i][1], r->b_bytes, cudaMemcpyDeviceToHost, sl.st));
    }
    FFGPU_CHECK_CUDA(cudaFreeAsync(sl.dev, sl.st));
    sl.dev = nullptr;
    FFGPU_CHECK_CUDA(cudaEventRecord(sl.done, sl.st));
}

void worker_main(ffgpu_server *S) {
    cudaSetDevice(S->device);
    std::unique_lock<std::mutex> lk(S->mu);
    while (true) {
        // retire finished slots
        bool progressed = false;
        for (Slot &sl : S->slots) {
            if (!sl.busy) continue;
            const cudaError_t q = cudaEventQuery(sl.done);
            if (q == cudaErrorNotReady) continue;
            const double t = S->now();
            for (SrvReq *r : sl.reqs) {
                if (q == cudaSuccess) {
                    r->state = 2;
                } else {
                    r->state = 3;
                    r->error = cudaGetErrorString(q);
                }
                r->t_done = t;
            }
            S->in_use -= sl.dev_bytes;
            sl.reqs.clear();
            sl.busy = false;
            progressed = true;
        }
        if (progressed) S->done_cv.notify_all();
        if (S->stop && S->queue.empty()) {
            bool any = false;
            for (Slot &sl : S->slots) any |= sl.busy;
            if (!any) break;
        }
        // admit queued requests into free slots, FIFO, within the HBM budget
        for (Slot &sl : S->slots) {
            if (sl.busy || S->queue.empty()) continue;
            size_t need = 0;
            while (!S->queue.empty() && sl.reqs.size() < S->max_batch) {
                SrvReq *r = S->queue.front();
                const size_t n = dev_need(*r);
                if (S->in_use + need + n > S->budget && !(sl.reqs.empty() && S->in_use == 0)) break;
                S->queue.pop_front();
                sl.reqs.push_back(r);
                need += n;
            }
            if (sl.reqs.empty()) break;  // the head does not fit yet: wait for memory
            const double t = S->now();
            for (SrvReq *r : sl.reqs) {
                r->state = 1;
                r->t_start = t;
            }
            S->in_use += need;
            sl.busy = true;
            lk.unlock();
            try {
                issue(*S, sl);
            } catch (const std::exception &e) {
                // copies already queued on the slot's stream may still read
                // or write the callers' host buffers: let them finish before
                // the requests are reported failed, then return the memory
                cudaStreamSynchronize(sl.st);
                if (sl.dev) {
                    cudaFreeAsync(sl.dev, sl.st);
                    cudaStreamSynchronize(sl.st);
                    sl.dev = nullptr;
                }
                cudaGetLastError();
                const auto *fe = dynamic_cast<const ffgpu::Error *>(&e);
                lk.lock();
                fail_slot_requests(*S, sl, e.what(), fe ? fe->code : FFGPU_ECUDA);
                S->in_use -= need;
                sl.reqs.clear();
                sl.busy = false;
                S->done_cv.notify_all();
                continue;
            }
            lk.lock();
        }
        bool busy = false;
        for (Slot &sl : S->slots) busy |= sl.busy;
        // sleep until a submission arrives, or poll the slots shortly
        S->cv.wait_for(lk, busy ? std::chrono::microseconds(20) : std::chrono::milliseconds(5));
    }
}

SrvReq *enqueue(ffgpu_server *S, std::unique_ptr<SrvReq> r, uint64_t *ticket) {
    std::lock_guard<std::mutex> lk(S->mu);
    FFGPU_REQUIRE(!S->stop, "server is shutting down");
    r->id = S->next_id++;
    r->t_submit = S->now();
    SrvReq *p = r.get();
    S->reqs[p->id] = std::move(r);
    S->queue.push_back(p);
    *ticket = p->id;
    S->cv.notify_one();
    return p;
}

}  // namespace

using namespace ffgpu;

extern "C" {

int ffgpu_server_create(size_t hbm_budget, int nslots, int max_batch, ffgpu_server **out) {
    return guarded([&] {
        FFGPU_REQUIRE(out, "out is NULL");
        FFGPU_REQUIRE(nslots >= 1 && nslots <= 64, "slots must be in [1, 64]");
        auto S = std::make_unique<ffgpu_server>();
        FFGPU_CHECK_CUDA(cudaGetDevice(&S->device));
        size_t free_b = 0, total_b = 0;
        FFGPU_CHECK_CUDA(cudaMemGetInfo(&free_b, &total_b));
        const size_t cap = free_b / 10 * 8;
        S->budget = hbm_budget ? std::min(hbm_budget, cap) : cap;
        S->max_batch = max_batch > 0 ? (size_t)max_batch : 64;
        S->slots.resize((size_t)nslots);
        for (Slot &sl : S->slots) {
            FFGPU_CHECK_CUDA(cudaStreamCreateWithFlags(&sl.st, cudaStreamNonBlocking));
            FFGPU_CHECK_CUDA(cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming));
            if (int rc = ffgpu_batch_create(&sl.batch)) throw ffgpu::Error(rc, ffgpu_last_error());
        }
        S->worker = std::thread(worker_main, S.get());
        *out = S.release();
    });
}

int ffgpu_server_destroy(ffgpu_server *S) {
    return guarded([&] {
        if (!S) return;
        {
            std::lock_guard<std::mutex> lk(S->mu);
            S->stop = true;
        }
        S->cv.notify_all();
        if (S->worker.joinable()) S->worker.join();
        for (Slot &sl : S->slots) {
            cudaStreamSynchronize(sl.st);
            ffgpu_batch_destroy(sl.batch);
            cudaEventDestroy(sl.done);
            cudaStreamDestroy(sl.st);
        }
        delete S;
    });
}

int ffgpu_server_submit_rs256(ffgpu_server *S, const ffgpu_rs256 *code, int op, uint8_t *data, uint8_t *parity,
                              size_t nblocks, size_t message_len, uint8_t *status, uint64_t *ticket) {
    return guarded([&] {
        FFGPU_REQUIRE(S && code && ticket, "server, code or ticket is NULL");
        FFGPU_REQUIRE(op == FFGPU_OP_ENCODE || op == FFGPU_OP_DECODE, "op must be FFGPU_OP_ENCODE or FFGPU_OP_DECODE");
        FFGPU_REQUIRE(nblocks > 0 && data && parity, "empty request");
        FFGPU_REQUIRE(op == FFGPU_OP_ENCODE || status, "decode needs a status array");
        const int ecc = code->code->ecc;
        FFGPU_REQUIRE(message_len >= 1 && message_len + (size_t)ecc <= 255,
                      "message_len + ecc_len must be in [ecc_len + 1, 255]");
        auto r = std::make_unique<SrvReq>();
        r->kind = SK_RS256;
        r->op = op;
        r->code = code;
        r->a = data;
        r->b = parity;
        r->status = status;
        r->nblocks = nblocks;
        r->msg_len = message_len;
        r->a_bytes = nblocks * message_len;
        r->b_bytes = nblocks * (size_t)ecc;
        r->s_bytes = op == FFGPU_OP_DECODE ? nblocks : 0;
        enqueue(S, std::move(r), ticket);
    });
}

int ffgpu_server_submit_rsi16(ffgpu_server *S, const ffgpu_rsi16 *code, int op, uint16_t *msg, uint16_t *parity,
                              size_t nblocks, uint8_t *status, uint64_t *ticket) {
    return guarded([&] {
        FFGPU_REQUIRE(S && code && ticket, "server, code or ticket is NULL");
        FFGPU_REQUIRE(op == FFGPU_OP_ENCODE || op == FFGPU_OP_DECODE, "op must be FFGPU_OP_ENCODE or FFGPU_OP_DECODE");
        FFGPU_REQUIRE(nblocks > 0 && msg && parity, "empty request");
        FFGPU_REQUIRE(op == FFGPU_OP_ENCODE || status, "decode needs a status array");
        const Rsi16Code &c = *code->code;
        auto r = std::make_unique<SrvReq>();
        r->kind = SK_RSI16;
        r->op = op;
        r->code = code;
        r->a = reinterpret_cast<uint8_t *>(msg);
        r->b = reinterpret_cast<uint8_t *>(parity);
        r->status = status;
        r->nblocks = nblocks;
        r->a_bytes = nblocks * c.message_len * 2;
        r->b_bytes = nblocks * c.ecc * 2;
        r->s_bytes = op == FFGPU_OP_DECODE ? nblocks : 0;
        enqueue(S, std::move(r), ticket);
    });
}

int ffgpu_server_submit_circ16(ffgpu_server *S, const ffgpu_circ16 *code, int op, uint16_t *msg, uint16_t *ecc,
                               size_t nblocks, uint8_t *status, uint64_t *ticket) {
    return guarded([&] {
        FFGPU_REQUIRE(S && code && ticket, "server, code or ticket is NULL");
        FFGPU_REQUIRE(op == FFGPU_OP_ENCODE || op == FFGPU_OP_DECODE, "op must be FFGPU_OP_ENCODE or FFGPU_OP_DECODE");
        FFGPU_REQUIRE(nblocks > 0 && msg && ecc, "empty request");
        FFGPU_REQUIRE(op == FFGPU_OP_ENCODE || status, "decode needs a status array");
        const Circ16Code &c = *code->code;
        auto r = std::make_unique<SrvReq>();
        r->kind = SK_CIRC16;
        r->op = op;
        r->code = code;
        r->a = reinterpret_cast<uint8_t *>(msg);
        r->b = reinterpret_cast<uint8_t *>(ecc);
        r->nblocks = nblocks;
        r->a_bytes = nblocks * c.message_len * 2;
        r->b_bytes = nblocks * c.ecc_len * 2;
        r->status = status;
        r->s_bytes = op == FFGPU_OP_DECODE ? nblocks : 0;
        enqueue(S, std::move(r), ticket);
    });
}

// state: 0 queued, 1 running, 2 done, 3 failed; times in seconds since the
// server was created (submit, admitted into a slot, completion seen)
int ffgpu_server_poll(ffgpu_server *S, uint64_t ticket, int *state, double *t_submit, double *t_start,
                      double *t_done) {
    return guarded([&] {
        FFGPU_REQUIRE(S, "server is NULL");
        std::lock_guard<std::mutex> lk(S->mu);
        auto it = S->reqs.find(ticket);
        FFGPU_REQUIRE(it != S->reqs.end(), "unknown ticket");
        const SrvReq &r = *it->second;
        if (state) *state = r.state;
        if (t_submit) *t_submit = r.t_submit;
        if (t_start) *t_start = r.t_start;
        if (t_done) *t_done = r.t_done;
    });
}

// wait until the request is done (or failed, or timeout_s passed; < 0: no limit)
int ffgpu_server_wait(ffgpu_server *S, uint64_t ticket, double timeout_s) {
    return guarded([&] {
        FFGPU_REQUIRE(S, "server is NULL");
        std::unique_lock<std::mutex> lk(S->mu);
        auto it = S->reqs.find(ticket);
        FFGPU_REQUIRE(it != S->reqs.end(), "unknown ticket");
        SrvReq *r = it->second.get();
        auto pred = [&] { return r->state >= 2; };
        if (timeout_s < 0)
            S->done_cv.wait(lk, pred);
        else if (!S->done_cv.wait_for(lk, std::chrono::duration<double>(timeout_s), pred))
            throw Error(FFGPU_ETIMEOUT, "request not finished within the timeout");
        if (r->state == 3) throw Error(r->error_code, "request failed: " + r->error);
        if (r->state == 4) throw Error(FFGPU_ECANCELLED, "request cancelled");
    });
}

// withdraw a request that is still queued; one already admitted into a slot
// runs to completion
int ffgpu_server_cancel(ffgpu_server *S, uint64_t ticket) {
    return guarded([&] {
        FFGPU_REQUIRE(S, "server is NULL");
        std::lock_guard<std::mutex> lk(S->mu);
        auto it = S->reqs.find(ticket);
        FFGPU_REQUIRE(it != S->reqs.end(), "unknown ticket");
        SrvReq *r = it->second.get();
        if (r->state == 4) return;
        FFGPU_REQUIRE(r->state == 0, "request already admitted: it runs to completion");
        auto q = std::find(S->queue.begin(), S->queue.end(), r);
        if (q != S->queue.end()) S->queue.erase(q);
        r->state = 4;
        r->t_done = S->now();
        S->done_cv.notify_all();
    });
}

int ffgpu_server_debug_fail_allocs(int n) {
    return guarded([&] {
        FFGPU_REQUIRE(n >= 0, "n must be >= 0");
        g_fail_allocs.store(n);
    });
}

// forget a finished request
int ffgpu_server_release(ffgpu_server *S, uint64_t ticket) {
    return guarded([&] {
        FFGPU_REQUIRE(S, "server is NULL");
        std::lock_guard<std::mutex> lk(S->mu);
        auto it = S->reqs.find(ticket);
        FFGPU_REQUIRE(it != S->reqs.end(), "unknown ticket");
        FFGPU_REQUIRE(it->second->state >= 2, "request still queued or running");
        S->reqs.erase(it);
    });
}

}  // extern "C"
