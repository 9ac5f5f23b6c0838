// Shared runtime pieces of libffgpu: error reporting, launch accounting, the
// library stream and reusable device / pinned staging buffers.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/ffgpu.h"

namespace ffgpu {

void set_error(const std::string &msg);

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

#define FFGPU_CHECK_CUDA(expr)                                                                        \
    do {                                                                                              \
        cudaError_t _e = (expr);                                                                      \
        if (_e != cudaSuccess)                                                                        \
            throw ::ffgpu::Error(FFGPU_ECUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
    } while (0)

#define FFGPU_REQUIRE(cond, msg)                                      \
    do {                                                              \
        if (!(cond)) throw ::ffgpu::Error(FFGPU_EINVAL, (msg));        \
    } while (0)

// Every kernel launch in the library goes through this counter so callers can
// report how many kernels ran inside a timed region.
extern std::atomic<uint64_t> g_launches;

inline void launched(int n = 1) { g_launches.fetch_add((uint64_t)n, std::memory_order_relaxed); }

inline void check_launch(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw Error(FFGPU_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
    launched();
}

cudaStream_t lib_stream();
// k-th compute stream (mod kPipeStreams) of the chunked host-buffer pipelines
constexpr size_t kPipeStreams = 4;
cudaStream_t pipe_stream(size_t k);
// the pipelines' upload and download streams
cudaStream_t pipe_up();
cudaStream_t pipe_down();

// Stream roles of one host-buffer pipeline call.  Every upload goes to
// pipe_up() and every download to pipe_down(), so the two directions sit on
// different copy engines and overlap (with the directions mixed over the
// same streams, uploads queued behind downloads on a shared engine); the
// kernels of chunk k run on compute stream k mod kPipeStreams.  Events order
// upload -> kernels -> download per chunk.
class HostPipeline {
  public:
    HostPipeline() = default;
    HostPipeline(const HostPipeline &) = delete;
    HostPipeline &operator=(const HostPipeline &) = delete;
    ~HostPipeline();
    cudaStream_t up() const { return pipe_up(); }
    cudaStream_t down() const { return pipe_down(); }
    // after chunk k's uploads: the compute stream its kernels go on
    cudaStream_t compute(size_t k);
    // after chunk k's kernels: the download stream, ordered behind them
    cudaStream_t to_down(size_t k);
    // waits for every download issued (and so for everything before them)
    void sync();

  private:
    cudaEvent_t record(cudaStream_t s);
    std::vector<cudaEvent_t> evs_;
};
// blocks per chunk of a host-buffer pipeline: ffgpu_set_host_chunk_blocks, or
// at least min_chunk and at most max_chunks chunks
size_t host_chunk_blocks(size_t nblocks, size_t min_chunk, size_t max_chunks);
// memcpy split over a small pool of host threads for large copies (the pages
// of a fresh pageable destination are also faulted in in parallel)
void host_copy(void *dst, const void *src, size_t n);

// Outputs of a host-buffer pipeline that land in pageable memory: each
// chunk's device-to-host copies go to page-locked staging, chunk() records an
// event behind them on the chunk's stream, and finish() copies every chunk
// out as soon as its event has completed, while later chunks are still in
// flight.  copy() with dst == src (the output was page-locked) is a no-op.
class OutputDrain {
  public:
    OutputDrain() = default;
    OutputDrain(const OutputDrain &) = delete;
    OutputDrain &operator=(const OutputDrain &) = delete;
    ~OutputDrain();
    void copy(void *dst, const void *src, size_t n);
    void chunk(cudaStream_t st);
    void finish();

  private:
    struct Part {
        void *dst;
        const void *src;
        size_t n;
    };
    struct Chunk {
        cudaEvent_t ev;
        size_t first, count;
    };
    std::vector<Part> parts_;
    std::vector<Chunk> chunks_;
    size_t open_ = 0;
};

// Optional per-kernel timing (ffgpu_timing_enable): while it is on, a
// KernelTimer records a CUDA event pair around one launch on the launching
// stream, and ffgpu_timing_collect adds the elapsed times up per kernel name.
bool timing_on();
cudaEvent_t timing_event();
void timing_push(const char *name, cudaEvent_t start, cudaEvent_t stop);

struct KernelTimer {
    const char *name;
    cudaStream_t st;
    cudaEvent_t start = nullptr;
    KernelTimer(const char *n, cudaStream_t s) : name(n), st(s) {
        if (timing_on()) {
            start = timing_event();
            cudaEventRecord(start, st);
        }
    }
    ~KernelTimer() {
        if (start) {
            cudaEvent_t stop = timing_event();
            cudaEventRecord(stop, st);
            timing_push(name, start, stop);
        }
    }
    KernelTimer(const KernelTimer &) = delete;
    KernelTimer &operator=(const KernelTimer &) = delete;
};

// Grow-only device scratch owned by one code object (not thread-safe by
// design: one code object is used from one host thread at a time).
struct DeviceBuffer {
    void *ptr = nullptr;
    size_t bytes = 0;
    void *get(size_t need) {
        if (need > bytes) {
            if (ptr) cudaFree(ptr);
            ptr = nullptr;
            bytes = 0;
            size_t want = need < 256 ? 256 : need;
            if (cudaMalloc(&ptr, want) != cudaSuccess) throw Error(FFGPU_ENOMEM, "cudaMalloc failed");
            bytes = want;
        }
        return ptr;
    }
    ~DeviceBuffer() {
        if (ptr) cudaFree(ptr);
    }
};

struct PinnedBuffer {
    void *ptr = nullptr;
    size_t bytes = 0;
    void *get(size_t need) {
        if (need > bytes) {
            if (ptr) cudaFreeHost(ptr);
            ptr = nullptr;
            bytes = 0;
            size_t want = need < 4096 ? 4096 : need;
            if (cudaMallocHost(&ptr, want) != cudaSuccess) throw Error(FFGPU_ENOMEM, "cudaMallocHost failed");
            bytes = want;
        }
        return ptr;
    }
    ~PinnedBuffer() {
        if (ptr) cudaFreeHost(ptr);
    }
};

// True when `p` is page-locked host memory.  A device-to-host copy into
// pageable memory blocks the calling thread until the stream's earlier work
// is done, which serialises the chunks of a host-buffer pipeline; such
// outputs go through a PinnedBuffer instead.
inline bool page_locked(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// Where a host-buffer pipeline lands one output: the caller's memory when it
// is page-locked or when the call is a single chunk (nothing to overlap: the
// one blocking copy at the end costs no more than a staging copy), else the
// page-locked staging buffer.
template <typename T>
T *pipeline_out(T *dst, bool chunked, PinnedBuffer &stage, size_t bytes) {
    return (!chunked || page_locked(dst)) ? dst : (T *)stage.get(bytes);
}

// Runs `f` and converts exceptions into a status code + last-error message.
template <typename F>
int guarded(F &&f) {
    try {
        f();
        return FFGPU_OK;
    } catch (const Error &e) {
        set_error(e.what());
        return e.code;
    } catch (const std::bad_alloc &) {
        set_error("out of host memory");
        return FFGPU_ENOMEM;
    } catch (const std::exception &e) {
        set_error(e.what());
        return FFGPU_EINVAL;
    }
}

inline unsigned grid_for(size_t n, unsigned block) { return (unsigned)((n + block - 1) / block); }

}  // namespace ffgpu
