// common.cuh -- shared infrastructure of the sqbem CUDA library: status codes,
// error propagation, launch accounting, device buffers.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "sqbem.h"

namespace sqbem {

// Failure carried from the implementation to the C ABI boundary.
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] inline void fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    throw Error(code, buf);
}

inline void cuda_check(cudaError_t e, const char* what, const char* file, int line) {
    if (e != cudaSuccess) fail(SQBEM_ERR_CUDA, "%s: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
}
#define CUDA_CHECK(x) ::sqbem::cuda_check((x), #x, __FILE__, __LINE__)

// Every kernel launch of the library goes through LAUNCH so the count is exact.
extern std::atomic<long long> g_launches;
#define LAUNCH(kernel, grid, block, smem, stream, ...)                                  \
    do {                                                                                \
        kernel<<<(grid), (block), (smem), (stream)>>>(__VA_ARGS__);                     \
        ::sqbem::g_launches.fetch_add(1, std::memory_order_relaxed);                    \
        ::sqbem::cuda_check(cudaGetLastError(), #kernel, __FILE__, __LINE__);           \
    } while (0)

// Host<->device bytes moved by the library (every copy goes through DevBuf or
// count_h2d/count_d2h).
extern std::atomic<long long> g_h2d_bytes, g_d2h_bytes;
inline void count_h2d(size_t b) { g_h2d_bytes.fetch_add((long long)b, std::memory_order_relaxed); }
inline void count_d2h(size_t b) { g_d2h_bytes.fetch_add((long long)b, std::memory_order_relaxed); }

// Opt-in per-kernel-class timing (sqbem_kernel_stats_*): CUDA events around the
// launches of one class on their own stream, with the algorithmic flops and
// bytes each launch is credited with.
bool kstats_on();
// free-form description attached to the next timed launch of this thread
void kstat_note(const std::string& note);
int kstat_begin(cudaStream_t st);
void kstat_end(int slot, const char* cls, cudaStream_t st, double flops, double bytes);
// Work known only on the device when the launch is issued: n counters that the
// caller copies (stream-ordered, before the timed launch) into pinned host
// ints from kstat_pinned_ints; the launch is credited with sum w[i] * counts[i]
// flops once its events have completed.
int* kstat_pinned_ints(int n);
void kstat_end_counted(int slot, const char* cls, cudaStream_t st, const int* counts, const double* w, int n,
                       double bytes);
#define TIMED_LAUNCH(cls, flops, bytes, kernel, grid, block, smem, stream, ...)          \
    do {                                                                                \
        const int _ks = ::sqbem::kstats_on() ? ::sqbem::kstat_begin(stream) : -1;      \
        LAUNCH(kernel, grid, block, smem, stream, __VA_ARGS__);                         \
        if (_ks >= 0) ::sqbem::kstat_end(_ks, cls, stream, (flops), (bytes));           \
    } while (0)

void require_device();
void set_last_error(const char* msg);

// Limits set by sqbem_set_limits: SM clock cycles a tensor-core GEMM role waits
// on one mbarrier phase before it gives up (SQBEM_ERR_TIMEOUT), and the cap on
// mixed-precision refinement steps (SQBEM_ERR_NOT_CONVERGED beyond it).
constexpr long long DEFAULT_WAIT_CYCLES = 4000000000LL;  // ~2 s at 2 GHz
constexpr int DEFAULT_REFINE_MAX_IT = 30;
long long gemm_wait_cycles();
int refine_max_iterations();
inline void set_last_error(const std::string& msg) { set_last_error(msg.c_str()); }

// Run f; convert a failure into a status code and the thread's error message.
template <class F>
int guarded(F&& f) {
    try {
        f();
        set_last_error("");
        return SQBEM_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::bad_alloc&) {
        set_last_error("host allocation failed");
        return SQBEM_ERR_ALLOC;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return SQBEM_ERR_ARG;
    }
}

// The library's stream-ordered device pool (keeps freed memory) and the
// host-to-device copy through pinned staging (memory.cu).
cudaMemPool_t device_pool();
void upload_bytes(void* dst, const void* src, size_t bytes, cudaStream_t st);

// Idle device blocks of one stream.  The stream-ordered allocator serialises
// its calls across host threads behind one driver lock: on GB300's Grace host a
// malloc/free pair took 0.6 us on one thread and 27 us per thread on six, and
// the six concurrent workers of a 48-swimmer ensemble group spent 51-54 of
// their 88 ms in it.  So a worker allocates through the cache of its slot
// (below): a block freed on the slot's stream goes back to the cache, and a
// later allocation on the same stream of the same size class takes it -- safe
// in stream order, as the allocator's own reuse is -- with no driver call.
// Size classes are 1/8 octave apart (at most 12.5% over the request).
class StreamCache {
public:
    explicit StreamCache(cudaStream_t s) : s_(s) {}
    StreamCache(const StreamCache&) = delete;
    StreamCache& operator=(const StreamCache&) = delete;
    cudaStream_t stream() const { return s_; }
    void* take(size_t bytes);          // a block of the request's class, or null if the pool is out of memory
    void give(void* p, size_t bytes);  // a block that take() returned, now idle
    void trim_to(size_t keep);         // idle blocks back to the pool until at most keep bytes stay
    size_t held() const { return held_; }

private:
    cudaStream_t s_;
    std::map<size_t, std::vector<void*>> idle_;
    size_t held_ = 0;
};

// Worker slot k of the current device: a stream and its block cache that last
// for the process, so that successive batched calls (an ensemble's RK stages,
// repeated sweeps) reuse each other's blocks.  The lease installs the cache for
// the calling thread; a slot already leased (a concurrent call from another
// host thread) leaves this lease with a stream of its own and no cache.
// sqbem_trim_pool() empties the caches.
class WorkerLease {
public:
    explicit WorkerLease(int k);
    ~WorkerLease();
    WorkerLease(const WorkerLease&) = delete;
    WorkerLease& operator=(const WorkerLease&) = delete;
    cudaStream_t stream() const { return st_; }
    void end_task();  // after a task: the slot's idle blocks trimmed to its share

private:
    int dev_ = 0, k_ = -1;
    cudaStream_t st_ = nullptr;
    bool own_stream_ = false;
    StreamCache* prev_ = nullptr;
};
void trim_worker_caches();

// Device allocation on stream s: from the calling thread's slot cache when it
// serves s (*cached set), else from the pool.  Fails with SQBEM_ERR_ALLOC.
void* dev_alloc(size_t bytes, cudaStream_t s, bool* cached);
void dev_free(void* p, size_t bytes, cudaStream_t s, bool cached);

// Owning device allocation (stream-ordered, from device_pool() or a worker's
// StreamCache).
template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaStream_t st = nullptr;
    bool cached = false;
    DevBuf() = default;
    DevBuf(size_t count, cudaStream_t s) { alloc(count, s); }
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n), st(o.st), cached(o.cached) { o.p = nullptr; o.n = 0; }
    DevBuf& operator=(DevBuf&& o) noexcept {
        if (this != &o) {
            release();
            p = o.p; n = o.n; st = o.st; cached = o.cached;
            o.p = nullptr; o.n = 0;
        }
        return *this;
    }
    ~DevBuf() { release(); }
    void alloc(size_t count, cudaStream_t s) {
        release();
        st = s;
        n = count;
        if (count == 0) return;
        p = static_cast<T*>(dev_alloc(count * sizeof(T), s, &cached));
    }
    void zero() {
        if (n) CUDA_CHECK(cudaMemsetAsync(p, 0, n * sizeof(T), st));
    }
    void release() {
        if (p) dev_free(p, n * sizeof(T), st, cached);
        p = nullptr;
        n = 0;
        cached = false;
    }
    void upload(const T* h, size_t count) { upload_bytes(p, h, count * sizeof(T), st); }
    void download(T* h, size_t count) const {
        CUDA_CHECK(cudaMemcpyAsync(h, p, count * sizeof(T), cudaMemcpyDeviceToHost, st));
        count_d2h(count * sizeof(T));
    }
    T* get() const { return p; }
};

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

// Column-major device matrix view: element (i, j) at a[i + j * ld].
template <class T>
struct MatView {
    T* a;
    int rows, cols;
    long long ld;
    __host__ __device__ T& operator()(int i, int j) const { return a[i + (long long)j * ld]; }
    MatView block(int i0, int j0, int r, int c) const { return {a + i0 + (long long)j0 * ld, r, c, ld}; }
};

constexpr double EIGHT_PI = 8.0 * 3.14159265358979323846;

}  // namespace sqbem
