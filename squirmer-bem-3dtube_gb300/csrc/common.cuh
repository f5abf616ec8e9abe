// common.cuh -- shared infrastructure of the sqbem CUDA library: status codes,
// error propagation, launch accounting, device buffers.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <stdexcept>
#include <string>

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

// Owning device allocation (stream-ordered, from device_pool()).
template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaStream_t st = nullptr;
    DevBuf() = default;
    DevBuf(size_t count, cudaStream_t s) { alloc(count, s); }
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n), st(o.st) { o.p = nullptr; o.n = 0; }
    DevBuf& operator=(DevBuf&& o) noexcept {
        if (this != &o) { release(); p = o.p; n = o.n; st = o.st; o.p = nullptr; o.n = 0; }
        return *this;
    }
    ~DevBuf() { release(); }
    void alloc(size_t count, cudaStream_t s) {
        release();
        st = s;
        n = count;
        if (count == 0) return;
        cudaError_t e = cudaMallocFromPoolAsync((void**)&p, count * sizeof(T), device_pool(), s);
        if (e != cudaSuccess) {
            p = nullptr;
            (void)cudaGetLastError();
            fail(SQBEM_ERR_ALLOC, "device allocation of %zu bytes failed: %s", count * sizeof(T),
                 cudaGetErrorString(e));
        }
    }
    void zero() {
        if (n) CUDA_CHECK(cudaMemsetAsync(p, 0, n * sizeof(T), st));
    }
    void release() {
        if (p) cudaFreeAsync(p, st);
        p = nullptr;
        n = 0;
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
