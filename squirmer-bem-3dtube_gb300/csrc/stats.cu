// stats.cu -- transfer counters and opt-in per-kernel-class event timing.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"

namespace sqbem {

std::atomic<long long> g_h2d_bytes{0}, g_d2h_bytes{0};

namespace {
constexpr int MAX_COUNTS = 8;
struct Pending {
    cudaEvent_t a = nullptr, b = nullptr;
    cudaStream_t st = nullptr;
    std::string cls, note;
    double flops = 0, bytes = 0;
    const int* counts = nullptr;  // pinned host counters, read at collection
    double w[MAX_COUNTS] = {};
    int ncounts = 0;
};
// pinned host ints for device-side counters (kstat_pinned_ints), used as a ring
constexpr int PINNED_INTS = 1 << 20;
int* g_pinned = nullptr;
int g_pinned_next = 0;
struct Agg {
    long long launches = 0;
    double seconds = 0, flops = 0, bytes = 0;
};
std::mutex g_mu;
std::atomic<bool> g_on{false};
std::vector<Pending> g_pending;
std::map<std::string, Agg> g_agg;
std::vector<cudaEvent_t> g_free;  // recorded-and-collected events, reused
// Per-launch log (profiling aid): with kernel stats enabled and SQBEM_KSTATS_LOG
// naming a file, every timed launch appends "class microseconds flops bytes note
// @start,end,stream": start and end in microseconds after the event recorded
// when the log was opened, and the launching stream, so that a run on several
// streams can be laid out as a timeline.
FILE* g_log = nullptr;
cudaEvent_t g_base = nullptr;
thread_local std::string t_note;

cudaEvent_t take_event() {
    if (!g_free.empty()) {
        cudaEvent_t e = g_free.back();
        g_free.pop_back();
        return e;
    }
    cudaEvent_t e;
    CUDA_CHECK(cudaEventCreate(&e));
    return e;
}

void collect_locked() {
    for (auto& p : g_pending) {
        if (p.b) {
            cudaEventSynchronize(p.b);
            float ms = 0;
            if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
                for (int i = 0; i < p.ncounts; ++i) p.flops += p.w[i] * (double)p.counts[i];
                Agg& g = g_agg[p.cls];
                g.launches += 1;
                g.seconds += ms * 1e-3;
                g.flops += p.flops;
                g.bytes += p.bytes;
                if (g_log) {
                    float t0 = 0, t1 = 0;
                    if (g_base) {
                        cudaEventElapsedTime(&t0, g_base, p.a);
                        cudaEventElapsedTime(&t1, g_base, p.b);
                    }
                    std::fprintf(g_log, "%s %.3f %.6g %.6g %s @%.3f,%.3f,%llx\n", p.cls.c_str(), ms * 1e3, p.flops,
                                 p.bytes, p.note.c_str(), t0 * 1e3, t1 * 1e3,
                                 (unsigned long long)(uintptr_t)p.st);
                }
            }
        }
        if (p.a) g_free.push_back(p.a);
        if (p.b) g_free.push_back(p.b);
    }
    g_pending.clear();
}
}  // namespace

bool kstats_on() { return g_on.load(std::memory_order_relaxed); }

int kstat_begin(cudaStream_t st) {
    std::lock_guard<std::mutex> lk(g_mu);
    Pending p;
    p.a = take_event();
    p.b = take_event();
    p.st = st;
    CUDA_CHECK(cudaEventRecord(p.a, st));
    g_pending.push_back(p);
    return (int)g_pending.size() - 1;
}

void kstat_end(int slot, const char* cls, cudaStream_t st, double flops, double bytes) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (slot < 0 || slot >= (int)g_pending.size()) return;
    Pending& p = g_pending[slot];
    CUDA_CHECK(cudaEventRecord(p.b, st));
    p.cls = cls;
    p.flops = flops;
    p.bytes = bytes;
    p.note.swap(t_note);
    t_note.clear();
}

void kstat_note(const std::string& note) { t_note = note; }

int* kstat_pinned_ints(int n) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (n <= 0 || n > 1024) fail(SQBEM_ERR_ARG, "kstat_pinned_ints: bad count");
    if (!g_pinned) CUDA_CHECK(cudaHostAlloc((void**)&g_pinned, sizeof(int) * PINNED_INTS, cudaHostAllocDefault));
    if (g_pinned_next + n > PINNED_INTS) {
        collect_locked();  // every earlier launch (and the copies before it) has completed
        g_pinned_next = 0;
    }
    int* p = g_pinned + g_pinned_next;
    g_pinned_next += n;
    return p;
}

void kstat_end_counted(int slot, const char* cls, cudaStream_t st, const int* counts, const double* w, int n,
                       double bytes) {
    kstat_end(slot, cls, st, 0.0, bytes);
    std::lock_guard<std::mutex> lk(g_mu);
    if (slot < 0 || slot >= (int)g_pending.size() || n > MAX_COUNTS) return;
    Pending& p = g_pending[slot];
    p.counts = counts;
    p.ncounts = n;
    for (int i = 0; i < n; ++i) p.w[i] = w[i];
}

// ---------------------------------------------------------------- pipe rates
// FMA throughput of the FP64 and FP32 pipes, measured with independent FMA
// chains on every SM: the denominators of the assembly kernels' rooflines
// (no FP64 or FP32 peak is published for this part in a form that matches
// what a kernel can issue).
namespace {
constexpr int PROBE_CHAINS = 8;

template <class T>
__global__ void __launch_bounds__(256) fma_probe_kernel(T a, T b, int iters, T* sink) {
    T x[PROBE_CHAINS];
#pragma unroll
    for (int c = 0; c < PROBE_CHAINS; ++c) x[c] = (T)(threadIdx.x + c) * b;
    for (int i = 0; i < iters; ++i)
#pragma unroll
        for (int c = 0; c < PROBE_CHAINS; ++c) x[c] = fma(x[c], a, b);
    T s = 0;
#pragma unroll
    for (int c = 0; c < PROBE_CHAINS; ++c) s += x[c];
    if (s == (T)-1) sink[0] = s;  // never true for these inputs; keeps the chains live
}

template <class T>
double probe_rate(int sms, int iters) {
    cudaStream_t st;
    CUDA_CHECK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    T* sink = nullptr;
    CUDA_CHECK(cudaMallocAsync((void**)&sink, sizeof(T), st));
    cudaEvent_t e0, e1;
    CUDA_CHECK(cudaEventCreate(&e0));
    CUDA_CHECK(cudaEventCreate(&e1));
    const int blocks = sms * 8, threads = 256;
    const T a = (T)0.999999, b = (T)1e-7;
    LAUNCH(fma_probe_kernel<T>, blocks, threads, 0, st, a, b, iters / 8, sink);  // warm-up
    CUDA_CHECK(cudaEventRecord(e0, st));
    LAUNCH(fma_probe_kernel<T>, blocks, threads, 0, st, a, b, iters, sink);
    CUDA_CHECK(cudaEventRecord(e1, st));
    CUDA_CHECK(cudaEventSynchronize(e1));
    float ms = 0;
    CUDA_CHECK(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeAsync(sink, st);
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    const double flops = 2.0 * PROBE_CHAINS * (double)iters * blocks * threads;
    return flops / (ms * 1e-3) / 1e12;
}
}  // namespace

}  // namespace sqbem

using namespace sqbem;

extern "C" int sqbem_pipe_rates(double* fp64_tflops, double* fp32_tflops) {
    return guarded([&] {
        require_device();
        int dev = 0, sms = 0;
        CUDA_CHECK(cudaGetDevice(&dev));
        CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        if (fp64_tflops) *fp64_tflops = probe_rate<double>(sms, 4096);
        if (fp32_tflops) *fp32_tflops = probe_rate<float>(sms, 262144);
    });
}

extern "C" int sqbem_transfer_bytes(long long* h2d, long long* d2h) {
    if (h2d) *h2d = g_h2d_bytes.load();
    if (d2h) *d2h = g_d2h_bytes.load();
    return SQBEM_OK;
}

extern "C" int sqbem_kernel_stats_enable(int on) {
    return guarded([&] {
        std::lock_guard<std::mutex> lk(g_mu);
        collect_locked();
        if (on) g_agg.clear();
        if (g_log) {
            std::fclose(g_log);
            g_log = nullptr;
        }
        const char* path = std::getenv("SQBEM_KSTATS_LOG");
        if (on && path && *path) {
            g_log = std::fopen(path, "a");
            if (!g_base) CUDA_CHECK(cudaEventCreate(&g_base));
            CUDA_CHECK(cudaEventRecord(g_base, 0));
            CUDA_CHECK(cudaEventSynchronize(g_base));
        }
        g_on.store(on != 0);
    });
}

extern "C" int sqbem_kernel_stats(const char* cls, long long* launches, double* seconds, double* flops,
                                  double* bytes) {
    return guarded([&] {
        if (!cls) fail(SQBEM_ERR_ARG, "kernel_stats: null class");
        std::lock_guard<std::mutex> lk(g_mu);
        collect_locked();
        Agg g;
        auto it = g_agg.find(cls);
        if (it != g_agg.end()) g = it->second;
        if (launches) *launches = g.launches;
        if (seconds) *seconds = g.seconds;
        if (flops) *flops = g.flops;
        if (bytes) *bytes = g.bytes;
    });
}

extern "C" int sqbem_kernel_stats_classes(char* buf, int cap) {
    return guarded([&] {
        std::lock_guard<std::mutex> lk(g_mu);
        collect_locked();
        std::string s;
        for (auto& kv : g_agg) s += (s.empty() ? "" : ",") + kv.first;
        if (!buf || cap <= (int)s.size()) fail(SQBEM_ERR_ARG, "kernel_stats_classes: buffer too small");
        std::memcpy(buf, s.c_str(), s.size() + 1);
    });
}
