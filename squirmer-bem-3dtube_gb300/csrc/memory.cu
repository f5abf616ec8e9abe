// memory.cu -- the library's device memory pool and pinned upload staging.
//
// Device buffers come from one stream-ordered pool per device that keeps freed
// memory (release threshold = max): the default pool returns it to the CUDA driver
// at every synchronisation, and the next large allocation then has to map
// fresh pages while the GPU waits.  The concurrent workers allocate through the
// block caches of persistent worker slots (WorkerLease, StreamCache in
// common.cuh) in front of that pool.  sqbem_trim_pool() gives the cached memory
// back.
//
// A host-to-device copy from pageable memory may wait for its stream to drain
// before it starts, which stalls the host thread that feeds that stream behind
// every kernel already queued.  Every upload therefore goes through pinned
// staging (copied on the host, then a truly asynchronous DMA): copies of up to
// 64 KB through a ring of fixed 64 KB slots, larger ones through blocks sized
// for them.  A slot or block is reused once the event recorded after its copy
// has completed.
#include <cuda_runtime.h>

#include <atomic>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>

#include "common.cuh"

namespace sqbem {

namespace {

constexpr int MAX_DEV = 64;
cudaMemPool_t g_pools[MAX_DEV] = {};
std::once_flag g_pool_once[MAX_DEV];

// A block is free, being filled (taken, its copy not yet enqueued) or in
// flight (its event recorded after the copy); only an in-flight block whose
// event has completed becomes free again.
enum class PinState { Free, Filling, InFlight };
struct Pinned {
    void* p = nullptr;
    size_t bytes = 0;
    cudaEvent_t ev = nullptr;
    PinState state = PinState::Free;
};
std::mutex g_pin_mu;
std::deque<Pinned> g_pinned;  // deque: references stay valid as it grows
size_t g_pinned_total = 0;
constexpr size_t PINNED_CAP = 1ull << 30;      // at most 1 GiB of block staging
constexpr size_t SLOT_BYTES = 64 * 1024;        // copies up to this size take a ring slot
constexpr int SLOTS = 512;                      // 32 MiB of slots

// The ring: slots handed out in turn.  A slot's mutex is held while it is filled
// and its copy enqueued; a thread that comes round to a slot whose previous copy
// has not yet completed waits for that copy's event (with 512 slots, only when
// hundreds of small copies are queued behind long kernels).
struct Slot {
    std::mutex mu;
    cudaEvent_t ev = nullptr;
    bool used = false;
};
std::once_flag g_ring_once;
char* g_ring = nullptr;  // SLOTS x SLOT_BYTES pinned, or null if that allocation failed
Slot g_slots[SLOTS];
std::atomic<unsigned> g_ring_next{0};

bool upload_small(void* dst, const void* src, size_t bytes, cudaStream_t st) {
    std::call_once(g_ring_once, [] {
        void* p = nullptr;
        if (cudaMallocHost(&p, (size_t)SLOTS * SLOT_BYTES) != cudaSuccess) {
            (void)cudaGetLastError();
            return;
        }
        for (Slot& sl : g_slots) CUDA_CHECK(cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming));
        g_ring = static_cast<char*>(p);
    });
    if (!g_ring) return false;
    const unsigned i = g_ring_next.fetch_add(1, std::memory_order_relaxed) % SLOTS;
    Slot& sl = g_slots[i];
    std::lock_guard<std::mutex> lk(sl.mu);
    if (sl.used) CUDA_CHECK(cudaEventSynchronize(sl.ev));
    char* buf = g_ring + (size_t)i * SLOT_BYTES;
    std::memcpy(buf, src, bytes);
    CUDA_CHECK(cudaMemcpyAsync(dst, buf, bytes, cudaMemcpyHostToDevice, st));
    CUDA_CHECK(cudaEventRecord(sl.ev, st));
    sl.used = true;
    return true;
}

}  // namespace

cudaMemPool_t device_pool() {
    int dev = 0;
    CUDA_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= MAX_DEV) fail(SQBEM_ERR_ARG, "device ordinal %d out of range", dev);
    std::call_once(g_pool_once[dev], [dev] {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        CUDA_CHECK(cudaMemPoolCreate(&g_pools[dev], &props));
        unsigned long long keep = ~0ull;
        CUDA_CHECK(cudaMemPoolSetAttribute(g_pools[dev], cudaMemPoolAttrReleaseThreshold, &keep));
    });
    return g_pools[dev];
}

// ---------------------------------------------------------------- allocation
namespace {
thread_local StreamCache* t_cache = nullptr;

// 1/8-octave size classes: a power of two, or the next multiple of an eighth of
// the power of two below (256 bytes at least)
size_t size_class(size_t b) {
    if (b <= 256) return 256;
    const int e = 63 - __builtin_clzll((unsigned long long)b);
    if (b == (size_t(1) << e)) return b;
    const size_t step = size_t(1) << (e - 3 > 8 ? e - 3 : 8);
    return (b + step - 1) / step * step;
}

void* pool_alloc(size_t bytes, cudaStream_t s) {
    void* p = nullptr;
    const cudaError_t e = cudaMallocFromPoolAsync(&p, bytes, device_pool(), s);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    return p;
}

// the worker slots: taken through busy (compare-exchange, so that a nested
// lease on the same thread simply finds the slot taken)
constexpr int MAX_SLOTS = 8;
struct WorkerSlot {
    std::atomic<bool> busy{false};
    cudaStream_t st = nullptr;
    std::unique_ptr<StreamCache> cache;
};
WorkerSlot g_wslots[MAX_DEV][MAX_SLOTS];
size_t g_slot_share[MAX_DEV];  // idle bytes a slot keeps between tasks: 1/32 of the device's memory
std::once_flag g_share_once[MAX_DEV];

bool try_take(WorkerSlot& s) {
    bool expect = false;
    return s.busy.compare_exchange_strong(expect, true, std::memory_order_acquire);
}
}  // namespace

void* StreamCache::take(size_t bytes) {
    const size_t cls = size_class(bytes);
    auto it = idle_.find(cls);
    if (it != idle_.end() && !it->second.empty()) {
        void* p = it->second.back();
        it->second.pop_back();
        held_ -= cls;
        return p;
    }
    void* p = pool_alloc(cls, s_);
    if (!p && held_ > 0) {  // the idle blocks of other classes go back first
        trim_to(0);
        p = pool_alloc(cls, s_);
    }
    return p;
}

void StreamCache::give(void* p, size_t bytes) {
    const size_t cls = size_class(bytes);
    idle_[cls].push_back(p);
    held_ += cls;
}

void StreamCache::trim_to(size_t keep) {
    for (auto it = idle_.rbegin(); it != idle_.rend() && held_ > keep; ++it)
        while (!it->second.empty() && held_ > keep) {
            cudaFreeAsync(it->second.back(), s_);
            it->second.pop_back();
            held_ -= it->first;
        }
}

WorkerLease::WorkerLease(int k) {
    CUDA_CHECK(cudaGetDevice(&dev_));
    prev_ = t_cache;
    if (dev_ >= 0 && dev_ < MAX_DEV && k >= 0 && k < MAX_SLOTS && try_take(g_wslots[dev_][k])) {
        WorkerSlot& s = g_wslots[dev_][k];
        if (!s.st) {
            const cudaError_t e = cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking);
            if (e != cudaSuccess) {
                s.st = nullptr;
                s.busy.store(false, std::memory_order_release);
                CUDA_CHECK(e);
            }
            s.cache = std::make_unique<StreamCache>(s.st);
        }
        std::call_once(g_share_once[dev_], [this] {
            size_t fr = 0, tot = 0;
            CUDA_CHECK(cudaMemGetInfo(&fr, &tot));
            g_slot_share[dev_] = tot / 32;
        });
        k_ = k;
        st_ = s.st;
        t_cache = s.cache.get();
    } else {
        CUDA_CHECK(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking));
        own_stream_ = true;
        t_cache = nullptr;
    }
}

WorkerLease::~WorkerLease() {
    t_cache = prev_;
    if (k_ >= 0) {
        g_wslots[dev_][k_].busy.store(false, std::memory_order_release);
    } else if (own_stream_) {
        cudaStreamSynchronize(st_);
        cudaStreamDestroy(st_);
    }
}

void WorkerLease::end_task() {
    if (k_ >= 0) g_wslots[dev_][k_].cache->trim_to(g_slot_share[dev_]);
}

void trim_worker_caches() {
    for (auto& dev : g_wslots)
        for (WorkerSlot& s : dev)
            if (try_take(s)) {
                if (s.cache) {
                    s.cache->trim_to(0);
                    cudaStreamSynchronize(s.st);
                }
                s.busy.store(false, std::memory_order_release);
            }
}

void* dev_alloc(size_t bytes, cudaStream_t s, bool* cached) {
    StreamCache* c = t_cache;
    void* p = nullptr;
    if (c && c->stream() == s) {
        p = c->take(bytes);
        *cached = true;
    } else {
        p = pool_alloc(bytes, s);
        *cached = false;
    }
    if (!p) fail(SQBEM_ERR_ALLOC, "device allocation of %zu bytes failed", bytes);
    return p;
}

void dev_free(void* p, size_t bytes, cudaStream_t s, bool cached) {
    StreamCache* c = t_cache;
    if (cached && c && c->stream() == s) c->give(p, bytes);
    else cudaFreeAsync(p, s);
}

void upload_bytes(void* dst, const void* src, size_t bytes, cudaStream_t st) {
    count_h2d(bytes);
    if (bytes == 0) return;
    if (bytes <= SLOT_BYTES) {
        if (!upload_small(dst, src, bytes, st))  // no pinned ring: the plain copy is still correct
            CUDA_CHECK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
        return;
    }
    Pinned* blk = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_pin_mu);
        for (Pinned& b : g_pinned) {
            if (b.state == PinState::InFlight && cudaEventQuery(b.ev) == cudaSuccess) b.state = PinState::Free;
            if (b.state == PinState::Free && b.bytes >= bytes && (!blk || b.bytes < blk->bytes)) blk = &b;
        }
        if (!blk && g_pinned_total + bytes <= PINNED_CAP) {
            Pinned b;
            size_t sz = 1u << 20;
            while (sz < bytes) sz <<= 1;
            if (cudaMallocHost(&b.p, sz) == cudaSuccess) {
                b.bytes = sz;
                CUDA_CHECK(cudaEventCreateWithFlags(&b.ev, cudaEventDisableTiming));
                g_pinned_total += sz;
                g_pinned.push_back(b);
                blk = &g_pinned.back();
            } else {
                (void)cudaGetLastError();
            }
        }
        if (blk) blk->state = PinState::Filling;
    }
    if (!blk) {  // staging full: the plain copy is still correct
        CUDA_CHECK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
        return;
    }
    std::memcpy(blk->p, src, bytes);
    const cudaError_t e1 = cudaMemcpyAsync(dst, blk->p, bytes, cudaMemcpyHostToDevice, st);
    const cudaError_t e2 = e1 == cudaSuccess ? cudaEventRecord(blk->ev, st) : e1;
    {
        std::lock_guard<std::mutex> lk(g_pin_mu);
        blk->state = e2 == cudaSuccess ? PinState::InFlight : PinState::Free;
    }
    CUDA_CHECK(e2);
}

}  // namespace sqbem

using namespace sqbem;

extern "C" int sqbem_trim_pool(void) {
    return guarded([&] {
        require_device();
        trim_worker_caches();
        CUDA_CHECK(cudaDeviceSynchronize());
        CUDA_CHECK(cudaMemPoolTrimTo(device_pool(), 0));
    });
}
