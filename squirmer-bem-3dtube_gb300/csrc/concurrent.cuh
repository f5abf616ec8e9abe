// concurrent.cuh -- independent tasks (instance chunks, swimmer groups) on
// several host threads, each with its own CUDA stream, under a device-memory
// budget.  One chunk's latency-bound phases (diagonal LU leaves, small updates,
// host synchronisations) then overlap another's large GEMMs.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstdlib>
#include <exception>
#include <mutex>
#include <thread>
#include <vector>

#include "common.cuh"
#include "solver.cuh"

namespace sqbem {

// SQBEM_STREAMS host threads / streams (default 6, at most 8).
inline int stream_count() {
    const char* e = std::getenv("SQBEM_STREAMS");
    const int v = e ? std::atoi(e) : 6;
    return std::max(1, std::min(v, 8));
}

// Concurrent chunks share a memory budget: free device memory plus what the
// library's pool holds unused, times 0.8.  A chunk waits while its estimate
// does not fit next to the running ones (one chunk always runs).
class MemBudget {
public:
    explicit MemBudget(double budget) : budget_(budget) {}
    void acquire(double b) {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return used_ == 0 || used_ + b <= budget_; });
        used_ += b;
    }
    void release(double b) {
        {
            std::lock_guard<std::mutex> lk(mu_);
            used_ -= b;
        }
        cv_.notify_all();
    }

private:
    std::mutex mu_;
    std::condition_variable cv_;
    double budget_, used_ = 0;
};

inline double device_budget() {
    size_t fr = 0, tot = 0;
    CUDA_CHECK(cudaMemGetInfo(&fr, &tot));
    cuuint64_t reserved = 0, in_use = 0;
    cudaMemPool_t pool = device_pool();
    CUDA_CHECK(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved));
    CUDA_CHECK(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &in_use));
    return 0.8 * ((double)fr + (double)(reserved > in_use ? reserved - in_use : 0));
}

// Runs work(k, stream) for k < ntasks on up to stream_count() host threads, each
// with its own stream, tasks taken in order from a shared counter, every task's
// estimated device bytes held against the memory budget while it runs.  Events
// make the batch stream bs cover all of it.  The first failure is rethrown.
template <class Work>
void run_concurrent(size_t ntasks, const std::vector<double>& task_bytes, cudaStream_t bs, Work&& work) {
    const int W = std::min<int>(stream_count(), (int)ntasks);
    MemBudget budget(device_budget());
    int dev = 0;
    CUDA_CHECK(cudaGetDevice(&dev));
    cudaEvent_t start;
    CUDA_CHECK(cudaEventCreateWithFlags(&start, cudaEventDisableTiming));
    CUDA_CHECK(cudaEventRecord(start, bs));
    std::atomic<size_t> next{0};
    std::atomic<bool> failed{false};
    std::exception_ptr first_error;
    std::mutex emu;
    auto worker = [&](int slot) {
        try {
            CUDA_CHECK(cudaSetDevice(dev));
            WorkerLease lease(slot);  // the slot's stream and block cache
            const cudaStream_t ws = lease.stream();
            CUDA_CHECK(cudaStreamWaitEvent(ws, start, 0));
            for (;;) {
                const size_t k = next.fetch_add(1);
                if (k >= ntasks || failed.load()) break;
                budget.acquire(task_bytes[k]);
                try {
                    work(k, ws);
                    CUDA_CHECK(cudaStreamSynchronize(ws));
                    lease.end_task();
                } catch (...) {
                    budget.release(task_bytes[k]);
                    throw;
                }
                budget.release(task_bytes[k]);
            }
            cudaEvent_t done;
            CUDA_CHECK(cudaEventCreateWithFlags(&done, cudaEventDisableTiming));
            CUDA_CHECK(cudaEventRecord(done, ws));
            CUDA_CHECK(cudaStreamWaitEvent(bs, done, 0));
            CUDA_CHECK(cudaEventDestroy(done));
        } catch (...) {
            failed.store(true);
            std::lock_guard<std::mutex> lk(emu);
            if (!first_error) first_error = std::current_exception();
        }
    };
    if (W <= 1) {
        worker(0);
    } else {
        std::vector<std::thread> th;
        for (int w = 0; w < W; ++w) th.emplace_back(worker, w);
        for (auto& t : th) t.join();
    }
    cudaEventDestroy(start);
    if (first_error) std::rethrow_exception(first_error);
}

}  // namespace sqbem
