// tube_cache.cu -- factored tubes kept across calls.
//
// A trajectory, an ensemble of trajectories and an ensemble field all solve
// swimmers against one tube, which moves with the swimmer and so is assembled
// and factored once (src/trajectory.hpp:47).  Successive calls with the same
// tube (the usual case: many trajectory segments, or the field after the
// ensemble that produced the states) reuse the factor from this cache instead
// of building it again.  Entries are keyed by every parameter the factor
// depends on -- R, L, a, n_theta, n_r, mu and the precision mode -- compared
// exactly, and evicted least-recently-used beyond SQBEM_TUBE_CACHE entries
// (default 4; 0 turns the cache off).  A mixed-precision tube at n_theta = 24
// holds about 0.2 GB.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <list>
#include <memory>
#include <mutex>

#include "common.cuh"
#include "solver.cuh"
#include "tube_cache.cuh"

namespace sqbem {

namespace {

struct Key {
    double R, L, a, mu;
    int n_theta, n_r, precision;
    bool operator==(const Key& o) const { return std::memcmp(this, &o, sizeof(Key)) == 0; }
};

struct Entry {
    Key key;
    std::shared_ptr<const sqbem_tube> tube;
};

std::mutex g_mu;
std::list<Entry> g_lru;  // most recently used first
long long g_builds = 0, g_hits = 0;

size_t capacity() {
    const char* e = std::getenv("SQBEM_TUBE_CACHE");
    const int v = e ? std::atoi(e) : 4;
    return (size_t)std::max(0, std::min(v, 64));
}

}  // namespace

std::shared_ptr<const sqbem_tube> cached_tube(double R, double L, double a, int n_theta, int n_r, double mu,
                                              int precision) {
    Key k;
    std::memset(&k, 0, sizeof k);  // padding compares equal
    k.R = R; k.L = L; k.a = a; k.mu = mu; k.n_theta = n_theta; k.n_r = n_r; k.precision = precision;
    std::lock_guard<std::mutex> lk(g_mu);
    for (auto it = g_lru.begin(); it != g_lru.end(); ++it)
        if (it->key == k) {
            g_lru.splice(g_lru.begin(), g_lru, it);
            ++g_hits;
            return it->tube;
        }
    // built under the lock: a concurrent caller with the same key waits for this
    // factor instead of building its own
    auto t = std::make_shared<sqbem_tube>();
    t->build(R, L, a, n_theta, n_r, mu, precision);  // synchronizes its stream before returning
    ++g_builds;
    std::shared_ptr<const sqbem_tube> out = t;
    const size_t cap = capacity();
    if (cap > 0) {
        g_lru.push_front({k, out});
        while (g_lru.size() > cap) g_lru.pop_back();  // users still holding an entry keep it alive
    }
    return out;
}

}  // namespace sqbem

using namespace sqbem;

extern "C" int sqbem_tube_cache_stats(long long* builds, long long* hits, int* entries) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (builds) *builds = g_builds;
    if (hits) *hits = g_hits;
    if (entries) *entries = (int)g_lru.size();
    return SQBEM_OK;
}

extern "C" int sqbem_tube_cache_clear(void) {
    return guarded([&] {
        std::lock_guard<std::mutex> lk(g_mu);
        g_lru.clear();  // a call still using an entry holds its own reference
    });
}
