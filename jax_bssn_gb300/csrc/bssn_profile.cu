// Launch counter and optional per-kernel-class event timing (see bssn_profile.h).
#include <atomic>
#include <mutex>
#include <vector>

#include "../../include/bssn_gb300.h"
#include "bssn_profile.h"

namespace bssn {
namespace {

struct Pending {
    int cls;
    cudaEvent_t start, stop;
};

std::atomic<long long> g_launches{0};
std::atomic<int> g_enabled{0};
std::mutex g_mu;
std::vector<Pending> g_pending;
std::vector<cudaEvent_t> g_pool;
double g_ms[KC_COUNT] = {0};
long long g_count[KC_COUNT] = {0};
thread_local cudaEvent_t t_start = nullptr;

cudaEvent_t take_event() {
    if (!g_pool.empty()) {
        cudaEvent_t e = g_pool.back();
        g_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}

}  // namespace

void prof_begin(int cls, cudaStream_t s) {
    (void)cls;
    g_launches.fetch_add(1, std::memory_order_relaxed);
    if (!g_enabled.load(std::memory_order_relaxed)) return;
    std::lock_guard<std::mutex> lock(g_mu);
    t_start = take_event();
    cudaEventRecord(t_start, s);
}

bool profiling_enabled() { return g_enabled.load(std::memory_order_relaxed) != 0; }

void count_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

void prof_end(int cls, cudaStream_t s) {
    if (!g_enabled.load(std::memory_order_relaxed) || t_start == nullptr) return;
    std::lock_guard<std::mutex> lock(g_mu);
    cudaEvent_t stop = take_event();
    cudaEventRecord(stop, s);
    g_pending.push_back(Pending{cls, t_start, stop});
    t_start = nullptr;
}

}  // namespace bssn

using namespace bssn;

extern "C" {

long long bssn_launch_count(void) { return g_launches.load(); }

void bssn_profile_enable(int on) { g_enabled.store(on ? 1 : 0); }

void bssn_profile_reset(void) {
    std::lock_guard<std::mutex> lock(g_mu);
    for (auto& p : g_pending) {
        g_pool.push_back(p.start);
        g_pool.push_back(p.stop);
    }
    g_pending.clear();
    for (int c = 0; c < KC_COUNT; ++c) { g_ms[c] = 0.0; g_count[c] = 0; }
}

int bssn_profile_read(double* ms, long long* counts, int n) {
    std::lock_guard<std::mutex> lock(g_mu);
    for (auto& p : g_pending) {
        cudaEventSynchronize(p.stop);
        float t = 0.f;
        cudaEventElapsedTime(&t, p.start, p.stop);
        g_ms[p.cls] += t;
        g_count[p.cls] += 1;
        g_pool.push_back(p.start);
        g_pool.push_back(p.stop);
    }
    g_pending.clear();
    const int m = n < KC_COUNT ? n : KC_COUNT;
    for (int c = 0; c < m; ++c) {
        if (ms) ms[c] = g_ms[c];
        if (counts) counts[c] = g_count[c];
    }
    return KC_COUNT;
}

}  // extern "C"
