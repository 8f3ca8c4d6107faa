// Opt-in launch tracing: CUDA events recorded on the launching stream around
// every kernel this library enqueues, aggregated per kernel name.  Off by
// default (one relaxed load per launch); SZxG_trace_enable(1) turns it on and
// SZxG_trace_collect() resolves the events and returns per-kernel totals.
#include <string.h>

#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/szx_gb300.h"
#include "kernels.h"

namespace szxg {

namespace {
std::atomic<int> g_on{0};
std::mutex g_mu;
struct Rec {
    const char* name;
    cudaEvent_t a, b;
};
std::vector<Rec> g_recs;
std::vector<cudaEvent_t> g_pool;

cudaEvent_t take_event() {
    if (!g_pool.empty()) {
        cudaEvent_t e = g_pool.back();
        g_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}
}  // namespace

TraceScope::TraceScope(const char* name, cudaStream_t s) : name_(name), s_(s), a_(nullptr) {
    if (!g_on.load(std::memory_order_relaxed)) return;
    std::lock_guard<std::mutex> lk(g_mu);
    a_ = take_event();
    cudaEventRecord((cudaEvent_t)a_, s_);
}

TraceScope::~TraceScope() {
    if (!a_) return;
    std::lock_guard<std::mutex> lk(g_mu);
    cudaEvent_t b = take_event();
    cudaEventRecord(b, s_);
    g_recs.push_back(Rec{name_, (cudaEvent_t)a_, b});
}

}  // namespace szxg

using namespace szxg;

extern "C" {

void SZxG_trace_enable(int on) {
    std::lock_guard<std::mutex> lk(g_mu);
    g_on.store(on ? 1 : 0);
    for (auto& r : g_recs) { g_pool.push_back(r.a); g_pool.push_back(r.b); }
    g_recs.clear();
}

int SZxG_trace_collect(char* names, size_t names_len, double* ms, unsigned long long* counts, int max_kernels) {
    std::lock_guard<std::mutex> lk(g_mu);
    std::vector<std::string> nm;
    std::vector<double> tot;
    std::vector<unsigned long long> cnt;
    for (auto& r : g_recs) {
        cudaEventSynchronize(r.b);
        float t = 0.f;
        cudaEventElapsedTime(&t, r.a, r.b);
        size_t k = 0;
        while (k < nm.size() && nm[k] != r.name) k++;
        if (k == nm.size()) { nm.emplace_back(r.name); tot.push_back(0); cnt.push_back(0); }
        tot[k] += t;
        cnt[k] += 1;
        g_pool.push_back(r.a);
        g_pool.push_back(r.b);
    }
    g_recs.clear();
    int n = (int)nm.size() < max_kernels ? (int)nm.size() : max_kernels;
    size_t off = 0;
    for (int k = 0; k < n; k++) {
        if (ms) ms[k] = tot[k];
        if (counts) counts[k] = cnt[k];
        if (names && off + nm[k].size() + 1 < names_len) {
            memcpy(names + off, nm[k].c_str(), nm[k].size());
            off += nm[k].size();
            names[off++] = '\n';
        }
    }
    if (names && off < names_len) names[off] = 0;
    return n;
}

}  // extern "C"
