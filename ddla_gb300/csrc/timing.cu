// Optional per-launch device timing of kernel classes, used by the benchmark
// to report the dominant kernel's achieved throughput against its roofline.
// When enabled, the drivers bracket each launch of a class with CUDA events on
// the launching stream; durations are summed when read.
#include <mutex>
#include <vector>

#include "common.cuh"
#include "timing.cuh"

namespace ddla {

namespace {
struct Rec {
    int cls;
    cudaEvent_t e0, e1;
    double flops, bytes;
};
std::mutex g_mu;
bool g_on = false;
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

bool timing_on() { return g_on; }

Timed::Timed(cudaStream_t s, int cls, double flops, double bytes) : s_(s), idx_(-1) {
    if (!g_on) return;
    std::lock_guard<std::mutex> g(g_mu);
    Rec r{cls, take_event(), take_event(), flops, bytes};
    cudaEventRecord(r.e0, s);
    g_recs.push_back(r);
    idx_ = (int)g_recs.size() - 1;
}

Timed::~Timed() {
    if (idx_ < 0) return;
    std::lock_guard<std::mutex> g(g_mu);
    if (idx_ < (int)g_recs.size()) cudaEventRecord(g_recs[idx_].e1, s_);
}

}  // namespace ddla

using namespace ddla;

extern "C" int ddla_timing_enable(int on) {
    std::lock_guard<std::mutex> g(g_mu);
    for (auto &r : g_recs) {
        cudaEventSynchronize(r.e1);
        g_pool.push_back(r.e0);
        g_pool.push_back(r.e1);
    }
    g_recs.clear();
    g_on = on != 0;
    return 0;
}

extern "C" int ddla_timing_read(int cls, double *total_ms, int64_t *launches, double *flops, double *bytes) {
    std::lock_guard<std::mutex> g(g_mu);
    double ms = 0, fl = 0, by = 0;
    int64_t n = 0;
    for (auto &r : g_recs) {
        if (r.cls != cls) continue;
        DDLA_CUDA(cudaEventSynchronize(r.e1));
        float t = 0;
        DDLA_CUDA(cudaEventElapsedTime(&t, r.e0, r.e1));
        ms += t;
        fl += r.flops;
        by += r.bytes;
        n++;
    }
    if (total_ms) *total_ms = ms;
    if (launches) *launches = n;
    if (flops) *flops = fl;
    if (bytes) *bytes = by;
    return 0;
}
