// trace.cpp -- launch accounting and opt-in per-kernel CUDA-event tracing.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "host.h"

namespace cy {

static std::atomic<uint64_t> g_launches{0};
static std::atomic<bool> g_trace_on{false};
static std::mutex g_mu;

struct TraceRecord {
    std::string name;
    cudaEvent_t start, stop;
};
static std::vector<TraceRecord> g_records;

// Called by every launch: counts it and, when tracing, records its start event.
int trace_begin(const char* name, int logn, cudaStream_t st) {
    g_launches.fetch_add(1, std::memory_order_relaxed);
    if (!g_trace_on.load(std::memory_order_relaxed)) return -1;
    TraceRecord r;
    char buf[48];
    if (logn > 0) std::snprintf(buf, sizeof(buf), "%s_n%d", name, 1 << logn);
    else std::snprintf(buf, sizeof(buf), "%s", name);
    r.name = buf;
    if (cudaEventCreate(&r.start) != cudaSuccess) return -1;
    if (cudaEventCreate(&r.stop) != cudaSuccess) {
        cudaEventDestroy(r.start);
        return -1;
    }
    cudaEventRecord(r.start, st);
    std::lock_guard<std::mutex> lock(g_mu);
    g_records.push_back(r);
    return (int)g_records.size() - 1;
}

void trace_end(int idx, cudaStream_t st) {
    if (idx < 0) return;
    std::lock_guard<std::mutex> lock(g_mu);
    if ((size_t)idx < g_records.size()) cudaEventRecord(g_records[idx].stop, st);
}

}  // namespace cy

using namespace cy;

extern "C" {

uint64_t cy_launch_count(void) { return g_launches.load(); }

cy_status cy_trace_start(void) {
    std::lock_guard<std::mutex> lock(g_mu);
    for (auto& r : g_records) {
        cudaEventDestroy(r.start);
        cudaEventDestroy(r.stop);
    }
    g_records.clear();
    g_trace_on = true;
    return CY_OK;
}

cy_status cy_trace_stop(cy_trace_entry* entries, int max_entries, int* n_entries) {
    g_trace_on = false;
    std::lock_guard<std::mutex> lock(g_mu);
    std::map<std::string, std::pair<int, double>> agg;
    cy_status st = CY_OK;
    for (auto& r : g_records) {
        float ms = 0.f;
        cudaError_t e = cudaEventSynchronize(r.stop);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, r.start, r.stop);
        if (e != cudaSuccess && st == CY_OK) st = cuda_error(e, "cy_trace_stop");
        auto& a = agg[r.name];
        a.first += 1;
        a.second += ms;
        cudaEventDestroy(r.start);
        cudaEventDestroy(r.stop);
    }
    g_records.clear();
    int n = 0;
    for (auto& kv : agg) {
        if (entries && n < max_entries) {
            std::memset(&entries[n], 0, sizeof(cy_trace_entry));
            std::strncpy(entries[n].name, kv.first.c_str(), sizeof(entries[n].name) - 1);
            entries[n].launches = kv.second.first;
            entries[n].total_ms = kv.second.second;
        }
        n++;
    }
    if (n_entries) *n_entries = n;
    return st;
}

}  // extern "C"
