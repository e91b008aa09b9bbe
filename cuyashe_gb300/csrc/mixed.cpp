// mixed.cpp -- host side of cy_polymul_batched: one persistent launch for a
// batch of products of different rings.
//
// The reference multiplies one polynomial pair per call, re-running
// CUDAFunctions::init whenever the size changes (src/common.h:139-146) and
// synchronising after each product (src/common.h:223). Here a mixed batch of
// up to thousands of products of N = 1024..8192 and q up to 192 bits is one
// work list for one persistent kernel (k_mixed.cu); products of other rings in
// the same submission go through the per-ring path.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "host.h"

namespace cy {

void* mixed_kernel();
size_t mixed_smem_bytes();
int mixed_threads();
int trace_begin(const char* name, int logn, cudaStream_t st);
void trace_end(int idx, cudaStream_t st);

// Per-device state of the mixed path. Calls are ordered on the device through
// `last_done` (a later call's stream waits for the previous launch), so that
// the shared scratch is never used by two launches at once.
struct MixedState {
    std::mutex mu;
    uint32_t* d_resid = nullptr;
    size_t resid_words = 0;
    char* d_meta = nullptr;  // jobs, units, done counters, control words
    size_t meta_bytes = 0;
    char* h_meta = nullptr;  // pinned staging of the same
    size_t h_bytes = 0;
    cudaEvent_t meta_copied = nullptr, last_done = nullptr;
    bool launched = false;
    uint32_t* d_ctl = nullptr;  // control words of the last launch
};

static MixedState& mixed_state(int dev) {
    static std::mutex mu;
    static std::map<int, MixedState*> states;
    std::lock_guard<std::mutex> lock(mu);
    auto it = states.find(dev);
    if (it != states.end()) return *it->second;
    MixedState* s = new MixedState();  // kept until process exit
    states[dev] = s;
    return *s;
}

static bool mixable(const cy_ring* r) { return r->logn >= 10 && r->logn <= 13 && r->l32 <= 6; }

static size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

cy_status run_mixed(const std::vector<const cy_polymul_job*>& jobs, cudaStream_t st) {
    if (jobs.empty()) return CY_OK;
    int dev = 0;
    CY_CUDA(cudaGetDevice(&dev));
    MixedState& S = mixed_state(dev);
    std::lock_guard<std::mutex> lock(S.mu);
    if (!S.meta_copied) {
        CY_CUDA(cudaEventCreateWithFlags(&S.meta_copied, cudaEventDisableTiming));
        CY_CUDA(cudaEventCreateWithFlags(&S.last_done, cudaEventDisableTiming));
    }
    const int nj = (int)jobs.size();
    // residue offsets and units
    std::vector<MixedJob> mj(nj);
    std::vector<MixedUnit> ntt_units, epi_units;
    size_t words = 0;
    std::vector<size_t> offset(nj);
    for (int j = 0; j < nj; j++) {
        const cy_ring* r = jobs[j]->ring;
        offset[j] = words;
        words += (size_t)r->mul.h.k * r->n;
        // primes side by side in one 1024-thread block (8 coefficients per thread)
        const int per = r->logn == 10 ? 8 : r->logn == 11 ? 4 : r->logn == 12 ? 2 : 1;
        for (int f = 0; f < r->mul.h.k; f += per) ntt_units.push_back({j, 0, f, std::min(per, r->mul.h.k - f)});
    }
    // largest transforms first (longest units first balances the tail)
    std::stable_sort(ntt_units.begin(), ntt_units.end(), [&](const MixedUnit& x, const MixedUnit& y) {
        return jobs[x.job]->ring->logn > jobs[y.job]->ring->logn;
    });
    // epilogues in the order in which the jobs' first units appear
    std::vector<int> order;
    std::vector<char> seen(nj, 0);
    for (const MixedUnit& u : ntt_units)
        if (!seen[u.job]) {
            seen[u.job] = 1;
            order.push_back(u.job);
        }
    for (int j : order) {
        const int n = jobs[j]->ring->n;
        for (int c0 = 0; c0 < n; c0 += 2048) epi_units.push_back({j, 1, c0, std::min(2048, n - c0)});
    }
    std::vector<MixedUnit> units(ntt_units);
    units.insert(units.end(), epi_units.begin(), epi_units.end());
    const int nu = (int)units.size();

    // device scratch
    if (words > S.resid_words) {
        if (S.launched) CY_CUDA(cudaEventSynchronize(S.last_done));
        if (S.d_resid) cudaFree(S.d_resid);
        S.d_resid = nullptr;
        S.resid_words = 0;
        CY_CUDA(cudaMalloc(&S.d_resid, words * sizeof(uint32_t)));
        S.resid_words = words;
    }
    for (int j = 0; j < nj; j++) {
        const cy_ring* r = jobs[j]->ring;
        mj[j] = MixedJob{r->mul.d, jobs[j]->d_a, jobs[j]->d_b, jobs[j]->d_c, S.d_resid + offset[j],
                         r->logn,  r->mul.h.k, r->l32,       r->l64};
    }
    const size_t jobs_b = align16(sizeof(MixedJob) * nj);
    const size_t units_b = align16(sizeof(MixedUnit) * nu);
    const size_t done_b = align16(sizeof(uint32_t) * nj);
    const size_t ctl_b = 16;
    const size_t meta = jobs_b + units_b + done_b + ctl_b;
    if (meta > S.meta_bytes) {
        if (S.launched) CY_CUDA(cudaEventSynchronize(S.last_done));
        if (S.d_meta) cudaFree(S.d_meta);
        if (S.h_meta) cudaFreeHost(S.h_meta);
        S.d_meta = nullptr;
        S.h_meta = nullptr;
        S.meta_bytes = S.h_bytes = 0;
        CY_CUDA(cudaMalloc(&S.d_meta, meta));
        CY_CUDA(cudaMallocHost(&S.h_meta, meta));
        S.meta_bytes = S.h_bytes = meta;
    }
    // the previous call's copy out of the staging buffer must be done before it is rewritten
    if (S.launched) CY_CUDA(cudaEventSynchronize(S.meta_copied));
    std::memcpy(S.h_meta, mj.data(), sizeof(MixedJob) * nj);
    std::memcpy(S.h_meta + jobs_b, units.data(), sizeof(MixedUnit) * nu);
    std::memset(S.h_meta + jobs_b + units_b, 0, done_b + ctl_b);
    // device order: wait for the previous mixed launch (it may be on another stream)
    if (S.launched) CY_CUDA(cudaStreamWaitEvent(st, S.last_done, 0));
    CY_CUDA(cudaMemcpyAsync(S.d_meta, S.h_meta, meta, cudaMemcpyHostToDevice, st));
    CY_CUDA(cudaEventRecord(S.meta_copied, st));
    const MixedJob* d_jobs = reinterpret_cast<const MixedJob*>(S.d_meta);
    const MixedUnit* d_units = reinterpret_cast<const MixedUnit*>(S.d_meta + jobs_b);
    uint32_t* d_done = reinterpret_cast<uint32_t*>(S.d_meta + jobs_b + units_b);
    uint32_t* d_ctl = reinterpret_cast<uint32_t*>(S.d_meta + jobs_b + units_b + done_b);
    S.d_ctl = d_ctl;

    void* func = mixed_kernel();
    const size_t smem = mixed_smem_bytes();
    static std::mutex attr_mu;
    {
        std::lock_guard<std::mutex> l(attr_mu);
        CY_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    }
    int per_sm = 0, sms = 0;
    CY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, func, mixed_threads(), smem));
    CY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int grid = std::max(1, std::min(nu, std::max(1, per_sm) * sms));
    void* args[] = {(void*)&d_jobs, (void*)&d_units, (void*)&nu, (void*)&d_done, (void*)&d_ctl};
    const int tr = trace_begin("mixed", 0, st);
    const cudaError_t e = cudaLaunchKernel(func, dim3(grid), dim3(mixed_threads()), args, smem, st);
    trace_end(tr, st);
    if (e != cudaSuccess) return cuda_error(e, "k_mixed");
    CY_CUDA(cudaEventRecord(S.last_done, st));
    S.launched = true;
    return CY_OK;
}

cy_status mixed_status(cudaStream_t st) {
    int dev = 0;
    CY_CUDA(cudaGetDevice(&dev));
    MixedState& S = mixed_state(dev);
    std::lock_guard<std::mutex> lock(S.mu);
    if (!S.launched) return CY_OK;
    CY_CUDA(cudaStreamWaitEvent(st, S.last_done, 0));
    CY_CUDA(cudaStreamSynchronize(st));
    uint32_t ctl[2] = {0, 0};
    CY_CUDA(cudaMemcpy(ctl, S.d_ctl, sizeof(ctl), cudaMemcpyDeviceToHost));
    if (ctl[1]) return set_error(CY_ERR_TIMEOUT, "a block of the mixed batch gave up waiting for its job's NTTs");
    return CY_OK;
}

bool mixed_supported(const cy_ring* r) { return mixable(r); }

}  // namespace cy
