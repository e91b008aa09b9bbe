// mixed.cpp -- host side of the mixed batches: cy_polymul_batched (a list of
// products submitted per call) and cy_mixed_plan_* (a prepared list of products
// and YASHE multiplies, launched as one persistent kernel, capturable in a CUDA
// graph and autotuned).
//
// The reference multiplies one polynomial pair per call, re-running
// CUDAFunctions::init whenever the size changes (src/common.h:139-146) and
// synchronising after each product (src/common.h:223); a homomorphic multiply is
// a chain of such calls plus host rounding and keyswitch loops
// (src/ciphertext.cpp:38-130). Here a batch of products and HE multiplies of
// N = 1024..8192 and q up to 192 bits is one work list for one persistent
// kernel (k_mixed.cu); products of other rings submitted to cy_polymul_batched
// go through the per-ring path in the same call.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "host.h"

namespace cy {

void* mixed_kernel(int sched);
size_t mixed_smem_bytes(int sched);
int mixed_threads(int sched);
int mixed_schedules();
unsigned mixed_spin_default();
unsigned long long epi_frac_limit();
int trace_begin(const char* name, int logn, cudaStream_t st);
void trace_end(int idx, cudaStream_t st);

static bool mixable(const cy_ring* r) { return r->logn >= 10 && r->logn <= 13 && r->l32 <= 6; }
static size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

// Primes of one ring run side by side in one unit (the same for both schedules).
static int primes_per_unit(int logn) { return logn == 10 ? 8 : logn == 11 ? 4 : logn == 12 ? 2 : 1; }
constexpr int kEpiUnitCoefs = 2048;

// Job record of a product of ring r (mod-q epilogue, no keyswitch).
static MixedJob product_job(const cy_ring* r, const uint64_t* a, const uint64_t* b, uint64_t* c) {
    MixedJob J{};
    J.B = r->mul.d;
    J.a = a;
    J.b = b;
    J.c = c;
    J.logn = r->logn;
    J.k = r->mul.h.k;
    J.l32 = r->l32;
    J.l64 = r->l64;
    J.mode = EPI_MODQ;
    J.centered = 0;
    J.n_epi = (r->n + kEpiUnitCoefs - 1) / kEpiUnitCoefs;
    J.need0 = J.k;
    return J;
}

// Job record of a YASHE multiply of y (tensor + rounding, keyswitch if relin).
static MixedJob yashe_job(const cy_yashe* y, const uint64_t* c1, const uint64_t* c2, uint64_t* out, bool relin) {
    const cy_ring* r = y->ring;
    MixedJob J{};
    J.B = y->tensor.d;
    J.B2 = relin ? y->relin.d : nullptr;
    J.a = c1;
    J.b = c2;
    J.c = out;
    J.evk = relin ? y->d_evk : nullptr;
    J.logn = r->logn;
    J.k = y->tensor.h.k;
    J.l32 = r->l32;
    J.l64 = r->l64;
    J.mode = EPI_YASHE;
    J.centered = 1;
    J.k2 = relin ? y->relin.h.k : 0;
    J.ell = relin ? y->ell : 0;
    J.n_epi = (r->n + kEpiUnitCoefs - 1) / kEpiUnitCoefs;
    J.need0 = J.k;
    return J;
}

// The work list: every job's transform units (largest transforms first), the
// first epilogues in the order the jobs first appear, the keyswitch transforms
// (largest first), the keyswitch epilogues. A unit only waits for units of its
// job in earlier phases, which lie earlier in the list.
static std::vector<MixedUnit> build_units(const std::vector<MixedJob>& jobs) {
    const int nj = (int)jobs.size();
    auto transform_units = [&](int kind) {
        std::vector<MixedUnit> out;
        for (int j = 0; j < nj; j++) {
            const int k = kind == 0 ? jobs[j].k : jobs[j].k2;
            const int per = primes_per_unit(jobs[j].logn);
            for (int f = 0; f < k; f += per) out.push_back({j, kind, f, std::min(per, k - f)});
        }
        std::stable_sort(out.begin(), out.end(), [&](const MixedUnit& x, const MixedUnit& y) {
            return jobs[x.job].logn > jobs[y.job].logn;  // longest units first balances the tail
        });
        return out;
    };
    auto epilogue_units = [&](const std::vector<MixedUnit>& after, int kind) {
        std::vector<MixedUnit> out;
        std::vector<char> seen(nj, 0);
        for (const MixedUnit& u : after) {
            if (seen[u.job]) continue;
            seen[u.job] = 1;
            const int n = 1 << jobs[u.job].logn;
            for (int c0 = 0; c0 < n; c0 += kEpiUnitCoefs) out.push_back({u.job, kind, c0, std::min(kEpiUnitCoefs, n - c0)});
        }
        return out;
    };
    std::vector<MixedUnit> a = transform_units(0), b = epilogue_units(a, 1);
    std::vector<MixedUnit> c = transform_units(2), d = epilogue_units(c, 3);
    std::vector<MixedUnit> units;
    units.reserve(a.size() + b.size() + c.size() + d.size());
    for (auto* v : {&a, &b, &c, &d}) units.insert(units.end(), v->begin(), v->end());
    return units;
}

// residue words of job j in the batch scratch
static size_t resid_words(const MixedJob& J) { return (size_t)std::max(J.k, J.k2) << J.logn; }

static cy_status set_smem_attr(int sched) {
    static std::mutex mu;
    std::lock_guard<std::mutex> l(mu);
    CY_CUDA(cudaFuncSetAttribute(mixed_kernel(sched), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)mixed_smem_bytes(sched)));
    return CY_OK;
}

static cy_status persistent_grid(int sched, int dev, int n_units, int* grid) {
    CY_TRY(set_smem_attr(sched));
    int per_sm = 0, sms = 0;
    CY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mixed_kernel(sched), mixed_threads(sched),
                                                          mixed_smem_bytes(sched)));
    CY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    *grid = std::max(1, std::min(n_units, std::max(1, per_sm) * sms));
    return CY_OK;
}

static cy_status launch_mixed(int sched, int grid, const MixedJob* d_jobs, const MixedUnit* d_units, int nu,
                              uint32_t* d_done, uint32_t* d_ctl, unsigned spin, cudaStream_t st) {
    unsigned long long fl = epi_frac_limit();
    void* args[] = {(void*)&d_jobs, (void*)&d_units, (void*)&nu, (void*)&d_done, (void*)&d_ctl, (void*)&spin,
                    (void*)&fl};
    const int tr = trace_begin("mixed", 0, st);
    const cudaError_t e = cudaLaunchKernel(mixed_kernel(sched), dim3(grid), dim3(mixed_threads(sched)), args,
                                           mixed_smem_bytes(sched), st);
    trace_end(tr, st);
    if (e != cudaSuccess) return cuda_error(e, "k_mixed");
    return CY_OK;
}

// ---- cy_polymul_batched: a list of products per call ------------------------------

// Per-device state of the per-call path. Calls are ordered on the device through
// `last_done` (a later call's stream waits for the previous launch), so that the
// shared scratch is never used by two launches at once.
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
    std::vector<MixedJob> mj(nj);
    std::vector<size_t> offset(nj);
    size_t words = 0;
    for (int j = 0; j < nj; j++) {
        mj[j] = product_job(jobs[j]->ring, jobs[j]->d_a, jobs[j]->d_b, jobs[j]->d_c);
        offset[j] = words;
        words += resid_words(mj[j]);
    }
    const std::vector<MixedUnit> units = build_units(mj);
    const int nu = (int)units.size();
    if (words > S.resid_words) {
        if (S.launched) CY_CUDA(cudaEventSynchronize(S.last_done));
        if (S.d_resid) cudaFree(S.d_resid);
        S.d_resid = nullptr;
        S.resid_words = 0;
        CY_CUDA(cudaMalloc(&S.d_resid, words * sizeof(uint32_t)));
        S.resid_words = words;
    }
    for (int j = 0; j < nj; j++) mj[j].resid = S.d_resid + offset[j];
    const size_t jobs_b = align16(sizeof(MixedJob) * nj);
    const size_t units_b = align16(sizeof(MixedUnit) * nu);
    const size_t done_b = align16(sizeof(uint32_t) * 4 * nj);
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
    int grid = 1;
    CY_TRY(persistent_grid(0, dev, nu, &grid));
    CY_TRY(launch_mixed(0, grid, d_jobs, d_units, nu, d_done, d_ctl, mixed_spin_default(), st));
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

using namespace cy;

// ---- cy_mixed_plan: a prepared batch ---------------------------------------------
struct cy_mixed_plan {
    int device = 0;
    std::vector<MixedJob> jobs;      // host copy of the job records (device pointers)
    std::vector<uint64_t*> outs;     // output buffers, for the autotuner's comparison
    std::vector<size_t> out_words;
    int n_units = 0;
    int sched = 0;
    int grid[2] = {1, 1};
    unsigned spin = 0;
    uint32_t* d_resid = nullptr;
    char* d_meta = nullptr;  // jobs, units
    uint32_t* d_done = nullptr;  // 4 counters per job, then 4 control words
    size_t done_bytes = 0;
    ~cy_mixed_plan() {
        if (d_resid) cudaFree(d_resid);
        if (d_meta) cudaFree(d_meta);
        if (d_done) cudaFree(d_done);
    }
};

static cy_status check_buffers(const void* a, const void* b, const void* c) {
    if (!a || !b || !c) return set_error(CY_ERR_INVALID_ARGUMENT, "NULL buffer in a mixed job");
    if (((uintptr_t)a | (uintptr_t)b | (uintptr_t)c) & 15)
        return set_error(CY_ERR_INVALID_ARGUMENT, "mixed job buffers must be 16-byte aligned");
    if (c == a || c == b) return set_error(CY_ERR_INVALID_ARGUMENT, "a mixed plan's outputs must not be its inputs");
    return CY_OK;
}

extern "C" {

cy_status cy_mixed_plan_create(const cy_mixed_job* jobs, int njobs, cy_mixed_plan** out) {
    if (!out || njobs < 1 || !jobs) return set_error(CY_ERR_INVALID_ARGUMENT, "bad job list");
    *out = nullptr;
    std::unique_ptr<cy_mixed_plan> P(new cy_mixed_plan());
    CY_CUDA(cudaGetDevice(&P->device));
    for (int i = 0; i < njobs; i++) {
        const cy_mixed_job& q = jobs[i];
        if ((q.ring == nullptr) == (q.yashe == nullptr))
            return set_error(CY_ERR_INVALID_ARGUMENT, "a mixed job names a ring or a YASHE scheme (one of them)");
        CY_TRY(check_buffers(q.d_a, q.d_b, q.d_c));
        const cy_ring* r = q.ring ? q.ring : q.yashe->ring;
        if (r->device != P->device) return set_error(CY_ERR_INVALID_ARGUMENT, "job of another CUDA device");
        if (!mixable(r))
            return set_error(CY_ERR_UNSUPPORTED, "mixed plans take N = 1024..8192 and q of up to 192 bits (job " +
                                                     std::to_string(i) + ")");
        if (q.yashe && q.relin && !q.yashe->d_evk) return set_error(CY_ERR_NO_KEYS, "YASHE job without keys");
        MixedJob J = q.ring ? product_job(q.ring, q.d_a, q.d_b, q.d_c)
                            : yashe_job(q.yashe, q.d_a, q.d_b, q.d_c, q.relin != 0);
        P->jobs.push_back(J);
        P->outs.push_back(q.d_c);
        P->out_words.push_back((size_t)r->n * r->l64);
    }
    const std::vector<MixedUnit> units = build_units(P->jobs);
    P->n_units = (int)units.size();
    size_t words = 0;
    for (const MixedJob& J : P->jobs) words += resid_words(J);
    CY_CUDA(cudaMalloc(&P->d_resid, words * sizeof(uint32_t)));
    size_t off = 0;
    for (MixedJob& J : P->jobs) {
        J.resid = P->d_resid + off;
        off += resid_words(J);
    }
    const size_t jobs_b = align16(sizeof(MixedJob) * njobs);
    const size_t units_b = align16(sizeof(MixedUnit) * units.size());
    CY_CUDA(cudaMalloc(&P->d_meta, jobs_b + units_b));
    CY_CUDA(cudaMemcpy(P->d_meta, P->jobs.data(), sizeof(MixedJob) * njobs, cudaMemcpyHostToDevice));
    CY_CUDA(cudaMemcpy(P->d_meta + jobs_b, units.data(), sizeof(MixedUnit) * units.size(), cudaMemcpyHostToDevice));
    P->done_bytes = sizeof(uint32_t) * (4 * (size_t)njobs + 4);
    CY_CUDA(cudaMalloc(&P->d_done, P->done_bytes));
    for (int s = 0; s < mixed_schedules(); s++) CY_TRY(persistent_grid(s, P->device, P->n_units, &P->grid[s]));
    P->spin = mixed_spin_default();
    *out = P.release();
    return CY_OK;
}

cy_status cy_mixed_plan_destroy(cy_mixed_plan* plan) {
    delete plan;
    return CY_OK;
}

cy_status cy_mixed_plan_launch(cy_mixed_plan* P, cy_stream_t stream) {
    if (!P) return set_error(CY_ERR_INVALID_ARGUMENT, "plan is NULL");
    int dev = -1;
    CY_CUDA(cudaGetDevice(&dev));
    if (dev != P->device) return set_error(CY_ERR_INVALID_ARGUMENT, "plan belongs to another CUDA device");
    cudaStream_t st = (cudaStream_t)stream;
    CY_CUDA(cudaMemsetAsync(P->d_done, 0, P->done_bytes, st));
    const size_t jobs_b = align16(sizeof(MixedJob) * P->jobs.size());
    const MixedJob* d_jobs = reinterpret_cast<const MixedJob*>(P->d_meta);
    const MixedUnit* d_units = reinterpret_cast<const MixedUnit*>(P->d_meta + jobs_b);
    uint32_t* d_ctl = P->d_done + 4 * P->jobs.size();
    return launch_mixed(P->sched, P->grid[P->sched], d_jobs, d_units, P->n_units, P->d_done, d_ctl, P->spin, st);
}

cy_status cy_mixed_plan_status(cy_mixed_plan* P, cy_stream_t stream) {
    if (!P) return set_error(CY_ERR_INVALID_ARGUMENT, "plan is NULL");
    CY_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    uint32_t ctl[4] = {0, 0, 0, 0};
    CY_CUDA(cudaMemcpy(ctl, P->d_done + 4 * P->jobs.size(), sizeof(ctl), cudaMemcpyDeviceToHost));
    if (ctl[1])
        return set_error(CY_ERR_TIMEOUT, "a block of the mixed batch gave up waiting for earlier units of its job (" +
                                             std::to_string(ctl[2]) + " units skipped)");
    return CY_OK;
}

cy_status cy_mixed_plan_set_schedule(cy_mixed_plan* P, int schedule) {
    if (!P || schedule < 0 || schedule >= mixed_schedules())
        return set_error(CY_ERR_INVALID_ARGUMENT, "schedule must be 0 or 1");
    P->sched = schedule;
    return CY_OK;
}

cy_status cy_mixed_plan_get_schedule(const cy_mixed_plan* P, int* schedule) {
    if (!P || !schedule) return set_error(CY_ERR_INVALID_ARGUMENT, "NULL argument");
    *schedule = P->sched;
    return CY_OK;
}

cy_status cy_mixed_plan_autotune(cy_mixed_plan* P, cy_stream_t stream) {
    if (!P) return set_error(CY_ERR_INVALID_ARGUMENT, "plan is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    size_t total = 0;
    for (size_t w : P->out_words) total += w;
    std::vector<uint64_t> ref(total), cur(total);
    auto fetch = [&](std::vector<uint64_t>& dst) -> cy_status {
        CY_CUDA(cudaStreamSynchronize(st));
        size_t off = 0;
        for (size_t j = 0; j < P->outs.size(); j++) {
            CY_CUDA(cudaMemcpy(dst.data() + off, P->outs[j], P->out_words[j] * 8, cudaMemcpyDeviceToHost));
            off += P->out_words[j];
        }
        return CY_OK;
    };
    cudaEvent_t e0, e1;
    CY_CUDA(cudaEventCreate(&e0));
    CY_CUDA(cudaEventCreate(&e1));
    float best = 0;
    int best_s = 0;
    cy_status status = CY_OK;
    for (int s = 0; s < mixed_schedules() && status == CY_OK; s++) {
        P->sched = s;
        status = cy_mixed_plan_launch(P, stream);
        if (status == CY_OK) status = cy_mixed_plan_status(P, stream);
        if (status == CY_OK) status = fetch(s == 0 ? ref : cur);
        if (status == CY_OK && s > 0 && std::memcmp(ref.data(), cur.data(), total * 8) != 0)
            status = set_error(CY_ERR_INTERNAL, "autotune: the mixed schedules disagree");
        if (status != CY_OK) break;
        cudaEventRecord(e0, st);
        for (int r = 0; r < 3 && status == CY_OK; r++) status = cy_mixed_plan_launch(P, stream);
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (s == 0 || ms < best) {
            best = ms;
            best_s = s;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    P->sched = best_s;
    return status;
}

cy_status cy_mixed_plan_test_starve(cy_mixed_plan* P, int job, unsigned spin_limit) {
    if (!P || job < 0 || job >= (int)P->jobs.size() || spin_limit < 1)
        return set_error(CY_ERR_INVALID_ARGUMENT, "bad argument");
    P->jobs[job].need0 = P->jobs[job].k + 1;  // one more prime than the job has: never reached
    P->spin = spin_limit;
    CY_CUDA(cudaMemcpy(P->d_meta + sizeof(MixedJob) * job, &P->jobs[job], sizeof(MixedJob), cudaMemcpyHostToDevice));
    return CY_OK;
}

}  // extern "C"
