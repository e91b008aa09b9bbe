// api.cpp -- the extern "C" boundary (include/cuyashe.h).
//
// Launch sequence of one product batch, per chunk of jobs:
//   k_mul / k_keyswitch  grid (k primes, jobs)  -> residues in the workspace
//   k_epi                grid (jobs * N / 256)  -> limbs (or plaintext words)
// all on the caller's stream, no host synchronisation, no allocation once the
// workspace has grown to the chunk size. The reference allocates 4 residue
// buffers per product and synchronises the device after every operation
// (src/cuda_functions.cu:670-738, src/common.h:223).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <map>
#include <mutex>
#include <set>
#include <tuple>
#include <utility>
#include <vector>

#include "host.h"

namespace cy {

const char* last_error_message();
void* addsub_kernel(int l64, bool sub);
void* crt_kernel();
void* shoup_pairs_kernel();
void* evk_rows_kernel();

static constexpr int kEpiThreads = 256;
// blocks of the epilogue kernel for `coefs` coefficients of a q of l32 words
static unsigned epi_blocks(long long coefs, int l32) {
    const long long per = (long long)kEpiThreads * epi_coefs_per_thread(l32);
    return (unsigned)((coefs + per - 1) / per);
}

int trace_begin(const char* name, int logn, cudaStream_t st);
void trace_end(int idx, cudaStream_t st);

// Jobs per launch: the residue scratch of one chunk (k residues of N words per
// job) is kept near CY_CHUNK_BYTES (default 24 MiB) so that it stays in L2
// between the NTT kernel that writes it and the epilogue that reads it.
static long long chunk_bytes() {
    static long long v = [] {
        const char* e = std::getenv("CY_CHUNK_BYTES");
        long long x = e ? std::atoll(e) : 0;
        return x > 0 ? x : (24ll << 20);
    }();
    return v;
}
int chunk_jobs(int n, int k) {
    long long c = chunk_bytes() / ((long long)n * k * 4);
    if (c < 1) c = 1;
    if (c > 65535) c = 65535;
    return (int)c;
}

static cy_status ensure_smem(void* func, size_t bytes) {
    static std::mutex mu;
    static std::set<std::pair<void*, int>> done;
    int dev = 0;
    CY_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    if (done.count({func, dev})) return CY_OK;
    if (bytes > 48 * 1024) CY_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    done.insert({func, dev});
    return CY_OK;
}

// Blocks of `func` (with `threads` threads and `smem` bytes of dynamic shared
// memory) resident on the whole device at once; 0 if it cannot be queried.
static int resident_blocks(void* func, int threads, size_t smem) {
    static std::mutex mu;
    static std::map<std::tuple<void*, int, int>, int> cache;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    {
        std::lock_guard<std::mutex> lock(mu);
        auto it = cache.find(std::make_tuple(func, dev, threads));
        if (it != cache.end()) return it->second;
    }
    int sms = 0, per_sm = 0;
    if (ensure_smem(func, smem) != CY_OK || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, func, threads, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    std::lock_guard<std::mutex> lock(mu);
    return cache[std::make_tuple(func, dev, threads)] = per_sm * sms;
}

// A chunk of `jobs` cut to whole waves of a kernel that runs `per_job` blocks per
// job, so that its last wave is not a tail: up to the next whole wave when that is
// at most a quarter more (the size target is soft), else down (unchanged when it
// holds less than one wave). At N = 4096 with the 64-coefficient keyswitch: 912
// slots, 6 blocks per job, chunks of 152 jobs instead of 170 (2.91 against 2.97 ms
// per 4096-pair HE multiply step). CY_WAVE_CHUNKS=0 turns this off.
static int wave_chunk(int jobs, void* func, int threads, size_t smem, int per_job) {
    static const bool on = [] {
        const char* e = std::getenv("CY_WAVE_CHUNKS");
        return !(e && std::atoi(e) == 0);
    }();
    const int w = (on && per_job > 0) ? resident_blocks(func, threads, smem) / per_job : 0;
    if (w < 1 || jobs <= w) return jobs;
    const long long up = ((long long)jobs + w - 1) / w * w;
    if (4 * up <= 5ll * jobs && up <= 65535) return (int)up;
    return jobs / w * w;
}

static cy_status launch(void* func, const char* name, int logn, dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                        void** args) {
    if (!func) return set_error(CY_ERR_INTERNAL, "missing kernel instantiation");
    CY_TRY(ensure_smem(func, smem));
    const int tr = trace_begin(name, logn, st);
    const cudaError_t e = cudaLaunchKernel(func, grid, block, args, smem, st);
    trace_end(tr, st);
    if (e != cudaSuccess) return cuda_error(e, name);
    return CY_OK;
}

// Fixed-point YASHE rounding: coefficients whose estimate has a fraction at or
// above this limit take the exact path (0: every coefficient does).
static std::atomic<int> g_epi_exact{0};
unsigned long long epi_frac_limit() { return g_epi_exact.load() ? 0ull : 0xFFFFFFF000000000ull; }

static const char* epi_name(int mode) {
    return mode == EPI_YASHE ? "epi_yashe" : mode == EPI_DECRYPT ? "epi_decrypt" : "epi_modq";
}

// Epilogues specialised for the basis's prime count are used unless this is set.
static std::atomic<int> g_epi_generic{0};

// ICRT epilogue of basis B over `nj` jobs of residues [job][k][N] into `out`: the
// kernel specialised for B's prime count (constants passed by value) when there
// is one, else the generic kernel.
// lm: outputs limb-major ([job][limb][N]), for the keyswitch that follows in an
// HE multiply (its digit loads then cover consecutive words)
static cy_status launch_epi(const Basis& B, const uint32_t* resid, void* out, int nj, cudaStream_t st,
                            const char* name, int lm = 0) {
    const BasisDev* Bd = B.d;
    unsigned long long fl = epi_frac_limit();
    const long long coefs = (long long)nj * B.h.n;
    if (B.epi && !g_epi_generic.load()) {
        const long long per = (long long)kEpiThreads * B.epi->coefs_per_thread;
        void* args[] = {(void*)B.epi_param.data(), (void*)&Bd, (void*)&resid, (void*)&out, (void*)&nj, (void*)&fl,
                        (void*)&lm};
        return launch(B.epi->func, name, B.h.logn, dim3((unsigned)((coefs + per - 1) / per)), dim3(kEpiThreads), 0,
                      st, args);
    }
    void* args[] = {(void*)&Bd, (void*)&resid, (void*)&out, (void*)&nj, (void*)&fl, (void*)&lm};
    return launch(epi_kernel(B.h.l32, B.h.mode), name, B.h.logn, dim3(epi_blocks(coefs, B.h.l32)), dim3(kEpiThreads),
                  0, st, args);
}

static cy_status check_device(int device) {
    int cur = -1;
    CY_CUDA(cudaGetDevice(&cur));
    if (cur != device) return set_error(CY_ERR_INVALID_ARGUMENT, "handle belongs to another CUDA device");
    return CY_OK;
}

int tuned_variant(int logn, int l64, int op);
cy_status run_mixed(const std::vector<const cy_polymul_job*>& jobs, cudaStream_t st);
cy_status mixed_status(cudaStream_t st);
bool mixed_supported(const cy_ring* r);

// Lanes for a call of several chunks: lane 0 is the caller's stream with the
// workspace's scratch, lanes 1.. side streams of the workspace with their own
// scratch. Chunk c runs on lane c mod lanes (one chunk's kernels fill the tails
// of the others'); begin() orders the side streams after the caller's work,
// end() orders the caller's stream after theirs. The lane count is
// CY_CHUNK_LANES (1 .. 1 + kMaxSide, default 3: measured 3.01-3.04 ms per 4096-pair
// HE multiply step against 3.08 with two lanes and 3.62 with one); cy_set_chunk_overlap(0)
// makes it 1.
static std::atomic<int> g_two_lanes{1};

static int lane_count() {
    static const int v = [] {
        const char* e = std::getenv("CY_CHUNK_LANES");
        const int x = e ? std::atoi(e) : 3;
        return x < 1 ? 1 : (x > 1 + kMaxSide ? 1 + kMaxSide : x);
    }();
    return g_two_lanes.load() ? v : 1;
}

struct Lanes {
    cudaStream_t s[1 + kMaxSide] = {};
    uint32_t* resid[1 + kMaxSide] = {};
    int n = 1;
    cy_status begin(Workspace& ws, cudaStream_t st, size_t words, int nchunks) {
        CY_TRY(ws.reserve(words));
        s[0] = st;
        resid[0] = ws.d_resid;
        n = std::min(nchunks, lane_count());
        if (n < 1) n = 1;
        if (n == 1) return CY_OK;
        for (int i = 0; i < n - 1; i++) CY_TRY(ws.reserve_side(i, words));
        CY_CUDA(cudaEventRecord(ws.fork, st));
        for (int i = 0; i < n - 1; i++) {
            CY_CUDA(cudaStreamWaitEvent(ws.side[i], ws.fork, 0));
            s[1 + i] = ws.side[i];
            resid[1 + i] = ws.d_side_resid[i];
        }
        return CY_OK;
    }
    cudaStream_t stream(int c) const { return s[c % n]; }
    uint32_t* scratch(int c) const { return resid[c % n]; }
    cy_status end(Workspace& ws, cudaStream_t st, cy_status status) {
        cudaError_t err = cudaSuccess;
        for (int i = 0; i < n - 1; i++) {
            cudaError_t e = cudaEventRecord(ws.join[i], ws.side[i]);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(st, ws.join[i], 0);
            if (err == cudaSuccess) err = e;
        }
        if (status != CY_OK) return status;
        if (err != cudaSuccess) return cuda_error(err, "joining the side streams");
        return CY_OK;
    }
};

// One chunk of products with basis B: out_j = epilogue(a_j * b_j), residues in
// `resid`; lm: outputs limb-major.
static cy_status product_chunk(const Basis& B, const KernelSet& ks, bool centered, const uint64_t* aj,
                               long long a_stride, const uint64_t* bj, long long b_stride, void* oj, int nj,
                               uint32_t* resid, cudaStream_t st, int lm = 0) {
    const int k = B.h.k;
    const BasisDev* Bd = B.d;
    void* args[] = {(void*)&Bd, (void*)&aj, (void*)&a_stride, (void*)&bj, (void*)&b_stride, (void*)&resid};
    CY_TRY(launch(ks.mul_for(B.h.l64, centered), centered ? "mul_centered" : "mul", B.h.logn,
                  dim3(k * ks.blocks_per_prime, nj), dim3(ks.threads), ks.smem_mul, st, args));
    return launch_epi(B, resid, oj, nj, st, epi_name(B.h.mode), lm);
}

// One chunk of keyswitches c_j -> out_j (out may alias c), residues in `resid`;
// lm: c is limb-major ([job][limb][N]).
static cy_status keyswitch_chunk(const Basis& B, const KernelSet& ks, int sel, const uint64_t* cj, const uint2* evk,
                                 int ell, uint64_t* oj, int nj, uint32_t* resid, cudaStream_t st, int lm = 0) {
    const int k = B.h.k;
    const BasisDev* Bd = B.d;
    int cs = lm ? 1 : B.h.l64, ls = lm ? B.h.n : 1;  // limb w of coefficient i at [i * cs + w * ls]
    void* args[] = {(void*)&Bd, (void*)&cj, (void*)&evk, (void*)&ell, (void*)&resid, (void*)&cs, (void*)&ls};
    CY_TRY(launch(ks.ks_for(B.h.l64, sel), "keyswitch", B.h.logn, dim3(k * ks.blocks_per_prime, nj),
                  dim3(ks.threads), ks.smem_ks[sel], st, args));
    return launch_epi(B, resid, oj, nj, st, epi_name(B.h.mode));
}

static cy_status keyswitch_digits_per_pass(const KernelSet& ks, int ell, int* sel) {
    int maxsm = 0, dev = 0;
    CY_CUDA(cudaGetDevice(&dev));
    CY_CUDA(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    *sel = (ell % 4 == 0 && ks.smem_ks[1] <= (size_t)maxsm) ? 1 : 0;
    return CY_OK;
}

// a product chunk cut to whole waves of the product kernel
static int product_chunk_jobs(const Basis& B, const KernelSet& ks, bool centered, int jobs) {
    return wave_chunk(jobs, ks.mul_for(B.h.l64, centered), ks.threads, ks.smem_mul, B.h.k * ks.blocks_per_prime);
}

// products of `batch` jobs with basis B: out_j = epilogue(a_j * b_j); `variant`
// selects the NTT schedule (-1: the tuned one for this device and size)
static cy_status run_product(const Basis& B, bool centered, const uint64_t* a, long long a_stride,
                             const uint64_t* b, long long b_stride, void* out, long long out_stride, int batch,
                             Workspace& ws, cudaStream_t st, int variant = -1) {
    if (batch == 0) return CY_OK;
    const KernelSet& ks = kernel_variant(
        B.h.logn, variant >= 0 ? variant : tuned_variant(B.h.logn, B.h.l64, centered ? TUNE_MULC : TUNE_MUL));
    const int n = B.h.n, k = B.h.k;
    const int chunk = product_chunk_jobs(B, ks, centered, std::min(batch, chunk_jobs(n, k)));
    const int nchunks = (batch + chunk - 1) / chunk;
    Lanes L;
    CY_TRY(L.begin(ws, st, (size_t)chunk * k * n, nchunks));
    cy_status status = CY_OK;
    for (int c = 0; c < nchunks && status == CY_OK; c++) {
        const int j0 = c * chunk, nj = std::min(chunk, batch - j0);
        status = product_chunk(B, ks, centered, a + (size_t)j0 * a_stride, a_stride, b + (size_t)j0 * b_stride,
                               b_stride, (char*)out + (size_t)j0 * out_stride * sizeof(uint64_t), nj, L.scratch(c),
                               L.stream(c));
    }
    return L.end(ws, st, status);
}

// keyswitch of `batch` polynomials c_j -> out_j (may alias c)
// chunk_k > 0 sizes the chunks as for a basis of that many primes (the tuner
// uses the HE multiply's chunks, which are sized by its larger basis).
// lm: c is limb-major (the tuner times the layout of the HE multiply's keyswitch)
static cy_status run_keyswitch(const Basis& B, const uint64_t* c, const uint2* evk, int ell, uint64_t* out,
                               int batch, Workspace& ws, cudaStream_t st, int variant = -1, int chunk_k = 0,
                               int lm = 0) {
    if (batch == 0) return CY_OK;
    const KernelSet& ks =
        kernel_variant(B.h.logn, variant >= 0 ? variant : tuned_variant(B.h.logn, B.h.l64, TUNE_KS));
    const int n = B.h.n, k = B.h.k, l64 = B.h.l64;
    int sel = 0;
    CY_TRY(keyswitch_digits_per_pass(ks, ell, &sel));
    const int chunk = wave_chunk(std::min(batch, chunk_jobs(n, chunk_k > 0 ? std::max(k, chunk_k) : k)),
                                 ks.ks_for(l64, sel), ks.threads, ks.smem_ks[sel], k * ks.blocks_per_prime);
    const int nchunks = (batch + chunk - 1) / chunk;
    Lanes L;
    CY_TRY(L.begin(ws, st, (size_t)chunk * k * n, nchunks));
    cy_status status = CY_OK;
    for (int cc = 0; cc < nchunks && status == CY_OK; cc++) {
        const int j0 = cc * chunk, nj = std::min(chunk, batch - j0);
        status = keyswitch_chunk(B, ks, sel, c + (size_t)j0 * n * l64, evk, ell, out + (size_t)j0 * n * l64, nj,
                                 L.scratch(cc), L.stream(cc), lm);
    }
    return L.end(ws, st, status);
}

// The HE multiply of `batch` pairs: per chunk, the tensor product with the
// YASHE rounding into out, then (relin) its keyswitch in place; chunks alternate
// between two lanes.
// ks_variant >= 0 forces the keyswitch schedule (the autotuner's timing runs).
cy_status run_yashe_mul(const Basis& tensor, const Basis& relin, const uint2* evk, int ell, const uint64_t* c1,
                        const uint64_t* c2, uint64_t* out, int batch, bool do_relin, Workspace& ws, cudaStream_t st,
                        int ks_variant) {
    if (batch == 0) return CY_OK;
    const int n = tensor.h.n, l64 = tensor.h.l64;
    const KernelSet& kt = kernel_variant(tensor.h.logn, tuned_variant(tensor.h.logn, l64, TUNE_MULC));
    const KernelSet& kr = kernel_variant(
        relin.h.logn, ks_variant >= 0 ? ks_variant : tuned_variant(relin.h.logn, l64, TUNE_KS));
    const int kmax = std::max(tensor.h.k, do_relin ? relin.h.k : 0);
    int sel = 0;
    if (do_relin) CY_TRY(keyswitch_digits_per_pass(kr, ell, &sel));
    int chunk = std::min(batch, chunk_jobs(n, kmax));
    if (do_relin)  // whole waves of the keyswitch
        chunk = wave_chunk(chunk, kr.ks_for(l64, sel), kr.threads, kr.smem_ks[sel], relin.h.k * kr.blocks_per_prime);
    const int nchunks = (batch + chunk - 1) / chunk;
    const long long stride = (long long)n * l64;
    Lanes L;
    CY_TRY(L.begin(ws, st, (size_t)chunk * kmax * n, nchunks));
    cy_status status = CY_OK;
    for (int c = 0; c < nchunks && status == CY_OK; c++) {
        const int j0 = c * chunk, nj = std::min(chunk, batch - j0);
        uint64_t* oj = out + (size_t)j0 * stride;
        // with relinearisation the rounded tensor product goes to `out` limb-major
        // (coalesced digit loads in the keyswitch), and the keyswitch's epilogue
        // writes the result over it in the [N][limb] layout
        status = product_chunk(tensor, kt, true, c1 + (size_t)j0 * stride, stride, c2 + (size_t)j0 * stride, stride,
                               oj, nj, L.scratch(c), L.stream(c), do_relin ? 1 : 0);
        if (status == CY_OK && do_relin)
            status = keyswitch_chunk(relin, kr, sel, oj, evk, ell, oj, nj, L.scratch(c), L.stream(c), 1);
    }
    return L.end(ws, st, status);
}

static cy_status run_crt(const Basis& B, const uint64_t* x, uint32_t* res, const uint32_t* d_scale, int batch,
                         cudaStream_t st) {
    if (batch == 0) return CY_OK;
    const BasisDev* Bd = B.d;
    long long threads = (long long)batch * B.h.n;
    void* args[] = {(void*)&Bd, (void*)&x, (void*)&res, (void*)&d_scale, (void*)&batch};
    return launch(crt_kernel(), "crt", B.h.logn, dim3((unsigned)((threads + 255) / 256)), dim3(256), 0, st, args);
}

static cy_status run_ntt(const Basis& B, uint32_t* res, int batch, bool inverse, cudaStream_t st,
                         int variant = -1) {
    if (batch == 0) return CY_OK;
    const KernelSet& ks =
        kernel_variant(B.h.logn, variant >= 0 ? variant : tuned_variant(B.h.logn, B.h.l64, TUNE_NTT));
    const BasisDev* Bd = B.d;
    const uint32_t* ninv = B.d_ninv;
    const long long rows = (long long)batch * B.h.k * (B.h.n / 64);
    if (inverse && ks.intt_tma && B.h.logn == 12 && ntt_tma_usable(res, rows)) {  // input tiles by TMA
        alignas(64) CUtensorMap map;
        dim3 grid;
        int* err = nullptr;
        CY_TRY(intt_tma_prepare(res, rows, B.h.k, batch, &map, &grid, &err));
        uint32_t spin = ntt_tma_spin_limit(), extra = ntt_tma_extra_tx();
        void* args[] = {(void*)&Bd, (void*)&map, (void*)&res, (void*)&ninv, (void*)&batch, (void*)&err, (void*)&spin,
                        (void*)&extra};
        return launch(intt_tma_kernel(), "ntt_inv", B.h.logn, grid, dim3(64), intt_tma_smem(), st, args);
    }
    if (ks.ntt_jobs_per_block == 1) {  // k_ntt1: grid (jobs, primes)
        void* args[] = {(void*)&Bd, (void*)&res, (void*)&ninv, (void*)&batch};
        return launch(ks.ntt[inverse ? 1 : 0], inverse ? "ntt_inv" : "ntt_fwd", B.h.logn, dim3(batch, B.h.k),
                      dim3(ks.threads), ks.smem_ntt, st, args);
    }
    for (int j0 = 0; j0 < batch; j0 += 2 * 65535) {  // two jobs per block
        int nj = std::min(2 * 65535, batch - j0);
        uint32_t* rj = res + (size_t)j0 * B.h.k * B.h.n;
        void* args[] = {(void*)&Bd, (void*)&rj, (void*)&ninv, (void*)&nj};
        CY_TRY(launch(ks.ntt[inverse ? 1 : 0], inverse ? "ntt_inv" : "ntt_fwd", B.h.logn, dim3(B.h.k, (nj + 1) / 2),
                      dim3(ks.threads), ks.smem_ntt, st, args));
    }
    return CY_OK;
}

cy_status run_ntt_api(const Basis& B, uint32_t* res, int batch, bool inverse, cudaStream_t st, int variant) {
    return run_ntt(B, res, batch, inverse, st, variant);
}

static cy_status run_addsub(const cy_ring* r, const uint64_t* a, const uint64_t* b, uint64_t* c, int batch, bool sub,
                            cudaStream_t st) {
    if (batch == 0) return CY_OK;
    long long count = (long long)batch * r->n;
    const uint64_t* q = r->d_q;
    void* args[] = {(void*)&a, (void*)&b, (void*)&c, (void*)&q, (void*)&count};
    return launch(addsub_kernel(r->l64, sub), sub ? "polysub" : "polyadd", r->logn,
                  dim3((unsigned)((count + 255) / 256)), dim3(256), 0, st, args);
}

// Buffers must be 16-byte aligned: the kernels load coefficients with 16-byte
// vector loads (cudaMalloc returns 256-byte aligned memory).
static cy_status check_aligned(const void* a, const void* b, const void* c) {
    if (((uintptr_t)a | (uintptr_t)b | (uintptr_t)c) & 15)
        return set_error(CY_ERR_INVALID_ARGUMENT, "buffers must be 16-byte aligned");
    return CY_OK;
}

static cy_status validate_poly_args(const cy_ring* r, const void* a, const void* b, const void* c, int batch) {
    if (!r) return set_error(CY_ERR_INVALID_ARGUMENT, "ring is NULL");
    if (batch < 0) return set_error(CY_ERR_INVALID_ARGUMENT, "batch < 0");
    if (batch > 0 && (!a || !b || !c)) return set_error(CY_ERR_INVALID_ARGUMENT, "NULL buffer");
    CY_TRY(check_aligned(a, b, c));
    return check_device(r->device);
}

// bound = 4 * N * q^2: |X| < N q^2 for products of values in [0, q)
static BigUInt product_bound(int n, const BigUInt& q) { return BigUInt(4ull * (uint64_t)n) * q * q; }

cy_status check_aligned_api(const void* a, const void* b, const void* c) { return check_aligned(a, b, c); }

cy_status run_product_api(const Basis& B, bool centered, const uint64_t* a, long long a_stride, const uint64_t* b,
                          long long b_stride, void* out, long long out_stride, int batch, Workspace& ws,
                          cudaStream_t st, int variant) {
    return run_product(B, centered, a, a_stride, b, b_stride, out, out_stride, batch, ws, st, variant);
}

// Jobs per chunk of an HE multiply of `batch` pairs, as run_yashe_mul cuts it
// (the host-buffer pipeline uses the same chunks).
int yashe_chunk_jobs(const Basis& tensor, const Basis& relin, int ell, bool do_relin) {
    const int n = tensor.h.n, l64 = tensor.h.l64;
    int chunk = chunk_jobs(n, std::max(tensor.h.k, do_relin ? relin.h.k : 0));
    if (do_relin) {
        const KernelSet& kr = kernel_variant(relin.h.logn, tuned_variant(relin.h.logn, l64, TUNE_KS));
        int sel = 0;
        if (keyswitch_digits_per_pass(kr, ell, &sel) == CY_OK)
            chunk = wave_chunk(chunk, kr.ks_for(l64, sel), kr.threads, kr.smem_ks[sel], relin.h.k * kr.blocks_per_prime);
    }
    return chunk;
}

cy_status run_keyswitch_api(const Basis& B, const uint64_t* c, const uint2* evk, int ell, uint64_t* out, int batch,
                            Workspace& ws, cudaStream_t st, int variant, int chunk_k, int lm) {
    return run_keyswitch(B, c, evk, ell, out, batch, ws, st, variant, chunk_k, lm);
}

// Evaluation key in the keyswitch basis, NTT domain, with Shoup companions:
// d_evk [ell][k][N] of (value, floor(value 2^32 / p)); at N = ROWS_N a second
// copy laid out by lane follows it (the 64-coefficient keyswitch reads that
// one). Synchronous.
cy_status prepare_evk(const Basis& relin, const uint64_t* h_evk, int ell, int n, int l64, uint2** d_evk) {
    const int k = relin.h.k;
    const size_t words = (size_t)ell * k * n;
    const bool rows = relin.h.logn == ROWS_LOGN;
    uint64_t* d_limbs = nullptr;
    uint32_t* d_res = nullptr;
    uint2* out = nullptr;
    cudaError_t e = cudaMalloc(&d_limbs, sizeof(uint64_t) * (size_t)ell * n * l64);
    if (e == cudaSuccess) e = cudaMalloc(&d_res, sizeof(uint32_t) * words);
    if (e == cudaSuccess) e = cudaMalloc(&out, sizeof(uint2) * words * (rows ? 2 : 1));
    if (e == cudaSuccess)
        e = cudaMemcpy(d_limbs, h_evk, sizeof(uint64_t) * (size_t)ell * n * l64, cudaMemcpyHostToDevice);
    cy_status st = (e == cudaSuccess) ? CY_OK : cuda_error(e, "evaluation key upload");
    if (st == CY_OK) st = run_crt(relin, d_limbs, d_res, nullptr, ell, 0);
    if (st == CY_OK) st = run_ntt(relin, d_res, ell, false, 0);
    if (st == CY_OK) {
        const BasisDev* Bd = relin.d;
        long long total = (long long)words;
        void* args[] = {(void*)&Bd, (void*)&d_res, (void*)&out, (void*)&total};
        st = launch(shoup_pairs_kernel(), "shoup_pairs", relin.h.logn, dim3((unsigned)((total + 255) / 256)), dim3(256),
                    0, 0, args);
        if (st == CY_OK && rows) {
            uint2* out_rows = out + words;
            void* rargs[] = {(void*)&out, (void*)&out_rows, (void*)&total};
            st = launch(evk_rows_kernel(), "evk_rows", relin.h.logn, dim3((unsigned)((total + 255) / 256)),
                        dim3(256), 0, 0, rargs);
        }
    }
    if (st == CY_OK) {
        e = cudaDeviceSynchronize();
        if (e != cudaSuccess) st = cuda_error(e, "evaluation key transform");
    }
    cudaFree(d_limbs);
    cudaFree(d_res);
    if (st != CY_OK) {
        cudaFree(out);
        return st;
    }
    *d_evk = out;
    return CY_OK;
}

}  // namespace cy

using namespace cy;

// ---- rings ----------------------------------------------------------------------
cy_ring::~cy_ring() {
    if (d_q) cudaFree(d_q);
}

extern "C" {

const char* cy_status_string(int status) {
    switch (status) {
        case CY_OK: return "ok";
        case CY_ERR_INVALID_ARGUMENT: return "invalid argument";
        case CY_ERR_UNSUPPORTED: return "unsupported parameters";
        case CY_ERR_CUDA: return "CUDA error";
        case CY_ERR_OUT_OF_MEMORY: return "out of device memory";
        case CY_ERR_NOT_INVERTIBLE: return "not invertible";
        case CY_ERR_NO_KEYS: return "no keys";
        case CY_ERR_TIMEOUT: return "timeout";
        case CY_ERR_BUSY: return "busy";
        case CY_ERR_INTERNAL: return "internal error";
        default: return "unknown status";
    }
}

const char* cy_last_error(void) { return last_error_message(); }

int cy_version(void) { return 1; }

cy_status cy_ring_create(int n, const uint64_t* h_q, int q_limbs, cy_ring** out) {
    if (!out || !h_q) return set_error(CY_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = nullptr;
    if (n < 2 || n > NMAX || (n & (n - 1))) return set_error(CY_ERR_UNSUPPORTED, "N must be a power of two in [2, 16384]");
    if (q_limbs < 1 || q_limbs > 6) return set_error(CY_ERR_UNSUPPORTED, "q_limbs must be 1..6");
    BigUInt q = BigUInt::from_limbs64(h_q, q_limbs);
    if (q.bits() < 2) return set_error(CY_ERR_INVALID_ARGUMENT, "q must be >= 2");
    if (q.bits() > 64 * q_limbs) return set_error(CY_ERR_INTERNAL, "limb conversion");
    int dev = 0;
    CY_CUDA(cudaGetDevice(&dev));
    std::unique_ptr<cy_ring> r(new cy_ring());
    r->device = dev;
    r->n = n;
    while ((1 << r->logn) < n) r->logn++;
    r->q = q;
    r->qbits = q.bits();
    r->l32 = (r->qbits + 31) / 32;
    r->l64 = (r->qbits + 63) / 64;
    r->q_limbs.assign(r->l64, 0);
    q.to_limbs64(r->q_limbs.data(), r->l64);
    CY_TRY(build_basis(r->mul, dev, n, q, EPI_MODQ, product_bound(n, q), 0, true, true, false));
    CY_TRY(build_basis(r->plain, dev, n, q, EPI_MODQ, product_bound(n, q), 0, false, false, false));
    CY_CUDA(cudaMalloc(&r->d_q, sizeof(uint64_t) * r->l64));
    CY_CUDA(cudaMemcpy(r->d_q, r->q_limbs.data(), sizeof(uint64_t) * r->l64, cudaMemcpyHostToDevice));
    r->own_ws.ws.device = dev;
    *out = r.release();
    return CY_OK;
}

cy_status cy_ring_destroy(cy_ring* ring) {
    delete ring;
    return CY_OK;
}

cy_status cy_ring_get_info(const cy_ring* r, cy_ring_info* info) {
    if (!r || !info) return set_error(CY_ERR_INVALID_ARGUMENT, "NULL argument");
    std::memset(info, 0, sizeof(*info));
    info->n = r->n;
    info->q_limbs = r->l64;
    info->q_bits = r->qbits;
    info->crt_primes = r->mul.h.k;
    info->crt_bits = r->mul.crt_bits;
    for (int i = 0; i < r->mul.h.k; i++) info->primes[i] = r->mul.h.p[i];
    return CY_OK;
}

cy_status cy_workspace_create(cy_workspace** out) {
    if (!out) return set_error(CY_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = new cy_workspace();
    CY_CUDA(cudaGetDevice(&(*out)->ws.device));
    return CY_OK;
}

cy_status cy_workspace_destroy(cy_workspace* ws) {
    delete ws;
    return CY_OK;
}

cy_status cy_polymul_ws(cy_ring* r, cy_workspace* ws, const uint64_t* d_a, const uint64_t* d_b, uint64_t* d_c,
                        int batch, cy_stream_t stream) {
    CY_TRY(validate_poly_args(r, d_a, d_b, d_c, batch));
    const long long stride = (long long)r->n * r->l64;
    if (!ws) {
        std::lock_guard<std::mutex> lock(r->mu);
        return run_product(r->mul, false, d_a, stride, d_b, stride, d_c, stride, batch, r->own_ws.ws,
                           (cudaStream_t)stream);
    }
    return run_product(r->mul, false, d_a, stride, d_b, stride, d_c, stride, batch, ws->ws, (cudaStream_t)stream);
}

cy_status cy_polymul(cy_ring* r, const uint64_t* d_a, const uint64_t* d_b, uint64_t* d_c, int batch,
                     cy_stream_t stream) {
    return cy_polymul_ws(r, nullptr, d_a, d_b, d_c, batch, stream);
}

cy_status cy_polymul_host(cy_ring* r, const uint64_t* h_a, const uint64_t* h_b, uint64_t* h_c, int batch) {
    CY_TRY(validate_poly_args(r, h_a, h_b, h_c, batch));
    if (batch == 0) return CY_OK;
    const KernelSet& ks = kernel_variant(r->mul.h.logn, tuned_variant(r->mul.h.logn, r->mul.h.l64, TUNE_MUL));
    const int chunk = product_chunk_jobs(r->mul, ks, false, chunk_jobs(r->n, r->mul.h.k));
    return run_host_pipeline((size_t)r->n * r->l64, batch, chunk, h_a, h_b, h_c,
                             [r](cy_workspace* ws, const uint64_t* a, const uint64_t* b, uint64_t* c, int nj,
                                 cudaStream_t st) { return cy_polymul_ws(r, ws, a, b, c, nj, st); });
}

cy_status cy_polyadd(cy_ring* r, const uint64_t* d_a, const uint64_t* d_b, uint64_t* d_c, int batch,
                     cy_stream_t stream) {
    CY_TRY(validate_poly_args(r, d_a, d_b, d_c, batch));
    return run_addsub(r, d_a, d_b, d_c, batch, false, (cudaStream_t)stream);
}

cy_status cy_polysub(cy_ring* r, const uint64_t* d_a, const uint64_t* d_b, uint64_t* d_c, int batch,
                     cy_stream_t stream) {
    CY_TRY(validate_poly_args(r, d_a, d_b, d_c, batch));
    return run_addsub(r, d_a, d_b, d_c, batch, true, (cudaStream_t)stream);
}

cy_status cy_poly_scalar_mul(cy_ring* r, const uint64_t* d_a, const uint64_t* h_scalar, uint64_t* d_c, int batch,
                             cy_stream_t stream) {
    CY_TRY(validate_poly_args(r, d_a, h_scalar, d_c, batch));
    if (batch == 0) return CY_OK;
    BigUInt s = BigUInt::from_limbs64(h_scalar, r->l64);
    if (s >= r->q) return set_error(CY_ERR_INVALID_ARGUMENT, "scalar must be < q");
    std::lock_guard<std::mutex> lock(r->mu);
    const Basis& B = r->plain;
    const int k = B.h.k, n = r->n;
    // residues of a times (s mod p_i), then the plain ICRT epilogue: |a s| < q^2 < M/4
    std::vector<uint32_t> scale(2 * (size_t)k);
    for (int i = 0; i < k; i++) {
        const uint32_t p = B.h.p[i], v = s.mod_u32(p);
        scale[2 * i] = v;
        scale[2 * i + 1] = (uint32_t)(((uint64_t)v << 32) / p);
    }
    cudaStream_t st = (cudaStream_t)stream;
    const int chunk = std::min(batch, chunk_jobs(n, k));
    Workspace& ws = r->own_ws.ws;
    CY_TRY(ws.reserve((size_t)chunk * k * n + 2 * (size_t)KMAX));
    uint32_t* d_scale = ws.d_resid + (size_t)chunk * k * n;
    CY_CUDA(cudaMemcpyAsync(d_scale, scale.data(), sizeof(uint32_t) * scale.size(), cudaMemcpyHostToDevice, st));
    for (int j0 = 0; j0 < batch; j0 += chunk) {
        int nj = std::min(chunk, batch - j0);
        const uint64_t* aj = d_a + (size_t)j0 * n * r->l64;
        CY_TRY(run_crt(B, aj, ws.d_resid, d_scale, nj, st));
        CY_TRY(launch_epi(B, ws.d_resid, d_c + (size_t)j0 * n * r->l64, nj, st, "epi_modq"));
    }
    // the scale vector is read by the kernels above before the stream moves on
    return CY_OK;
}

cy_status cy_set_chunk_overlap(int on) {
    g_two_lanes.store(on ? 1 : 0);
    return CY_OK;
}

cy_status cy_set_epilogue_generic(int on) {
    g_epi_generic.store(on ? 1 : 0);
    return CY_OK;
}

cy_status cy_set_epilogue_exact(int on) {
    g_epi_exact.store(on ? 1 : 0);
    return CY_OK;
}

cy_status cy_polymul_batched(const cy_polymul_job* jobs, int njobs, cy_stream_t stream) {
    if (njobs < 0 || (njobs > 0 && !jobs)) return set_error(CY_ERR_INVALID_ARGUMENT, "bad job list");
    std::vector<const cy_polymul_job*> mixed, other;
    for (int i = 0; i < njobs; i++) {
        CY_TRY(validate_poly_args(jobs[i].ring, jobs[i].d_a, jobs[i].d_b, jobs[i].d_c, 1));
        (mixed_supported(jobs[i].ring) ? mixed : other).push_back(&jobs[i]);
    }
    cudaStream_t st = (cudaStream_t)stream;
    CY_TRY(run_mixed(mixed, st));
    // other rings: consecutive jobs of one ring with contiguous buffers share a launch
    size_t i = 0;
    while (i < other.size()) {
        cy_ring* r = other[i]->ring;
        const long long stride = (long long)r->n * r->l64;
        size_t j = i + 1;
        while (j < other.size() && other[j]->ring == r && other[j]->d_a == other[i]->d_a + (j - i) * stride &&
               other[j]->d_b == other[i]->d_b + (j - i) * stride && other[j]->d_c == other[i]->d_c + (j - i) * stride)
            j++;
        CY_TRY(cy_polymul(r, other[i]->d_a, other[i]->d_b, other[i]->d_c, (int)(j - i), stream));
        i = j;
    }
    return CY_OK;
}

cy_status cy_polymul_batched_status(cy_stream_t stream) { return mixed_status((cudaStream_t)stream); }

cy_status cy_ntt(cy_ring* r, uint32_t* d_res, int batch, int inverse, cy_stream_t stream) {
    CY_TRY(validate_poly_args(r, d_res, d_res, d_res, batch));
    return run_ntt(r->plain, d_res, batch, inverse != 0, (cudaStream_t)stream);
}

cy_status cy_ntt_check(void) {
    CY_CUDA(cudaDeviceSynchronize());
    return ntt_tma_check(true);
}

cy_status cy_ntt_test_wait(unsigned spin_limit, unsigned extra_bytes) {
    ntt_tma_set_test(spin_limit, extra_bytes);
    return CY_OK;
}

cy_status cy_crt(cy_ring* r, const uint64_t* d_x, uint32_t* d_res, int batch, cy_stream_t stream) {
    CY_TRY(validate_poly_args(r, d_x, d_res, d_res, batch));
    return run_crt(r->plain, d_x, d_res, nullptr, batch, (cudaStream_t)stream);
}

cy_status cy_icrt(cy_ring* r, const uint32_t* d_res, uint64_t* d_x, int batch, cy_stream_t stream) {
    CY_TRY(validate_poly_args(r, d_res, d_x, d_x, batch));
    if (batch == 0) return CY_OK;
    const Basis& B = r->plain;
    for (int j0 = 0; j0 < batch; j0 += 65536) {
        int nj = std::min(65536, batch - j0);
        const uint32_t* rj = d_res + (size_t)j0 * B.h.k * r->n;
        CY_TRY(launch_epi(B, rj, d_x + (size_t)j0 * r->n * r->l64, nj, (cudaStream_t)stream, "epi_modq"));
    }
    return CY_OK;
}

}  // extern "C"
