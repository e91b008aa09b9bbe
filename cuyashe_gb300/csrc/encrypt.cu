// encrypt.cu -- YASHE encryption on the GPU with on-device sampling.
//
// Replaces Yashe::encrypt (src/yashe.cpp:104-142) and its samplers
// (src/distribution.cpp:4-60, src/cuda_distribution.cu:11-35, which draw
// uniform values with cuRAND where the scheme asks for an error distribution):
//   ct = [h*s + e + Delta*m]_q,  Delta = floor(q/t),  s, e ~ D_sigma (discrete
//   Gaussian on [-B, B], B = ceil(6 sigma)).
//
// Randomness is counter-based, so that every coefficient is drawn
// independently on its own thread and the draws can be reproduced exactly on
// the CPU: draw number c of a call with seed S is the c-th output of splitmix64
// seeded with S, i.e. mix(S + (c+1) * 0x9E3779B97F4A7C15). Coefficient i of s
// (of e) for ciphertext b uses counter (2b) * N + i ((2b+1) * N + i). A draw
// u is mapped to x = j - B with j the first index of the CDT table with
// u < T[j] (T: 64-bit cumulative thresholds, see gaussian_cdt).
//
// Three steps on the caller's stream: k_enc_sample writes s (as limbs mod q)
// into the output, the product kernels compute h*s in place (a chunk's product
// kernel reads its inputs before its epilogue writes), and k_enc_finish adds e
// and Delta*m and reduces mod q.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "host.h"
#include "kernels.cuh"

namespace cy {

cy_status run_product_api(const Basis& B, bool centered, const uint64_t* a, long long a_stride, const uint64_t* b,
                          long long b_stride, void* out, long long out_stride, int batch, Workspace& ws,
                          cudaStream_t st, int variant = -1);
int trace_begin(const char* name, int logn, cudaStream_t st);
void trace_end(int idx, cudaStream_t st);

constexpr int kCdtMax = 512;  // thresholds (sigma up to 42)

// Host: the 64-bit CDT thresholds of D_sigma on [-B, B], B = ceil(6 sigma):
// w_j = exp(-x^2 / (2 sigma^2)) for x = j - B, acc_j = sum_{i<=j} w_i / total,
// T_j = floor(acc_j * 2^64) (2^64 - 1 for the last entry and when acc_j >= 1).
std::vector<uint64_t> gaussian_cdt(double sigma) {
    const int bound = (int)std::ceil(6.0 * sigma);
    std::vector<double> w(2 * bound + 1);
    double total = 0.0;
    for (int j = 0; j <= 2 * bound; j++) {
        const int x = j - bound;
        w[j] = std::exp(-(double)(x * x) / (2.0 * sigma * sigma));
        total += w[j];
    }
    std::vector<uint64_t> T(w.size());
    double acc = 0.0;
    for (size_t j = 0; j < w.size(); j++) {
        acc += w[j] / total;
        T[j] = acc >= 1.0 ? ~0ULL : (uint64_t)(acc * 18446744073709551616.0);
    }
    T.back() = ~0ULL;
    return T;
}

struct EncConsts {
    uint64_t q[6];
    uint64_t delta[6];  // floor(q / t)
    uint64_t seed;
    uint32_t t;
    int l64, logn, bound, ncdt;
};

__device__ __forceinline__ uint64_t counter_draw(uint64_t seed, uint64_t ctr) {
    uint64_t z = seed + (ctr + 1) * 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

// first j with u < T[j] (the last threshold is 2^64 - 1, so j <= ncdt - 1)
__device__ __forceinline__ int cdt_sample(const uint64_t* T, int ncdt, int bound, uint64_t u) {
    int lo = 0, hi = ncdt - 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (T[mid] <= u) lo = mid + 1;
        else hi = mid;
    }
    return lo - bound;
}

__device__ __forceinline__ void load_cdt(uint64_t* sT, const uint64_t* __restrict__ T, int ncdt) {
    for (int i = threadIdx.x; i < ncdt; i += blockDim.x) sT[i] = T[i];
    __syncthreads();
}

// s -> out as limbs of [s]_q
__global__ void k_enc_sample(EncConsts C, const uint64_t* __restrict__ T, uint64_t* __restrict__ out, int batch) {
    __shared__ uint64_t sT[kCdtMax];
    load_cdt(sT, T, C.ncdt);
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= ((long long)batch << C.logn)) return;
    const long long b = idx >> C.logn, i = idx & ((1LL << C.logn) - 1);
    const int s = cdt_sample(sT, C.ncdt, C.bound, counter_draw(C.seed, ((uint64_t)(2 * b) << C.logn) + i));
    uint64_t* dst = out + idx * C.l64;
    if (s >= 0) {
        dst[0] = (uint64_t)s;
        for (int w = 1; w < C.l64; w++) dst[w] = 0;
    } else {  // q - |s|
        unsigned __int128 borrow = (uint64_t)(-s);
        for (int w = 0; w < C.l64; w++) {
            const unsigned __int128 d = (unsigned __int128)C.q[w] - borrow;
            dst[w] = (uint64_t)d;
            borrow = (d >> 64) ? 1 : 0;
        }
    }
}

// x (l64 + 1 limbs, x < 4q) -> x mod q, written to dst
__device__ __forceinline__ void reduce_small_multiple(uint64_t* x, const uint64_t* q, int l64, uint64_t* dst) {
    for (int it = 0; it < 3; it++) {
        uint64_t t[7];
        uint64_t borrow = 0;
        for (int w = 0; w <= l64; w++) {
            const uint64_t qw = w < l64 ? q[w] : 0;
            const unsigned __int128 d = (unsigned __int128)x[w] - qw - borrow;
            t[w] = (uint64_t)d;
            borrow = (d >> 64) ? 1 : 0;
        }
        if (borrow) break;  // x < q
        for (int w = 0; w <= l64; w++) x[w] = t[w];
    }
    for (int w = 0; w < l64; w++) dst[w] = x[w];
}

// ct = [hs + e + Delta*(m mod t)]_q in place (hs in [0, q), e in [-B, B])
__global__ void k_enc_finish(EncConsts C, const uint64_t* __restrict__ T, const uint64_t* __restrict__ m,
                             uint64_t* __restrict__ ct, int batch) {
    __shared__ uint64_t sT[kCdtMax];
    load_cdt(sT, T, C.ncdt);
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= ((long long)batch << C.logn)) return;
    const long long b = idx >> C.logn, i = idx & ((1LL << C.logn) - 1);
    const int e = cdt_sample(sT, C.ncdt, C.bound, counter_draw(C.seed, ((uint64_t)(2 * b + 1) << C.logn) + i));
    const uint64_t mv = m[idx] % C.t;
    uint64_t* c = ct + idx * C.l64;
    // x = Delta * mv + hs (+ q - |e| or + e): < Delta t + 2q <= 3q
    uint64_t x[7];
    unsigned __int128 carry = 0;
    for (int w = 0; w < C.l64; w++) {
        const unsigned __int128 v = (unsigned __int128)C.delta[w] * mv + c[w] + carry;
        x[w] = (uint64_t)v;
        carry = v >> 64;
    }
    x[C.l64] = (uint64_t)carry;
    carry = 0;
    if (e >= 0) {
        carry = (uint64_t)e;
        for (int w = 0; w <= C.l64; w++) {
            const unsigned __int128 v = (unsigned __int128)x[w] + carry;
            x[w] = (uint64_t)v;
            carry = v >> 64;
        }
    } else {  // + (q - |e|)
        const uint64_t ae = (uint64_t)(-e);
        uint64_t borrow = ae;
        for (int w = 0; w <= C.l64; w++) {  // x += q
            const uint64_t qw = w < C.l64 ? C.q[w] : 0;
            const unsigned __int128 v = (unsigned __int128)x[w] + qw + carry;
            x[w] = (uint64_t)v;
            carry = v >> 64;
        }
        for (int w = 0; w <= C.l64; w++) {  // x -= |e|
            const unsigned __int128 d = (unsigned __int128)x[w] - borrow;
            x[w] = (uint64_t)d;
            borrow = (d >> 64) ? 1 : 0;
        }
    }
    reduce_small_multiple(x, C.q, C.l64, c);
}

// out = [c + Delta*(m mod t)]_q (plaintext addition)
__global__ void k_add_plain(EncConsts C, const uint64_t* __restrict__ m, const uint64_t* __restrict__ cin,
                            uint64_t* __restrict__ out, int batch) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= ((long long)batch << C.logn)) return;
    const uint64_t mv = m[idx] % C.t;
    const uint64_t* c = cin + idx * C.l64;
    uint64_t x[7];
    unsigned __int128 carry = 0;
    for (int w = 0; w < C.l64; w++) {  // < Delta t + q <= 2q
        const unsigned __int128 v = (unsigned __int128)C.delta[w] * mv + c[w] + carry;
        x[w] = (uint64_t)v;
        carry = v >> 64;
    }
    x[C.l64] = (uint64_t)carry;
    reduce_small_multiple(x, C.q, C.l64, out + idx * C.l64);
}

// out = [m_c]_q with m_c the representative of m mod t in (-t/2, t/2]
__global__ void k_lift_plain(EncConsts C, const uint64_t* __restrict__ m, uint64_t* __restrict__ out, int batch) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= ((long long)batch << C.logn)) return;
    const uint64_t v = m[idx] % C.t;
    uint64_t* dst = out + idx * C.l64;
    if (v <= C.t / 2) {
        dst[0] = v;
        for (int w = 1; w < C.l64; w++) dst[w] = 0;
    } else {  // q - (t - v)
        uint64_t borrow = C.t - v;
        for (int w = 0; w < C.l64; w++) {
            const unsigned __int128 d = (unsigned __int128)C.q[w] - borrow;
            dst[w] = (uint64_t)d;
            borrow = (d >> 64) ? 1 : 0;
        }
    }
}

}  // namespace cy

using namespace cy;

namespace {

cy_status plain_consts(cy_yashe* y, EncConsts& C) {
    cy_ring* r = y->ring;
    int cur = -1;
    CY_CUDA(cudaGetDevice(&cur));
    if (cur != r->device) return set_error(CY_ERR_INVALID_ARGUMENT, "handle belongs to another CUDA device");
    if (r->l64 > 6) return set_error(CY_ERR_UNSUPPORTED, "plaintext operations support q of up to 384 bits");
    C = EncConsts{};
    r->q.to_limbs64(C.q, r->l64);
    (r->q / BigUInt(y->t)).to_limbs64(C.delta, r->l64);
    C.t = (uint32_t)y->t;
    C.l64 = r->l64;
    C.logn = r->logn;
    return CY_OK;
}

cy_status plain_args(cy_yashe* y, const void* a, const void* b, const void* out, int batch) {
    if (!y) return set_error(CY_ERR_INVALID_ARGUMENT, "yashe handle is NULL");
    if (batch < 0 || (batch > 0 && (!a || !b || !out))) return set_error(CY_ERR_INVALID_ARGUMENT, "bad argument");
    for (const void* p : {a, out})
        if (((uintptr_t)p & 15) != 0) return set_error(CY_ERR_INVALID_ARGUMENT, "buffer not 16-byte aligned");
    return CY_OK;
}

}  // namespace

extern "C" cy_status cy_yashe_add_plain(cy_yashe* y, const uint64_t* d_c, const uint64_t* d_m, uint64_t* d_out,
                                        int batch, cy_stream_t stream) {
    CY_TRY(plain_args(y, d_c, d_m, d_out, batch));
    if (batch == 0) return CY_OK;
    EncConsts C;
    CY_TRY(plain_consts(y, C));
    const long long total = (long long)batch << C.logn;
    cudaStream_t st = (cudaStream_t)stream;
    const int tr = trace_begin("add_plain", C.logn, st);
    k_add_plain<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(C, d_m, d_c, d_out, batch);
    trace_end(tr, st);
    CY_CUDA(cudaGetLastError());
    return CY_OK;
}

extern "C" cy_status cy_yashe_mul_plain(cy_yashe* y, const uint64_t* d_c, const uint64_t* d_m, uint64_t* d_out,
                                        int batch, cy_stream_t stream) {
    CY_TRY(plain_args(y, d_c, d_m, d_out, batch));
    if (batch == 0) return CY_OK;
    if (d_out == d_c) return set_error(CY_ERR_INVALID_ARGUMENT, "out must not alias the ciphertext");
    EncConsts C;
    CY_TRY(plain_consts(y, C));
    cy_ring* r = y->ring;
    std::lock_guard<std::mutex> lock(r->mu);
    const long long total = (long long)batch << C.logn;
    cudaStream_t st = (cudaStream_t)stream;
    const int tr = trace_begin("lift_plain", C.logn, st);
    k_lift_plain<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(C, d_m, d_out, batch);
    trace_end(tr, st);
    CY_CUDA(cudaGetLastError());
    const long long stride = (long long)r->n * r->l64;
    return run_product_api(r->mul, false, d_c, stride, d_out, stride, d_out, stride, batch, r->own_ws.ws, st);
}

extern "C" cy_status cy_gaussian_cdt(double sigma, uint64_t* out, int max_entries, int* n_entries) {
    if (!(sigma > 0.0) || !n_entries || max_entries < 0 || (max_entries > 0 && !out))
        return set_error(CY_ERR_INVALID_ARGUMENT, "bad argument");
    const std::vector<uint64_t> T = gaussian_cdt(sigma);
    *n_entries = (int)T.size();
    if ((int)T.size() > max_entries) return set_error(CY_ERR_INVALID_ARGUMENT, "table does not fit");
    std::copy(T.begin(), T.end(), out);
    return CY_OK;
}

extern "C" cy_status cy_yashe_encrypt(cy_yashe* y, const uint64_t* d_m, uint64_t* d_ct, int batch, uint64_t seed,
                                      cy_stream_t stream) {
    if (!y) return set_error(CY_ERR_INVALID_ARGUMENT, "yashe handle is NULL");
    if (batch < 0 || (batch > 0 && (!d_m || !d_ct))) return set_error(CY_ERR_INVALID_ARGUMENT, "bad argument");
    if (!y->has_keys || !y->d_h) return set_error(CY_ERR_NO_KEYS, "no keys installed");
    if (batch == 0) return CY_OK;
    if (((uintptr_t)d_ct & 15) != 0) return set_error(CY_ERR_INVALID_ARGUMENT, "ciphertext buffer not 16-byte aligned");
    cy_ring* r = y->ring;
    int cur = -1;
    CY_CUDA(cudaGetDevice(&cur));
    if (cur != r->device) return set_error(CY_ERR_INVALID_ARGUMENT, "handle belongs to another CUDA device");
    if (r->l64 > 6) return set_error(CY_ERR_UNSUPPORTED, "GPU encryption supports q of up to 384 bits");
    cudaStream_t st = (cudaStream_t)stream;
    std::lock_guard<std::mutex> lock(r->mu);
    if (!y->d_cdt) {
        const std::vector<uint64_t> T = gaussian_cdt(y->sigma);
        if ((int)T.size() > kCdtMax) return set_error(CY_ERR_UNSUPPORTED, "sigma too large for the sampler table");
        CY_CUDA(cudaMalloc(&y->d_cdt, T.size() * sizeof(uint64_t)));
        CY_CUDA(cudaMemcpy(y->d_cdt, T.data(), T.size() * sizeof(uint64_t), cudaMemcpyHostToDevice));
        y->n_cdt = (int)T.size();
    }
    EncConsts C{};
    r->q.to_limbs64(C.q, r->l64);
    (r->q / BigUInt(y->t)).to_limbs64(C.delta, r->l64);
    C.seed = seed;
    C.t = (uint32_t)y->t;
    C.l64 = r->l64;
    C.logn = r->logn;
    C.bound = (y->n_cdt - 1) / 2;
    C.ncdt = y->n_cdt;
    const long long total = (long long)batch << r->logn;
    const dim3 grid((unsigned)((total + 255) / 256)), block(256);
    int tr = trace_begin("enc_sample", r->logn, st);
    k_enc_sample<<<grid, block, 0, st>>>(C, y->d_cdt, d_ct, batch);
    trace_end(tr, st);
    CY_CUDA(cudaGetLastError());
    const long long stride = (long long)r->n * r->l64;
    CY_TRY(run_product_api(r->mul, false, y->d_h, 0, d_ct, stride, d_ct, stride, batch, r->own_ws.ws, st));
    tr = trace_begin("enc_finish", r->logn, st);
    k_enc_finish<<<grid, block, 0, st>>>(C, y->d_cdt, d_m, d_ct, batch);
    trace_end(tr, st);
    CY_CUDA(cudaGetLastError());
    return CY_OK;
}
