// ICRT epilogues, CRT split, elementwise mod-q kernels and the dispatch tables.
#include <mutex>
#include <vector>

#include <algorithm>

#include "host.h"
#include "kernels.cuh"

namespace cy {

void fill_small(KernelSet* t);
void fill_n10_e3(KernelSet& ks);
void fill_n10_e4(KernelSet& ks);
void fill_n11_e3(KernelSet& ks);
void fill_n11_e4(KernelSet& ks);
void fill_n12_e3(KernelSet& ks);
void fill_n12_e4(KernelSet& ks);
void fill_n13_e3(KernelSet& ks);
void fill_n13_e4(KernelSet& ks);
void fill_n14_e4(KernelSet& ks);
void fill_n12_e3r(KernelSet& ks);
void fill_n12_e4r(KernelSet& ks);
void fill_n13_e4r(KernelSet& ks);
void fill_n14_e5(KernelSet& ks);
void fill_n12_e4s(KernelSet& ks);
void fill_n12_e3s(KernelSet& ks);
void fill_n12_e4m(KernelSet& ks);
void fill_n13_e4s(KernelSet& ks);
void fill_n12_e4t(KernelSet& ks);
void fill_n14_e4d1(KernelSet& ks);
void fill_n12_e4u(KernelSet& ks);
void fill_n14_pair(KernelSet& ks);
void fill_n12_e6(KernelSet& ks);
void fill_n12_e6t(KernelSet& ks);

struct VariantTable {
    std::vector<KernelSet> v[LOGN_MAX + 1];
};

static const VariantTable& variants() {
    static VariantTable T;
    static std::once_flag once;
    std::call_once(once, [] {
        KernelSet small[LOGN_MAX + 1];
        fill_small(small);
        for (int logn = 1; logn <= 9; logn++) T.v[logn].push_back(small[logn]);
        auto add = [](int logn, void (*fill)(KernelSet&)) {
            KernelSet ks;
            fill(ks);
            T.v[logn].push_back(ks);
        };
        // variant 0 first: the default schedule of each length
        add(10, fill_n10_e3);
        add(10, fill_n10_e4);
        add(11, fill_n11_e3);
        add(11, fill_n11_e4);
        add(12, fill_n12_e3);
        add(12, fill_n12_e4);
        add(13, fill_n13_e4);
        add(13, fill_n13_e3);
        add(14, fill_n14_e4);
        // larger register budgets per thread (fewer blocks per SM)
        add(12, fill_n12_e3r);
        add(12, fill_n12_e4r);
        add(13, fill_n13_e4r);
        add(14, fill_n14_e5);
        add(12, fill_n12_e4s);  // one keyswitch exchange region: two blocks per SM
        add(12, fill_n12_e3s);
        add(12, fill_n12_e4m);
        add(13, fill_n13_e4s);
        add(12, fill_n12_e4t);
        add(14, fill_n14_e4d1);
        add(12, fill_n12_e4u);
        add(12, fill_n12_e6);  // 64 coefficients per thread: two passes, one transpose
        add(12, fill_n12_e6t);  // the same, the standalone inverse NTT's input by TMA
        {
            KernelSet ks = T.v[14][0];  // the default set's standalone NTT
            fill_n14_pair(ks);
            T.v[14].push_back(ks);
        }
    });
    return T;
}

int variant_count(int logn) { return (logn >= 1 && logn <= LOGN_MAX) ? (int)variants().v[logn].size() : 0; }
const KernelSet& kernel_variant(int logn, int v) {
    const std::vector<KernelSet>& vs = variants().v[logn];
    return vs[(v >= 0 && v < (int)vs.size()) ? v : 0];
}
const KernelSet& kernel_set(int logn) { return kernel_variant(logn, 0); }

#define CY_EPI_ROW(L) {(void*)k_epi<L, EPI_MODQ>, (void*)k_epi<L, EPI_YASHE>, (void*)k_epi<L, EPI_DECRYPT>}

void* epi_kernel(int l32, int mode) {
    static void* table[L32MAX + 1][3] = {
        {nullptr, nullptr, nullptr}, CY_EPI_ROW(1), CY_EPI_ROW(2), CY_EPI_ROW(3), CY_EPI_ROW(4),
        CY_EPI_ROW(5),  CY_EPI_ROW(6), CY_EPI_ROW(7), CY_EPI_ROW(8), CY_EPI_ROW(9), CY_EPI_ROW(10),
        CY_EPI_ROW(11), CY_EPI_ROW(12)};
    if (l32 < 1 || l32 > L32MAX || mode < 0 || mode > 2) return nullptr;
    return table[l32][mode];
}

// Residues [job][k][N] in [0, p) of limbs [job][N][l64]; each residue is also
// multiplied by scale[i] (value, Shoup companion) when `scale` is not null.
__global__ void k_crt(const BasisDev* __restrict__ B, const uint64_t* __restrict__ X, uint32_t* __restrict__ res,
                      const uint32_t* __restrict__ scale, int njobs) {
    __shared__ uint32_t s_crt[KMAX * L32MAX];
    const int k = B->k, logn = B->logn, l64 = B->l64;
    for (int i = threadIdx.x; i < k * L32MAX; i += blockDim.x) s_crt[i] = B->crt[i / L32MAX][i % L32MAX];
    __syncthreads();
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int n = 1 << logn;
    const long long job = idx >> logn;
    if (job >= njobs) return;
    const int coef = (int)(idx & (n - 1));
    const uint64_t* x = X + (size_t)job * n * l64;
    for (int i = 0; i < k; i++) {
        const PrimeCtx c = load_prime_ctx(B, i);
        uint32_t r = crt_coef<false>(x, coef, l64, &s_crt[i * L32MAX], nullptr, c);
        if (scale) r = shoup(r, scale[2 * i], scale[2 * i + 1], c.p);
        r = red(red(r, 2 * c.p), c.p);
        res[((size_t)job * k + i) * n + coef] = r;
    }
}

// Shoup companions of NTT-domain values: out[j] = (v, floor(v 2^32 / p_i)) for
// the residue vectors of a [ell][k][N] array.
__global__ void k_shoup_pairs(const BasisDev* __restrict__ B, const uint32_t* __restrict__ v, uint2* __restrict__ out,
                              long long total) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const int prime = (int)((idx >> B->logn) % B->k);
    const uint32_t p = B->p[prime];
    const uint32_t x = v[idx];
    out[idx] = make_uint2(x, (uint32_t)(((uint64_t)x << 32) / p));
}

// The copy of an NTT-domain evaluation key [ell][k][ROWS_N] of (value, Shoup)
// pairs laid out by lane for the row pass of the 64-coefficient schedule: the
// entry at position 64 tau + u goes to record [u/2][tau], word u mod 2.
__global__ void k_evk_rows(const uint2* __restrict__ in, uint2* __restrict__ out, long long total) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const long long row = idx / ROWS_N;
    const int pos = (int)(idx % ROWS_N);
    const int tau = pos >> 6, u = pos & 63;
    out[row * ROWS_N + (u >> 1) * 2 * ROWS_G + 2 * tau + (u & 1)] = in[idx];
}

// Elementwise c = a +/- b mod q over [count][l64] limbs (inputs in [0, q)).
template <int L64, bool SUB>
__global__ void k_addsub(const uint64_t* __restrict__ a, const uint64_t* __restrict__ b, uint64_t* __restrict__ c,
                         const uint64_t* __restrict__ q, long long count) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= count) return;
    uint64_t x[L64], y[L64], s[L64], t[L64], qq[L64];
#pragma unroll
    for (int j = 0; j < L64; j++) {
        x[j] = a[idx * L64 + j];
        y[j] = b[idx * L64 + j];
        qq[j] = q[j];
    }
    if (!SUB) {
        // s = x + y; t = s - q; pick t unless it borrows (and s did not carry)
        uint64_t carry = 0;
#pragma unroll
        for (int j = 0; j < L64; j++) {
            const uint64_t u = x[j] + y[j];
            const uint64_t c1 = u < x[j];
            s[j] = u + carry;
            carry = c1 | (s[j] < u);
        }
        uint64_t br = 0;
#pragma unroll
        for (int j = 0; j < L64; j++) {
            const uint64_t d = s[j] - qq[j];
            const uint64_t b1 = s[j] < qq[j];
            t[j] = d - br;
            br = b1 | (d < br);
        }
        const bool use_t = carry || !br;
#pragma unroll
        for (int j = 0; j < L64; j++) c[idx * L64 + j] = use_t ? t[j] : s[j];
    } else {
        // s = x - y; if it borrows, add q
        uint64_t br = 0;
#pragma unroll
        for (int j = 0; j < L64; j++) {
            const uint64_t d = x[j] - y[j];
            const uint64_t b1 = x[j] < y[j];
            s[j] = d - br;
            br = b1 | (d < br);
        }
        uint64_t carry = 0;
#pragma unroll
        for (int j = 0; j < L64; j++) {
            const uint64_t u = s[j] + qq[j];
            const uint64_t c1 = u < s[j];
            t[j] = u + carry;
            carry = c1 | (t[j] < u);
        }
#pragma unroll
        for (int j = 0; j < L64; j++) c[idx * L64 + j] = br ? t[j] : s[j];
    }
}

void* addsub_kernel(int l64, bool sub) {
    static void* table[7][2] = {{nullptr, nullptr},
                                {(void*)k_addsub<1, false>, (void*)k_addsub<1, true>},
                                {(void*)k_addsub<2, false>, (void*)k_addsub<2, true>},
                                {(void*)k_addsub<3, false>, (void*)k_addsub<3, true>},
                                {(void*)k_addsub<4, false>, (void*)k_addsub<4, true>},
                                {(void*)k_addsub<5, false>, (void*)k_addsub<5, true>},
                                {(void*)k_addsub<6, false>, (void*)k_addsub<6, true>}};
    if (l64 < 1 || l64 > 6) return nullptr;
    return table[l64][sub ? 1 : 0];
}

// Polynomials of `words` uint64 words between a list of device pointers and one
// contiguous array (16-byte moves): gather ptrs[i] -> flat + i*words, or scatter
// flat + i*words -> ptrs[i]. The serving loop's device-resident requests.
template <bool GATHER>
__global__ void k_poly_move(uint64_t* const* __restrict__ ptrs, uint64_t* __restrict__ flat, long long count,
                            long long words) {
    const long long half = words / 2;  // 16-byte units per polynomial (words is even: N >= 2)
    const long long total = count * half;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long i = idx / half, w = idx - i * half;
        uint4* f = reinterpret_cast<uint4*>(flat + i * words) + w;
        uint4* q = reinterpret_cast<uint4*>(ptrs[i]) + w;
        if (GATHER) *f = __ldg(q);
        else *q = *f;
    }
}

int trace_begin(const char* name, int logn, cudaStream_t st);
void trace_end(int idx, cudaStream_t st);

// Sets *differ to 1 if the `words` 32-bit words at a and b are not all equal
// (the autotuner's check that a schedule gives the default's output).
__global__ void k_words_differ(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b, size_t words,
                               int* __restrict__ differ) {
    bool d = false;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < words; i += (size_t)gridDim.x * blockDim.x)
        d |= a[i] != b[i];
    if (__syncthreads_or(d) && threadIdx.x == 0) atomicExch(differ, 1);
}

cy_status words_differ(const void* a, const void* b, size_t bytes, int* d_flag, cudaStream_t st, bool* differ) {
    size_t words = bytes / 4;
    CY_CUDA(cudaMemsetAsync(d_flag, 0, sizeof(int), st));
    const unsigned blocks = (unsigned)std::max<size_t>(1, std::min<size_t>((words + 255) / 256, 4096));
    void* args[] = {(void*)&a, (void*)&b, (void*)&words, (void*)&d_flag};
    CY_CUDA(cudaLaunchKernel((void*)k_words_differ, dim3(blocks), dim3(256), args, 0, st));
    int h = 0;
    CY_CUDA(cudaMemcpyAsync(&h, d_flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    CY_CUDA(cudaStreamSynchronize(st));
    *differ = h != 0;
    return CY_OK;
}

cy_status move_polys(uint64_t* const* d_ptrs, uint64_t* flat, int count, size_t words, bool gather,
                     cudaStream_t st) {
    if (count <= 0) return CY_OK;
    const long long total = (long long)count * (long long)(words / 2);
    long long blocks = (total + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    long long cnt = count, w = (long long)words;
    void* args[] = {(void*)&d_ptrs, (void*)&flat, (void*)&cnt, (void*)&w};
    const int tr = trace_begin(gather ? "serve_gather" : "serve_scatter", 0, st);
    const cudaError_t e = cudaLaunchKernel(gather ? (void*)k_poly_move<true> : (void*)k_poly_move<false>,
                                           dim3((unsigned)blocks), dim3(256), args, 0, st);
    trace_end(tr, st);
    return e == cudaSuccess ? CY_OK : cuda_error(e, "serving gather/scatter");
}

void* crt_kernel() { return (void*)k_crt; }
void* shoup_pairs_kernel() { return (void*)k_shoup_pairs; }
void* evk_rows_kernel() { return (void*)k_evk_rows; }

}  // namespace cy
