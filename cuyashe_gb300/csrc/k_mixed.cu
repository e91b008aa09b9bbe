// k_mixed: one persistent launch for a batch of products of different rings
// (N from 1024 to 8192, q up to 192 bits): the fused CRT -> NTT -> pointwise ->
// INTT -> ICRT -> mod q path over a work list.
//
// Blocks of 1024 threads claim units from an atomic counter. The NTT units come
// first, largest transforms first; with 8 coefficients per thread a unit of
// N = 8192 fills the block and a unit of N = 4096, 2048 or 1024 runs 2, 4 or 8
// primes of its job side by side, each on its own named barrier. The epilogue units of
// a job follow all NTT units; a block that claims one waits until every prime of
// that job is done. Those primes were claimed earlier by running blocks that
// never wait, so the wait ends; the spin is still bounded, and on expiry the
// block records an error word and skips the unit instead of hanging.
#include "kernels.cuh"

namespace cy {

constexpr int kMixedThreads = 1024;
constexpr unsigned kMixedSpinLimit = 1u << 24;  // ~ seconds with the back-off below

// L64: limbs per coefficient (1..3, compile-time load and CRT split), or 0 to
// read the count at run time.
template <int LOGN, int LOGE, int L64>
__device__ __forceinline__ void mixed_ntt_unit(const MixedJob& J, const MixedUnit& U, uint32_t* smem,
                                               uint32_t* __restrict__ done) {
    using PL = NttPlan<LOGN, LOGE>;
    constexpr int E = PL::E, G = PL::G;
    constexpr int NSUB = kMixedThreads / G;
    // two exchange regions of two operands per sub-group (147 KB per block at every N)
    constexpr int SUBW = 4 * PL::SMW;
    constexpr int STRIDE = 2 * PL::SMW;
    const int sub = threadIdx.x / G, tau = threadIdx.x % G;
    if (sub >= U.count) return;  // fewer primes than sub-groups in this unit
    const int prime = U.first + sub;
    const GroupSync bar{1 + sub, G};
    uint32_t* sm = smem + sub * SUBW;
    const BasisDev* __restrict__ B = J.B;
    const PrimeCtx c = load_prime_ctx(B, prime);
    uint32_t x[2][E];
    if constexpr (L64 > 0) {
        constexpr int W = 2 * L64;
        uint32_t cc[W], qh[W];
#pragma unroll
        for (int w = 0; w < W; w++) {
            cc[w] = B->crt[prime][w];
            qh[w] = 0;  // no centring
        }
#pragma unroll
        for (int e = 0; e < E; e++) {
            const int pos = slot_pos<PL, 0>(tau, e);
            uint32_t wa[W], wb[W];
            load_words<L64>(J.a + (size_t)pos * L64, wa);
            load_words<L64>(J.b + (size_t)pos * L64, wb);
            x[0][e] = crt_words<W, false>(wa, cc, qh, c);
            x[1][e] = crt_words<W, false>(wb, cc, qh, c);
        }
    } else {
        const uint32_t* crt = B->crt[prime];
#pragma unroll
        for (int e = 0; e < E; e++) {
            const int pos = slot_pos<PL, 0>(tau, e);
            x[0][e] = crt_coef<false>(J.a, pos, J.l64, crt, nullptr, c);
            x[1][e] = crt_coef<false>(J.b, pos, J.l64, crt, nullptr, c);
        }
    }
    const Mod m = mod_of(c.p);  // 64 registers per thread: constants folded
    int buf = ntt_forward<PL, 2, GroupSync>(x, B->psi[prime], m, tau, sm, STRIDE, 0, bar);
    uint32_t z[1][E];
#pragma unroll
    for (int e = 0; e < E; e++) z[0][e] = mont(red(x[0][e], 2 * c.p), red(x[1][e], 2 * c.p), c.p, c.pinv);
    ntt_inverse<PL, 1, GroupSync>(z, B->ipsi[prime], m, tau, sm, STRIDE, buf, bar);
    uint32_t* out = J.resid + (size_t)prime * PL::N;
#pragma unroll
    for (int e = 0; e < E; e++) out[slot_pos<PL, 0>(tau, e)] = z[0][e];
    __threadfence();  // residues visible device-wide before the count says so
    bar.sync();
    if (tau == 0) atomicAdd(&done[U.job], 1u);
}

template <int L>
__device__ __forceinline__ void mixed_epi_coefs(const MixedJob& J, const MixedUnit& U, EpiShared& S) {
    epi_stage<L, EPI_MODQ>(S, J.B, threadIdx.x, kMixedThreads);
    __syncthreads();
    const size_t n = (size_t)1 << J.logn;
    for (int coef = U.first + threadIdx.x; coef < U.first + U.count; coef += kMixedThreads)
        epi_coef<L, EPI_MODQ>(S, J.B, J.resid + coef, n, J.c + (size_t)coef * J.l64);
}

__device__ __forceinline__ uint32_t load_acquire(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__global__ void __launch_bounds__(kMixedThreads, 1)
    k_mixed(const MixedJob* __restrict__ jobs, const MixedUnit* __restrict__ units, int n_units,
            uint32_t* __restrict__ done, uint32_t* __restrict__ ctl) {
    extern __shared__ uint32_t smem[];
    __shared__ EpiShared S;
    __shared__ int s_unit, s_ok;
    for (;;) {
        if (threadIdx.x == 0) s_unit = (int)atomicAdd(&ctl[0], 1u);
        __syncthreads();
        const int u = s_unit;
        if (u >= n_units) break;
        const MixedUnit U = units[u];
        const MixedJob J = jobs[U.job];
        if (U.kind == 0) {
            switch (J.logn * 4 + J.l64) {
#define CY_MIXED_NTT(LOGN, LOGE)                                                    \
    case LOGN * 4 + 1: mixed_ntt_unit<LOGN, LOGE, 1>(J, U, smem, done); break; \
    case LOGN * 4 + 2: mixed_ntt_unit<LOGN, LOGE, 2>(J, U, smem, done); break; \
    case LOGN * 4 + 3: mixed_ntt_unit<LOGN, LOGE, 3>(J, U, smem, done); break;
                CY_MIXED_NTT(10, 3)
                CY_MIXED_NTT(11, 3)
                CY_MIXED_NTT(12, 3)
                CY_MIXED_NTT(13, 3)
#undef CY_MIXED_NTT
                default: break;
            }
        } else {
            if (threadIdx.x == 0) {
                unsigned spins = 0;
                while (load_acquire(&done[U.job]) < (uint32_t)J.k && spins < kMixedSpinLimit) {
                    __nanosleep(256);
                    spins++;
                }
                s_ok = spins < kMixedSpinLimit;
                if (!s_ok) atomicExch(&ctl[1], 1u);
            }
            __syncthreads();
            if (s_ok) {
                __threadfence();
                switch (J.l32) {
                    case 1: mixed_epi_coefs<1>(J, U, S); break;
                    case 2: mixed_epi_coefs<2>(J, U, S); break;
                    case 3: mixed_epi_coefs<3>(J, U, S); break;
                    case 4: mixed_epi_coefs<4>(J, U, S); break;
                    case 5: mixed_epi_coefs<5>(J, U, S); break;
                    case 6: mixed_epi_coefs<6>(J, U, S); break;
                    default: break;
                }
            }
        }
        __syncthreads();  // shared memory and s_unit are reused by the next unit
    }
}

void* mixed_kernel() { return (void*)k_mixed; }
// the same at every N: (1024 / (N/8)) sub-groups x 4 operand buffers of N + N/8 words
size_t mixed_smem_bytes() { return (size_t)2 * 4 * NttPlan<12, 3>::SMW * sizeof(uint32_t); }
static_assert(1 * 4 * NttPlan<13, 3>::SMW == 2 * 4 * NttPlan<12, 3>::SMW &&
                  4 * 4 * NttPlan<11, 3>::SMW == 2 * 4 * NttPlan<12, 3>::SMW &&
                  8 * 4 * NttPlan<10, 3>::SMW == 2 * 4 * NttPlan<12, 3>::SMW,
              "one shared-memory size serves every transform length");
int mixed_threads() { return kMixedThreads; }

}  // namespace cy
