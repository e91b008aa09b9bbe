// k_mixed: one persistent launch for a batch of polynomial products and YASHE
// multiplies of different rings (N from 1024 to 8192, q up to 192 bits): the
// fused CRT -> NTT -> pointwise -> INTT -> ICRT -> mod q (or YASHE rounding)
// path, then for relinearised YASHE jobs the keyswitch (digits -> NTT -> MAC
// with the resident evaluation key -> INTT -> ICRT -> mod q), over a work list.
//
// Blocks claim units from an atomic counter, in list order: every job's
// transform units (largest transforms first), then the first epilogues, then
// the keyswitch transforms, then the keyswitch epilogues. A unit of N = 8192
// fills a block; units of N = 4096, 2048 and 1024 run 2, 4 or 8 primes side by
// side, each on its own named barrier. A block that claims a unit whose inputs
// come from earlier units of its job waits until their count is complete. Those
// units were claimed earlier by blocks that are running, and the earliest
// unfinished unit waits for nothing, so every wait ends; no cooperative launch is
// needed. The spin is still bounded: on expiry the block records an error word
// and skips the unit instead of hanging.
//
// Two schedules (the autotuner picks per batch): 8 coefficients per thread in
// 1024-thread blocks, or 16 in 512-thread blocks. Both give a unit the same
// number of primes at every N, so one work list serves both.
#include "kernels.cuh"

namespace cy {

// Spin limit (iterations of a 256 ns back-off) a launch uses unless its plan
// sets a shorter one: about seconds, far beyond any unit's run time.
constexpr unsigned kMixedSpinDefault = 1u << 24;

template <int LOGE>
struct MixedSched {
    static constexpr int THREADS = LOGE == 3 ? 1024 : 512;
    static constexpr int MINB = 1;
};

// L64: limbs per coefficient (1..3, compile-time load and CRT split).
template <int LOGN, int LOGE, int L64, bool CENTER>
__device__ __forceinline__ void mixed_ntt_unit(const MixedJob& J, const MixedUnit& U, uint32_t* smem,
                                               uint32_t* __restrict__ done) {
    using PL = NttPlan<LOGN, LOGE>;
    constexpr int E = PL::E, G = PL::G;
    // two exchange regions of two operands per sub-group (the same size at every N)
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
    constexpr int W = 2 * L64;
    uint32_t cc[W], qh[W];
#pragma unroll
    for (int w = 0; w < W; w++) {
        cc[w] = B->crt[prime][w];
        qh[w] = CENTER ? B->qhalf[w] : 0u;
    }
#pragma unroll
    for (int e = 0; e < E; e++) {
        const int pos = slot_pos<PL, 0>(tau, e);
        uint32_t wa[W], wb[W];
        load_words<L64>(J.a + (size_t)pos * L64, wa);
        load_words<L64>(J.b + (size_t)pos * L64, wb);
        x[0][e] = crt_words<W, CENTER>(wa, cc, qh, c);
        x[1][e] = crt_words<W, CENTER>(wb, cc, qh, c);
    }
    // 1024-thread schedule: 64 registers per thread, constants folded from p
    const Mod m = LOGE == 3 ? mod_of(c.p) : c.m;
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
    if (tau == 0) atomicAdd(&done[4 * U.job], 1u);
}

// Keyswitch transforms of `count` primes of the keyswitch basis: digits of c
// (written by this launch's first epilogues, so read through L2), two digits
// per pass, multiply-accumulate with the evaluation key in the NTT domain.
template <int LOGN, int LOGE>
__device__ __forceinline__ void mixed_ks_unit(const MixedJob& J, const MixedUnit& U, uint32_t* smem,
                                              uint32_t* __restrict__ done) {
    using PL = NttPlan<LOGN, LOGE>;
    constexpr int E = PL::E, G = PL::G;
    constexpr int LAST = PL::NPASS - 1;
    constexpr int SUBW = 4 * PL::SMW;
    constexpr int STRIDE = 2 * PL::SMW;
    const int sub = threadIdx.x / G, tau = threadIdx.x % G;
    if (sub >= U.count) return;
    const int prime = U.first + sub;
    const GroupSync bar{1 + sub, G};
    uint32_t* sm = smem + sub * SUBW;
    const BasisDev* __restrict__ B = J.B2;
    const Mod m = LOGE == 3 ? mod_of(B->p[prime]) : load_mod(B, prime);
    const int k2 = J.k2, ell = J.ell;
    uint32_t acc[1][E];
#pragma unroll
    for (int e = 0; e < E; e++) acc[0][e] = 0;
    int buf = 0;
    for (int d0 = 0; d0 < ell; d0 += 2) {
        uint32_t x[2][E];
#pragma unroll
        for (int e = 0; e < E; e++) {
            const int pos = slot_pos<PL, 0>(tau, e);
#pragma unroll
            for (int o = 0; o < 2; o++) {
                const int d = d0 + o;
                uint32_t w = 0;
                if (d < ell) {  // c is limb-major here ([limb][N]): a warp's loads are contiguous
                    const uint64_t limb = __ldcg(reinterpret_cast<const unsigned long long*>(J.c) +
                                                 (size_t)(d >> 1) * PL::N + pos);
                    w = (uint32_t)(limb >> (32 * (d & 1)));
                }
                x[o][e] = __viaddmin_u32(w, m.np2, w);  // digit < 2^32 < 6p -> [0, 4p)
            }
        }
        buf = ntt_forward<PL, 2, GroupSync>(x, B->psi[prime], m, tau, sm, STRIDE, buf, bar);
#pragma unroll
        for (int o = 0; o < 2; o++) {
            const int d = d0 + o;
            if (d < ell) {
                const uint2* __restrict__ g = J.evk + ((size_t)d * k2 + prime) * PL::N;
#pragma unroll
                for (int e = 0; e < E; e++) {
                    const uint2 W = __ldg(g + slot_pos<PL, LAST>(tau, e));
                    acc[0][e] = mac_red(acc[0][e], shoup_m(x[o][e], W.x, W.y, m), m);
                }
            }
        }
    }
    ntt_inverse<PL, 1, GroupSync>(acc, B->ipsi[prime], m, tau, sm, STRIDE, buf, bar);
    uint32_t* out = J.resid + (size_t)prime * PL::N;
#pragma unroll
    for (int e = 0; e < E; e++) out[slot_pos<PL, 0>(tau, e)] = acc[0][e];
    __threadfence();
    bar.sync();
    if (tau == 0) atomicAdd(&done[4 * U.job + 2], 1u);
}

// C coefficients per thread and step (the constants of a prime are read once for
// all of them): 1 in the 64-register schedule, 2 in the 128-register one.
template <int L, int MODE, int C>
__device__ __forceinline__ void mixed_epi_coefs(const MixedJob& J, const BasisDev* __restrict__ B,
                                                const MixedUnit& U, EpiShared& S, int threads,
                                                unsigned long long frac_limit) {
    epi_stage<L, MODE>(S, B, threadIdx.x, threads);
    __syncthreads();
    const size_t n = (size_t)1 << J.logn;
    // a job with a keyswitch gets its first epilogue's output limb-major (the
    // keyswitch units' digit loads), and the keyswitch's epilogue writes over it
    const bool lm = U.kind == 1 && J.k2 > 0;
    const int end = U.first + U.count;
    for (int c0 = U.first + threadIdx.x; c0 < end; c0 += C * threads) {
        const uint32_t* r0[C];
        uint64_t* dst[C];
        bool st[C];
#pragma unroll
        for (int c = 0; c < C; c++) {
            int coef = c0 + c * threads;
            st[c] = coef < end;
            if (!st[c]) coef = c0;  // computed and not written
            r0[c] = J.resid + coef;
            dst[c] = J.c + (lm ? (size_t)coef : (size_t)coef * J.l64);
        }
        epi_coefs<L, MODE, C>(S, B, r0, n, dst, st, frac_limit, lm ? n : 1);
    }
}

template <int MODE, int C>
__device__ __forceinline__ void mixed_epi(const MixedJob& J, const BasisDev* __restrict__ B, const MixedUnit& U,
                                          EpiShared& S, int threads, unsigned long long frac_limit) {
    switch (J.l32) {
        case 1: mixed_epi_coefs<1, MODE, C>(J, B, U, S, threads, frac_limit); break;
        case 2: mixed_epi_coefs<2, MODE, C>(J, B, U, S, threads, frac_limit); break;
        case 3: mixed_epi_coefs<3, MODE, C>(J, B, U, S, threads, frac_limit); break;
        case 4: mixed_epi_coefs<4, MODE, C>(J, B, U, S, threads, frac_limit); break;
        case 5: mixed_epi_coefs<5, MODE, C>(J, B, U, S, threads, frac_limit); break;
        case 6: mixed_epi_coefs<6, MODE, C>(J, B, U, S, threads, frac_limit); break;
        default: break;
    }
}

__device__ __forceinline__ uint32_t load_acquire(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// ctl[0]: unit counter; ctl[1]: set when a wait expired; ctl[2]: units skipped.
template <int LOGE>
__global__ void __launch_bounds__(MixedSched<LOGE>::THREADS, MixedSched<LOGE>::MINB)
    k_mixed(const MixedJob* __restrict__ jobs, const MixedUnit* __restrict__ units, int n_units,
            uint32_t* __restrict__ done, uint32_t* __restrict__ ctl, unsigned spin_limit,
            unsigned long long frac_limit) {
    constexpr int THREADS = MixedSched<LOGE>::THREADS;
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
        if (U.kind != 0) {
            // inputs of this unit: every earlier-phase unit of its job
            const uint32_t need = U.kind == 1 ? (uint32_t)J.need0 : U.kind == 2 ? (uint32_t)J.n_epi : (uint32_t)J.k2;
            const uint32_t* cnt = &done[4 * U.job + (U.kind - 1)];
            if (threadIdx.x == 0) {
                unsigned spins = 0;
                while (load_acquire(cnt) < need && spins < spin_limit) {
                    __nanosleep(256);
                    spins++;
                }
                s_ok = load_acquire(cnt) >= need;
                if (!s_ok) {
                    atomicExch(&ctl[1], 1u);
                    atomicAdd(&ctl[2], 1u);
                }
            }
            __syncthreads();
            if (s_ok) __threadfence();
        }
        if (U.kind == 0) {
            switch (J.logn * 8 + J.l64 * 2 + J.centered) {
#define CY_MIXED_NTT(LOGN)                                                                            \
    case LOGN * 8 + 2: mixed_ntt_unit<LOGN, LOGE, 1, false>(J, U, smem, done); break;                 \
    case LOGN * 8 + 4: mixed_ntt_unit<LOGN, LOGE, 2, false>(J, U, smem, done); break;                 \
    case LOGN * 8 + 6: mixed_ntt_unit<LOGN, LOGE, 3, false>(J, U, smem, done); break;                 \
    case LOGN * 8 + 3: mixed_ntt_unit<LOGN, LOGE, 1, true>(J, U, smem, done); break;                  \
    case LOGN * 8 + 5: mixed_ntt_unit<LOGN, LOGE, 2, true>(J, U, smem, done); break;                  \
    case LOGN * 8 + 7: mixed_ntt_unit<LOGN, LOGE, 3, true>(J, U, smem, done); break;
                CY_MIXED_NTT(10)
                CY_MIXED_NTT(11)
                CY_MIXED_NTT(12)
                CY_MIXED_NTT(13)
#undef CY_MIXED_NTT
                default: break;
            }
        } else if (U.kind == 2) {
            if (s_ok) {
                switch (J.logn) {
                    case 10: mixed_ks_unit<10, LOGE>(J, U, smem, done); break;
                    case 11: mixed_ks_unit<11, LOGE>(J, U, smem, done); break;
                    case 12: mixed_ks_unit<12, LOGE>(J, U, smem, done); break;
                    case 13: mixed_ks_unit<13, LOGE>(J, U, smem, done); break;
                    default: break;
                }
            }
        } else if (s_ok) {  // kinds 1 and 3: epilogues
            constexpr int C = LOGE == 3 ? 1 : 2;
            if (U.kind == 1 && J.mode == EPI_YASHE) mixed_epi<EPI_YASHE, C>(J, J.B, U, S, THREADS, frac_limit);
            else mixed_epi<EPI_MODQ, C>(J, U.kind == 1 ? J.B : J.B2, U, S, THREADS, frac_limit);
            __threadfence();
            __syncthreads();
            if (threadIdx.x == 0) atomicAdd(&done[4 * U.job + (U.kind == 1 ? 1 : 3)], 1u);
        }
        __syncthreads();  // shared memory and s_unit are reused by the next unit
    }
}

// Dynamic shared memory: the same at every N for one schedule
// ((threads / (N/E)) sub-groups x 4 operand buffers of N + N/E words).
template <int LOGE>
constexpr size_t mixed_smem() {
    return (size_t)(MixedSched<LOGE>::THREADS / NttPlan<13, LOGE>::G) * 4 * NttPlan<13, LOGE>::SMW * sizeof(uint32_t);
}
static_assert(mixed_smem<3>() == (size_t)2 * 4 * NttPlan<12, 3>::SMW * 4 &&
                  mixed_smem<3>() == (size_t)8 * 4 * NttPlan<10, 3>::SMW * 4 &&
                  mixed_smem<4>() == (size_t)2 * 4 * NttPlan<12, 4>::SMW * 4 &&
                  mixed_smem<4>() == (size_t)8 * 4 * NttPlan<10, 4>::SMW * 4,
              "one shared-memory size serves every transform length");

// schedule 0: 8 coefficients per thread, 1024 threads; 1: 16 per thread, 512 threads
int mixed_schedules() { return 2; }
void* mixed_kernel(int sched) { return sched == 1 ? (void*)k_mixed<4> : (void*)k_mixed<3>; }
size_t mixed_smem_bytes(int sched) { return sched == 1 ? mixed_smem<4>() : mixed_smem<3>(); }
int mixed_threads(int sched) { return sched == 1 ? MixedSched<4>::THREADS : MixedSched<3>::THREADS; }
unsigned mixed_spin_default() { return kMixedSpinDefault; }

}  // namespace cy
