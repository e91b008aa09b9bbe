// kernels_pair.cuh -- product and keyswitch kernels for N = 16384 that run each
// (prime, job) on a cluster of two blocks.
//
// A length-16384 transform in one block needs 16 coefficients per thread (1024
// threads at most per block), and at the 64 registers a 1024-thread block allows
// its kernels spill. Here block h of the pair owns positions [h N/2, (h+1) N/2)
// with 8 coefficients per thread:
//   * the first forward stage (pairs j, j + N/2, twiddle psi^bitrev(1)) is the only
//     one that mixes the halves. The product kernel splits only its own half of
//     the inputs into residues and sends them to the peer through distributed
//     shared memory; the keyswitch reads both halves' digits (cheap) itself. Each
//     block then computes the stage and keeps its half;
//   * stages 1 .. 13 of half h are a length-8192 transform whose stage-s twiddles
//     start at (2 + h) 2^s (NttPlan<13, 3> with tm = 2 + h);
//   * the last inverse stage needs both halves: each block stores its half into the
//     other block's shared memory (distributed shared memory), both wait on the
//     cluster barrier, and each finishes its own half.
// The residues come out in natural order, as from the one-block kernels, so the
// epilogues are unchanged.
#pragma once

#include "kernels.cuh"

namespace cy {

__device__ __forceinline__ void cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

// word v at local shared address `local` of cluster block `peer`
__device__ __forceinline__ void store_peer(const uint32_t* local, uint32_t peer, uint32_t v) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(local);
    uint32_t remote;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(remote) : "r"(a), "r"(peer));
    asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(remote), "r"(v) : "memory");
}

using PairPlan = NttPlan<13, 3>;  // one half of N = 16384, 8 coefficients per thread, 1024 threads
constexpr int kPairHalf = PairPlan::N;

// Exchange words (two regions when they fit) plus the half received from the peer.
template <int NOPS>
__host__ __device__ constexpr size_t pair_smem_bytes() {
    return region_bytes<PairPlan, NOPS>() + (size_t)kPairHalf * 4;
}

// Last inverse stage across the pair, then the store of this block's half:
// x[e] holds half h at local position slot_pos<PairPlan, 0>(tau, e), in [0, 2p).
__device__ __forceinline__ void pair_finish(uint32_t (&x)[1][PairPlan::E], uint32_t* recv, uint32_t h, int tau,
                                            uint32_t p, uint2 w, uint32_t* __restrict__ out) {
    constexpr int E = PairPlan::E;
#pragma unroll
    for (int e = 0; e < E; e++) store_peer(&recv[slot_pos<PairPlan, 0>(tau, e)], h ^ 1u, x[0][e]);
    cluster_barrier();  // the peer's half has arrived
#pragma unroll
    for (int e = 0; e < E; e++) {
        const int pos = slot_pos<PairPlan, 0>(tau, e);
        const uint32_t other = recv[pos];
        const uint32_t lo = h ? other : x[0][e], hi = h ? x[0][e] : other;
        out[h * kPairHalf + pos] = h ? shoup(lo - hi + 2 * p, w.x, w.y, p) : red(lo + hi, 2 * p);
    }
}

// k_mul for N = 16384 on a block pair (see k_mul for the arguments).
template <int L64, bool CENTER>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(PairPlan::G, 1)
    k_mul_pair(const BasisDev* __restrict__ B, const uint64_t* __restrict__ A, long long a_stride,
               const uint64_t* __restrict__ Bv, long long b_stride, uint32_t* __restrict__ resid) {
    using PL = PairPlan;
    constexpr int E = PL::E;
    extern __shared__ uint32_t smem[];
    __shared__ uint32_t s_crt[L32MAX];
    __shared__ uint32_t s_qhalf[L32MAX];
    const int tau = threadIdx.x;
    const uint32_t h = cluster_rank();
    const int prime = blockIdx.x >> 1;
    const int job = blockIdx.y;
    const int k = B->k, l64 = B->l64;
    for (int i = tau; i < L32MAX; i += PL::G) {
        s_crt[i] = B->crt[prime][i];
        s_qhalf[i] = B->qhalf[i];
    }
    const PrimeCtx c = load_prime_ctx(B, prime);
    const uint2* __restrict__ psi = B->psi[prime];
    const uint2* __restrict__ ipsi = B->ipsi[prime];
    uint32_t* recv = smem + region_bytes<PL, 2>() / 4;
    cluster_barrier();  // both blocks have started before any remote store; s_crt is ready

    // CRT split of this block's half of a and b only; the peer's half arrives in
    // the first words of this block's exchange region (unused until the first
    // exchange, which follows the barrier below)
    const uint64_t* a = A + (size_t)job * a_stride + (size_t)h * kPairHalf * l64;
    const uint64_t* b = Bv + (size_t)job * b_stride + (size_t)h * kPairHalf * l64;
    uint32_t x[2][E];
#pragma unroll
    for (int e = 0; e < E; e++) {
        const int pos = slot_pos<PL, 0>(tau, e);
        if constexpr (L64 > 0) {
            constexpr int W = 2 * L64;
            uint32_t cc[W], qh[W];
#pragma unroll
            for (int j = 0; j < W; j++) {
                cc[j] = s_crt[j];
                qh[j] = s_qhalf[j];
            }
            uint32_t w[W];
            load_words<L64>(a + (size_t)pos * L64, w);
            x[0][e] = crt_words<W, CENTER>(w, cc, qh, c);
            load_words<L64>(b + (size_t)pos * L64, w);
            x[1][e] = crt_words<W, CENTER>(w, cc, qh, c);
        } else {
            x[0][e] = crt_coef<CENTER>(a, pos, l64, s_crt, s_qhalf, c);
            x[1][e] = crt_coef<CENTER>(b, pos, l64, s_crt, s_qhalf, c);
        }
#pragma unroll
        for (int o = 0; o < 2; o++) store_peer(&smem[o * kPairHalf + pos], h ^ 1u, x[o][e]);
    }
    cluster_barrier();  // the peer's half of a and b has arrived
    const uint2 w0 = __ldg(psi + 1);
#pragma unroll
    for (int e = 0; e < E; e++) {
        const int pos = slot_pos<PL, 0>(tau, e);
#pragma unroll
        for (int o = 0; o < 2; o++) {
            const uint32_t other = smem[o * kPairHalf + pos];
            uint32_t lo = h ? other : x[o][e], hi = h ? x[o][e] : other;
            ct_bfly(lo, hi, w0.x, w0.y, c.m);  // first stage of the whole transform
            x[o][e] = h ? hi : lo;
        }
    }
    __syncthreads();  // every thread has read region 0 before the first exchange writes it
    constexpr int STRIDE = region_stride<PL, 2>();
    const int tm = 2 + (int)h;
    int buf = ntt_forward<PL, 2>(x, psi, c.m, tau, smem, STRIDE, 0, CtaSync(), tm);
    uint32_t z[1][E];
#pragma unroll
    for (int e = 0; e < E; e++) z[0][e] = mont(red(x[0][e], 2 * c.p), red(x[1][e], 2 * c.p), c.p, c.pinv);
    ntt_inverse<PL, 1>(z, ipsi, c.m, tau, smem, STRIDE, buf, CtaSync(), tm);
    pair_finish(z, recv, h, tau, c.p, __ldg(ipsi + 1), resid + ((size_t)job * k + prime) * (2 * kPairHalf));
}

// k_keyswitch for N = 16384 on a block pair, ND digits per pass (see k_keyswitch).
template <int L64, int ND>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(PairPlan::G, 1)
    k_keyswitch_pair(const BasisDev* __restrict__ B, const uint64_t* __restrict__ C, const uint2* __restrict__ evk,
                     int ell, uint32_t* __restrict__ resid, int cs, int ls) {
    using PL = PairPlan;
    constexpr int E = PL::E;
    constexpr int LAST = PL::NPASS - 1;
    static_assert(PL::LOGD(LAST) == 0 && PL::R(LAST) == PL::LOGE, "contiguous last-pass positions");
    extern __shared__ uint32_t smem[];
    const int tau = threadIdx.x;
    const uint32_t h = cluster_rank();
    const int prime = blockIdx.x >> 1;
    const int job = blockIdx.y;
    const int k = B->k, l64 = L64 > 0 ? L64 : B->l64;
    const Mod m = load_mod(B, prime);
    const uint32_t p = m.p;
    const uint2* __restrict__ psi = B->psi[prime];
    const uint2* __restrict__ ipsi = B->ipsi[prime];
    const uint64_t* cj = C + (size_t)job * (2 * kPairHalf) * l64;
    // limb w of coefficient pos at cj[pos * cs + w * ls]: (limbs, 1) for [N][limb],
    // (1, N) for limb-major
    uint32_t* recv = smem + region_bytes<PL, ND>() / 4;
    constexpr int STRIDE = region_stride<PL, ND>();
    const int tm = 2 + (int)h;
    const uint2 w0 = __ldg(psi + 1);
    cluster_barrier();  // both blocks have started before any remote store

    uint32_t acc[1][E];
#pragma unroll
    for (int e = 0; e < E; e++) acc[0][e] = 0;
    int buf = 0;
    for (int d0 = 0; d0 < ell; d0 += ND) {
        uint32_t x[ND][E];
#pragma unroll
        for (int e = 0; e < E; e++) {
            const int pos = slot_pos<PL, 0>(tau, e);
            uint32_t lo[ND], hi[ND];
#pragma unroll
            for (int o = 0; o < ND; o++) {
                const int d = d0 + o;
                uint32_t wl = 0, wh = 0;
                if (L64 > 0 || d < ell) {  // digits past the top word of q are zero
                    const uint64_t ll = __ldg(cj + (size_t)pos * cs + (size_t)(d >> 1) * ls);
                    const uint64_t lh = __ldg(cj + (size_t)(pos + kPairHalf) * cs + (size_t)(d >> 1) * ls);
                    wl = (uint32_t)(ll >> (32 * (d & 1)));
                    wh = (uint32_t)(lh >> (32 * (d & 1)));
                }
                lo[o] = red(wl, 2 * p);  // digit < 2^32 < 6p -> [0, 4p)
                hi[o] = red(wh, 2 * p);
                ct_bfly(lo[o], hi[o], w0.x, w0.y, m);  // first stage of the whole transform
                x[o][e] = h ? hi[o] : lo[o];
            }
        }
        buf = ntt_forward<PL, ND>(x, psi, m, tau, smem, STRIDE, buf, CtaSync(), tm);
#pragma unroll
        for (int o = 0; o < ND; o++) {
            const int d = d0 + o;
            if (d < ell) {
                const uint2* __restrict__ g = evk + ((size_t)d * k + prime) * (2 * kPairHalf) + h * kPairHalf;
                const uint4* g4 = reinterpret_cast<const uint4*>(g + group_base<PL, LAST>(tau, 0));
#pragma unroll
                for (int q = 0; q < E / 2; q++) {
                    const uint4 W = __ldg(g4 + q);
                    acc[0][2 * q] = mac_red(acc[0][2 * q], shoup_m(x[o][2 * q], W.x, W.y, m), m);
                    acc[0][2 * q + 1] = mac_red(acc[0][2 * q + 1], shoup_m(x[o][2 * q + 1], W.z, W.w, m), m);
                }
            }
        }
    }
    ntt_inverse<PL, 1>(acc, ipsi, m, tau, smem, STRIDE, buf, CtaSync(), tm);
    pair_finish(acc, recv, h, tau, p, __ldg(ipsi + 1), resid + ((size_t)job * k + prime) * (2 * kPairHalf));
}

}  // namespace cy
