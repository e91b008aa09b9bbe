// kernels.cuh -- CUDA kernels of the multiply path (templates; instantiated in
// the k_*.cu translation units).
//
//   k_mul        per (job, prime): CRT split of a and b -> forward NTTs ->
//                pointwise Montgomery product -> inverse NTT -> residues.
//                Replaces callCRT (src/cuda_bn.cu:970-1002) and the NTT branch of
//                callPolynomialMul (src/cuda_functions.cu:658-738).
//   k_keyswitch  per (job, prime): base-2^32 digits of c -> forward NTTs ->
//                sum_d D_d * evk_d in the NTT domain -> inverse NTT -> residues.
//                Replaces Ciphertext::keyswitch (src/ciphertext.cpp:81-107).
//   k_epi        per coefficient: ICRT of the k residues to the exact integer,
//                then mod q, round(t/q .) or decryption. Replaces cuPreICRT /
//                cuICRT / cuModN (src/cuda_bn.cu:759-968), Polynomial::reduce's
//                mod q (src/cuda_functions.cu:1076) and the host rounding loop
//                of Ciphertext::operator* (src/ciphertext.cpp:55-63).
//   k_ntt, k_crt standalone transforms (callNTT, callCRT).
#pragma once

#include <stdint.h>

#include "arith.cuh"
#include "common.h"
#include "dispatch.h"
#include "ntt_core.cuh"

namespace cy {

// Exchange-region stride (words) for a kernel whose widest exchange carries
// NOPS operands: two alternating regions when they fit, else one (stride 0).
template <class PL, int NOPS>
__host__ __device__ constexpr int region_stride() {
    return (size_t)2 * NOPS * PL::SMW * 4 <= kSmemDoubleLimit ? NOPS * PL::SMW : 0;
}
template <class PL, int NOPS>
__host__ __device__ constexpr size_t region_bytes() {
    return (size_t)(region_stride<PL, NOPS>() ? 2 : 1) * NOPS * PL::SMW * 4;
}

// The modulus of prime i with its derived constants, each read on its own.
__device__ __forceinline__ Mod load_mod(const BasisDev* __restrict__ B, int i) {
    Mod m;
    m.p = B->p[i];
    m.p2 = B->p2[i];
    m.np = B->np[i];
    m.np2 = B->np2[i];
    return m;
}

// a + b reduced from [0, 4p) to [0, 2p) (a, b in [0, 2p)): one add, one add-then-min
__device__ __forceinline__ uint32_t mac_red(uint32_t a, uint32_t b, const Mod& m) {
    return __viaddmin_u32(a, b, a + b + m.np2);
}

// Per-prime constants a product kernel keeps in registers.
struct PrimeCtx {
    uint32_t p, pinv, r32, r32_sh, one_sh, qmodp;
    Mod m;
};

__device__ __forceinline__ PrimeCtx load_prime_ctx(const BasisDev* __restrict__ B, int i) {
    PrimeCtx c;
    c.m = load_mod(B, i);
    c.p = c.m.p;
    c.pinv = B->pinv[i];
    c.r32 = B->r32[i];
    c.r32_sh = B->r32_sh[i];
    c.one_sh = (uint32_t)(0x100000000ULL / c.p);  // Shoup companion of 1
    c.qmodp = B->qmodp[i];
    return c;
}

// 64-bit partial sum T (< 2^64) -> value in [0, 2p)
__device__ __forceinline__ uint32_t fold64(uint64_t T, const PrimeCtx& c) {
    const uint32_t hi = (uint32_t)(T >> 32), lo = (uint32_t)T;
    const uint32_t a = shoup(hi, c.r32, c.r32_sh, c.p) + shoup(lo, 1u, c.one_sh, c.p);
    return red(a, 2 * c.p);
}

// Residue of coefficient `pos` of a polynomial stored as [N][l64] limbs, in
// [0, 4p) (valid forward-NTT input). `crt` (shared memory) holds 2^(32 j) mod p
// for j < 2*l64 <= L32MAX. With CENTER, values above (q-1)/2 stand for x - q.
template <bool CENTER>
__device__ __forceinline__ uint32_t crt_coef(const uint64_t* __restrict__ src, int pos, int l64,
                                             const uint32_t* crt, const uint32_t* qhalf, const PrimeCtx& c) {
    const uint64_t* s = src + (size_t)pos * l64;
    uint64_t T = 0;
    uint32_t acc = 0;
    bool gt = false;
    for (int j = 0; j < l64; j++) {
        const uint64_t limb = __ldg(s + j);
        const uint32_t lo = (uint32_t)limb, hi = (uint32_t)(limb >> 32);
        T += (uint64_t)lo * crt[2 * j] + (uint64_t)hi * crt[2 * j + 1];
        if (CENTER) {
            const uint32_t h0 = qhalf[2 * j], h1 = qhalf[2 * j + 1];
            gt = (lo > h0) || (lo == h0 && gt);
            gt = (hi > h1) || (hi == h1 && gt);
        }
        if ((j & 1) || j == l64 - 1) {  // at most 4 products of < 2^62 per partial sum
            acc = red(acc + fold64(T, c), 2 * c.p);
            T = 0;
        }
    }
    if (CENTER && gt) acc = acc + 2 * c.p - c.qmodp;  // [0, 4p)
    return acc;
}

// The limbs of one coefficient as 32-bit words (16-byte loads when L64 is even).
template <int L64>
__device__ __forceinline__ void load_words(const uint64_t* __restrict__ p, uint32_t (&w)[2 * L64]) {
    if constexpr (L64 % 2 == 0) {
#pragma unroll
        for (int i = 0; i < L64 / 2; i++) {
            const uint4 v = __ldg(reinterpret_cast<const uint4*>(p) + i);
            w[4 * i] = v.x;
            w[4 * i + 1] = v.y;
            w[4 * i + 2] = v.z;
            w[4 * i + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int i = 0; i < L64; i++) {
            const uint2 v = __ldg(reinterpret_cast<const uint2*>(p) + i);
            w[2 * i] = v.x;
            w[2 * i + 1] = v.y;
        }
    }
}

// Residue in [0, 4p) of the coefficient whose 32-bit words are w (compile-time
// count W); cc[j] = 2^(32 j) mod p. With CENTER, values above (q-1)/2 (words
// qh) stand for x - q.
template <int W, bool CENTER>
__device__ __forceinline__ uint32_t crt_words(const uint32_t (&w)[W], const uint32_t (&cc)[W],
                                              const uint32_t (&qh)[W], const PrimeCtx& c) {
    uint32_t acc = 0;
#pragma unroll
    for (int j0 = 0; j0 < W; j0 += 4) {
        uint64_t T = 0;
#pragma unroll
        for (int j = j0; j < j0 + 4 && j < W; j++) T += (uint64_t)w[j] * cc[j];  // < 4 * 2^62
        const uint32_t f = fold64(T, c);
        acc = (j0 == 0) ? f : red(acc + f, 2 * c.p);
    }
    if (CENTER) {
        // x > (q-1)/2: one 64- or 128-bit compare (no branch) for two or four
        // words; for more, the top words decide unless they are equal (rare),
        // then the lower words do
        bool gt;
        if constexpr (W == 2) {
            gt = ((uint64_t)w[1] << 32 | w[0]) > ((uint64_t)qh[1] << 32 | qh[0]);
        } else if constexpr (W == 4) {
            // (q-1)/2 - x borrows exactly when x > (q-1)/2: one subtract-with-borrow
            // chain, its final borrow spread to a mask (no compares, no selects)
            uint32_t mask;
            asm("{\n\t.reg .u32 d;\n\t"
                "sub.cc.u32 d, %1, %5;\n\t"
                "subc.cc.u32 d, %2, %6;\n\t"
                "subc.cc.u32 d, %3, %7;\n\t"
                "subc.cc.u32 d, %4, %8;\n\t"
                "subc.u32 %0, 0, 0;\n\t}"
                : "=r"(mask)
                : "r"(qh[0]), "r"(qh[1]), "r"(qh[2]), "r"(qh[3]), "r"(w[0]), "r"(w[1]), "r"(w[2]), "r"(w[3]));
            return acc + (mask & (2 * c.p - c.qmodp));  // [0, 4p)
        } else {
            gt = w[W - 1] > qh[W - 1];
            if (w[W - 1] == qh[W - 1]) {
                bool g = false;
#pragma unroll
                for (int j = 0; j < W - 1; j++) g = (w[j] > qh[j]) || (w[j] == qh[j] && g);
                gt = g;
            }
        }
        acc += gt ? 2 * c.p - c.qmodp : 0u;  // [0, 4p)
    }
    return acc;
}

// --------------------------------------------------------------------------
// k_mul: one block per (prime, job); G = N/E threads
// --------------------------------------------------------------------------
// L64 > 0: coefficients have exactly L64 limbs (specialised load and CRT
// split); L64 == 0: the limb count is read from the basis at run time.
// Blocks per SM the product kernel is compiled for: 48 resident warps with 8
// coefficients per thread, 32 with 16 (more registers per thread).
template <int LOGN, int LOGE>
constexpr int mul_min_blocks() {
    constexpr int G = NttPlan<LOGN, LOGE>::G;
    constexpr int target = (LOGE <= 3 ? 1536 : 1024) / G;
    return target < 1 ? 1 : (target > 16 ? 16 : target);
}
template <int LOGN, int LOGE>
constexpr int ks_min_blocks() {
    constexpr int G = NttPlan<LOGN, LOGE>::G;
    constexpr int target = 1024 / G;
    return target < 1 ? 1 : (target > 16 ? 16 : target);
}

// MINB > 0 overrides the blocks per SM the kernel is compiled for (a schedule
// with a larger register budget per thread).
// SINGLE: one exchange region (two barriers per exchange), so that more blocks
// fit in shared memory.
template <int LOGN, int LOGE, int L64, bool CENTER, int MINB = 0, bool SINGLE = false>
__global__ void __launch_bounds__(NttPlan<LOGN, LOGE>::G, (MINB > 0 ? MINB : mul_min_blocks<LOGN, LOGE>()))
    k_mul(const BasisDev* __restrict__ B, const uint64_t* __restrict__ A, long long a_stride,
          const uint64_t* __restrict__ Bv, long long b_stride, uint32_t* __restrict__ resid) {
    using PL = NttPlan<LOGN, LOGE>;
    constexpr int E = PL::E;
    extern __shared__ uint32_t smem[];  // exchange regions, 2 operands x SMW each
    __shared__ uint32_t s_crt[L32MAX];
    __shared__ uint32_t s_qhalf[L32MAX];
    const int tau = threadIdx.x;
    const int prime = blockIdx.x;
    const int job = blockIdx.y;
    const int k = B->k, l64 = B->l64;
    for (int i = tau; i < L32MAX; i += PL::G) {  // blocks of small N have fewer than L32MAX threads
        s_crt[i] = B->crt[prime][i];
        s_qhalf[i] = B->qhalf[i];
    }
    const PrimeCtx c = load_prime_ctx(B, prime);
    const uint2* __restrict__ psi = B->psi[prime];
    const uint2* __restrict__ ipsi = B->ipsi[prime];
    __syncthreads();

    const uint64_t* a = A + (size_t)job * a_stride;
    const uint64_t* b = Bv + (size_t)job * b_stride;
    uint32_t x[2][E];
    if constexpr (L64 > 0) {
        constexpr int W = 2 * L64;
        uint32_t cc[W], qh[W];
#pragma unroll
        for (int j = 0; j < W; j++) {
            cc[j] = s_crt[j];
            qh[j] = s_qhalf[j];
        }
#pragma unroll
        for (int e = 0; e < E; e++) {
            const int pos = slot_pos<PL, 0>(tau, e);
            uint32_t wa[W], wb[W];
            load_words<L64>(a + (size_t)pos * L64, wa);
            load_words<L64>(b + (size_t)pos * L64, wb);
            x[0][e] = crt_words<W, CENTER>(wa, cc, qh, c);
            x[1][e] = crt_words<W, CENTER>(wb, cc, qh, c);
        }
    } else {
#pragma unroll
        for (int e = 0; e < E; e++) {
            const int pos = slot_pos<PL, 0>(tau, e);
            x[0][e] = crt_coef<CENTER>(a, pos, l64, s_crt, s_qhalf, c);
            x[1][e] = crt_coef<CENTER>(b, pos, l64, s_crt, s_qhalf, c);
        }
    }
    constexpr int STRIDE = SINGLE ? 0 : region_stride<PL, 2>();
    // 64 coefficients per thread at N = 4096: both transforms loop over one copy of
    // the pass code (the unrolled three transforms overflow the instruction cache)
    constexpr bool LOOP64 = LOGN == 12 && LOGE == 6;
    int buf = 0;
    if constexpr (LOOP64) ntt64_forward<PL, 2>(x, psi, B->psi_r[prime], c.m, tau, smem);
    else buf = ntt_forward<PL, 2>(x, psi, c.m, tau, smem, STRIDE, 0, CtaSync(), 1, B->psi_r[prime]);
    uint32_t z[1][E];
#pragma unroll
    for (int e = 0; e < E; e++) z[0][e] = mont(red(x[0][e], 2 * c.p), red(x[1][e], 2 * c.p), c.p, c.pinv);
    if constexpr (LOOP64) ntt64_inverse<PL, 1>(z, ipsi, B->ipsi_r[prime], c.m, tau, smem + STRIDE, STRIDE == 0, nullptr);
    else ntt_inverse<PL, 1>(z, ipsi, c.m, tau, smem, STRIDE, buf, CtaSync(), 1, B->ipsi_r[prime]);
    uint32_t* out = resid + ((size_t)job * k + prime) * PL::N;
#pragma unroll
    for (int e = 0; e < E; e++) out[slot_pos<PL, 0>(tau, e)] = z[0][e];
}

// --------------------------------------------------------------------------
// k_keyswitch: one block per (prime, job). Digits are the 32-bit words of the
// coefficients of c in [0, q) (w = 2^32), processed ND at a time.
// evk: [ell][k][N] (value, Shoup companion) in the forward-NTT output order.
// --------------------------------------------------------------------------
// SINGLE: one exchange region (two barriers per exchange) instead of two, so
// that more blocks fit in shared memory.
template <int LOGN, int LOGE, int L64, int ND, int MINB = 0, bool SINGLE = false>
__global__ void __launch_bounds__(NttPlan<LOGN, LOGE>::G, (MINB > 0 ? MINB : ks_min_blocks<LOGN, LOGE>()))
    k_keyswitch(const BasisDev* __restrict__ B, const uint64_t* __restrict__ C, const uint2* __restrict__ evk,
                int ell, uint32_t* __restrict__ resid, int cs, int ls) {
    using PL = NttPlan<LOGN, LOGE>;
    constexpr int E = PL::E;
    constexpr int LAST = PL::NPASS - 1;
    extern __shared__ uint32_t smem[];  // exchange regions, ND operands x SMW each
    const int tau = threadIdx.x;
    const int prime = blockIdx.x;
    const int job = blockIdx.y;
    const int k = B->k, l64 = L64 > 0 ? L64 : B->l64;
    const Mod m = load_mod(B, prime);
    const uint32_t p = m.p;
    const uint2* __restrict__ psi = B->psi[prime];
    const uint2* __restrict__ ipsi = B->ipsi[prime];
    const uint64_t* cj = C + (size_t)job * PL::N * l64;
    // limb w of coefficient pos at cj[pos * cs + w * ls]: (cs, ls) = (limbs, 1) for
    // [N][limb], (1, N) for limb-major (the HE multiply's intermediate: a warp's
    // loads of one limb are then contiguous). Kernel parameters, so that they stay
    // in the constant bank.
    constexpr int STRIDE = SINGLE ? 0 : region_stride<PL, ND>();

    uint32_t acc[1][E];
#pragma unroll
    for (int e = 0; e < E; e++) acc[0][e] = 0;
    int buf = 0;
    for (int d0 = 0; d0 < ell; d0 += ND) {
        uint32_t x[ND][E];
#pragma unroll
        for (int e = 0; e < E; e++) {
            const int pos = slot_pos<PL, 0>(tau, e);
            if constexpr (L64 > 0 && ND % 2 == 0) {
                // digits d0 .. d0+ND-1 are limbs d0/2 .. d0/2+ND/2-1 of the coefficient;
                // digits past the last word of q are zero (coefficients are < q)
                const uint64_t* src = cj + (size_t)pos * cs + (size_t)(d0 >> 1) * ls;
                uint32_t w[ND];
                bool both = false;  // two limbs side by side: one 16-byte load
                if constexpr (ND == 4 && L64 % 2 == 0) {
                    if (ls == 1) {
                        const uint4 v = __ldg(reinterpret_cast<const uint4*>(src));
                        w[0] = v.x;
                        w[1] = v.y;
                        w[ND - 2] = v.z;
                        w[ND - 1] = v.w;
                        both = true;
                    }
                }
                if (!both) {
#pragma unroll
                    for (int o = 0; o < ND; o += 2) {
                        const uint2 v = __ldg(reinterpret_cast<const uint2*>(src + (o >> 1) * ls));
                        w[o] = v.x;
                        w[o + 1] = v.y;
                    }
                }
#pragma unroll
                for (int o = 0; o < ND; o++) x[o][e] = red(w[o], 2 * p);  // digit < 2^32 < 6p -> [0, 4p)
            } else {
#pragma unroll
                for (int o = 0; o < ND; o++) {
                    const int d = d0 + o;
                    uint32_t w = 0;
                    if (d < ell) {
                        const uint64_t limb = __ldg(cj + (size_t)pos * cs + (size_t)(d >> 1) * ls);
                        w = (uint32_t)(limb >> (32 * (d & 1)));
                    }
                    x[o][e] = red(w, 2 * p);  // digit < 2^32 < 6p -> [0, 4p)
                }
            }
        }
        if constexpr (LOGN == 12 && LOGE == 6) {  // one copy of the pass code (see k_mul)
            ntt64_forward<PL, ND>(x, psi, B->psi_r[prime], m, tau, smem, true);
            buf++;
        } else {
            buf = ntt_forward<PL, ND>(x, psi, m, tau, smem, STRIDE, buf, CtaSync(), 1, B->psi_r[prime]);
        }
#pragma unroll
        for (int o = 0; o < ND; o++) {
            const int d = d0 + o;
            if (d < ell) {
                const uint2* __restrict__ g = evk + ((size_t)d * k + prime) * PL::N;
                if constexpr (rows_pass<PL, LAST>()) {
                    // the key's copy laid out by lane (after the [ell][k][N] table): the
                    // pair (u, u+1) of lane tau is the 16-byte record [u/2][tau]
                    const uint4* g4 = reinterpret_cast<const uint4*>(g + (size_t)ell * k * PL::N) + tau;
#pragma unroll
                    for (int h = 0; h < E / 2; h++) {
                        const uint4 W = __ldg(g4 + h * PL::G);
                        acc[0][2 * h] = mac_red(acc[0][2 * h], shoup_m(x[o][2 * h], W.x, W.y, m), m);
                        acc[0][2 * h + 1] = mac_red(acc[0][2 * h + 1], shoup_m(x[o][2 * h + 1], W.z, W.w, m), m);
                    }
                } else if constexpr (PL::LOGD(LAST) == 0 && PL::R(LAST) == PL::LOGE) {
                    // after the last pass a thread's E positions are contiguous: 16-byte loads
                    const uint4* g4 = reinterpret_cast<const uint4*>(g + group_base<PL, LAST>(tau, 0));
#pragma unroll
                    for (int h = 0; h < E / 2; h++) {
                        const uint4 W = __ldg(g4 + h);
                        acc[0][2 * h] = mac_red(acc[0][2 * h], shoup_m(x[o][2 * h], W.x, W.y, m), m);
                        acc[0][2 * h + 1] = mac_red(acc[0][2 * h + 1], shoup_m(x[o][2 * h + 1], W.z, W.w, m), m);
                    }
                } else {
#pragma unroll
                    for (int e = 0; e < E; e++) {
                        const uint2 W = __ldg(g + slot_pos<PL, LAST>(tau, e));
                        acc[0][e] = mac_red(acc[0][e], shoup_m(x[o][e], W.x, W.y, m), m);
                    }
                }
            }
        }
    }
    if constexpr (LOGN == 12 && LOGE == 6) ntt64_inverse<PL, 1>(acc, ipsi, B->ipsi_r[prime], m, tau, smem, true, nullptr);
    else ntt_inverse<PL, 1>(acc, ipsi, m, tau, smem, STRIDE, buf, CtaSync(), 1, B->ipsi_r[prime]);
    uint32_t* out = resid + ((size_t)job * k + prime) * PL::N;
#pragma unroll
    for (int e = 0; e < E; e++) out[slot_pos<PL, 0>(tau, e)] = acc[0][e];
}

// --------------------------------------------------------------------------
// k_ntt: in-place transform of residue vectors [batch][k][N], values in [0, p).
// Forward output in bit-reversed order; inverse includes N^-1. A block runs the
// transforms of two jobs for one prime side by side (shared twiddle loads and
// barriers); with an odd job count the last block repeats its job and stores it
// once.
// --------------------------------------------------------------------------
template <int LOGN, int LOGE, bool INV>
__global__ void __launch_bounds__(NttPlan<LOGN, LOGE>::G)
    k_ntt(const BasisDev* __restrict__ B, uint32_t* __restrict__ res, const uint32_t* __restrict__ ninv,
          int njobs) {
    using PL = NttPlan<LOGN, LOGE>;
    constexpr int E = PL::E;
    constexpr int LAST = PL::NPASS - 1;
    extern __shared__ uint32_t smem[];
    const int tau = threadIdx.x;
    const int prime = blockIdx.x;
    const int job0 = 2 * blockIdx.y;
    const bool two = job0 + 1 < njobs;
    const int k = B->k;
    const Mod m = load_mod(B, prime);
    const uint32_t p = m.p;
    uint32_t* v[2] = {res + ((size_t)job0 * k + prime) * PL::N, res + ((size_t)(two ? job0 + 1 : job0) * k + prime) * PL::N};
    uint32_t x[2][E];
    constexpr int STRIDE = region_stride<PL, 2>();
    // after the last pass a thread's E positions are contiguous (16-byte accesses)
    constexpr bool VEC = PL::LOGD(LAST) == 0 && PL::R(LAST) == PL::LOGE && E % 4 == 0;
    if (!INV) {
#pragma unroll
        for (int o = 0; o < 2; o++)
#pragma unroll
            for (int e = 0; e < E; e++) x[o][e] = v[o][slot_pos<PL, 0>(tau, e)];
        ntt_forward<PL, 2>(x, B->psi[prime], m, tau, smem, STRIDE, 0);
#pragma unroll
        for (int o = 0; o < 2; o++) {
            if (o == 1 && !two) break;
            if constexpr (VEC) {
                uint4* d4 = reinterpret_cast<uint4*>(v[o] + group_base<PL, LAST>(tau, 0));
#pragma unroll
                for (int h = 0; h < E / 4; h++)
                    d4[h] = make_uint4(red(red(x[o][4 * h], 2 * p), p), red(red(x[o][4 * h + 1], 2 * p), p),
                                       red(red(x[o][4 * h + 2], 2 * p), p), red(red(x[o][4 * h + 3], 2 * p), p));
            } else {
#pragma unroll
                for (int e = 0; e < E; e++) v[o][slot_pos<PL, LAST>(tau, e)] = red(red(x[o][e], 2 * p), p);
            }
        }
    } else {
        const uint32_t w = ninv[4 * prime], ws = ninv[4 * prime + 1];
#pragma unroll
        for (int o = 0; o < 2; o++) {
            if constexpr (VEC) {
                const uint4* s4 = reinterpret_cast<const uint4*>(v[o] + group_base<PL, LAST>(tau, 0));
#pragma unroll
                for (int h = 0; h < E / 4; h++) {
                    const uint4 q4 = s4[h];
                    x[o][4 * h] = q4.x;
                    x[o][4 * h + 1] = q4.y;
                    x[o][4 * h + 2] = q4.z;
                    x[o][4 * h + 3] = q4.w;
                }
            } else {
#pragma unroll
                for (int e = 0; e < E; e++) x[o][e] = v[o][slot_pos<PL, LAST>(tau, e)];
            }
        }
        ntt_inverse<PL, 2>(x, B->ipsi[prime], m, tau, smem, STRIDE, 0);
#pragma unroll
        for (int o = 0; o < 2; o++) {
            if (o == 1 && !two) break;
#pragma unroll
            for (int e = 0; e < E; e++) v[o][slot_pos<PL, 0>(tau, e)] = red(shoup(x[o][e], w, ws, p), p);
        }
    }
}

// --------------------------------------------------------------------------
// k_ntt1: the same transform, one residue vector per block, for schedules whose
// threads hold many coefficients (E = 64: 64 threads, two register passes of six
// stages and one exchange, a transpose through shared memory). Grid (jobs,
// primes): consecutive blocks share a prime, so the blocks resident on an SM
// read the same twiddle table (L1 hits).
// MINB > 0: blocks per SM the kernel is compiled for.
// COAL (two passes of six stages): the row side of the transform (forward
// output, inverse input) goes through the exchange region once more, so that
// every global access of a warp covers 128 consecutive bytes instead of 32
// rows 256 bytes apart.
// TPB: transforms per block (TPB groups of G threads, one exchange region each,
// block-wide barriers). Several transforms in step keep the warps of an SM on
// nearby instructions (the unrolled transform is larger than the instruction
// cache). Jobs past the last are computed on the last job and not stored.
// --------------------------------------------------------------------------
// LOOP (N = 4096, E = 64): the two passes run as a loop over one copy of the pass
// code (ntt_core.cuh, ntt64_forward / ntt64_inverse).
template <int LOGN, int LOGE, bool INV, int MINB = 0, bool COAL = false, int TPB = 1, bool LOOP = false>
__global__ void __launch_bounds__(NttPlan<LOGN, LOGE>::G * TPB, (MINB > 0 ? MINB : 1))
    k_ntt1(const BasisDev* __restrict__ B, uint32_t* __restrict__ res, const uint32_t* __restrict__ ninv,
           int njobs) {
    using PL = NttPlan<LOGN, LOGE>;
    constexpr int E = PL::E;
    constexpr int LAST = PL::NPASS - 1;
    static_assert(!COAL || (PL::NPASS == 2 && LOGE == 6 && LOGN == 12), "row-side staging: N = 4096, E = 64");
    extern __shared__ uint32_t smem_all[];
    const int sub = TPB > 1 ? (int)threadIdx.x / PL::G : 0;
    const int tau = TPB > 1 ? (int)threadIdx.x % PL::G : (int)threadIdx.x;
    uint32_t* smem = smem_all + sub * PL::SMW;
    const int job_raw = blockIdx.x * TPB + sub;
    const bool store = job_raw < njobs;
    const int job = store ? job_raw : njobs - 1;
    const int prime = blockIdx.y;
    const int k = B->k;
    const Mod m = load_mod(B, prime);
    const uint32_t p = m.p;
    uint32_t* v = res + ((size_t)job * k + prime) * PL::N;
    uint32_t x[1][E];
    // one exchange (two passes) needs no barrier ahead of its writes: a second,
    // never used region offset stands in for the alternation; more passes share
    // one region with a barrier before each exchange
    constexpr int STRIDE = PL::NPASS <= 2 ? PL::SMW : 0;
    constexpr bool VEC = PL::LOGD(LAST) == 0 && PL::R(LAST) == PL::LOGE && E % 4 == 0;
    if (!INV) {
#pragma unroll
        for (int e = 0; e < E; e++) x[0][e] = COAL ? __ldcs(v + slot_pos<PL, 0>(tau, e)) : v[slot_pos<PL, 0>(tau, e)];
        if constexpr (LOOP) ntt64_forward<PL, 1>(x, B->psi[prime], B->psi_r[prime], m, tau, smem);
        else ntt_forward<PL, 1>(x, B->psi[prime], m, tau, smem, STRIDE, 0, CtaSync(), 1, B->psi_r[prime]);
        if constexpr (COAL) {
            // row tau (positions 64 tau + u) into the padded region (word 65 tau + u),
            // then column tau (positions tau + 64 m, word 65 m + tau) to global memory
            __syncthreads();
#pragma unroll
            for (int u = 0; u < E; u++) smem[65 * tau + u] = red(red(x[0][u], 2 * p), p);
            __syncthreads();
            if (store) {
#pragma unroll
                for (int m = 0; m < E; m++) __stcs(v + tau + 64 * m, smem[tau + 65 * m]);
            }
        } else if constexpr (VEC) {
            if (store) {
                uint4* d4 = reinterpret_cast<uint4*>(v + group_base<PL, LAST>(tau, 0));
#pragma unroll
                for (int h = 0; h < E / 4; h++)
                    d4[h] = make_uint4(red(red(x[0][4 * h], 2 * p), p), red(red(x[0][4 * h + 1], 2 * p), p),
                                       red(red(x[0][4 * h + 2], 2 * p), p), red(red(x[0][4 * h + 3], 2 * p), p));
            }
        } else if (store) {
#pragma unroll
            for (int e = 0; e < E; e++) v[slot_pos<PL, LAST>(tau, e)] = red(red(x[0][e], 2 * p), p);
        }
    } else {
        int stride = STRIDE;
        if constexpr (COAL) {
            // columns in (coalesced), rows out of the padded region; the exchange
            // of the inverse then reuses the region after a barrier (stride 0)
#pragma unroll
            for (int m = 0; m < E; m++) smem[tau + 65 * m] = __ldcs(v + tau + 64 * m);
            __syncthreads();
#pragma unroll
            for (int u = 0; u < E; u++) x[0][u] = smem[65 * tau + u];
            stride = 0;
        } else if constexpr (VEC) {
            const uint4* s4 = reinterpret_cast<const uint4*>(v + group_base<PL, LAST>(tau, 0));
#pragma unroll
            for (int h = 0; h < E / 4; h++) {
                const uint4 q4 = s4[h];
                x[0][4 * h] = q4.x;
                x[0][4 * h + 1] = q4.y;
                x[0][4 * h + 2] = q4.z;
                x[0][4 * h + 3] = q4.w;
            }
        } else {
#pragma unroll
            for (int e = 0; e < E; e++) x[0][e] = v[slot_pos<PL, LAST>(tau, e)];
        }
        // N^-1 is applied inside the last stage (outputs in [0, p))
        if constexpr (LOOP)
            ntt64_inverse<PL, 1>(x, B->ipsi[prime], B->ipsi_r[prime], m, tau, smem, stride == 0, ninv + 4 * prime);
        else
            ntt_inverse<PL, 1>(x, B->ipsi[prime], m, tau, smem, stride, 0, CtaSync(), 1, B->ipsi_r[prime],
                               ninv + 4 * prime);
        if (store) {
#pragma unroll
            for (int e = 0; e < E; e++) {
                if constexpr (COAL) __stcs(v + slot_pos<PL, 0>(tau, e), x[0][e]);
                else v[slot_pos<PL, 0>(tau, e)] = x[0][e];
            }
        }
    }
}

// --------------------------------------------------------------------------
// k_epi: ICRT + mod q / round(t/q) / decrypt. One thread per coefficient.
// L = 32-bit words of q.
// --------------------------------------------------------------------------
template <int L>
struct Cols {
    uint64_t c[L + 2];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int w = 0; w < L + 2; w++) c[w] = 0;
    }
    __device__ __forceinline__ void mac(uint32_t y, const uint32_t* a) {
#pragma unroll
        for (int w = 0; w < L; w++) c[w] += (uint64_t)y * a[w];
    }
    __device__ __forceinline__ void add(const uint32_t* a) {
#pragma unroll
        for (int w = 0; w < L; w++) c[w] += a[w];
    }
    // carry-propagate so that c[w] < 2^32 for w <= L
    __device__ __forceinline__ void norm() {
#pragma unroll
        for (int w = 0; w < L + 1; w++) {
            c[w + 1] += c[w] >> 32;
            c[w] &= 0xFFFFFFFFULL;
        }
    }
};

// Barrett division of a normalised column value x (< 2^(32L+37)) by q' (top bit
// of word L-1 set): returns the quotient, writes the remainder (< q') to r.
template <int L>
__device__ __forceinline__ uint64_t barrett(const Cols<L>& x, const uint32_t* qn, uint64_t mu, uint32_t (&r)[L]) {
    const uint64_t x1 = (x.c[L + 1] << 33) | (x.c[L] << 1) | (x.c[L - 1] >> 31);  // floor(x / 2^(32L-1)) < 2^38
    const uint64_t hi = __umul64hi(x1, mu), lo = x1 * mu;
    uint64_t Q = (hi << 26) | (lo >> 38);  // Q-2 <= Q <= Q_true
    const uint32_t Ql = (uint32_t)Q, Qh = (uint32_t)(Q >> 32);
    uint32_t P[L + 2];
    uint64_t carry = 0;
#pragma unroll
    for (int w = 0; w < L; w++) {
        const uint64_t t = (uint64_t)Ql * qn[w] + carry;
        P[w] = (uint32_t)t;
        carry = t >> 32;
    }
    P[L] = (uint32_t)carry;
    carry = 0;
#pragma unroll
    for (int w = 0; w < L; w++) {
        const uint64_t t = (uint64_t)Qh * qn[w] + P[w + 1] + carry;
        P[w + 1] = (uint32_t)t;
        carry = t >> 32;
    }
    P[L + 1] = (uint32_t)carry;
    uint32_t rr[L + 1];
    int64_t br = 0;
#pragma unroll
    for (int w = 0; w <= L; w++) {
        const int64_t d = (int64_t)x.c[w] - (int64_t)P[w] - br;
        rr[w] = (uint32_t)d;
        br = d < 0;
    }
#pragma unroll
    for (int it = 0; it < 2; it++) {
        uint32_t t[L + 1];
        int64_t b2 = 0;
#pragma unroll
        for (int w = 0; w < L; w++) {
            const int64_t d = (int64_t)rr[w] - (int64_t)qn[w] - b2;
            t[w] = (uint32_t)d;
            b2 = d < 0;
        }
        const int64_t d = (int64_t)rr[L] - b2;
        t[L] = (uint32_t)d;
        b2 = d < 0;
        if (!b2) {
#pragma unroll
            for (int w = 0; w <= L; w++) rr[w] = t[w];
            Q++;
        }
    }
#pragma unroll
    for (int w = 0; w < L; w++) r[w] = rr[w];
    return Q;
}

// Epilogue constants in shared memory. The per-prime rows are padded to a
// multiple of three primes with zero factors (ycon = 0, zero rows), so that a
// padded prime contributes exactly nothing and the prime loop runs whole
// groups of three without guards.
constexpr int KPAD = KMAX + 2;

// Scalars of one prime, read with two 16-byte shared loads.
struct __align__(16) EpiPrime {
    uint32_t p, ycon, ycon_sh, fhi, flo;
    uint32_t F0, F1;  // YASHE: R_i / q in units of 2^-64 (lo, hi)
    uint32_t pad;
};
struct EpiShared {
    EpiPrime pr[KPAD];
    __align__(16) uint32_t A0[KPAD * L32MAX];
    __align__(16) uint32_t A1[KPAD * L32MAX];
    uint32_t B0[L32MAX], B1[L32MAX], qn[L32MAX], qhalf_n[L32MAX];
    uint32_t FM[2];  // YASHE: (q - R_M) / q in units of 2^-64
};

// Copy the epilogue constants of basis B into shared memory (threads tid, tid +
// nthreads, ... of the caller's group), with the zero padding up to 3*ceil(k/3).
template <int L, int MODE>
__device__ __forceinline__ void epi_stage(EpiShared& S, const BasisDev* __restrict__ B, int tid, int nthreads) {
    const int k = B->k, kp = 3 * ((k + 2) / 3);
    for (int i = tid; i < kp; i += nthreads) {
        EpiPrime e{1u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
        if (i < k) {
            e.p = B->p[i];
            e.ycon = B->ycon[i];
            e.ycon_sh = B->ycon_sh[i];
            e.fhi = B->fhi[i];
            e.flo = B->flo[i];
            if (MODE == EPI_YASHE) {
                e.F0 = B->frac[i][0];
                e.F1 = B->frac[i][1];
            }
        }
        S.pr[i] = e;
    }
    for (int i = tid; i < kp * L; i += nthreads) {
        const bool in = i < k * L;
        S.A0[i] = in ? B->A0[i / L][i % L] : 0u;
        if (MODE == EPI_YASHE) S.A1[i] = in ? B->A1[i / L][i % L] : 0u;
    }
    if (MODE == EPI_YASHE && tid < 2) S.FM[tid] = B->frac_m[tid];
    for (int i = tid; i < L; i += nthreads) {
        S.B0[i] = B->B0[i];
        S.B1[i] = B->B1[i];
        S.qn[i] = B->qn[i];
        S.qhalf_n[i] = B->qhalf_n[i];
    }
}

// Row of L words of shared memory (16- or 8-byte loads when L allows).
template <int L>
__device__ __forceinline__ void load_row(const uint32_t* src, uint32_t (&a)[L]) {
    if constexpr (L % 4 == 0) {
#pragma unroll
        for (int w = 0; w < L; w += 4) {
            const uint4 v = *reinterpret_cast<const uint4*>(src + w);
            a[w] = v.x;
            a[w + 1] = v.y;
            a[w + 2] = v.z;
            a[w + 3] = v.w;
        }
    } else if constexpr (L % 2 == 0) {
#pragma unroll
        for (int w = 0; w < L; w += 2) {
            const uint2 v = *reinterpret_cast<const uint2*>(src + w);
            a[w] = v.x;
            a[w + 1] = v.y;
        }
    } else {
#pragma unroll
        for (int w = 0; w < L; w++) a[w] = src[w];
    }
}

// YASHE rounding, exact: Q = floor((S' + (q-1)/2) / q) with S' = sum y_i R_i +
// v (q - R_M), from the residues again (the rare case that the fixed-point
// estimate cannot decide).
template <int L>
__device__ __noinline__ uint64_t yashe_round_exact(const EpiShared& S, const BasisDev* __restrict__ B,
                                                   const uint32_t* __restrict__ r0, size_t stride, uint32_t v) {
    const int k = B->k;
    Cols<L> c1;
    c1.zero();
    for (int i = 0; i < k; i++) {
        const EpiPrime P = S.pr[i];
        const uint32_t y = red(shoup(__ldcg(r0 + (size_t)i * stride), P.ycon, P.ycon_sh, P.p), P.p);
        c1.mac(y, &S.A1[i * L]);
        if (i % 3 == 2) c1.norm();
    }
    c1.norm();
    c1.mac(v, S.B1);
    c1.add(S.qhalf_n);
    c1.norm();
    uint32_t rdummy[L];
    return barrett<L>(c1, S.qn, B->mu, rdummy);
}

// Epilogue of C coefficients: r0[c] points at the residue of coefficient c for
// prime 0, residues of the next primes follow `stride` words apart. Writes the
// limbs of dst[c] (MODQ, YASHE) or one word (DECRYPT) where store[c] is set.
// The constants of a prime are read once for all C coefficients.
//
// YASHE rounding: Q = round(S'/q) is first estimated in 64-bit fixed point,
// Z = sum y_i F_i + v F_M + 2^63 (F = floor(R 2^64 / q)), which undershoots the
// true value by less than (k+1) 2^30 2^-64 < 2^-28. floor(Z / 2^64) is exact
// unless the fraction of Z is within 2^-28 of the next integer; those
// coefficients (about one in 2^28), and all of them when frac_limit is 0, take
// the exact multiword path.
// lstride: distance in words between the limbs of an output coefficient (1, or
// N for the limb-major layout)
template <int L, int MODE, int C>
__device__ __forceinline__ void epi_coefs(const EpiShared& S, const BasisDev* __restrict__ B,
                                          const uint32_t* const (&r0)[C], size_t stride, uint64_t* const (&dst)[C],
                                          const bool (&store)[C], uint64_t frac_limit, size_t lstride = 1) {
    const int k = B->k, shift = B->shift, l64 = B->l64;
    const int groups = (k + 2) / 3;
    const uint64_t mu = B->mu;
    Cols<L> c0[C];
    Cols<2> fz[C];  // YASHE: Z in 32-bit columns
    uint64_t vacc[C];
#pragma unroll
    for (int c = 0; c < C; c++) {
        c0[c].zero();
        fz[c].zero();
        vacc[c] = 0;
    }
    // One prime's contribution to every coefficient: y = [X Mhat_i^-1]_{p_i}, the
    // fixed-point estimate of y/p_i for v, y times the row of constants into the
    // columns and (YASHE) y F_i into Z.
    auto absorb = [&](int i, const uint32_t (&r)[C]) {
        const EpiPrime P = S.pr[i];
        uint32_t a[L];
        load_row<L>(&S.A0[i * L], a);
        const uint32_t F[2] = {P.F0, P.F1};
#pragma unroll
        for (int c = 0; c < C; c++) {
            const uint32_t y = red(shoup(r[c], P.ycon, P.ycon_sh, P.p), P.p);
            vacc[c] += (uint64_t)y * P.fhi + __umulhi(y, P.flo);  // sum y_i/p_i in 2^-32 units
            c0[c].mac(y, a);
            if (MODE == EPI_YASHE) fz[c].mac(y, F);
        }
    };
    // Residues come from L2: the loads of the next two groups of three primes are
    // in flight while a group is absorbed. Loads past the last prime re-read its
    // residue (a valid address); its padded factors make the contribution zero.
    auto load3 = [&](int g, uint32_t (&d)[3][C]) {
#pragma unroll
        for (int j = 0; j < 3; j++) {
            const size_t off = (size_t)min(3 * g + j, k - 1) * stride;
#pragma unroll
            for (int c = 0; c < C; c++) d[j][c] = __ldcg(r0[c] + off);
        }
    };
    uint32_t g0[3][C], g1[3][C], g2[3][C];
    load3(0, g0);
    load3(min(1, groups - 1), g1);
    for (int g = 0; g < groups; g++) {
        load3(min(g + 2, groups - 1), g2);
#pragma unroll
        for (int j = 0; j < 3; j++) absorb(3 * g + j, g0[j]);
#pragma unroll
        for (int c = 0; c < C; c++) {
            c0[c].norm();  // columns take three products of < 2^62 between carry passes
            if (MODE == EPI_YASHE) fz[c].norm();
        }
#pragma unroll
        for (int j = 0; j < 3; j++)
#pragma unroll
            for (int c = 0; c < C; c++) {
                g0[j][c] = g1[j][c];
                g1[j][c] = g2[j][c];
            }
    }
#pragma unroll
    for (int c = 0; c < C; c++) {
        const uint32_t v = (uint32_t)((vacc[c] + 0x80000000ULL) >> 32);  // X = sum y_i Mhat_i - v M
        Cols<L>& x = c0[c];
        x.norm();
        x.mac(v, S.B0);
        if (MODE == EPI_YASHE) {
            Cols<2>& z = fz[c];
            z.mac(v, S.FM);
            z.c[1] += 0x80000000u;  // + 1/2
            z.norm();
            const uint64_t frac = z.c[0] | (z.c[1] << 32);
            uint64_t Q2 = z.c[2] | (z.c[3] << 32);  // round(S/q) + v, S = sum y_i R_i - v R_M
            if (frac >= frac_limit) Q2 = yashe_round_exact<L>(S, B, r0[c], stride, v);
            // x += Q2 << shift
            const uint64_t lo = Q2 << shift;
            const uint64_t hi = shift ? (Q2 >> (64 - shift)) : 0;
            x.c[0] += (uint32_t)lo;
            x.c[1] += (uint32_t)(lo >> 32);
            x.c[2] += hi;
        }
        x.norm();
        uint32_t r[L];
        barrett<L>(x, S.qn, mu, r);  // r = (result mod q) << shift
        if (!store[c]) continue;
        if constexpr (MODE == EPI_DECRYPT) {
            Cols<L> c2;
            c2.zero();
            c2.mac(B->t, r);
            c2.add(S.qhalf_n);
            c2.norm();
            uint32_t rd[L];
            uint64_t Q = barrett<L>(c2, S.qn, mu, rd);  // round(t x / q) in [0, t]
            if (Q >= B->t) Q -= B->t;
            dst[c][0] = Q;
        } else {
            uint32_t o[L];
#pragma unroll
            for (int w = 0; w < L; w++) {
                const uint32_t nx = (w + 1 < L) ? r[w + 1] : 0u;
                o[w] = __funnelshift_r(r[w], nx, shift);
            }
#pragma unroll
            for (int j = 0; j < (L + 1) / 2; j++) {
                const uint64_t lo32 = o[2 * j];
                const uint64_t hi32 = (2 * j + 1 < L) ? o[2 * j + 1] : 0u;
                if (j < l64) dst[c][j * lstride] = lo32 | (hi32 << 32);
            }
        }
    }
}

// One coefficient (the mixed-batch kernel's epilogue units).
template <int L, int MODE>
__device__ __forceinline__ void epi_coef(const EpiShared& S, const BasisDev* __restrict__ B,
                                         const uint32_t* __restrict__ r0, size_t stride, uint64_t* __restrict__ dst,
                                         uint64_t frac_limit = 0) {
    const uint32_t* const rr[1] = {r0};
    uint64_t* const dd[1] = {dst};
    const bool st[1] = {true};
    epi_coefs<L, MODE, 1>(S, B, rr, stride, dd, st, frac_limit);
}

// lm: outputs limb-major ([job][limb][N]) instead of [job][N][limb] (modes
// MODQ and YASHE; the HE multiply's intermediate before its keyswitch)
template <int L, int MODE>
__global__ void __launch_bounds__(256) k_epi(const BasisDev* __restrict__ B, const uint32_t* __restrict__ resid,
                                             void* __restrict__ out, int njobs, unsigned long long frac_limit,
                                             int lm) {
    constexpr int C = epi_coefs_per_thread(L);  // coefficients per thread
    __shared__ EpiShared S;
    epi_stage<L, MODE>(S, B, threadIdx.x, blockDim.x);
    __syncthreads();
    const int logn = B->logn, k = B->k, l64 = B->l64;
    const int n = 1 << logn;
    const long long total = (long long)njobs << logn;
    const long long base = (long long)blockIdx.x * blockDim.x * C + threadIdx.x;
    if (base >= total) return;
    const uint32_t* r0[C];
    uint64_t* dst[C];
    bool store[C];
#pragma unroll
    for (int c = 0; c < C; c++) {
        long long idx = base + (long long)c * blockDim.x;  // coalesced across the warp for every c
        store[c] = idx < total;
        if (!store[c]) idx = base;  // computed and not written
        const long long job = idx >> logn;
        const int coef = (int)(idx & (n - 1));
        r0[c] = resid + (size_t)job * k * n + coef;
        dst[c] = reinterpret_cast<uint64_t*>(out) +
                 (MODE == EPI_DECRYPT ? (size_t)job * n + coef
                                      : (size_t)job * n * l64 + (lm ? (size_t)coef : (size_t)coef * l64));
    }
    epi_coefs<L, MODE, C>(S, B, r0, (size_t)n, dst, store, frac_limit, lm ? (size_t)n : 1);
}

// --------------------------------------------------------------------------
// k_epi_k: the MODQ / YASHE epilogue for a compile-time prime count K. The
// basis constants travel by value as a kernel parameter (constant bank), so each
// constant is a uniform operand of the instruction that uses it: no shared-memory
// staging, no address arithmetic, no guards. The prime loop is straight-line
// code with a carry pass every four primes (four products of < 2^62 plus a
// normalised word stay below 2^64).
// --------------------------------------------------------------------------
template <int L, int K>
struct EpiConst {
    uint32_t p[K], np[K], ycon[K], ycon_sh[K], fhi[K], flo[K], F0[K], F1[K];
    uint32_t A0[K][L];
    uint32_t B0[L], qn[L], qhalf_n[L];
    uint32_t FM[2];
    uint64_t mu;
    int shift, l64, logn;
};

// x in [0, 2m) -> [0, m) with nm = -m
__device__ __forceinline__ uint32_t red_neg(uint32_t x, uint32_t nm) { return __viaddmin_u32(x, nm, x); }

// The exact YASHE rounding of yashe_round_exact with the constants read from
// the basis in global memory (the rare path of k_epi_k).
template <int L>
__device__ __noinline__ uint64_t yashe_round_exact_g(const BasisDev* __restrict__ B, const uint32_t* __restrict__ r0,
                                                     size_t stride, uint32_t v) {
    const int k = B->k;
    Cols<L> c1;
    c1.zero();
    for (int i = 0; i < k; i++) {
        const uint32_t p = B->p[i];
        const uint32_t y = red(shoup(__ldcg(r0 + (size_t)i * stride), B->ycon[i], B->ycon_sh[i], p), p);
        c1.mac(y, B->A1[i]);
        if (i % 3 == 2) c1.norm();
    }
    c1.norm();
    c1.mac(v, B->B1);
    c1.add(B->qhalf_n);
    c1.norm();
    uint32_t rdummy[L];
    return barrett<L>(c1, B->qn, B->mu, rdummy);
}

template <int L, int MODE, int K, int C>
__global__ void __launch_bounds__(256) k_epi_k(const __grid_constant__ EpiConst<L, K> P,
                                               const BasisDev* __restrict__ B, const uint32_t* __restrict__ resid,
                                               void* __restrict__ out, int njobs, unsigned long long frac_limit,
                                               int lm) {
    static_assert(MODE == EPI_MODQ || MODE == EPI_YASHE, "mod-q and YASHE epilogues only");
    const int logn = P.logn;
    const int n = 1 << logn;
    const long long total = (long long)njobs << logn;
    const long long base = (long long)blockIdx.x * blockDim.x * C + threadIdx.x;
    if (base >= total) return;
    const uint32_t* r0[C];
    uint64_t* dst[C];
    bool store[C];
#pragma unroll
    for (int c = 0; c < C; c++) {
        long long idx = base + (long long)c * blockDim.x;  // coalesced across the warp for every c
        store[c] = idx < total;
        if (!store[c]) idx = base;  // computed and not written
        const long long job = idx >> logn;
        const int coef = (int)(idx & (n - 1));
        r0[c] = resid + (size_t)job * K * n + coef;
        dst[c] = reinterpret_cast<uint64_t*>(out) + (size_t)job * n * P.l64 +
                 (lm ? (size_t)coef : (size_t)coef * P.l64);
    }
    const size_t lstride = lm ? (size_t)n : 1;
    uint32_t r[K][C];
#pragma unroll
    for (int i = 0; i < K; i++)
#pragma unroll
        for (int c = 0; c < C; c++) r[i][c] = __ldcg(r0[c] + (size_t)i * n);

    Cols<L> c0[C];
    Cols<2> fz[C];
    uint64_t vacc[C];
#pragma unroll
    for (int c = 0; c < C; c++) {
        c0[c].zero();
        fz[c].zero();
        vacc[c] = 0;
    }
#pragma unroll
    for (int i = 0; i < K; i++) {
#pragma unroll
        for (int c = 0; c < C; c++) {
            const uint32_t y = red_neg(shoup(r[i][c], P.ycon[i], P.ycon_sh[i], P.p[i]), P.np[i]);
            vacc[c] += (uint64_t)y * P.fhi[i] + __umulhi(y, P.flo[i]);  // sum y_i/p_i in 2^-32 units
#pragma unroll
            for (int w = 0; w < L; w++) c0[c].c[w] += (uint64_t)y * P.A0[i][w];
            if (MODE == EPI_YASHE) {
                fz[c].c[0] += (uint64_t)y * P.F0[i];
                fz[c].c[1] += (uint64_t)y * P.F1[i];
            }
        }
        if (i % 4 == 3 && i + 1 < K) {
#pragma unroll
            for (int c = 0; c < C; c++) {
                c0[c].norm();
                if (MODE == EPI_YASHE) fz[c].norm();
            }
        }
    }
    // products since the last carry pass; v adds one more
    constexpr bool NORM_BEFORE_V = (K % 4 == 0);
#pragma unroll
    for (int c = 0; c < C; c++) {
        const uint32_t v = (uint32_t)((vacc[c] + 0x80000000ULL) >> 32);  // X = sum y_i Mhat_i - v M
        Cols<L>& x = c0[c];
        if (NORM_BEFORE_V) x.norm();
#pragma unroll
        for (int w = 0; w < L; w++) x.c[w] += (uint64_t)v * P.B0[w];
        if (MODE == EPI_YASHE) {
            Cols<2>& z = fz[c];
            if (NORM_BEFORE_V) z.norm();
            z.c[0] += (uint64_t)v * P.FM[0];
            z.c[1] += (uint64_t)v * P.FM[1];
            z.c[1] += 0x80000000u;  // + 1/2
            z.norm();
            const uint64_t frac = z.c[0] | (z.c[1] << 32);
            uint64_t Q2 = z.c[2] | (z.c[3] << 32);  // round(S/q) + v, S = sum y_i R_i - v R_M
            if (frac >= frac_limit) Q2 = yashe_round_exact_g<L>(B, r0[c], (size_t)n, v);
            // x += Q2 << shift (each added word < 2^32: the columns stay below 2^64)
            const uint64_t lo = Q2 << P.shift;
            const uint64_t hi = P.shift ? (Q2 >> (64 - P.shift)) : 0;
            x.c[0] += (uint32_t)lo;
            x.c[1] += (uint32_t)(lo >> 32);
            x.c[2] += hi;
        }
        x.norm();
        uint32_t rm[L];
        barrett<L>(x, P.qn, P.mu, rm);  // rm = (result mod q) << shift
        if (!store[c]) continue;
        uint32_t o[L];
#pragma unroll
        for (int w = 0; w < L; w++) {
            const uint32_t nx = (w + 1 < L) ? rm[w + 1] : 0u;
            o[w] = __funnelshift_r(rm[w], nx, P.shift);
        }
#pragma unroll
        for (int j = 0; j < (L + 1) / 2; j++) {
            const uint64_t lo32 = o[2 * j];
            const uint64_t hi32 = (2 * j + 1 < L) ? o[2 * j + 1] : 0u;
            if (j < P.l64) dst[c][j * lstride] = lo32 | (hi32 << 32);
        }
    }
}

}  // namespace cy

namespace cy {

template <int LOGN, int LOGE, int L64, int MB_MUL, int MB_KS, bool SINGLE_KS, bool SINGLE_MUL, int ND_LO, int ND_HI>
void fill_l64(KernelSet& ks) {
    ks.mul[L64][0] = (void*)k_mul<LOGN, LOGE, L64, false, MB_MUL, SINGLE_MUL>;
    ks.mul[L64][1] = (void*)k_mul<LOGN, LOGE, L64, true, MB_MUL, SINGLE_MUL>;
    ks.ks[L64][0] = (void*)k_keyswitch<LOGN, LOGE, L64, ND_LO, MB_KS, SINGLE_KS>;
    ks.ks[L64][1] = (void*)k_keyswitch<LOGN, LOGE, L64, ND_HI, MB_KS, SINGLE_KS>;
}

// SPECIALISE: also instantiate the kernels for 1, 2, 3 and 6 limbs (q of up to
// 64, 128, 192 and 384 bits); other limb counts use the generic kernels.
// MB_MUL / MB_KS > 0: blocks per SM the product / keyswitch kernels are
// compiled for (0: the defaults above).
// SINGLE_KS / SINGLE_MUL: the keyswitch / product kernels use one exchange region.
// ND_LO: digits per pass of the keyswitch kernel used when four do not fit (2, or 1
// for fewer registers); ND_HI: digits per pass of the one used when the digit
// count is a multiple of four and it fits (4, or 2 for fewer registers).
// SPEC_MASK: the limb counts (bit L64) that get specialised kernels when
// SPECIALISE is set.
template <int LOGN, int LOGE, bool SPECIALISE, int MB_MUL = 0, int MB_KS = 0, bool SINGLE_KS = false,
          bool SINGLE_MUL = false, int ND_LO = 2, int ND_HI = 4, unsigned SPEC_MASK = 0x4Eu>
void fill_kernel_set(KernelSet& ks) {
    using PL = NttPlan<LOGN, LOGE>;
    ks.logn = LOGN;
    ks.loge = LOGE;
    ks.threads = PL::G;
    fill_l64<LOGN, LOGE, 0, MB_MUL, MB_KS, SINGLE_KS, SINGLE_MUL, ND_LO, ND_HI>(ks);
    if constexpr (SPECIALISE && (SPEC_MASK & 2u))
        fill_l64<LOGN, LOGE, 1, MB_MUL, MB_KS, SINGLE_KS, SINGLE_MUL, ND_LO, ND_HI>(ks);
    if constexpr (SPECIALISE && (SPEC_MASK & 4u))
        fill_l64<LOGN, LOGE, 2, MB_MUL, MB_KS, SINGLE_KS, SINGLE_MUL, ND_LO, ND_HI>(ks);
    if constexpr (SPECIALISE && (SPEC_MASK & 8u))
        fill_l64<LOGN, LOGE, 3, MB_MUL, MB_KS, SINGLE_KS, SINGLE_MUL, ND_LO, ND_HI>(ks);
    if constexpr (SPECIALISE && (SPEC_MASK & 64u))
        fill_l64<LOGN, LOGE, 6, MB_MUL, MB_KS, SINGLE_KS, SINGLE_MUL, ND_LO, ND_HI>(ks);
    if constexpr (LOGE >= 6) {  // one transform per block (k_ntt1), coalesced row side at N = 4096
        // N = 4096: coalesced row side, the two passes as a loop over one copy of the
        // pass code, 96 registers (10 blocks per SM), measured best in both directions
        constexpr bool COAL = LOGN == 12 && LOGE == 6;
        ks.ntt[0] = (void*)k_ntt1<LOGN, LOGE, false, 10, COAL, 1, COAL>;
        ks.ntt[1] = (void*)k_ntt1<LOGN, LOGE, true, 10, COAL, 1, COAL>;
        ks.ntt_jobs_per_block = 1;
    } else {
        ks.ntt[0] = (void*)k_ntt<LOGN, LOGE, false>;
        ks.ntt[1] = (void*)k_ntt<LOGN, LOGE, true>;
    }
    ks.smem_mul = SINGLE_MUL ? (size_t)2 * PL::SMW * 4 : region_bytes<PL, 2>();
    ks.smem_ks[0] = SINGLE_KS ? (size_t)ND_LO * PL::SMW * 4 : region_bytes<PL, ND_LO>();
    ks.smem_ks[1] = SINGLE_KS ? (size_t)ND_HI * PL::SMW * 4 : region_bytes<PL, ND_HI>();
    ks.smem_ntt = LOGE >= 6 ? (size_t)PL::SMW * 4 : region_bytes<PL, 2>();
}

}  // namespace cy
