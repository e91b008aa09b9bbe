// ntt_core.cuh -- negacyclic NTT of length N = 2^LOGN held in registers.
//
// The reference runs one radix-2 Stockham stage per kernel launch, through
// global memory, with one block per residue (NTT / NTTIteration,
// src/cuda_functions.cu:404-458; 3*log2(n) launches per product). Here a thread
// block of G = N/E threads owns one length-N transform: every thread keeps E
// coefficients in registers, the log2(N) stages are grouped into passes of at
// most LOGE stages that run entirely in registers, and consecutive passes swap
// data through a padded shared-memory buffer (one barrier per swap, two
// alternating buffers). Several operands (NOPS) of the same prime share the
// twiddle loads and interleave for instruction-level parallelism.
//
// Transform (merged negacyclic twist): forward Cooley-Tukey on natural-order
// input with twiddles psi^bitrev(m+i), output in bit-reversed order; inverse
// Gentleman-Sande on bit-reversed input with psi^-bitrev(m+i), natural-order
// output, without the N^-1 factor (folded into the ICRT constants). So
// INTT(NTT(a) . NTT(b)) = N * a*b mod (x^N + 1, p): the fold by x^N + 1 that the
// reference does on the host (src/cuda_functions.cu:1061-1072) is implicit.
//
// Index map of a pass that covers stages s0 .. s0+R-1 (stage s pairs j and
// j + N/2^(s+1)): with d = N >> (s0 + R), a butterfly group is the 2^R
// positions g*2^R*d + r + u*d (u < 2^R); thread tau owns groups
// gamma = tau + v*G (v < E/2^R) with g = gamma / d, r = gamma % d. The
// twiddle of stage s0+l for element u is tw[2^(s0+l) + g*2^l + (u >> (R-l))].
#pragma once

#include <stdint.h>

#include "arith.cuh"

namespace cy {

template <int LOGN_, int LOGE_>
struct NttPlan {
    static constexpr int LOGN = LOGN_;
    static constexpr int LOGE = LOGE_;
    static constexpr int N = 1 << LOGN;
    static constexpr int E = 1 << LOGE;
    static constexpr int G = N >> LOGE;  // threads per transform
    static constexpr int NPASS = (LOGN + LOGE - 1) / LOGE;
    static constexpr int R0 = LOGN - (NPASS - 1) * LOGE;  // the first pass takes the remainder
    static constexpr int SMW = N + (N >> LOGE);            // words per operand buffer (with padding)
    __host__ __device__ static constexpr int R(int pass) { return pass == 0 ? R0 : LOGE; }
    __host__ __device__ static constexpr int S0(int pass) { return pass == 0 ? 0 : R0 + (pass - 1) * LOGE; }
    __host__ __device__ static constexpr int LOGD(int pass) { return LOGN - S0(pass) - R(pass); }
};

// Barrier of the threads that own one transform: the whole block, or a named
// barrier (ids 1..15) shared by `count` threads when a block runs several
// independent transforms side by side.
struct CtaSync {
    __device__ __forceinline__ void sync() const { __syncthreads(); }
};
struct GroupSync {
    int id, count;
    __device__ __forceinline__ void sync() const {
        asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
    }
};

// Shared-memory layout of the exchange between two passes whose butterflies
// span 2^DA and 2^DB positions (LOGD of the writing and the reading pass), for
// E = 2^R coefficients per thread. For one register slot a warp touches 32
// consecutive positions when LOGD >= 5, else 32/2^D runs of 2^D positions that
// are 2^(D+R) apart. Banks are kept distinct on both sides by
//   * P padding words after every 32 (an address stays base + constant): P = 1
//     when the strided side has LOGD = 0, P = 2^(5-R) when it has LOGD = R;
//   * an XOR of the low 5 bits with bits of the row (pos >> 5) when both sides
//     are strided (LOGD = R and 0), which permutes words inside each 32-word row.
// Every layout is a bijection into SMW = N + N/2^R words.
// With R = 6 (64 coefficients per thread) one word is added after every 64:
// the side with LOGD = 0 then reads 64 consecutive positions per thread at a
// stride of 65 words between lanes (all banks distinct), and the side whose
// lanes hold consecutive positions stays conflict free.
template <int R, int DA, int DB>
struct XLayout {
    static constexpr int DMIN = DA < DB ? DA : DB;
    static constexpr int DMAX = DA < DB ? DB : DA;
    static constexpr bool SWZ = DMAX < 5 && (R == 3 || R == 4);
    static constexpr int PAD = (DMIN >= 5 || DMIN == 0 || DMIN != R || R >= 5) ? 1 : (1 << (5 - R));
    static constexpr int PSH = R >= 6 ? 6 : 5;  // padding period 2^PSH words
    // the padded word of a position whose bits below PSH and above are independent
    __host__ __device__ static constexpr int pad(int pos) { return pos + PAD * (pos >> PSH); }
    __device__ __forceinline__ static int swz(int pos) {
        const int x = pos >> 5;
        if constexpr (R == 3) return pos ^ (x & 7) ^ (((x >> 1) & 3) << 3);
        else return pos ^ (x & 15) ^ (((x >> 3) & 1) << 4);
    }
};

// position of the first element of group v of thread tau in pass PASS
template <class PL, int PASS>
__device__ __forceinline__ int group_base(int tau, int v) {
    constexpr int R = PL::R(PASS), LOGD = PL::LOGD(PASS);
    const int gam = tau + (v << (PL::LOGN - PL::LOGE));
    const int g = gam >> LOGD;
    const int r = gam & ((1 << LOGD) - 1);
    return (g << (LOGD + R)) | r;
}

// position of slot e (= v*2^R + u) of thread tau in pass PASS
template <class PL, int PASS>
__device__ __forceinline__ int slot_pos(int tau, int e) {
    constexpr int R = PL::R(PASS), LOGD = PL::LOGD(PASS);
    return group_base<PL, PASS>(tau, e >> R) + ((e & ((1 << R) - 1)) << LOGD);
}

// Twiddle h of a stage with 2^l twiddles per group. For l >= 1 the group
// starts at an even index of a 16-byte aligned table, so twiddles h and h+1 come
// from one 16-byte load (issued at even h; the compiler keeps the odd half).
__device__ __forceinline__ uint2 load_twiddle(const uint2* __restrict__ twl, int h, int l) {
    if (l == 0) return __ldg(twl);
    const uint4 W2 = __ldg(reinterpret_cast<const uint4*>(twl + (h & ~1)));
    return (h & 1) ? make_uint2(W2.z, W2.w) : make_uint2(W2.x, W2.y);
}

// Plans with 64 coefficients per thread end (forward) or start (inverse) with a
// pass in which thread tau owns the 64 consecutive positions of row tau, and
// needs twiddles tw[2^(S0+l) + tau 2^l + h] (h < 2^l): 2^l consecutive entries
// per thread, 512 bytes apart between lanes at l = 6. Those passes read a copy
// of the table laid out by lane ("rows" table, one per prime and length):
// stage l starts at entry G (2^l - 1); its twiddle pairs (h, h+1) are 16-byte
// records [h/2][tau], so that a warp's load covers 512 consecutive bytes.
template <class PL, int PASS>
__host__ __device__ constexpr bool rows_pass() {
    return PL::LOGE == 6 && PASS == PL::NPASS - 1 && PL::LOGD(PASS) == 0;
}
__device__ __forceinline__ uint2 load_twiddle_rows(const uint2* __restrict__ twl, int h, int l, int G) {
    if (l == 0) return __ldg(twl);
    const uint4 W2 = __ldg(reinterpret_cast<const uint4*>(twl + (h >> 1) * 2 * G));
    return (h & 1) ? make_uint2(W2.z, W2.w) : make_uint2(W2.x, W2.y);
}

// tm: twiddle-offset multiplier. A transform of length N is stages 0.. of one of
// length 2N restricted to half h of it when its stage-s twiddles start at
// (2 + h) * 2^s instead of 2^s (tm = 2 + h); tm = 1 for a whole transform.
// twr: the rows table of this prime and length (plans with 64 coefficients per
// thread; unused otherwise).
template <class PL, int PASS, int NOPS>
__device__ __forceinline__ void fwd_pass(uint32_t (&x)[NOPS][PL::E], const uint2* __restrict__ tw, const Mod& m,
                                         int tau, int tm = 1, const uint2* __restrict__ twr = nullptr) {
    constexpr int R = PL::R(PASS), S0 = PL::S0(PASS), LOGD = PL::LOGD(PASS);
    constexpr int GS = 1 << R;
    constexpr int NV = PL::E >> R;
    constexpr bool ROWS = rows_pass<PL, PASS>();
#pragma unroll
    for (int v = 0; v < NV; v++) {
        const int gam = tau + (v << (PL::LOGN - PL::LOGE));
        const int g = (S0 == 0) ? 0 : (gam >> LOGD);
#pragma unroll
        for (int l = 0; l < R; l++) {
            const int half = 1 << (R - 1 - l);
            const uint2* twl = ROWS ? twr + PL::G * ((1 << l) - 1) + (l == 0 ? tau : 2 * tau)
                                    : tw + (tm << (S0 + l)) + (g << l);  // 16-byte aligned for l >= 1
            // one flat loop of 2^(R-1) butterflies per stage (a trip count that does
            // not depend on l, so that every loop unrolls fully for R = 6 too):
            // butterfly b is j = b mod half of twiddle group h = b / half
            uint2 W = make_uint2(0u, 0u);
#pragma unroll
            for (int b = 0; b < GS / 2; b++) {
                const int h = b >> (R - 1 - l), j = b & (half - 1);
                if (j == 0) W = ROWS ? load_twiddle_rows(twl, h, l, PL::G) : load_twiddle(twl, h, l);
                const int u = (h << (R - l)) + j;
#pragma unroll
                for (int o = 0; o < NOPS; o++) ct_bfly(x[o][v * GS + u], x[o][v * GS + u + half], W.x, W.y, m);
            }
        }
    }
}

// scale (inverse, pass 0, optional): {N^-1, Shoup, N^-1 w1, Shoup} with w1 the
// twiddle of the last stage; that stage then writes (X + Y) N^-1 and
// (X - Y) w1 N^-1 in [0, p), so no separate scaling pass is needed.
template <class PL, int PASS, int NOPS>
__device__ __forceinline__ void inv_pass(uint32_t (&x)[NOPS][PL::E], const uint2* __restrict__ tw, const Mod& m,
                                         int tau, int tm = 1, const uint2* __restrict__ twr = nullptr,
                                         const uint32_t* __restrict__ scale = nullptr) {
    constexpr int R = PL::R(PASS), S0 = PL::S0(PASS), LOGD = PL::LOGD(PASS);
    constexpr int GS = 1 << R;
    constexpr int NV = PL::E >> R;
    constexpr bool ROWS = rows_pass<PL, PASS>();
#pragma unroll
    for (int v = 0; v < NV; v++) {
        const int gam = tau + (v << (PL::LOGN - PL::LOGE));
        const int g = (S0 == 0) ? 0 : (gam >> LOGD);
#pragma unroll
        for (int l = R - 1; l >= 0; l--) {
            const int half = 1 << (R - 1 - l);
            const uint2* twl = ROWS ? twr + PL::G * ((1 << l) - 1) + (l == 0 ? tau : 2 * tau)
                                    : tw + (tm << (S0 + l)) + (g << l);  // 16-byte aligned for l >= 1
            uint2 W = make_uint2(0u, 0u);
            if (PASS == 0 && l == 0 && scale != nullptr) {  // last stage, N^-1 folded in (S0 = 0, g = 0)
                const uint32_t n0 = __ldg(scale), n0s = __ldg(scale + 1), n1 = __ldg(scale + 2),
                               n1s = __ldg(scale + 3);
#pragma unroll
                for (int b = 0; b < GS / 2; b++) {
                    const int u = b;  // l = 0: half = 2^(R-1), one twiddle group
#pragma unroll
                    for (int o = 0; o < NOPS; o++) {
                        uint32_t& X = x[o][v * GS + u];
                        uint32_t& Y = x[o][v * GS + u + half];
                        const uint32_t s = shoup_m(X + Y, n0, n0s, m);         // [0, 2p)
                        const uint32_t d = shoup_m(X - Y + m.p2, n1, n1s, m);  // [0, 2p)
                        X = __viaddmin_u32(s, m.np, s);
                        Y = __viaddmin_u32(d, m.np, d);
                    }
                }
                continue;
            }
#pragma unroll
            for (int b = 0; b < GS / 2; b++) {  // as in fwd_pass
                const int h = b >> (R - 1 - l), j = b & (half - 1);
                if (j == 0) W = ROWS ? load_twiddle_rows(twl, h, l, PL::G) : load_twiddle(twl, h, l);
                const int u = (h << (R - l)) + j;
#pragma unroll
                for (int o = 0; o < NOPS; o++) gs_bfly(x[o][v * GS + u], x[o][v * GS + u + half], W.x, W.y, m);
            }
        }
    }
}

// Registers laid out for pass PA -> registers laid out for pass PB, through
// shared memory `sm` (NOPS buffers of SMW words). Callers that alternate
// between two such regions need one barrier (the next write cannot race with a
// slow reader of this region); a caller with a single region passes
// `sync_before` to add a barrier ahead of the writes.
template <class PL, int PA, int PB, int NOPS, class Sync = CtaSync>
__device__ __forceinline__ void exchange(uint32_t (&x)[NOPS][PL::E], uint32_t* sm, int tau, bool sync_before,
                                         Sync bar = Sync()) {
    constexpr int RA = PL::R(PA), LA = PL::LOGD(PA), NVA = PL::E >> RA;
    constexpr int RB = PL::R(PB), LB = PL::LOGD(PB), NVB = PL::E >> RB;
    using X = XLayout<PL::LOGE, LA, LB>;
    if (sync_before) bar.sync();
#pragma unroll
    for (int v = 0; v < NVA; v++) {
        const int g = group_base<PL, PA>(tau, v);  // bits of u << LA are zero in g
        const int base = X::pad(g);
#pragma unroll
        for (int u = 0; u < (1 << RA); u++) {
            const int a = X::SWZ ? X::swz(g | (u << LA)) : base + X::pad(u << LA);
#pragma unroll
            for (int o = 0; o < NOPS; o++) sm[o * PL::SMW + a] = x[o][(v << RA) + u];
        }
    }
    bar.sync();
#pragma unroll
    for (int v = 0; v < NVB; v++) {
        const int g = group_base<PL, PB>(tau, v);
        const int base = X::pad(g);
#pragma unroll
        for (int u = 0; u < (1 << RB); u++) {
            const int a = X::SWZ ? X::swz(g | (u << LB)) : base + X::pad(u << LB);
#pragma unroll
            for (int o = 0; o < NOPS; o++) x[o][(v << RB) + u] = sm[o * PL::SMW + a];
        }
    }
}

// Forward passes PASS .. NPASS-1. `buf` counts the exchanges made so far by the
// block; exchange number b uses region (b & 1) of `sm`, regions `stride` words
// apart (stride >= NOPS * SMW for every NOPS the kernel uses), or the single
// region `sm` when stride == 0. Returns the updated count.
template <class PL, int PASS, int NOPS, class Sync = CtaSync>
struct FwdFrom {
    __device__ __forceinline__ static int run(uint32_t (&x)[NOPS][PL::E], const uint2* __restrict__ tw,
                                              const Mod& m, int tau, uint32_t* sm, int stride, int buf,
                                              Sync bar = Sync(), int tm = 1, const uint2* __restrict__ twr = nullptr) {
        if constexpr (PASS >= PL::NPASS) {
            return buf;
        } else {
            exchange<PL, PASS - 1, PASS, NOPS, Sync>(x, sm + (buf & 1) * stride, tau, stride == 0, bar);
            fwd_pass<PL, PASS, NOPS>(x, tw, m, tau, tm, twr);
            return FwdFrom<PL, PASS + 1, NOPS, Sync>::run(x, tw, m, tau, sm, stride, buf + 1, bar, tm, twr);
        }
    }
};

// Inverse passes PASS .. 0 where pass PASS+1 was the previous one.
template <class PL, int PASS, int NOPS, class Sync = CtaSync>
struct InvFrom {
    __device__ __forceinline__ static int run(uint32_t (&x)[NOPS][PL::E], const uint2* __restrict__ tw,
                                              const Mod& m, int tau, uint32_t* sm, int stride, int buf,
                                              Sync bar = Sync(), int tm = 1, const uint2* __restrict__ twr = nullptr,
                                              const uint32_t* __restrict__ scale = nullptr) {
        if constexpr (PASS < 0) {
            return buf;
        } else {
            exchange<PL, PASS + 1, PASS, NOPS, Sync>(x, sm + (buf & 1) * stride, tau, stride == 0, bar);
            inv_pass<PL, PASS, NOPS>(x, tw, m, tau, tm, twr, scale);
            return InvFrom<PL, PASS - 1, NOPS, Sync>::run(x, tw, m, tau, sm, stride, buf + 1, bar, tm, twr, scale);
        }
    }
};

// Full forward transform: registers in pass-0 layout (natural order) ->
// registers in last-pass layout (bit-reversed order).
template <class PL, int NOPS, class Sync = CtaSync>
__device__ __forceinline__ int ntt_forward(uint32_t (&x)[NOPS][PL::E], const uint2* __restrict__ tw, const Mod& m,
                                           int tau, uint32_t* sm, int stride, int buf, Sync bar = Sync(),
                                           int tm = 1, const uint2* __restrict__ twr = nullptr) {
    fwd_pass<PL, 0, NOPS>(x, tw, m, tau, tm, twr);
    return FwdFrom<PL, 1, NOPS, Sync>::run(x, tw, m, tau, sm, stride, buf, bar, tm, twr);
}

// Full inverse transform: registers in last-pass layout -> pass-0 layout.
template <class PL, int NOPS, class Sync = CtaSync>
__device__ __forceinline__ int ntt_inverse(uint32_t (&x)[NOPS][PL::E], const uint2* __restrict__ tw, const Mod& m,
                                           int tau, uint32_t* sm, int stride, int buf, Sync bar = Sync(),
                                           int tm = 1, const uint2* __restrict__ twr = nullptr,
                                           const uint32_t* __restrict__ scale = nullptr) {
    inv_pass<PL, PL::NPASS - 1, NOPS>(x, tw, m, tau, tm, twr, scale);
    return InvFrom<PL, PL::NPASS - 2, NOPS, Sync>::run(x, tw, m, tau, sm, stride, buf, bar, tm, twr, scale);
}

// ---------------------------------------------------------------------------
// Two-pass transforms of 64 coefficients per thread (N = 4096) with ONE copy of
// the pass code: both passes pair the same register slots at every stage (slot
// u with u + 2^(5-l)); only their twiddles differ (the first pass's are the same
// for every thread, the row pass's come from the lane-ordered table). The passes
// therefore run as two iterations of a loop that is not unrolled, with the
// twiddle pointers of the iteration in registers: half the instructions of the
// unrolled transform in the instruction cache.
// twp[l]: twiddle 0 of stage l (pairs (h, h+1) start there for l >= 1);
// tws: distance in uint2 between consecutive pairs (2, or 2G in the rows table).
template <int NOPS>
__device__ __forceinline__ uint2 tw_dyn(const uint2* __restrict__ base, int h, int l, int tws) {
    if (l == 0) return __ldg(base);
    const uint4 W2 = __ldg(reinterpret_cast<const uint4*>(base + (h >> 1) * tws));
    return (h & 1) ? make_uint2(W2.z, W2.w) : make_uint2(W2.x, W2.y);
}

template <int NOPS>
__device__ __forceinline__ void fwd_pass64(uint32_t (&x)[NOPS][64], const uint2* const (&twp)[6], int tws,
                                           const Mod& m) {
#pragma unroll
    for (int l = 0; l < 6; l++) {
        const int half = 1 << (5 - l);
        uint2 W = make_uint2(0u, 0u);
#pragma unroll
        for (int b = 0; b < 32; b++) {
            const int h = b >> (5 - l), j = b & (half - 1);
            if (j == 0) W = tw_dyn<NOPS>(twp[l], h, l, tws);
            const int u = (h << (6 - l)) + j;
#pragma unroll
            for (int o = 0; o < NOPS; o++) ct_bfly(x[o][u], x[o][u + half], W.x, W.y, m);
        }
    }
}

template <int NOPS>
__device__ __forceinline__ void inv_pass64(uint32_t (&x)[NOPS][64], const uint2* const (&twp)[6], int tws,
                                           const Mod& m, const uint32_t* __restrict__ scale) {
#pragma unroll
    for (int l = 5; l >= 0; l--) {
        const int half = 1 << (5 - l);
        if (l == 0 && scale != nullptr) {  // the transform's last stage with N^-1 folded in
            const uint32_t n0 = __ldg(scale), n0s = __ldg(scale + 1), n1 = __ldg(scale + 2), n1s = __ldg(scale + 3);
#pragma unroll
            for (int u = 0; u < 32; u++)
#pragma unroll
                for (int o = 0; o < NOPS; o++) {
                    uint32_t& X = x[o][u];
                    uint32_t& Y = x[o][u + 32];
                    const uint32_t sv = shoup_m(X + Y, n0, n0s, m);
                    const uint32_t dv = shoup_m(X - Y + m.p2, n1, n1s, m);
                    X = __viaddmin_u32(sv, m.np, sv);
                    Y = __viaddmin_u32(dv, m.np, dv);
                }
            continue;
        }
        uint2 W = make_uint2(0u, 0u);
#pragma unroll
        for (int b = 0; b < 32; b++) {
            const int h = b >> (5 - l), j = b & (half - 1);
            if (j == 0) W = tw_dyn<NOPS>(twp[l], h, l, tws);
            const int u = (h << (6 - l)) + j;
#pragma unroll
            for (int o = 0; o < NOPS; o++) gs_bfly(x[o][u], x[o][u + half], W.x, W.y, m);
        }
    }
}

// twiddle pointers of pass `pass` (0: column pass, shared by all threads; 1: row
// pass, lane-ordered table) of a transform of 4096 with 64 threads
__device__ __forceinline__ void pass64_twiddles(int pass, const uint2* __restrict__ tw, const uint2* __restrict__ twr,
                                                int tau, const uint2* (&twp)[6], int& tws) {
#pragma unroll
    for (int l = 0; l < 6; l++)
        twp[l] = pass == 0 ? tw + (1 << l) : twr + 64 * ((1 << l) - 1) + (l == 0 ? tau : 2 * tau);
    tws = pass == 0 ? 2 : 128;
}

// Forward transform, registers in column layout (positions tau + 64 u) ->
// row layout (64 tau + u); exchange region `sm` (one, SMW = 4160 words per operand).
template <class PL, int NOPS>
__device__ __forceinline__ void ntt64_forward(uint32_t (&x)[NOPS][64], const uint2* __restrict__ tw,
                                              const uint2* __restrict__ twr, const Mod& m, int tau, uint32_t* sm,
                                              bool sync_before = false) {
    static_assert(PL::LOGN == 12 && PL::LOGE == 6, "two passes of six stages");
#pragma unroll 1
    for (int pass = 0; pass < 2; pass++) {
        const uint2* twp[6];
        int tws;
        pass64_twiddles(pass, tw, twr, tau, twp, tws);
        fwd_pass64<NOPS>(x, twp, tws, m);
        if (pass == 0) exchange<PL, 0, 1, NOPS>(x, sm, tau, sync_before);
    }
}

// Inverse transform, row layout -> column layout; `sync_before`: a barrier
// before the exchange's writes (the region was read just before); scale as in
// inv_pass (or null).
template <class PL, int NOPS>
__device__ __forceinline__ void ntt64_inverse(uint32_t (&x)[NOPS][64], const uint2* __restrict__ tw,
                                              const uint2* __restrict__ twr, const Mod& m, int tau, uint32_t* sm,
                                              bool sync_before, const uint32_t* __restrict__ scale) {
    static_assert(PL::LOGN == 12 && PL::LOGE == 6, "two passes of six stages");
#pragma unroll 1
    for (int it = 0; it < 2; it++) {
        const int pass = 1 - it;
        const uint2* twp[6];
        int tws;
        pass64_twiddles(pass, tw, twr, tau, twp, tws);
        inv_pass64<NOPS>(x, twp, tws, m, pass == 0 ? scale : nullptr);
        if (pass == 1) exchange<PL, 1, 0, NOPS>(x, sm, tau, sync_before);
    }
}

}  // namespace cy
