// common.h -- definitions shared by the host set-up code and the CUDA kernels.
#pragma once

#include <stdint.h>
#include <vector_types.h>

namespace cy {

constexpr int KMAX = 40;          // primes per CRT basis
constexpr int L32MAX = 12;        // 32-bit words of q (384 bits)
constexpr int LOGN_MAX = 14;      // N <= 16384
constexpr int NMAX = 1 << LOGN_MAX;
constexpr int TABLE_PRIMES = 64;  // word-sized NTT primes with device twiddle tables
constexpr int PRIME_TWO_ADIC = 16;  // every table prime is 1 mod 2^16
// Length with a 64-coefficients-per-thread schedule (two passes of six stages):
// its row-pass twiddles have a per-lane table of ROWS_WORDS entries per prime.
constexpr int ROWS_LOGN = 12;
constexpr int ROWS_N = 1 << ROWS_LOGN;
constexpr int ROWS_G = ROWS_N >> 6;       // threads per transform
constexpr int ROWS_WORDS = 63 * ROWS_G;   // sum over the six stages of 2^l * G

// What the epilogue of a product kernel computes from the recombined integer X
// (|X| < M/4, M the basis product):
//   MODQ     X mod q                                  -> [N][L] limbs
//   YASHE    round(t*X/q) mod q                       -> [N][L] limbs
//   DECRYPT  round(t*(X mod q)/q) mod t               -> [N] uint64
enum EpiMode { EPI_MODQ = 0, EPI_YASHE = 1, EPI_DECRYPT = 2 };

// Coefficients per thread of the ICRT epilogue kernel for q of l32 words (the
// constants of a prime are read once for all of them); the launch grid is
// ceil(coefficients / (threads * this)).
#ifdef __CUDACC__
__host__ __device__
#endif
constexpr int epi_coefs_per_thread(int l32) { return l32 <= 6 ? 2 : 1; }

// Constants of one CRT basis for one ring (N, q). Lives in device memory; the
// kernels read the per-prime fields of their own prime and the epilogue copies
// what it needs into shared memory.
//
// Notation: p_i the basis primes, M = prod p_i, Mhat_i = M/p_i, s = 32*l32 -
// bits(q) the normalising shift so that q' = q << s has its top bit set.
struct BasisDev {
    int n, logn, k, l32, l64, mode, shift, qbits;
    uint32_t t;        // plaintext modulus (YASHE / DECRYPT)
    uint32_t centered; // inputs are taken as symmetric representatives (YASHE)
    uint64_t mu;       // floor(2^(32*l32+37) / q')
    uint32_t qn[L32MAX];       // q'
    uint32_t q[L32MAX];        // q
    uint32_t qhalf[L32MAX];    // (q-1)/2
    uint32_t qhalf_n[L32MAX];  // ((q-1)/2) << s
    uint32_t B0[L32MAX];       // MODQ: ((-M) mod q) << s        YASHE: ((-I_M) mod q) << s
    uint32_t B1[L32MAX];       //                                YASHE: (q - R_M) << s
    uint32_t p[KMAX];
    uint32_t p2[KMAX], np[KMAX], np2[KMAX];  // 2p, -p, -2p (mod 2^32), read apart from p (arith.cuh, Mod)
    uint32_t pinv[KMAX];       // -p^-1 mod 2^32
    uint32_t ycon[KMAX];       // residue -> [X * Mhat_i^-1]_{p_i} factor (N^-1, Montgomery folded)
    uint32_t ycon_sh[KMAX];    // Shoup companion of ycon
    uint32_t flo[KMAX], fhi[KMAX];  // floor(2^64/p_i) split in words (estimate of X'/M)
    uint32_t qmodp[KMAX];      // q mod p_i (centering)
    uint32_t r32[KMAX], r32_sh[KMAX];  // 2^32 mod p_i with Shoup companion
    uint32_t crt[KMAX][L32MAX];        // 2^(32 j) mod p_i
    uint32_t A0[KMAX][L32MAX];  // MODQ: (Mhat_i mod q) << s     YASHE: (I_i mod q) << s, t*Mhat_i = I_i q + R_i
    uint32_t A1[KMAX][L32MAX];  //                                YASHE: R_i << s
    uint32_t frac[KMAX][2];     // YASHE: floor(R_i 2^64 / q) (lo, hi words)
    uint32_t frac_m[2];         // YASHE: floor((q - R_M) 2^64 / q)
    const uint2* psi[KMAX];     // forward twiddles (w, floor(w 2^32/p)), bit-reversed powers of psi
    const uint2* ipsi[KMAX];    // inverse twiddles
    // N = ROWS_N only: the twiddles of the row pass of the 64-coefficient schedule,
    // laid out by lane (ntt_core.cuh, load_twiddle_rows); null for other N
    const uint2* psi_r[KMAX];
    const uint2* ipsi_r[KMAX];
};

// One job of a mixed batch (different N and q per job) for the persistent
// kernel k_mixed: a polynomial product (mode MODQ, no keyswitch) or a YASHE
// multiply (tensor with the rounding epilogue, then optionally the keyswitch).
struct MixedJob {
    const BasisDev* B;   // product / tensor basis
    const BasisDev* B2;  // keyswitch basis (YASHE with relinearisation), else null
    const uint64_t* a;
    const uint64_t* b;
    uint64_t* c;
    uint32_t* resid;     // [max(k, k2)][N] residues of this job in the batch scratch
    const uint2* evk;    // keyswitch key [ell][k2][N] (NTT domain, Shoup pairs)
    int logn, k, l32, l64;
    int mode;            // EPI_MODQ (product) or EPI_YASHE (tensor rounding)
    int centered;        // inputs taken as symmetric representatives (YASHE)
    int k2, ell;         // keyswitch primes and digits (k2 = 0: none)
    int n_epi;           // epilogue units of the job (each phase)
    int need0;           // NTT units' primes the first epilogue waits for (k unless a test starves it)
};

// A unit of work claimed by one block: kind 0 runs the forward/pointwise/inverse
// transforms of `count` consecutive primes of a job starting at `first`; kind 1
// the job's first epilogue over coefficients [first, first + count) once all
// its kind-0 primes are done; kind 2 the keyswitch transforms of `count` primes
// once every kind-1 unit of the job is done; kind 3 the keyswitch's mod-q
// epilogue once every kind-2 prime is done.
struct MixedUnit {
    int job, kind, first, count;
};

}  // namespace cy
