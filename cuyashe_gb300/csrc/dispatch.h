// dispatch.h -- table of kernel instantiations per transform length.
#pragma once

#include <stddef.h>

#include "common.h"

namespace cy {

// [l64][...]: index 0 holds the generic kernels (limb count read at run time),
// index L64 the kernels specialised for coefficients of L64 limbs (or null).
struct KernelSet {
    int logn = 0, loge = 0, threads = 0;
    void* mul[7][2] = {};  // [l64][centered]
    void* ks[7][2] = {};   // [l64][keyswitch with ND_LO (2 or 1) / ND_HI (4 or 2) digits per pass]
    void* ntt[2] = {nullptr, nullptr};  // forward / inverse
    size_t smem_mul = 0, smem_ks[2] = {0, 0}, smem_ntt = 0;
    int blocks_per_prime = 1;  // product / keyswitch blocks per (prime, job): 2 for block pairs
    int ntt_jobs_per_block = 2;  // k_ntt: two jobs per block, grid (primes, jobs/2); k_ntt1: one, grid (jobs, primes)
    bool intt_tma = false;  // N = 4096: the standalone inverse NTT takes its input tile by TMA (k_intt_tma)
    void* mul_for(int l64, bool centered) const { return mul[mul[l64][0] ? l64 : 0][centered ? 1 : 0]; }
    void* ks_for(int l64, int nd4) const { return ks[ks[l64][0] ? l64 : 0][nd4]; }
};

// Kernel sets for transforms of length 2^logn (1 <= logn <= LOGN_MAX). Each
// length has one or more schedules ("variants": coefficients per thread, hence
// threads per transform and passes); variant 0 is the default, the autotuner
// may pick another per ring (tuning.cpp).
const KernelSet& kernel_set(int logn);
int variant_count(int logn);
const KernelSet& kernel_variant(int logn, int v);

// Tuned operations (keys of the autotuner's table).
enum TuneOp { TUNE_MUL = 0, TUNE_MULC = 1, TUNE_KS = 2, TUNE_NTT = 3, TUNE_OPS = 4 };

// ICRT epilogue for `l32` words of q and epilogue mode (EpiMode).
void* epi_kernel(int l32, int mode);

// Epilogue specialised for a prime count (k_epi_k): the kernel, the size of its
// first parameter (the basis constants by value) and the function that writes
// that parameter from a basis. Null when (l32, k, mode) has no specialisation.
struct EpiSpecial {
    void* func;
    size_t param_bytes;
    void (*fill)(const BasisDev& h, void* param);
    int coefs_per_thread;
};
const EpiSpecial* epi_special(int l32, int k, int mode);

// Bytes of shared memory an exchange region set needs, and whether the kernel
// alternates two regions (one barrier per exchange) or reuses one (two).
constexpr size_t kSmemDoubleLimit = 200 * 1024;

}  // namespace cy
