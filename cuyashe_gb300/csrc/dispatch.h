// dispatch.h -- table of kernel instantiations per transform length.
#pragma once

#include <stddef.h>

#include "common.h"

namespace cy {

struct KernelSet {
    int logn = 0, loge = 0, threads = 0;
    void* mul[2] = {nullptr, nullptr};  // [centered]
    void* ks[2] = {nullptr, nullptr};   // keyswitch with 2 / 4 digits per pass
    void* ntt[2] = {nullptr, nullptr};  // forward / inverse
    size_t smem_mul = 0, smem_ks[2] = {0, 0}, smem_ntt = 0;
};

// Kernel set for transforms of length 2^logn (1 <= logn <= LOGN_MAX).
const KernelSet& kernel_set(int logn);

// ICRT epilogue for `l32` words of q and epilogue mode (EpiMode).
void* epi_kernel(int l32, int mode);

// Bytes of shared memory an exchange region set needs, and whether the kernel
// alternates two regions (one barrier per exchange) or reuses one (two).
constexpr size_t kSmemDoubleLimit = 200 * 1024;

}  // namespace cy
