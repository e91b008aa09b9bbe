// Kernel instantiations for N = 4096 with 2^6 coefficients per thread: 64
// threads per transform, two register passes of six stages joined by one
// transpose through shared memory (65-word rows). Products and keyswitches use
// one exchange region and take one digit per pass; six blocks per SM. Only
// two-limb coefficients (q of 65..128 bits) get specialised kernels.
#include "kernels.cuh"

namespace cy {
void fill_n12_e6(KernelSet& ks) { fill_kernel_set<12, 6, true, 6, 6, true, true, 1, 1, 0x4u>(ks); }
// the same kernels, with the standalone inverse NTT taking its input tile by
// TMA (k_ntt_tma.cu)
void fill_n12_e6t(KernelSet& ks) {
    fill_n12_e6(ks);
    ks.intt_tma = true;
}
}  // namespace cy
