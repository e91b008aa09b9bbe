// Kernel instantiations for N = 4096 with 2^3 coefficients per thread and one
// keyswitch exchange region, so that two 512-thread keyswitch blocks (64
// registers per thread) fit on an SM.
#include "kernels.cuh"

namespace cy {
void fill_n12_e3s(KernelSet& ks) { fill_kernel_set<12, 3, true, 0, 2, true>(ks); }
}  // namespace cy
