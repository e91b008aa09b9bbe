// Kernel instantiations for N = 4096 with 2^4 coefficients per thread, 128
// registers per thread and one keyswitch exchange region, so that two 256-thread
// keyswitch blocks fit on an SM.
#include "kernels.cuh"

namespace cy {
void fill_n12_e4s(KernelSet& ks) { fill_kernel_set<12, 4, true, 2, 2, true>(ks); }
}  // namespace cy
