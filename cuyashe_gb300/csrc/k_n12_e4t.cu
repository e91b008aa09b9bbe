// Kernel instantiations for N = 4096 with 2^4 coefficients per thread, 85
// registers and one exchange region in both kernels: three 256-thread blocks
// per SM.
#include "kernels.cuh"

namespace cy {
void fill_n12_e4t(KernelSet& ks) { fill_kernel_set<12, 4, true, 3, 3, true, true>(ks); }
}  // namespace cy
