// Kernel instantiations for N = 4096 with 2^4 coefficients per thread, 64 registers and one exchange region in both kernels: four 256-thread product blocks per SM.
#include "kernels.cuh"

namespace cy {
void fill_n12_e4m(KernelSet& ks) { fill_kernel_set<12, 4, true, 4, 4, true, true>(ks); }
}  // namespace cy
