// Kernel instantiations for N = 8192 with 2^4 coefficients per thread, 64 registers and one exchange region in both kernels: two 512-thread blocks per SM.
#include "kernels.cuh"

namespace cy {
void fill_n13_e4s(KernelSet& ks) { fill_kernel_set<13, 4, true, 2, 2, true, true>(ks); }
}  // namespace cy
