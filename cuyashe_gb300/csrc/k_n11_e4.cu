// Kernel instantiations for N = 2048 with 2^4 coefficients per thread.
#include "kernels.cuh"

namespace cy {
void fill_n11_e4(KernelSet& ks) { fill_kernel_set<11, 4, true>(ks); }
}  // namespace cy
