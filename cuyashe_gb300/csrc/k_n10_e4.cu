// Kernel instantiations for N = 1024 with 2^4 coefficients per thread.
#include "kernels.cuh"

namespace cy {
void fill_n10_e4(KernelSet& ks) { fill_kernel_set<10, 4, true>(ks); }
}  // namespace cy
