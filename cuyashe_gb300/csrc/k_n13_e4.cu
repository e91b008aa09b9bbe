// Kernel instantiations for N = 8192 with 2^4 coefficients per thread.
#include "kernels.cuh"

namespace cy {
void fill_n13_e4(KernelSet& ks) { fill_kernel_set<13, 4, true>(ks); }
}  // namespace cy
