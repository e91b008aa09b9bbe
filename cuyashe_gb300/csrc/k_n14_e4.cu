// Kernel instantiations for N = 16384 with 2^4 coefficients per thread.
#include "kernels.cuh"

namespace cy {
void fill_n14_e4(KernelSet& ks) { fill_kernel_set<14, 4, true>(ks); }
}  // namespace cy
