// Kernel instantiations for N = 4096 with 2^4 coefficients per thread.
#include "kernels.cuh"

namespace cy {
void fill_n12_e4(KernelSet& ks) { fill_kernel_set<12, 4, true>(ks); }
}  // namespace cy
