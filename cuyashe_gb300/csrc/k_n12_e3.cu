// Kernel instantiations for N = 4096 with 2^3 coefficients per thread.
#include "kernels.cuh"

namespace cy {
void fill_n12_e3(KernelSet& ks) { fill_kernel_set<12, 3, true>(ks); }
}  // namespace cy
