// Kernel instantiations for N = 1024 with 2^3 coefficients per thread.
#include "kernels.cuh"

namespace cy {
void fill_n10_e3(KernelSet& ks) { fill_kernel_set<10, 3, true>(ks); }
}  // namespace cy
