// Kernel instantiations for N = 8192 with 2^3 coefficients per thread.
#include "kernels.cuh"

namespace cy {
void fill_n13_e3(KernelSet& ks) { fill_kernel_set<13, 3, true>(ks); }
}  // namespace cy
