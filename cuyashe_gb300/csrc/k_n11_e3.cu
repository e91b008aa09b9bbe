// Kernel instantiations for N = 2048 with 2^3 coefficients per thread.
#include "kernels.cuh"

namespace cy {
void fill_n11_e3(KernelSet& ks) { fill_kernel_set<11, 3, true>(ks); }
}  // namespace cy
