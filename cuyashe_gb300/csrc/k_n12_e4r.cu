// Kernel instantiations for N = 4096 with 2^4 coefficients per thread and a larger register budget (two blocks per SM).
#include "kernels.cuh"

namespace cy {
void fill_n12_e4r(KernelSet& ks) { fill_kernel_set<12, 4, true, 2, 2>(ks); }
}  // namespace cy
