// Kernel instantiations for N = 8192 with 2^4 coefficients per thread and a larger register budget (one block per SM).
#include "kernels.cuh"

namespace cy {
void fill_n13_e4r(KernelSet& ks) { fill_kernel_set<13, 4, true, 1, 1>(ks); }
}  // namespace cy
