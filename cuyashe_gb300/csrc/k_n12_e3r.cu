// Kernel instantiations for N = 4096 with 2^3 coefficients per thread and a larger register budget (two product blocks / one keyswitch block per SM).
#include "kernels.cuh"

namespace cy {
void fill_n12_e3r(KernelSet& ks) { fill_kernel_set<12, 3, true, 2, 1>(ks); }
}  // namespace cy
