// Kernel instantiations for N = 4096 with 2^4 coefficients per thread and two
// exchange regions, compiled for the three product blocks per SM that their 69.6 KB
// of shared memory allows (85 registers per thread instead of 64). The
// keyswitch, whose two four-operand regions admit one block per SM, gets the
// whole register file.
#include "kernels.cuh"

namespace cy {
void fill_n12_e4u(KernelSet& ks) { fill_kernel_set<12, 4, true, 3, 1>(ks); }
}  // namespace cy
