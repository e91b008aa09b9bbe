// Kernel instantiations for N = 16384 with 2^4 coefficients per thread (1024
// threads, 64 registers) and a keyswitch that transforms one digit per pass
// (no register spills at this size).
#include "kernels.cuh"

namespace cy {
void fill_n14_e4d1(KernelSet& ks) { fill_kernel_set<14, 4, true, 0, 0, false, false, 1>(ks); }
}  // namespace cy
