// Kernel instantiations for N = 16384 with 2^5 coefficients per thread (512 threads, up to 128 registers each).
#include "kernels.cuh"

namespace cy {
void fill_n14_e5(KernelSet& ks) { fill_kernel_set<14, 5, true, 1, 1>(ks); }
}  // namespace cy
