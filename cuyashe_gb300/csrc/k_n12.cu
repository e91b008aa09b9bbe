// Kernel instantiations for N = 4096 (the headline ring size).
#include "kernels.cuh"

namespace cy {
void fill_n12(KernelSet* t) { fill_kernel_set<12, 3>(t[12]); }
}  // namespace cy
