// Kernel instantiations for N = 1024 and 2048.
#include "kernels.cuh"

namespace cy {
void fill_n10_11(KernelSet* t) {
    fill_kernel_set<10, 3>(t[10]);
    fill_kernel_set<11, 3>(t[11]);
}
}  // namespace cy
