// Kernel instantiations for N = 2 .. 512 (parity tests and small rings).
#include "kernels.cuh"

namespace cy {
void fill_small(KernelSet* t) {
    fill_kernel_set<1, 1, false>(t[1]);
    fill_kernel_set<2, 2, false>(t[2]);
    fill_kernel_set<3, 3, false>(t[3]);
    fill_kernel_set<4, 3, false>(t[4]);
    fill_kernel_set<5, 3, false>(t[5]);
    fill_kernel_set<6, 3, false>(t[6]);
    fill_kernel_set<7, 3, false>(t[7]);
    fill_kernel_set<8, 3, false>(t[8]);
    fill_kernel_set<9, 3, false>(t[9]);
}
}  // namespace cy
