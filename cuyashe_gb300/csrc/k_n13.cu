// Kernel instantiations for N = 8192 (generic and limb-specialised).
#include "kernels.cuh"

namespace cy {
void fill_n13(KernelSet* t) { fill_kernel_set<13, 4, true>(t[13]); }
}  // namespace cy
