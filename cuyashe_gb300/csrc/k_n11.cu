// Kernel instantiations for N = 2048 (generic and limb-specialised).
#include "kernels.cuh"

namespace cy {
void fill_n11(KernelSet* t) { fill_kernel_set<11, 3, true>(t[11]); }
}  // namespace cy
