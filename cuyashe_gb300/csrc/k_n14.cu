// Kernel instantiations for N = 16384 (generic and limb-specialised).
#include "kernels.cuh"

namespace cy {
void fill_n14(KernelSet* t) { fill_kernel_set<14, 4, true>(t[14]); }
}  // namespace cy
