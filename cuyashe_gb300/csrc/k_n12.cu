// Kernel instantiations for N = 4096 (generic and limb-specialised).
#include "kernels.cuh"

namespace cy {
void fill_n12(KernelSet* t) { fill_kernel_set<12, 3, true>(t[12]); }
}  // namespace cy
