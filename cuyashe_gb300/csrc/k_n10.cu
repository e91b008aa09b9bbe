// Kernel instantiations for N = 1024 (generic and limb-specialised).
#include "kernels.cuh"

namespace cy {
void fill_n10(KernelSet* t) { fill_kernel_set<10, 3, true>(t[10]); }
}  // namespace cy
