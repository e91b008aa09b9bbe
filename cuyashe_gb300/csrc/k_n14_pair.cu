// Kernel instantiations for N = 16384 whose product and keyswitch kernels run each
// (prime, job) on a cluster of two 1024-thread blocks, 8 coefficients per thread
// (kernels_pair.cuh); the standalone NTT is that of the default schedule.
#include "kernels_pair.cuh"

namespace cy {

// Two digits per pass in both keyswitch slots: with four the kernel spills at
// the 64 registers of a 1024-thread block.
template <int L64>
static void fill_pair_l64(KernelSet& ks) {
    ks.mul[L64][0] = (void*)k_mul_pair<L64, false>;
    ks.mul[L64][1] = (void*)k_mul_pair<L64, true>;
    ks.ks[L64][0] = (void*)k_keyswitch_pair<L64, 2>;
    ks.ks[L64][1] = (void*)k_keyswitch_pair<L64, 2>;
}

// `ks` arrives as a copy of the default N = 16384 set (its standalone NTT stays);
// every product and keyswitch entry of that set is replaced.
void fill_n14_pair(KernelSet& ks) {
    static_assert(PairPlan::G == NttPlan<14, 4>::G, "one thread count for the whole set");
    for (int l = 0; l < 7; l++)
        for (int j = 0; j < 2; j++) ks.mul[l][j] = ks.ks[l][j] = nullptr;
    fill_pair_l64<0>(ks);
    fill_pair_l64<1>(ks);
    fill_pair_l64<2>(ks);
    fill_pair_l64<3>(ks);
    fill_pair_l64<6>(ks);
    ks.smem_mul = pair_smem_bytes<2>();
    ks.smem_ks[0] = ks.smem_ks[1] = pair_smem_bytes<2>();
    ks.blocks_per_prime = 2;
}

}  // namespace cy
