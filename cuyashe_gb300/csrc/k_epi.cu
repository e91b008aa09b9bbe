// Epilogues specialised for the prime counts of the common parameter sets
// (k_epi_k): 4-word q (N = 4096, 127-bit q: tensor 9, keyswitch 6, product 9
// primes), 2-word q (62-bit, N = 2048: 5 / 4), 6-word q (190-bit, N = 8192:
// 14 / 8) and 12-word q (380-bit, N = 16384: 26 / 15). Other bases use the
// generic k_epi.
#include <string.h>

#include "kernels.cuh"

namespace cy {

template <int L, int K>
static void fill_epi_const(const BasisDev& h, void* param) {
    EpiConst<L, K> c;
    memset(&c, 0, sizeof c);
    for (int i = 0; i < K; i++) {
        c.p[i] = h.p[i];
        c.np[i] = 0u - h.p[i];
        c.ycon[i] = h.ycon[i];
        c.ycon_sh[i] = h.ycon_sh[i];
        c.fhi[i] = h.fhi[i];
        c.flo[i] = h.flo[i];
        c.F0[i] = h.frac[i][0];
        c.F1[i] = h.frac[i][1];
        for (int w = 0; w < L; w++) c.A0[i][w] = h.A0[i][w];
    }
    for (int w = 0; w < L; w++) {
        c.B0[w] = h.B0[w];
        c.qn[w] = h.qn[w];
        c.qhalf_n[w] = h.qhalf_n[w];
    }
    c.FM[0] = h.frac_m[0];
    c.FM[1] = h.frac_m[1];
    c.mu = h.mu;
    c.shift = h.shift;
    c.l64 = h.l64;
    c.logn = h.logn;
    memcpy(param, &c, sizeof c);
}

namespace {
struct EpiEntry {
    int l32, k, mode;
    EpiSpecial s;
};
}  // namespace

// One coefficient per thread: with the constants as instruction operands a
// second coefficient saves no loads, and half the registers admit more warps.
#define CY_EPI_K(L, K, MODE) \
    {L, K, MODE, {(void*)k_epi_k<L, MODE, K, 1>, sizeof(EpiConst<L, K>), fill_epi_const<L, K>, 1}}

static const EpiEntry kEpiSpecial[] = {
    CY_EPI_K(4, 9, EPI_YASHE),   CY_EPI_K(4, 6, EPI_MODQ),  CY_EPI_K(4, 9, EPI_MODQ),
    CY_EPI_K(2, 5, EPI_YASHE),   CY_EPI_K(2, 4, EPI_MODQ),  CY_EPI_K(6, 14, EPI_YASHE),
    CY_EPI_K(6, 8, EPI_MODQ),    CY_EPI_K(12, 26, EPI_YASHE), CY_EPI_K(12, 15, EPI_MODQ),
};

const EpiSpecial* epi_special(int l32, int k, int mode) {
    for (const EpiEntry& e : kEpiSpecial)
        if (e.l32 == l32 && e.k == k && e.mode == mode) return &e.s;
    return nullptr;
}

}  // namespace cy
