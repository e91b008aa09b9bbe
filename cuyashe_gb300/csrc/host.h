// host.h -- internal host-side objects behind the C ABI.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <memory>
#include <functional>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/cuyashe.h"
#include "../../include/cuyashe_bigint.h"
#include "common.h"
#include "dispatch.h"

namespace cy {

// ---- errors ---------------------------------------------------------------
cy_status set_error(cy_status st, const std::string& msg);
cy_status cuda_error(cudaError_t e, const char* what);
#define CY_CUDA(call)                                          \
    do {                                                       \
        cudaError_t _e = (call);                               \
        if (_e != cudaSuccess) return cy::cuda_error(_e, #call); \
    } while (0)
#define CY_TRY(call)                    \
    do {                                \
        cy_status _s = (call);          \
        if (_s != CY_OK) return _s;     \
    } while (0)

// ---- word-sized NTT primes with device twiddle tables ----------------------
// The TABLE_PRIMES largest primes p < 2^30 with p = 1 (mod 2^16), descending.
// For each, psi is a primitive 2^(LOGN_MAX+1)-th root of unity; the forward
// table holds psi^bitrev(i) and the inverse table psi^-bitrev(i) (bit reversal
// over LOGN_MAX bits) with Shoup companions. A prefix of length N of these
// tables is the table of the length-N transform (psi_N = psi^(NMAX/N)).
struct PrimeTable {
    int device = -1;
    std::vector<uint32_t> primes;
    uint2* d_psi = nullptr;   // [TABLE_PRIMES][NMAX]
    uint2* d_ipsi = nullptr;  // [TABLE_PRIMES][NMAX]
    uint2* d_psi_r = nullptr;   // [TABLE_PRIMES][ROWS_WORDS] row-pass twiddles of N = ROWS_N by lane
    uint2* d_ipsi_r = nullptr;  // [TABLE_PRIMES][ROWS_WORDS]
};
// Entry of the row-pass table of stage l (0..5), twiddle h (< 2^l) and lane tau
// (< ROWS_G): stage l starts at ROWS_G (2^l - 1); for l >= 1 the pairs (h, h+1)
// are 16-byte records [h/2][tau].
inline size_t rows_index(int l, int h, int tau) {
    const size_t base = (size_t)ROWS_G * ((1u << l) - 1);
    return l == 0 ? base + tau : base + (size_t)(h >> 1) * 2 * ROWS_G + 2 * (size_t)tau + (h & 1);
}
cy_status prime_table(int device, const PrimeTable** out);
const std::vector<uint32_t>& table_primes();  // host-only, no CUDA

// ---- a CRT basis for one ring and one epilogue ------------------------------
struct Basis {
    BasisDev h{};
    BasisDev* d = nullptr;
    uint32_t* d_ninv = nullptr;  // [k][4]: N^-1 mod p_i, N^-1 psi_i^-(NMAX/2), each with its Shoup companion
    int crt_bits = 0;
    const EpiSpecial* epi = nullptr;     // specialised epilogue of this basis, if any
    std::vector<unsigned char> epi_param;  // its parameter block (constants by value)
    Basis() = default;
    Basis(const Basis&) = delete;
    Basis& operator=(const Basis&) = delete;
    ~Basis();
};

// Host constants only (no device memory): smallest prefix of the table primes
// whose product exceeds `bound`.
// `scale_n` folds N^-1 (inverse NTT without scaling) and `mont` folds 2^32
// (Montgomery pointwise product) into the residue factors of the epilogue.
cy_status basis_constants(BasisDev& h, int* crt_bits, int n, const BigUInt& q, int mode, const BigUInt& bound,
                          uint32_t t, bool mont, bool scale_n, bool centered);
cy_status build_basis(Basis& b, int device, int n, const BigUInt& q, int mode, const BigUInt& bound, uint32_t t,
                      bool mont, bool scale_n, bool centered);

// ---- scratch ------------------------------------------------------------------
// Residue scratch of the product kernels. Calls of several chunks spread them
// over the caller's stream and up to kMaxSide side streams (created on first
// use), each with its own scratch, so that one chunk's kernels fill the others'
// tails; `fork` / `join` order the side streams after and before the caller's.
constexpr int kMaxSide = 3;
struct Workspace {
    int device = -1;
    uint32_t* d_resid = nullptr;
    size_t resid_words = 0;
    uint32_t* d_side_resid[kMaxSide] = {};
    size_t side_words[kMaxSide] = {};
    cudaStream_t side[kMaxSide] = {};
    cudaEvent_t fork = nullptr, join[kMaxSide] = {};
    cy_status reserve(size_t words);
    cy_status reserve_side(int i, size_t words);  // scratch, stream and events of side lane i
    ~Workspace();
};

// Jobs per launch of the product kernels (residue scratch near CY_CHUNK_BYTES).
int chunk_jobs(int n, int k);

// Host-buffer calls (hostpipe.cpp): `batch` jobs of `words` uint64 words per
// operand, `chunk` jobs at a time through three device slots, copies
// overlapping the kernels. op(ws, d_in0, d_in1, d_out, jobs, stream) runs one
// chunk; h_in1 may be NULL for a one-operand call.
using ChunkOp = std::function<cy_status(cy_workspace*, const uint64_t*, const uint64_t*, uint64_t*, int, cudaStream_t)>;
cy_status run_host_pipeline(size_t words, int batch, int chunk, const uint64_t* h_in0, const uint64_t* h_in1,
                            uint64_t* h_out, const ChunkOp& op);

// *differ: whether the bytes at a and b (multiple of 4) differ; synchronises `st`;
// d_flag: one device int of scratch (k_misc.cu)
cy_status words_differ(const void* a, const void* b, size_t bytes, int* d_flag, cudaStream_t st, bool* differ);

// ---- inverse NTT of length 4096 with its input tile by TMA (k_ntt_tma.cu) ----
void* intt_tma_kernel();
size_t intt_tma_smem();
// whether `res` ([jobs][k][4096] words, rows = jobs * k * 64) can be tiled
bool ntt_tma_usable(const void* res, long long rows);
// the tensor map of `res`, the grid and the error word of the launch
cy_status intt_tma_prepare(uint32_t* res, long long rows, int k, int njobs, CUtensorMap* map, dim3* grid,
                           int** d_err);
// CY_ERR_TIMEOUT if a launch gave up waiting for a tile since the last check
cy_status ntt_tma_check(bool reset);
// polls of the tile wait (default 2^22) and bytes the tile's barrier is told to
// expect beyond the tile (0; > 0 makes the wait run out, for its test)
uint32_t ntt_tma_spin_limit();
uint32_t ntt_tma_extra_tx();
void ntt_tma_set_test(uint32_t spin_limit, uint32_t extra_tx);

}  // namespace cy

struct cy_workspace {
    cy::Workspace ws;
};

struct cy_ring {
    int device = -1;
    int n = 0, logn = 0, l64 = 0, l32 = 0, qbits = 0;
    cy::BigUInt q;
    std::vector<uint64_t> q_limbs;
    uint64_t* d_q = nullptr;   // q as l64 limbs (elementwise kernels)
    cy::Basis mul;             // product basis, mod-q epilogue (N^-1 and 2^32 folded)
    cy::Basis plain;           // same primes, plain residues (ICRT, scalar multiply, NTT)
    cy_workspace own_ws;
    std::mutex mu;
    ~cy_ring();
};

struct cy_yashe {
    cy_ring* ring = nullptr;
    uint64_t t = 0;
    int w_bits = 32, ell = 0;
    double sigma = 8.0;
    cy::Basis tensor;  // centered inputs, round(t/q .) epilogue
    cy::Basis relin;   // keyswitch basis, mod-q epilogue
    cy::Basis dec;     // key * ciphertext, decryption epilogue
    bool has_keys = false;
    std::vector<uint64_t> h_f, h_h, h_evk;
    uint64_t* d_f = nullptr;
    uint64_t* d_f2 = nullptr;
    uint64_t* d_h = nullptr;    // public key (GPU encryption)
    uint2* d_evk = nullptr;     // [ell][k'][N] NTT-domain evaluation key
    uint64_t* d_cdt = nullptr;  // discrete Gaussian thresholds (GPU sampling)
    int n_cdt = 0;
    ~cy_yashe();
};
