// k_ntt_tma.cu -- the inverse NTT of length 4096 with its input tile by TMA.
//
// The 4096 residues of one transform are a [64][64] matrix of words, M[r][c] =
// v[64 r + c]. The two-pass schedule of 64 coefficients per thread (64 threads)
// leaves thread t's row t as the forward output, so the inverse starts from rows
// and ends with thread tau's column (positions tau + 64 e). Here the input rows
// come in as one shared-memory tile written by the TMA (two bulk tensor copies
// of 32 columns x 64 rows, completion on an mbarrier) with the 128-byte
// swizzle: chunk j (16 bytes) of row r of a box sits at chunk j ^ (r & 7), so
//   - 8 threads reading 16-byte chunks of 8 consecutive rows touch 8 distinct
//     16-byte bank groups (a thread's row is 16 conflict-free 16-byte reads), and
//   - a warp reading or writing one element of 32 consecutive columns touches 32
//     distinct banks,
// and the same tile then serves the transpose between the passes (16 row writes
// of 16 bytes, 64 column reads). The output columns leave by coalesced stores.
// One tile per block (10 blocks per SM, 96 registers), one job per block, grid
// (jobs, primes): the blocks an SM holds at a time share a prime and its
// twiddles (L1), and the other blocks of the SM cover a block's wait for its
// tile. Against the register schedule (k_ntt1: coalesced loads, a transpose
// through padded shared memory, then the exchange) this replaces 64 loads, 64
// stores and 64 shared-memory reads per thread by one tile copy and 16 reads.
// Measured alternatives (N = 4096, forward / inverse): the forward by TMA tiles
// (its input columns are coalesced loads already, and a tile only adds a wait)
// and tiles stored by bulk tensor stores were slower; so were blocks holding two
// tiles (the next job's prefetched: 6 blocks per SM) and blocks looping over the
// jobs of a prime (blocks of several primes on an SM thrash the twiddles in L1).
//
// Every wait on the tile's mbarrier is bounded: when it runs out the block
// records CY_ERR_TIMEOUT in the error word, waits (bounded again) for its copy
// and returns.
//
// Replaces the reference's inverse NTT launch (callNTT / NTTIteration with the
// inverse table, src/cuda_functions.cu:385-458) for N = 4096, as the other
// standalone schedules do.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <map>
#include <mutex>
#include <string>

#include "host.h"
#include "kernels.cuh"

namespace cy {

namespace tma {

constexpr int kBoxBytes = 64 * 128;        // 64 rows x 32 words
constexpr int kTileBytes = 2 * kBoxBytes;  // one transform
constexpr size_t kSmemBytes = 1024 + kTileBytes;  // one tile, 1024-byte aligned

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of M[r][c] in a swizzled tile
__device__ __forceinline__ uint32_t swz(int r, int c) {
    return ((uint32_t)(c >> 5) << 13) + ((uint32_t)r << 7) + ((uint32_t)(((c >> 2) & 7) ^ (r & 7)) << 4) +
           ((uint32_t)(c & 3) << 2);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(saddr(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(saddr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// at most `limit` polls; true once the phase of `parity` has completed
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit) {
    for (uint32_t i = 0; i < limit; i++)
        if (mbar_test(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void load_box(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
            "r"(saddr(dst)),
        "l"(map), "r"(x), "r"(y), "r"(saddr(bar))
        : "memory");
}

__device__ __forceinline__ void issue_tile(uint8_t* tile, const CUtensorMap* map, int row, uint64_t* bar,
                                           uint32_t extra_tx) {
    mbar_expect(bar, kTileBytes + extra_tx);
    load_box(tile, map, 0, row, bar);
    load_box(tile + kBoxBytes, map, 32, row, bar);
}

// column tau of the tile -> x (x[e] = M[e][tau])
__device__ __forceinline__ void read_column(const uint8_t* t, int tau, uint32_t (&x)[1][64]) {
#pragma unroll
    for (int e = 0; e < 64; e++) x[0][e] = *reinterpret_cast<const uint32_t*>(t + swz(e, tau));
}
// row r of the tile -> x (x[u] = M[r][u]), 16 bytes at a time
__device__ __forceinline__ void read_row(const uint8_t* t, int r, uint32_t (&x)[1][64]) {
#pragma unroll
    for (int q = 0; q < 16; q++) {
        const uint4 v = *reinterpret_cast<const uint4*>(t + swz(r, 4 * q));
        x[0][4 * q] = v.x;
        x[0][4 * q + 1] = v.y;
        x[0][4 * q + 2] = v.z;
        x[0][4 * q + 3] = v.w;
    }
}
__device__ __forceinline__ void write_row(uint8_t* t, int r, const uint32_t (&x)[1][64]) {
#pragma unroll
    for (int q = 0; q < 16; q++)
        *reinterpret_cast<uint4*>(t + swz(r, 4 * q)) =
            make_uint4(x[0][4 * q], x[0][4 * q + 1], x[0][4 * q + 2], x[0][4 * q + 3]);
}

}  // namespace tma

// Jobs blockIdx.x, +gridDim.x, ... of prime blockIdx.y (the host launches one
// job per block). `map`: the residues (`res`) as a [jobs * k * 64][64] word
// matrix, boxes of 32 x 64. `err`: set to CY_ERR_TIMEOUT by a block that gave
// up waiting for a tile (spin_limit polls). `extra_tx` > 0 only in the test of
// that path (the tile's barrier then waits for bytes that never come).
__global__ void __launch_bounds__(64, 10)
    k_intt_tma(const BasisDev* __restrict__ B, const __grid_constant__ CUtensorMap map, uint32_t* __restrict__ res,
               const uint32_t* __restrict__ ninv, int njobs, int* __restrict__ err, uint32_t spin_limit,
               uint32_t extra_tx) {
    extern __shared__ uint8_t smem_raw[];
    __shared__ uint64_t bar;
    uint8_t* tile = smem_raw + ((1024u - (tma::saddr(smem_raw) & 1023u)) & 1023u);  // the swizzle's 1024-byte period
    const int tau = threadIdx.x;
    const int prime = blockIdx.y;
    const int k = B->k;
    const Mod m = load_mod(B, prime);
    const uint2* __restrict__ tw = B->ipsi[prime];
    const uint2* __restrict__ twr = B->ipsi_r[prime];
    const int step = gridDim.x;
    int job = blockIdx.x;
    if (tau == 0) {
        asm volatile("prefetch.tensormap [%0];" ::"l"(&map) : "memory");
        tma::mbar_init(&bar);
    }
    __syncthreads();
    if (tau == 0 && job < njobs) tma::issue_tile(tile, &map, (job * k + prime) * 64, &bar, extra_tx);
    uint32_t parity = 0;
    for (; job < njobs; job += step) {
        const bool ok = tma::mbar_wait(&bar, parity, spin_limit);
        if (!__syncthreads_and(ok)) {
            if (tau == 0) {
                atomicExch(err, (int)CY_ERR_TIMEOUT);
                tma::mbar_wait(&bar, parity, spin_limit);  // the copy in flight, if it still lands
            }
            return;
        }
        parity ^= 1u;
        uint32_t x[1][64];
        tma::read_row(tile, tau, x);
#pragma unroll 1
        for (int pass = 1; pass >= 0; pass--) {
            const uint2* twp[6];
            int tws;
            pass64_twiddles(pass, tw, twr, tau, twp, tws);
            inv_pass64<1>(x, twp, tws, m, pass == 0 ? ninv + 4 * prime : nullptr);  // last stage: N^-1, [0, p)
            if (pass == 1) {  // rows -> columns through the tile
                __syncthreads();
                tma::write_row(tile, tau, x);
                __syncthreads();
                tma::read_column(tile, tau, x);
            }
        }
        if (job + step < njobs) {
            __syncthreads();  // every thread has read the tile
            if (tau == 0) tma::issue_tile(tile, &map, ((job + step) * k + prime) * 64, &bar, extra_tx);
        }
        uint32_t* v = res + ((size_t)job * k + prime) * 4096;
#pragma unroll
        for (int e = 0; e < 64; e++) __stcs(v + tau + 64 * e, x[0][e]);
    }
}

// ---- host side --------------------------------------------------------------

namespace {

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
    static EncodeTiled fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<EncodeTiled>(p);
    }();
    return fn;
}

struct DevState {
    int* d_err = nullptr;
};

cy_status dev_state(DevState** out) {
    static std::mutex mu;
    static std::map<int, DevState> states;
    int dev = 0;
    CY_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    DevState& s = states[dev];
    if (!s.d_err) {
        CY_CUDA(cudaFuncSetAttribute((const void*)k_intt_tma, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     cudaSharedmemCarveoutMaxShared));
        int* e = nullptr;
        CY_CUDA(cudaMalloc(&e, sizeof(int)));
        CY_CUDA(cudaMemset(e, 0, sizeof(int)));
        s.d_err = e;
    }
    *out = &s;
    return CY_OK;
}

}  // namespace

static std::atomic<uint32_t> g_spin_limit{1u << 22};
static std::atomic<uint32_t> g_extra_tx{0};
uint32_t ntt_tma_spin_limit() { return g_spin_limit.load(); }
uint32_t ntt_tma_extra_tx() { return g_extra_tx.load(); }
void ntt_tma_set_test(uint32_t spin_limit, uint32_t extra_tx) {
    g_spin_limit = spin_limit ? spin_limit : (1u << 22);
    g_extra_tx = extra_tx;
}

void* intt_tma_kernel() { return (void*)k_intt_tma; }
size_t intt_tma_smem() { return tma::kSmemBytes; }

bool ntt_tma_usable(const void* res, long long rows) {
    return encode_fn() != nullptr && ((uintptr_t)res & 15) == 0 && rows > 0 && rows < (1ll << 31);
}

cy_status intt_tma_prepare(uint32_t* res, long long rows, int k, int njobs, CUtensorMap* map, dim3* grid,
                           int** d_err) {
    EncodeTiled enc = encode_fn();
    if (!enc) return set_error(CY_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
    const cuuint64_t dims[2] = {64, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {64 * sizeof(uint32_t)};
    const cuuint32_t box[2] = {32, 64};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, res, dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(CY_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    DevState* s = nullptr;
    CY_TRY(dev_state(&s));
    // one job per block, blocks in job-major order: the blocks an SM holds at a
    // time share a prime (and its twiddles in L1)
    *grid = dim3((unsigned)njobs, (unsigned)k);
    *d_err = s->d_err;
    return CY_OK;
}

cy_status ntt_tma_check(bool reset) {
    DevState* s = nullptr;
    CY_TRY(dev_state(&s));
    int v = 0;
    CY_CUDA(cudaMemcpy(&v, s->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (reset && v != 0) CY_CUDA(cudaMemset(s->d_err, 0, sizeof(int)));
    if (v != 0) return set_error((cy_status)v, "a TMA transform gave up waiting for its input tile");
    return CY_OK;
}

}  // namespace cy
