// noalloc.cu -- the polynomial product without any device allocation.
//
// Who needs it: callers that are not allowed to call cudaMalloc. A
// latency-critical or serving path cannot afford cudaMalloc's implicit
// device-wide synchronisation, which stalls every other stream; and a host whose device
// memory belongs to another allocator (a framework's caching allocator, or a
// process that admits work against a fixed memory budget) must not have a
// library grab memory behind that allocator's back. cy_polymul grows a
// workspace with cudaMalloc the first time a batch needs it; this entry point
// instead keeps its scratch in a fixed array that is part of the library's
// device image, so the call itself never allocates.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "host.h"

namespace cy {

int trace_begin(const char* name, int logn, cudaStream_t st);
void trace_end(int idx, cudaStream_t st);

// Residue scratch of every cy_polymul_noalloc call on this device. Every GPU
// that loads the library holds these CY_NOALLOC_SCRATCH_BYTES until the
// process exits. All calls share it: calls that may overlap on the GPU (other
// streams, other host threads) race on it and must be serialised by the caller.
static __device__ __align__(256) uint32_t g_noalloc_scratch[CY_NOALLOC_SCRATCH_BYTES / sizeof(uint32_t)];

// In host code g_noalloc_scratch names a host-side stand-in, not device memory:
// the kernels must be given the device address, looked up once per device with
// that device current.
static cy_status scratch_address(uint32_t** out) {
    static std::mutex mu;
    static uint32_t* addr[256] = {};
    int dev = 0;
    CY_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256) return set_error(CY_ERR_UNSUPPORTED, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(noalloc scratch)");
        addr[dev] = static_cast<uint32_t*>(p);
    }
    *out = addr[dev];
    return CY_OK;
}

static cy_status launch_noalloc(void* func, const char* name, int logn, dim3 grid, dim3 block, size_t smem,
                                cudaStream_t st, void** args) {
    if (!func) return set_error(CY_ERR_INTERNAL, "missing kernel instantiation");
    if (smem > 48 * 1024) CY_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int tr = trace_begin(name, logn, st);
    const cudaError_t e = cudaLaunchKernel(func, grid, block, args, smem, st);
    trace_end(tr, st);
    if (e != cudaSuccess) return cuda_error(e, name);
    return CY_OK;
}

}  // namespace cy

using namespace cy;

extern "C" cy_status cy_polymul_noalloc(cy_ring* r, const uint64_t* d_a, const uint64_t* d_b, uint64_t* d_c,
                                        int batch, cy_stream_t stream) {
    if (!r) return set_error(CY_ERR_INVALID_ARGUMENT, "ring is NULL");
    if (batch < 0) return set_error(CY_ERR_INVALID_ARGUMENT, "batch < 0");
    if (batch == 0) return CY_OK;
    if (!d_a || !d_b || !d_c) return set_error(CY_ERR_INVALID_ARGUMENT, "NULL buffer");
    if (((uintptr_t)d_a | (uintptr_t)d_b | (uintptr_t)d_c) & 15)
        return set_error(CY_ERR_INVALID_ARGUMENT, "buffers must be 16-byte aligned");
    int cur = -1;
    CY_CUDA(cudaGetDevice(&cur));
    if (cur != r->device) return set_error(CY_ERR_INVALID_ARGUMENT, "handle belongs to another CUDA device");
    const Basis& B = r->mul;
    const int n = B.h.n, k = B.h.k;
    const size_t per_product = (size_t)k * n * sizeof(uint32_t);
    size_t max_batch = CY_NOALLOC_SCRATCH_BYTES / per_product;
    if (max_batch > 65535) max_batch = 65535;  // one launch: the grid's y dimension holds the products
    if ((size_t)batch > max_batch) {
        char msg[200];
        std::snprintf(msg, sizeof(msg),
                      "cy_polymul_noalloc: batch %d exceeds the limit of one call (static scratch and one launch); "
                      "at most %zu products of this ring (N=%d, %d CRT primes) per call",
                      batch, max_batch, n, k);
        return set_error(CY_ERR_INVALID_ARGUMENT, msg);
    }
    uint32_t* scratch = nullptr;
    CY_TRY(scratch_address(&scratch));
    // Nothing in the scratch has to start at zero: the product kernel writes every
    // residue word that the epilogue of the same call reads.
    cudaStream_t st = (cudaStream_t)stream;
    const KernelSet& ks = kernel_set(B.h.logn);
    const BasisDev* Bd = B.d;
    long long stride = (long long)n * r->l64;
    void* args[] = {(void*)&Bd, (void*)&d_a, (void*)&stride, (void*)&d_b, (void*)&stride, (void*)&scratch};
    // blocks_per_prime > 1 for schedules that run one product on a pair of blocks
    CY_TRY(launch_noalloc(ks.mul_for(B.h.l64, false), "mul_noalloc", B.h.logn, dim3(k * ks.blocks_per_prime, batch),
                          dim3(ks.threads), ks.smem_mul, st, args));
    void* epi = epi_kernel(B.h.l32, EPI_MODQ);
    unsigned long long fl = 0;  // mod-q epilogue: no rounding estimate
    int lm = 0;                 // outputs in the [job][N][limb] layout
    void* eargs[] = {(void*)&Bd, (void*)&scratch, (void*)&d_c, (void*)&batch, (void*)&fl, (void*)&lm};
    const long long threads = (long long)batch * n;
    const long long per = 256ll * epi_coefs_per_thread(B.h.l32);
    return launch_noalloc(epi, "epi_modq_noalloc", B.h.logn, dim3((unsigned)((threads + per - 1) / per)), dim3(256),
                          0, st, eargs);
}
