// api_yashe.cpp -- YASHE entry points of the C ABI (include/cuyashe.h).
//
// The homomorphic multiply is two product batches on the GPU:
//   tensor:    centered c1*c2 over Z[x]/(x^N+1) in a CRT basis with M > N q^2,
//              epilogue round(t/q X) mod q            (k_mul + k_epi<YASHE>)
//   keyswitch: base-2^32 digits of the result times the NTT-domain evaluation
//              key in a basis with M > 4 ell N 2^32 q, epilogue mod q
//                                                     (k_keyswitch + k_epi<MODQ>)
// The reference computes the product on the GPU and everything after it on the
// host with NTL (src/ciphertext.cpp:38-130).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>

#include "host.h"

namespace cy {
cy_status check_aligned_api(const void* a, const void* b, const void* c);
cy_status run_product_api(const Basis& B, bool centered, const uint64_t* a, long long a_stride, const uint64_t* b,
                          long long b_stride, void* out, long long out_stride, int batch, Workspace& ws,
                          cudaStream_t st, int variant = -1);
cy_status run_yashe_mul(const Basis& tensor, const Basis& relin, const uint2* evk, int ell, const uint64_t* c1,
                        const uint64_t* c2, uint64_t* out, int batch, bool do_relin, Workspace& ws, cudaStream_t st,
                        int ks_variant = -1);
cy_status run_keyswitch_api(const Basis& B, const uint64_t* c, const uint2* evk, int ell, uint64_t* out, int batch,
                            Workspace& ws, cudaStream_t st, int variant = -1, int chunk_k = 0, int lm = 0);
int yashe_chunk_jobs(const Basis& tensor, const Basis& relin, int ell, bool do_relin);
cy_status prepare_evk(const Basis& relin, const uint64_t* h_evk, int ell, int n, int l64, uint2** d_evk);
cy_status host_keygen(cy_yashe* y, uint64_t seed, std::vector<uint64_t>& f, std::vector<uint64_t>& h,
                      std::vector<uint64_t>& evk);
cy_status host_encrypt(cy_yashe* y, const uint64_t* m, uint64_t* ct, int batch, uint64_t seed);
}  // namespace cy

using namespace cy;

cy_yashe::~cy_yashe() {
    if (d_f) cudaFree(d_f);
    if (d_f2) cudaFree(d_f2);
    if (d_h) cudaFree(d_h);
    if (d_cdt) cudaFree(d_cdt);
    if (d_evk) cudaFree(d_evk);
    if (ring) cy_ring_destroy(ring);
}

static cy_status yashe_check(const cy_yashe* y, const void* a, const void* b, int batch) {
    if (!y) return set_error(CY_ERR_INVALID_ARGUMENT, "yashe handle is NULL");
    if (batch < 0) return set_error(CY_ERR_INVALID_ARGUMENT, "batch < 0");
    if (batch > 0 && (!a || !b)) return set_error(CY_ERR_INVALID_ARGUMENT, "NULL buffer");
    CY_TRY(check_aligned_api(a, b, nullptr));
    int cur = -1;
    CY_CUDA(cudaGetDevice(&cur));
    if (cur != y->ring->device) return set_error(CY_ERR_INVALID_ARGUMENT, "handle belongs to another CUDA device");
    return CY_OK;
}

extern "C" {

cy_status cy_yashe_create(const cy_yashe_params* prm, cy_yashe** out) {
    if (!prm || !out || !prm->q) return set_error(CY_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = nullptr;
    if (prm->t < 2 || prm->t >= (1ull << 32)) return set_error(CY_ERR_UNSUPPORTED, "t must be in [2, 2^32)");
    if (prm->w_bits != 32) return set_error(CY_ERR_UNSUPPORTED, "w_bits must be 32");
    std::unique_ptr<cy_yashe> y(new cy_yashe());
    CY_TRY(cy_ring_create(prm->n, prm->q, prm->q_limbs, &y->ring));
    const cy_ring* r = y->ring;
    if (!(r->q.w[0] & 1)) return set_error(CY_ERR_UNSUPPORTED, "q must be odd");
    y->t = prm->t;
    y->w_bits = prm->w_bits;
    y->sigma = prm->sigma > 0 ? prm->sigma : 8.0;
    y->ell = (r->qbits + y->w_bits - 1) / y->w_bits;
    const BigUInt& q = r->q;
    const int n = r->n;
    // |centered c1 * centered c2| <= N ((q-1)/2)^2 < N q^2 / 4
    CY_TRY(build_basis(y->tensor, r->device, n, q, EPI_YASHE, BigUInt((uint64_t)n) * q * q, (uint32_t)prm->t, true,
                       true, true));
    // 0 <= sum_d D_d evk_d < ell N 2^w q
    CY_TRY(build_basis(y->relin, r->device, n, q, EPI_MODQ,
                       BigUInt(4ull * (uint64_t)y->ell * (uint64_t)n).shl(y->w_bits) * q, 0, false, true, false));
    CY_TRY(build_basis(y->dec, r->device, n, q, EPI_DECRYPT, BigUInt(4ull * (uint64_t)n) * q * q, (uint32_t)prm->t,
                       true, true, false));
    *out = y.release();
    return CY_OK;
}

cy_status cy_yashe_destroy(cy_yashe* y) {
    delete y;
    return CY_OK;
}

cy_status cy_yashe_get_info(const cy_yashe* y, cy_yashe_info* info) {
    if (!y || !info) return set_error(CY_ERR_INVALID_ARGUMENT, "NULL argument");
    std::memset(info, 0, sizeof(*info));
    info->n = y->ring->n;
    info->q_limbs = y->ring->l64;
    info->q_bits = y->ring->qbits;
    info->ell = y->ell;
    info->w_bits = y->w_bits;
    info->t = y->t;
    info->tensor_primes = y->tensor.h.k;
    info->relin_primes = y->relin.h.k;
    info->has_keys = y->has_keys ? 1 : 0;
    return CY_OK;
}

cy_status cy_yashe_get_ring(cy_yashe* y, cy_ring** ring) {
    if (!y || !ring) return set_error(CY_ERR_INVALID_ARGUMENT, "NULL argument");
    *ring = y->ring;
    return CY_OK;
}

cy_status cy_yashe_set_keys(cy_yashe* y, const uint64_t* h_f, const uint64_t* h_h, const uint64_t* h_evk) {
    if (!y || !h_f || !h_h || !h_evk) return set_error(CY_ERR_INVALID_ARGUMENT, "NULL argument");
    cy_ring* r = y->ring;
    int cur = -1;
    CY_CUDA(cudaGetDevice(&cur));
    if (cur != r->device) return set_error(CY_ERR_INVALID_ARGUMENT, "handle belongs to another CUDA device");
    const size_t poly = (size_t)r->n * r->l64;
    // every coefficient must be in [0, q)
    for (const uint64_t* src : {h_f, h_h}) {
        for (int i = 0; i < r->n; i++)
            if (BigUInt::from_limbs64(src + (size_t)i * r->l64, r->l64) >= r->q)
                return set_error(CY_ERR_INVALID_ARGUMENT, "key coefficient not in [0, q)");
    }
    for (size_t i = 0; i < (size_t)y->ell * r->n; i++)
        if (BigUInt::from_limbs64(h_evk + i * r->l64, r->l64) >= r->q)
            return set_error(CY_ERR_INVALID_ARGUMENT, "evaluation key coefficient not in [0, q)");
    y->h_f.assign(h_f, h_f + poly);
    y->h_h.assign(h_h, h_h + poly);
    y->h_evk.assign(h_evk, h_evk + poly * y->ell);
    y->has_keys = false;
    if (!y->d_f) CY_CUDA(cudaMalloc(&y->d_f, poly * sizeof(uint64_t)));
    if (!y->d_f2) CY_CUDA(cudaMalloc(&y->d_f2, poly * sizeof(uint64_t)));
    if (!y->d_h) CY_CUDA(cudaMalloc(&y->d_h, poly * sizeof(uint64_t)));
    CY_CUDA(cudaMemcpy(y->d_f, h_f, poly * sizeof(uint64_t), cudaMemcpyHostToDevice));
    CY_CUDA(cudaMemcpy(y->d_h, h_h, poly * sizeof(uint64_t), cudaMemcpyHostToDevice));
    CY_TRY(cy_polymul(r, y->d_f, y->d_f, y->d_f2, 1, nullptr));
    if (y->d_evk) {
        cudaFree(y->d_evk);
        y->d_evk = nullptr;
    }
    CY_TRY(prepare_evk(y->relin, h_evk, y->ell, r->n, r->l64, &y->d_evk));
    CY_CUDA(cudaDeviceSynchronize());
    y->has_keys = true;
    return CY_OK;
}

cy_status cy_yashe_get_keys(const cy_yashe* y, uint64_t* h_f, uint64_t* h_h, uint64_t* h_evk) {
    if (!y) return set_error(CY_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!y->has_keys) return set_error(CY_ERR_NO_KEYS, "no keys installed");
    if (h_f) std::copy(y->h_f.begin(), y->h_f.end(), h_f);
    if (h_h) std::copy(y->h_h.begin(), y->h_h.end(), h_h);
    if (h_evk) std::copy(y->h_evk.begin(), y->h_evk.end(), h_evk);
    return CY_OK;
}

cy_status cy_yashe_keygen(cy_yashe* y, uint64_t seed) {
    if (!y) return set_error(CY_ERR_INVALID_ARGUMENT, "NULL argument");
    std::vector<uint64_t> f, h, evk;
    CY_TRY(host_keygen(y, seed, f, h, evk));
    return cy_yashe_set_keys(y, f.data(), h.data(), evk.data());
}

cy_status cy_yashe_encrypt_host(cy_yashe* y, const uint64_t* h_m, uint64_t* h_ct, int batch, uint64_t seed) {
    if (!y || batch < 0 || (batch > 0 && (!h_m || !h_ct))) return set_error(CY_ERR_INVALID_ARGUMENT, "bad argument");
    if (!y->has_keys) return set_error(CY_ERR_NO_KEYS, "no keys installed");
    return host_encrypt(y, h_m, h_ct, batch, seed);
}

cy_status cy_yashe_decrypt(cy_yashe* y, const uint64_t* d_ct, uint64_t* d_m, int batch, int aftermul,
                           cy_stream_t stream) {
    CY_TRY(yashe_check(y, d_ct, d_m, batch));
    if (!y->has_keys) return set_error(CY_ERR_NO_KEYS, "no keys installed");
    cy_ring* r = y->ring;
    std::lock_guard<std::mutex> lock(r->mu);
    const long long stride = (long long)r->n * r->l64;
    return run_product_api(y->dec, false, aftermul ? y->d_f2 : y->d_f, 0, d_ct, stride, d_m, r->n, batch,
                           r->own_ws.ws, (cudaStream_t)stream);
}

cy_status cy_yashe_mul_ws(cy_yashe* y, cy_workspace* ws, const uint64_t* d_c1, const uint64_t* d_c2,
                          uint64_t* d_out, int batch, int relin, cy_stream_t stream) {
    CY_TRY(yashe_check(y, d_c1, d_c2, batch));
    if (batch > 0 && !d_out) return set_error(CY_ERR_INVALID_ARGUMENT, "NULL buffer");
    CY_TRY(check_aligned_api(d_out, nullptr, nullptr));
    if (relin && !y->has_keys) return set_error(CY_ERR_NO_KEYS, "relinearisation needs keys");
    cy_ring* r = y->ring;
    cudaStream_t st = (cudaStream_t)stream;
    std::unique_lock<std::mutex> lock(r->mu, std::defer_lock);
    Workspace* w = ws ? &ws->ws : &r->own_ws.ws;
    if (!ws) lock.lock();
    return run_yashe_mul(y->tensor, y->relin, y->d_evk, y->ell, d_c1, d_c2, d_out, batch, relin != 0, *w, st);
}

cy_status cy_yashe_mul(cy_yashe* y, const uint64_t* d_c1, const uint64_t* d_c2, uint64_t* d_out, int batch,
                       int relin, cy_stream_t stream) {
    return cy_yashe_mul_ws(y, nullptr, d_c1, d_c2, d_out, batch, relin, stream);
}

cy_status cy_yashe_mul_host(cy_yashe* y, const uint64_t* h_c1, const uint64_t* h_c2, uint64_t* h_out, int batch,
                            int relin) {
    CY_TRY(yashe_check(y, h_c1, h_c2, batch));
    if (batch > 0 && !h_out) return set_error(CY_ERR_INVALID_ARGUMENT, "NULL buffer");
    if (relin && !y->has_keys) return set_error(CY_ERR_NO_KEYS, "relinearisation needs keys");
    if (batch == 0) return CY_OK;
    cy_ring* r = y->ring;
    return run_host_pipeline((size_t)r->n * r->l64, batch, yashe_chunk_jobs(y->tensor, y->relin, y->ell, relin != 0),
                             h_c1, h_c2, h_out,
                             [y, relin](cy_workspace* ws, const uint64_t* a, const uint64_t* b, uint64_t* c, int nj,
                                        cudaStream_t st) { return cy_yashe_mul_ws(y, ws, a, b, c, nj, relin, st); });
}

cy_status cy_yashe_keyswitch(cy_yashe* y, const uint64_t* d_c, uint64_t* d_out, int batch, cy_stream_t stream) {
    CY_TRY(yashe_check(y, d_c, d_out, batch));
    if (!y->has_keys) return set_error(CY_ERR_NO_KEYS, "no keys installed");
    cy_ring* r = y->ring;
    std::lock_guard<std::mutex> lock(r->mu);
    return run_keyswitch_api(y->relin, d_c, y->d_evk, y->ell, d_out, batch, r->own_ws.ws, (cudaStream_t)stream);
}

cy_status cy_yashe_add(cy_yashe* y, const uint64_t* d_c1, const uint64_t* d_c2, uint64_t* d_out, int batch,
                       cy_stream_t stream) {
    if (!y) return set_error(CY_ERR_INVALID_ARGUMENT, "yashe handle is NULL");
    return cy_polyadd(y->ring, d_c1, d_c2, d_out, batch, stream);
}

}  // extern "C"
