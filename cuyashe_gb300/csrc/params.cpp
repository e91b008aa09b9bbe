// params.cpp -- CRT bases, twiddle tables and ICRT constants (host, set-up time).
//
// Replaces Polynomial::gen_crt_primes (src/polynomial.h:898-955), which takes
// 29-bit primes from a fixed bucket (src/polynomial.cpp:22) that are not NTT
// friendly, compute_reciprocal (src/polynomial.cpp:554-582),
// CUDAFunctions::write_crt_primes (src/cuda_bn.cu:1047-1146) and the twiddle
// set-up of CUDAFunctions::init (src/cuda_functions.cu:878-930).
#include <cuda_runtime.h>

#include <map>
#include <mutex>

#include "host.h"

namespace cy {

// ---- errors ------------------------------------------------------------------
static thread_local std::string g_last_error;

cy_status set_error(cy_status st, const std::string& msg) {
    g_last_error = msg;
    return st;
}
cy_status cuda_error(cudaError_t e, const char* what) {
    cy_status st = (e == cudaErrorMemoryAllocation) ? CY_ERR_OUT_OF_MEMORY : CY_ERR_CUDA;
    return set_error(st, std::string(what) + ": " + cudaGetErrorString(e));
}
const char* last_error_message() { return g_last_error.c_str(); }

// ---- 32-bit number theory ----------------------------------------------------
static uint32_t mulmod32(uint32_t a, uint32_t b, uint32_t m) { return (uint32_t)((uint64_t)a * b % m); }
static uint32_t powmod32(uint32_t b, uint64_t e, uint32_t m) {
    uint32_t r = 1 % m;
    while (e) {
        if (e & 1) r = mulmod32(r, b, m);
        b = mulmod32(b, b, m);
        e >>= 1;
    }
    return r;
}
static uint32_t invmod32(uint32_t a, uint32_t m) { return powmod32(a % m, m - 2, m); }  // m prime

// deterministic Miller-Rabin for n < 2^32 (bases 2, 7, 61)
static bool is_prime32(uint32_t n) {
    if (n < 2) return false;
    for (uint32_t p : {2u, 3u, 5u, 7u, 11u, 13u, 61u})
        if (n % p == 0) return n == p;
    uint32_t d = n - 1;
    int s = 0;
    while (!(d & 1)) {
        d >>= 1;
        s++;
    }
    for (uint32_t a : {2u, 7u, 61u}) {
        uint32_t x = powmod32(a, d, n);
        if (x == 1 || x == n - 1) continue;
        bool comp = true;
        for (int r = 1; r < s; r++) {
            x = mulmod32(x, x, n);
            if (x == n - 1) {
                comp = false;
                break;
            }
        }
        if (comp) return false;
    }
    return true;
}

const std::vector<uint32_t>& table_primes() {
    static std::vector<uint32_t> primes;
    static std::once_flag once;
    std::call_once(once, [] {
        for (uint32_t c = (1u << (30 - PRIME_TWO_ADIC)) - 1; c > 0 && (int)primes.size() < TABLE_PRIMES; c--) {
            uint32_t p = (c << PRIME_TWO_ADIC) + 1;
            if (is_prime32(p)) primes.push_back(p);
        }
    });
    return primes;
}

static uint32_t bitrev(uint32_t x, int bits) {
    uint32_t r = 0;
    for (int i = 0; i < bits; i++) r |= ((x >> i) & 1u) << (bits - 1 - i);
    return r;
}

// psi of exact order 2^(LOGN_MAX+1) modulo p
static uint32_t find_psi(uint32_t p) {
    const uint64_t order = 2ull * NMAX;
    for (uint32_t g = 2; g < 1000; g++) {
        uint32_t w = powmod32(g, (p - 1) / order, p);
        if (powmod32(w, order / 2, p) == p - 1) return w;
    }
    return 0;
}

static uint32_t shoup_of(uint32_t w, uint32_t p) { return (uint32_t)(((uint64_t)w << 32) / p); }

cy_status prime_table(int device, const PrimeTable** out) {
    static std::mutex mu;
    static std::map<int, PrimeTable*> tables;
    std::lock_guard<std::mutex> lock(mu);
    auto it = tables.find(device);
    if (it != tables.end()) {
        *out = it->second;
        return CY_OK;
    }
    const std::vector<uint32_t>& primes = table_primes();
    if ((int)primes.size() < TABLE_PRIMES) return set_error(CY_ERR_INTERNAL, "prime table generation failed");
    std::vector<uint2> psi((size_t)TABLE_PRIMES * NMAX), ipsi((size_t)TABLE_PRIMES * NMAX);
    std::vector<uint32_t> pw(2 * NMAX);
    for (int i = 0; i < TABLE_PRIMES; i++) {
        const uint32_t p = primes[i];
        const uint32_t root = find_psi(p);
        if (!root) return set_error(CY_ERR_INTERNAL, "no root of unity for table prime");
        pw[0] = 1;
        for (int j = 1; j < 2 * NMAX; j++) pw[j] = mulmod32(pw[j - 1], root, p);
        for (int j = 0; j < NMAX; j++) {
            const uint32_t e = bitrev((uint32_t)j, LOGN_MAX);
            const uint32_t w = pw[e];
            const uint32_t wi = pw[(2 * NMAX - e) % (2 * NMAX)];
            psi[(size_t)i * NMAX + j] = make_uint2(w, shoup_of(w, p));
            ipsi[(size_t)i * NMAX + j] = make_uint2(wi, shoup_of(wi, p));
        }
    }
    // row-pass tables of N = ROWS_N: entry (l, h, tau) = tw[2^(S0+l) + tau 2^l + h]
    // with S0 = ROWS_LOGN - 6 the first stage of the row pass
    std::vector<uint2> psi_r((size_t)TABLE_PRIMES * ROWS_WORDS), ipsi_r((size_t)TABLE_PRIMES * ROWS_WORDS);
    for (int i = 0; i < TABLE_PRIMES; i++)
        for (int l = 0; l < 6; l++)
            for (int h = 0; h < (1 << l); h++)
                for (int tau = 0; tau < ROWS_G; tau++) {
                    const size_t src = (size_t)i * NMAX + ((size_t)1 << (ROWS_LOGN - 6 + l)) + ((size_t)tau << l) + h;
                    const size_t dst = (size_t)i * ROWS_WORDS + rows_index(l, h, tau);
                    psi_r[dst] = psi[src];
                    ipsi_r[dst] = ipsi[src];
                }
    PrimeTable* t = new PrimeTable();
    t->device = device;
    t->primes = primes;
    const size_t bytes = sizeof(uint2) * (size_t)TABLE_PRIMES * NMAX;
    const size_t rbytes = sizeof(uint2) * psi_r.size();
    cudaError_t e = cudaMalloc(&t->d_psi, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&t->d_ipsi, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&t->d_psi_r, rbytes);
    if (e == cudaSuccess) e = cudaMalloc(&t->d_ipsi_r, rbytes);
    if (e == cudaSuccess) e = cudaMemcpy(t->d_psi, psi.data(), bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(t->d_ipsi, ipsi.data(), bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(t->d_psi_r, psi_r.data(), rbytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(t->d_ipsi_r, ipsi_r.data(), rbytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(t->d_psi);
        cudaFree(t->d_ipsi);
        cudaFree(t->d_psi_r);
        cudaFree(t->d_ipsi_r);
        delete t;
        return cuda_error(e, "prime table upload");
    }
    tables[device] = t;  // kept until process exit
    *out = t;
    return CY_OK;
}

// ---- basis constants -------------------------------------------------------------
cy_status basis_constants(BasisDev& h, int* crt_bits, int n, const BigUInt& q, int mode, const BigUInt& bound,
                          uint32_t t, bool mont, bool scale_n, bool centered) {
    h = BasisDev{};
    const std::vector<uint32_t>& primes = table_primes();
    int logn = 0;
    while ((1 << logn) < n) logn++;
    const int qbits = q.bits();
    if (qbits < 2 || qbits > 32 * L32MAX) return set_error(CY_ERR_UNSUPPORTED, "q must have 2..384 bits");
    BigUInt M(1);
    int k = 0;
    while (M <= bound) {
        if (k >= KMAX || k >= (int)primes.size())
            return set_error(CY_ERR_UNSUPPORTED, "CRT basis needs more than CY_MAX_CRT_PRIMES primes");
        M = M * BigUInt(primes[k]);
        k++;
    }
    *crt_bits = M.bits();
    h.n = n;
    h.logn = logn;
    h.k = k;
    h.l32 = (qbits + 31) / 32;
    h.l64 = (qbits + 63) / 64;
    h.mode = mode;
    h.shift = 32 * h.l32 - qbits;
    h.qbits = qbits;
    h.t = t;
    h.centered = centered ? 1 : 0;
    const BigUInt qn = q.shl(h.shift);
    const BigUInt mu = BigUInt::pow2(32 * h.l32 + 37) / qn;
    h.mu = mu.low64();
    qn.to_words32(h.qn, L32MAX);
    q.to_words32(h.q, L32MAX);
    const BigUInt qhalf = (q - BigUInt(1)).shr(1);
    qhalf.to_words32(h.qhalf, L32MAX);
    qhalf.shl(h.shift).to_words32(h.qhalf_n, L32MAX);

    const BigUInt Mq = M % q;
    BigUInt tM, IM, RM;
    if (mode == EPI_YASHE) {
        tM = M * BigUInt(t);
        BigUInt::divmod(tM, q, &IM, &RM);
        BigUInt im1 = (IM + BigUInt(1)) % q;
        BigUInt b0 = im1.is_zero() ? BigUInt() : q - im1;
        b0.shl(h.shift).to_words32(h.B0, L32MAX);
        (q - RM).shl(h.shift).to_words32(h.B1, L32MAX);
        ((q - RM).shl(64) / q).to_words32(h.frac_m, 2);
    } else {
        BigUInt b0 = Mq.is_zero() ? BigUInt() : q - Mq;
        b0.shl(h.shift).to_words32(h.B0, L32MAX);
    }
    for (int i = 0; i < k; i++) {
        const uint32_t p = primes[i];
        h.p[i] = p;
        h.p2[i] = 2 * p;
        h.np[i] = 0u - p;
        h.np2[i] = 0u - 2 * p;
        // -p^-1 mod 2^32 by Newton iteration
        uint32_t inv = p;
        for (int it = 0; it < 5; it++) inv *= 2u - p * inv;
        h.pinv[i] = (uint32_t)(0u - inv);
        const BigUInt Mhat = M / BigUInt(p);
        const uint32_t mh = Mhat.mod_u32(p);
        uint32_t f = invmod32(mh, p);
        if (scale_n) f = mulmod32(f, invmod32((uint32_t)(n % p), p), p);
        if (mont) f = mulmod32(f, (uint32_t)((1ull << 32) % p), p);
        h.ycon[i] = f;
        h.ycon_sh[i] = shoup_of(f, p);
        const uint64_t F = (uint64_t)(((unsigned __int128)1 << 64) / p);
        h.fhi[i] = (uint32_t)(F >> 32);
        h.flo[i] = (uint32_t)F;
        h.qmodp[i] = q.mod_u32(p);
        const uint32_t r32 = (uint32_t)((1ull << 32) % p);
        h.r32[i] = r32;
        h.r32_sh[i] = shoup_of(r32, p);
        uint32_t c = 1;
        for (int j = 0; j < L32MAX; j++) {
            h.crt[i][j] = c;
            c = mulmod32(c, r32, p);
        }
        if (mode == EPI_YASHE) {
            BigUInt I, R;
            BigUInt::divmod(Mhat * BigUInt(t), q, &I, &R);
            (I % q).shl(h.shift).to_words32(h.A0[i], L32MAX);
            R.shl(h.shift).to_words32(h.A1[i], L32MAX);
            (R.shl(64) / q).to_words32(h.frac[i], 2);
        } else {
            (Mhat % q).shl(h.shift).to_words32(h.A0[i], L32MAX);
        }
    }
    return CY_OK;
}

Basis::~Basis() {
    if (d) cudaFree(d);
    if (d_ninv) cudaFree(d_ninv);
}

cy_status build_basis(Basis& b, int device, int n, const BigUInt& q, int mode, const BigUInt& bound, uint32_t t,
                      bool mont, bool scale_n, bool centered) {
    const PrimeTable* tab = nullptr;
    CY_TRY(prime_table(device, &tab));
    CY_TRY(basis_constants(b.h, &b.crt_bits, n, q, mode, bound, t, mont, scale_n, centered));
    for (int i = 0; i < b.h.k; i++) {
        b.h.psi[i] = tab->d_psi + (size_t)i * NMAX;
        b.h.ipsi[i] = tab->d_ipsi + (size_t)i * NMAX;
        if (b.h.logn == ROWS_LOGN) {
            b.h.psi_r[i] = tab->d_psi_r + (size_t)i * ROWS_WORDS;
            b.h.ipsi_r[i] = tab->d_ipsi_r + (size_t)i * ROWS_WORDS;
        }
    }
    // per prime: N^-1, and N^-1 times the twiddle of the last inverse stage
    // (psi^-bitrev(1) = psi^-(NMAX/2)), each with its Shoup companion
    std::vector<uint32_t> ninv(4 * (size_t)b.h.k);
    for (int i = 0; i < b.h.k; i++) {
        const uint32_t p = b.h.p[i];
        const uint32_t v = invmod32((uint32_t)(n % p), p);
        const uint32_t psi = find_psi(p);
        const uint32_t w1 = powmod32(psi, 2ull * NMAX - NMAX / 2, p);
        const uint32_t vw = mulmod32(v, w1, p);
        ninv[4 * i] = v;
        ninv[4 * i + 1] = shoup_of(v, p);
        ninv[4 * i + 2] = vw;
        ninv[4 * i + 3] = shoup_of(vw, p);
    }
    b.epi = epi_special(b.h.l32, b.h.k, b.h.mode);
    if (b.epi) {
        b.epi_param.assign(b.epi->param_bytes, 0);
        b.epi->fill(b.h, b.epi_param.data());
    }
    CY_CUDA(cudaMalloc(&b.d, sizeof(BasisDev)));
    CY_CUDA(cudaMemcpy(b.d, &b.h, sizeof(BasisDev), cudaMemcpyHostToDevice));
    CY_CUDA(cudaMalloc(&b.d_ninv, sizeof(uint32_t) * ninv.size()));
    CY_CUDA(cudaMemcpy(b.d_ninv, ninv.data(), sizeof(uint32_t) * ninv.size(), cudaMemcpyHostToDevice));
    return CY_OK;
}

// ---- scratch --------------------------------------------------------------------
cy_status Workspace::reserve(size_t words) {
    if (words <= resid_words) return CY_OK;
    if (d_resid) {
        cudaFree(d_resid);
        d_resid = nullptr;
        resid_words = 0;
    }
    CY_CUDA(cudaMalloc(&d_resid, words * sizeof(uint32_t)));
    resid_words = words;
    return CY_OK;
}

cy_status Workspace::reserve_side(int i, size_t words) {
    if (!fork) CY_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
    if (!side[i]) {
        CY_CUDA(cudaStreamCreateWithFlags(&side[i], cudaStreamNonBlocking));
        CY_CUDA(cudaEventCreateWithFlags(&join[i], cudaEventDisableTiming));
    }
    if (words <= side_words[i]) return CY_OK;
    if (d_side_resid[i]) {
        cudaFree(d_side_resid[i]);
        d_side_resid[i] = nullptr;
        side_words[i] = 0;
    }
    CY_CUDA(cudaMalloc(&d_side_resid[i], words * sizeof(uint32_t)));
    side_words[i] = words;
    return CY_OK;
}

Workspace::~Workspace() {
    if (d_resid) cudaFree(d_resid);
    for (int i = 0; i < kMaxSide; i++) {
        if (d_side_resid[i]) cudaFree(d_side_resid[i]);
        if (join[i]) cudaEventDestroy(join[i]);
        if (side[i]) cudaStreamDestroy(side[i]);
    }
    if (fork) cudaEventDestroy(fork);
}

}  // namespace cy
