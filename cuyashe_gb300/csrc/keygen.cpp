// keygen.cpp -- YASHE key generation and encryption (set-up time, host side).
//
// Replaces Yashe::generate_keys / Yashe::encrypt (src/yashe.cpp:17-142) and the
// samplers of src/distribution.cpp:4-60. Differences from the reference:
//   * f^-1 is a real inverse in R_q (the reference uses f itself,
//     src/yashe.cpp:48-50). It is computed on the host: pointwise inversion in
//     an NTT modulo q when q = 1 (mod 2N), the extended Euclidean algorithm over
//     F_q[x] for small N otherwise.
//   * the error distribution is a discrete Gaussian (CDT sampling, tail cut at
//     6 sigma); the reference draws uniform values mod 7 (src/distribution.cpp:9-51).
//   * every polynomial product (h = t g f^-1, h s_d, h s) runs on the GPU through
//     cy_polymul.
// Randomness: splitmix64 streams seeded by the caller.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "host.h"

namespace cy {

// ---- randomness -----------------------------------------------------------------
struct SplitMix64 {
    uint64_t s;
    explicit SplitMix64(uint64_t seed) : s(seed) {}
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        return z ^ (z >> 31);
    }
};

struct Gaussian {
    int bound;
    std::vector<double> cdf;
    explicit Gaussian(double sigma) {
        bound = (int)std::ceil(6.0 * sigma);
        double total = 0;
        std::vector<double> w(2 * bound + 1);
        for (int x = -bound; x <= bound; x++) total += (w[x + bound] = std::exp(-(double)x * x / (2 * sigma * sigma)));
        double acc = 0;
        cdf.resize(w.size());
        for (size_t i = 0; i < w.size(); i++) cdf[i] = (acc += w[i] / total);
        cdf.back() = 1.0;
    }
    int sample(SplitMix64& g) const {
        const double u = (double)(g.next() >> 11) * (1.0 / 9007199254740992.0);
        size_t lo = 0, hi = cdf.size() - 1;
        while (lo < hi) {
            size_t mid = (lo + hi) / 2;
            if (cdf[mid] < u) lo = mid + 1;
            else hi = mid;
        }
        return (int)lo - bound;
    }
};

// ---- fixed-width Montgomery arithmetic modulo q (L <= 6 limbs) ----------------------
struct MontQ {
    int L = 0;
    uint64_t q[6] = {0}, qinv = 0, r2[6] = {0}, one[6] = {0};

    explicit MontQ(const BigUInt& qq) {
        L = (qq.bits() + 63) / 64;
        qq.to_limbs64(q, L);
        uint64_t inv = q[0];
        for (int i = 0; i < 6; i++) inv *= 2 - q[0] * inv;
        qinv = (uint64_t)0 - inv;
        (BigUInt::pow2(128 * L) % qq).to_limbs64(r2, L);
        (BigUInt::pow2(64 * L) % qq).to_limbs64(one, L);
    }
    bool geq_q(const uint64_t* t) const {
        for (int i = L - 1; i >= 0; i--)
            if (t[i] != q[i]) return t[i] > q[i];
        return true;
    }
    void sub_q(uint64_t* t) const {
        unsigned __int128 br = 0;
        for (int i = 0; i < L; i++) {
            unsigned __int128 d = (unsigned __int128)t[i] - q[i] - br;
            t[i] = (uint64_t)d;
            br = (d >> 127) & 1;
        }
    }
    // out = a b R^-1 mod q (CIOS); out may alias a or b
    void mul(const uint64_t* a, const uint64_t* b, uint64_t* out) const {
        uint64_t t[8] = {0};
        for (int i = 0; i < L; i++) {
            unsigned __int128 C = 0;
            for (int j = 0; j < L; j++) {
                C += (unsigned __int128)a[j] * b[i] + t[j];
                t[j] = (uint64_t)C;
                C >>= 64;
            }
            C += t[L];
            t[L] = (uint64_t)C;
            t[L + 1] = (uint64_t)(C >> 64);
            const uint64_t m = t[0] * qinv;
            C = (unsigned __int128)m * q[0] + t[0];
            C >>= 64;
            for (int j = 1; j < L; j++) {
                C += (unsigned __int128)m * q[j] + t[j];
                t[j - 1] = (uint64_t)C;
                C >>= 64;
            }
            C += t[L];
            t[L - 1] = (uint64_t)C;
            t[L] = t[L + 1] + (uint64_t)(C >> 64);
        }
        if (t[L] || geq_q(t)) sub_q(t);
        std::memcpy(out, t, sizeof(uint64_t) * L);
    }
    void add(const uint64_t* a, const uint64_t* b, uint64_t* out) const {
        uint64_t t[7];
        unsigned __int128 c = 0;
        for (int i = 0; i < L; i++) {
            c += (unsigned __int128)a[i] + b[i];
            t[i] = (uint64_t)c;
            c >>= 64;
        }
        if (c || geq_q(t)) sub_q(t);
        std::memcpy(out, t, sizeof(uint64_t) * L);
    }
    void sub(const uint64_t* a, const uint64_t* b, uint64_t* out) const {
        uint64_t t[7];
        unsigned __int128 br = 0;
        for (int i = 0; i < L; i++) {
            unsigned __int128 d = (unsigned __int128)a[i] - b[i] - br;
            t[i] = (uint64_t)d;
            br = (d >> 127) & 1;
        }
        if (br) {
            unsigned __int128 c = 0;
            for (int i = 0; i < L; i++) {
                c += (unsigned __int128)t[i] + q[i];
                t[i] = (uint64_t)c;
                c >>= 64;
            }
        }
        std::memcpy(out, t, sizeof(uint64_t) * L);
    }
    void to_mont(const uint64_t* a, uint64_t* out) const { mul(a, r2, out); }
    void from_mont(const uint64_t* a, uint64_t* out) const {
        uint64_t o[6] = {1, 0, 0, 0, 0, 0};
        mul(a, o, out);
    }
    bool is_zero(const uint64_t* a) const {
        for (int i = 0; i < L; i++)
            if (a[i]) return false;
        return true;
    }
    // a^e (Montgomery domain in and out)
    void pow(const uint64_t* a, const BigUInt& e, uint64_t* out) const {
        uint64_t r[6], b[6];
        std::memcpy(r, one, sizeof(r));
        std::memcpy(b, a, sizeof(b));
        for (int i = e.bits() - 1; i >= 0; i--) {
            mul(r, r, r);
            if (e.bit(i)) mul(r, b, r);
        }
        std::memcpy(out, r, sizeof(uint64_t) * L);
    }
};

// f^-1 in Z_q[x]/(x^N+1) by pointwise inversion in a negacyclic NTT mod q
// (q = 1 mod 2N). f, out: [N][L] plain limbs.
static cy_status inverse_ntt_modq(const BigUInt& qq, int n, const std::vector<uint64_t>& f, std::vector<uint64_t>& out) {
    MontQ M(qq);
    const int L = M.L;
    // psi: element of order 2N
    const BigUInt qm1 = qq - BigUInt(1);
    const BigUInt e = qm1 / BigUInt(2ull * n);
    uint64_t psi[6] = {0};
    bool found = false;
    for (uint64_t g = 2; g < 1000 && !found; g++) {
        uint64_t gm[6] = {0}, gp[6] = {0};
        gm[0] = g;
        M.to_mont(gm, gm);
        M.pow(gm, e, psi);
        M.pow(psi, BigUInt((uint64_t)n), gp);  // psi^N must be -1
        uint64_t minus1[6];
        M.sub(M.one, M.one, minus1);
        M.sub(minus1, M.one, minus1);
        found = std::memcmp(gp, minus1, sizeof(uint64_t) * L) == 0;
    }
    if (!found) return set_error(CY_ERR_INTERNAL, "no 2N-th root of unity mod q");
    int logn = 0;
    while ((1 << logn) < n) logn++;
    // bit-reversed powers psi^bitrev(i), psi^-bitrev(i)
    std::vector<uint64_t> pw((size_t)2 * n * L), tw((size_t)n * L), itw((size_t)n * L);
    std::memcpy(&pw[0], M.one, sizeof(uint64_t) * L);
    for (int i = 1; i < 2 * n; i++) M.mul(&pw[(size_t)(i - 1) * L], psi, &pw[(size_t)i * L]);
    for (int i = 0; i < n; i++) {
        uint32_t r = 0;
        for (int b = 0; b < logn; b++) r |= ((i >> b) & 1u) << (logn - 1 - b);
        std::memcpy(&tw[(size_t)i * L], &pw[(size_t)r * L], sizeof(uint64_t) * L);
        std::memcpy(&itw[(size_t)i * L], &pw[(size_t)((2 * n - r) % (2 * n)) * L], sizeof(uint64_t) * L);
    }
    std::vector<uint64_t> a((size_t)n * L);
    for (int i = 0; i < n; i++) M.to_mont(&f[(size_t)i * L], &a[(size_t)i * L]);
    uint64_t U[6], V[6];
    // forward (Cooley-Tukey, natural in, bit-reversed out)
    for (int m = 1, t = n / 2; m < n; m *= 2, t /= 2) {
        for (int i = 0; i < m; i++) {
            const uint64_t* S = &tw[(size_t)(m + i) * L];
            for (int j = 2 * i * t; j < 2 * i * t + t; j++) {
                std::memcpy(U, &a[(size_t)j * L], sizeof(uint64_t) * L);
                M.mul(&a[(size_t)(j + t) * L], S, V);
                M.add(U, V, &a[(size_t)j * L]);
                M.sub(U, V, &a[(size_t)(j + t) * L]);
            }
        }
    }
    // batch inversion (Montgomery's trick)
    std::vector<uint64_t> pre((size_t)n * L);
    uint64_t acc[6];
    std::memcpy(acc, M.one, sizeof(acc));
    for (int i = 0; i < n; i++) {
        if (M.is_zero(&a[(size_t)i * L])) return set_error(CY_ERR_NOT_INVERTIBLE, "f is not invertible mod q");
        std::memcpy(&pre[(size_t)i * L], acc, sizeof(uint64_t) * L);
        M.mul(acc, &a[(size_t)i * L], acc);
    }
    uint64_t inv[6];
    M.pow(acc, qq - BigUInt(2), inv);
    for (int i = n - 1; i >= 0; i--) {
        uint64_t ai[6];
        M.mul(inv, &pre[(size_t)i * L], ai);
        M.mul(inv, &a[(size_t)i * L], inv);
        std::memcpy(&a[(size_t)i * L], ai, sizeof(uint64_t) * L);
    }
    // inverse (Gentleman-Sande, bit-reversed in, natural out)
    for (int m = n / 2, t = 1; m >= 1; m /= 2, t *= 2) {
        for (int i = 0, j1 = 0; i < m; i++, j1 += 2 * t) {
            const uint64_t* S = &itw[(size_t)(m + i) * L];
            for (int j = j1; j < j1 + t; j++) {
                std::memcpy(U, &a[(size_t)j * L], sizeof(uint64_t) * L);
                std::memcpy(V, &a[(size_t)(j + t) * L], sizeof(uint64_t) * L);
                M.add(U, V, &a[(size_t)j * L]);
                uint64_t d[6];
                M.sub(U, V, d);
                M.mul(d, S, &a[(size_t)(j + t) * L]);
            }
        }
    }
    uint64_t ninv[6] = {0}, nm[6] = {0};
    nm[0] = (uint64_t)n;
    M.to_mont(nm, nm);
    M.pow(nm, qq - BigUInt(2), ninv);
    out.assign((size_t)n * L, 0);
    for (int i = 0; i < n; i++) {
        uint64_t x[6];
        M.mul(&a[(size_t)i * L], ninv, x);
        M.from_mont(x, &out[(size_t)i * L]);
    }
    return CY_OK;
}

// ---- extended Euclid over F_q[x] (small N) ------------------------------------------
typedef std::vector<BigUInt> PolyQ;  // coefficients mod q, low degree first

static void trim(PolyQ& p) {
    while (!p.empty() && p.back().is_zero()) p.pop_back();
}
static BigUInt mod_sub(const BigUInt& a, const BigUInt& b, const BigUInt& q) { return a >= b ? a - b : a + q - b; }

static cy_status inverse_euclid(const BigUInt& q, int n, const std::vector<uint64_t>& f, int L,
                                std::vector<uint64_t>& out) {
    PolyQ r0(n + 1), r1(n), s0, s1(1, BigUInt(1));
    r0[0] = BigUInt(1);
    r0[n] = BigUInt(1);
    for (int i = 0; i < n; i++) r1[i] = BigUInt::from_limbs64(&f[(size_t)i * L], L) % q;
    trim(r1);
    const BigUInt qm2 = q - BigUInt(2);
    while (r1.size() > 1) {
        PolyQ rem = r0, quo(r0.size() - r1.size() + 1);
        const BigUInt inv_lead = BigUInt::powmod(r1.back(), qm2, q);
        trim(rem);
        while (rem.size() >= r1.size()) {
            const size_t d = rem.size() - r1.size();
            const BigUInt coef = (rem.back() * inv_lead) % q;
            quo[d] = coef;
            for (size_t i = 0; i < r1.size(); i++) rem[d + i] = mod_sub(rem[d + i], (coef * r1[i]) % q, q);
            trim(rem);
        }
        PolyQ prod(quo.size() + s1.size(), BigUInt());
        for (size_t i = 0; i < quo.size(); i++)
            for (size_t j = 0; j < s1.size(); j++) prod[i + j] = (prod[i + j] + quo[i] * s1[j]) % q;
        PolyQ sn(std::max(s0.size(), prod.size()), BigUInt());
        for (size_t i = 0; i < sn.size(); i++)
            sn[i] = mod_sub(i < s0.size() ? s0[i] : BigUInt(), i < prod.size() ? prod[i] : BigUInt(), q);
        trim(sn);
        r0 = r1;
        r1 = rem;
        s0 = s1;
        s1 = sn;
    }
    if (r1.empty()) return set_error(CY_ERR_NOT_INVERTIBLE, "f is not invertible mod q");
    const BigUInt c = BigUInt::powmod(r1[0], qm2, q);
    out.assign((size_t)n * L, 0);
    for (size_t i = 0; i < s1.size() && i < (size_t)n; i++) ((s1[i] * c) % q).to_limbs64(&out[i * L], L);
    return CY_OK;
}

// ---- helpers ---------------------------------------------------------------------------
static void put_signed(std::vector<uint64_t>& dst, size_t idx, long long v, const BigUInt& q, int L) {
    BigUInt x = v >= 0 ? BigUInt((uint64_t)v) % q : q - (BigUInt((uint64_t)(-v)) % q);
    if (x == q) x = BigUInt();
    x.to_limbs64(&dst[idx * L], L);
}

// c = a * b mod (x^N + 1, q) on the GPU for host arrays [count][N][L]
static cy_status gpu_mul(cy_ring* r, const std::vector<uint64_t>& a, const std::vector<uint64_t>& b,
                         std::vector<uint64_t>& c, int count) {
    c.assign(a.size(), 0);
    return cy_polymul_host(r, a.data(), b.data(), c.data(), count);
}

cy_status host_keygen(cy_yashe* y, uint64_t seed, std::vector<uint64_t>& f, std::vector<uint64_t>& h,
                      std::vector<uint64_t>& evk) {
    cy_ring* r = y->ring;
    const int n = r->n, L = r->l64;
    const BigUInt& q = r->q;
    SplitMix64 g(seed);
    Gaussian gauss(y->sigma);
    std::vector<uint64_t> gpoly((size_t)n * L), finv;
    for (int i = 0; i < n; i++) put_signed(gpoly, i, (long long)(g.next() % 3) - 1, q, L);
    const bool ntt_ok = ((q - BigUInt(1)) % BigUInt(2ull * n)).is_zero();
    if (!ntt_ok && n > 256)
        return set_error(CY_ERR_UNSUPPORTED, "keygen needs q = 1 mod 2N for N > 256 (NTT inversion)");
    for (int attempt = 0;; attempt++) {
        if (attempt > 64) return set_error(CY_ERR_NOT_INVERTIBLE, "no invertible f found");
        f.assign((size_t)n * L, 0);
        for (int i = 0; i < n; i++) {
            long long v = (long long)y->t * ((long long)(g.next() % 3) - 1) + (i == 0 ? 1 : 0);
            put_signed(f, i, v, q, L);
        }
        cy_status st = ntt_ok ? inverse_ntt_modq(q, n, f, finv) : inverse_euclid(q, n, f, L, finv);
        if (st == CY_OK) break;
        if (st != CY_ERR_NOT_INVERTIBLE) return st;
    }
    // h = t * g * f^-1
    std::vector<uint64_t> tg((size_t)n * L);
    for (int i = 0; i < n; i++) {
        BigUInt v = (BigUInt::from_limbs64(&gpoly[(size_t)i * L], L) * BigUInt(y->t)) % q;
        v.to_limbs64(&tg[(size_t)i * L], L);
    }
    CY_TRY(gpu_mul(r, tg, finv, h, 1));
    // evk_d = f w^d + e_d + h s_d
    const int ell = y->ell;
    std::vector<uint64_t> hs((size_t)ell * n * L), s((size_t)ell * n * L), e((size_t)ell * n * L), prod;
    for (int d = 0; d < ell; d++) {
        for (int i = 0; i < n; i++) put_signed(e, (size_t)d * n + i, gauss.sample(g), q, L);
        for (int i = 0; i < n; i++) put_signed(s, (size_t)d * n + i, gauss.sample(g), q, L);
        std::memcpy(&hs[(size_t)d * n * L], h.data(), sizeof(uint64_t) * n * L);
    }
    CY_TRY(gpu_mul(r, hs, s, prod, ell));
    evk.assign((size_t)ell * n * L, 0);
    for (int d = 0; d < ell; d++) {
        const BigUInt wd = BigUInt::pow2(y->w_bits * d) % q;
        for (int i = 0; i < n; i++) {
            const size_t idx = ((size_t)d * n + i) * L;
            BigUInt v = (BigUInt::from_limbs64(&f[(size_t)i * L], L) * wd) % q;
            v = v + BigUInt::from_limbs64(&e[idx], L);
            v = v + BigUInt::from_limbs64(&prod[idx], L);
            (v % q).to_limbs64(&evk[idx], L);
        }
    }
    return CY_OK;
}

cy_status host_encrypt(cy_yashe* y, const uint64_t* m, uint64_t* ct, int batch, uint64_t seed) {
    if (batch == 0) return CY_OK;
    cy_ring* r = y->ring;
    const int n = r->n, L = r->l64;
    const BigUInt& q = r->q;
    const BigUInt delta = q / BigUInt(y->t);
    Gaussian gauss(y->sigma);
    std::vector<uint64_t> hb((size_t)batch * n * L), s((size_t)batch * n * L), e((size_t)batch * n * L), prod;
    for (int b = 0; b < batch; b++) {
        SplitMix64 g(seed + 0x632BE59BD9B4E019ULL * (uint64_t)b);
        std::memcpy(&hb[(size_t)b * n * L], y->h_h.data(), sizeof(uint64_t) * n * L);
        for (int i = 0; i < n; i++) put_signed(s, (size_t)b * n + i, gauss.sample(g), q, L);
        for (int i = 0; i < n; i++) put_signed(e, (size_t)b * n + i, gauss.sample(g), q, L);
    }
    CY_TRY(gpu_mul(r, hb, s, prod, batch));
    for (int b = 0; b < batch; b++) {
        for (int i = 0; i < n; i++) {
            const size_t idx = ((size_t)b * n + i) * L;
            const uint64_t mv = m[(size_t)b * n + i];
            if (mv >= y->t) return set_error(CY_ERR_INVALID_ARGUMENT, "plaintext coefficient not in [0, t)");
            BigUInt v = delta * BigUInt(mv) + BigUInt::from_limbs64(&e[idx], L) + BigUInt::from_limbs64(&prod[idx], L);
            (v % q).to_limbs64(&ct[idx], L);
        }
    }
    return CY_OK;
}

}  // namespace cy
