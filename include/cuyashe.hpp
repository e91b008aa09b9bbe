// cuyashe.hpp -- the reference's C++ API (Polynomial, Ciphertext, Yashe) on top
// of the C ABI in cuyashe.h.
//
// The reference's classes (src/polynomial.h, src/ciphertext.h, src/yashe.h) keep
// NTL::ZZ coefficients on the host, device residues behind HOST_IS_UPDATED /
// CRT_COMPUTED flags, and process-wide statics for q, phi, the CRT basis and the
// YASHE keys. This header keeps the method names and their meaning:
//   Polynomial: set_coeff / get_coeff / get_coeffs / deg / set_coeffs / random,
//               operator* (= the reference's a*b followed by reduce()), +, -,
//               * by an integer, update_device_data / update_host_data,
//               reduce (kept for compatibility; results are already reduced);
//   Ciphertext: operator* (tensor product, marked `aftermul` as in the
//               reference, relinearised lazily), convert (keyswitch), +;
//   Yashe:      generate_keys, encrypt (on the GPU), decrypt; Ciphertext + and *
//               by a plaintext polynomial.
// Differences: the statics become a Context (the ring) and a Yashe object;
// coefficients are cuyashe::ZZ (a host big integer, NTL is not needed); every
// product runs on the GPU through cy_polymul / cy_yashe_mul; errors throw
// cuyashe::Error (the reference throws const char*).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "cuyashe.h"
#include "cuyashe_bigint.h"

namespace cuyashe {

using ZZ = cy::BigUInt;

struct Error : std::runtime_error {
    int status;
    Error(int st, const std::string& where)
        : std::runtime_error(where + ": " + cy_status_string(st) + " (" + cy_last_error() + ")"), status(st) {}
};

inline void check(cy_status st, const char* where) {
    if (st != CY_OK) throw Error(st, where);
}

inline void check_cuda(cudaError_t e, const char* where) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(where) + ": " + cudaGetErrorString(e));
}

// The ring Z_q[x]/(x^N+1): replaces Polynomial::global_mod / global_phi,
// Polynomial::gen_crt_primes and CUDAFunctions::init.
class Context {
   public:
    Context(int n, const ZZ& q) : n_(n), q_(q), limbs_((q.bits() + 63) / 64) {
        std::vector<uint64_t> ql(limbs_);
        q.to_limbs64(ql.data(), limbs_);
        check(cy_ring_create(n, ql.data(), limbs_, &ring_), "cy_ring_create");
        own_ = true;
    }
    // wraps a ring owned elsewhere (a Yashe context's)
    Context(cy_ring* ring, int n, const ZZ& q) : ring_(ring), n_(n), q_(q), limbs_((q.bits() + 63) / 64) {}
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    ~Context() {
        if (own_) cy_ring_destroy(ring_);
    }
    int n() const { return n_; }
    const ZZ& q() const { return q_; }
    int limbs() const { return limbs_; }
    cy_ring* ring() const { return ring_; }

   private:
    cy_ring* ring_ = nullptr;
    bool own_ = false;
    int n_;
    ZZ q_;
    int limbs_;
};

// A device copy of host words (owned, freed on destruction).
class DeviceWords {
   public:
    explicit DeviceWords(const std::vector<uint64_t>& h) : n_(h.size()) {
        check_cuda(cudaMalloc(&d_, n_ * sizeof(uint64_t)), "cudaMalloc");
        check_cuda(cudaMemcpy(d_, h.data(), n_ * sizeof(uint64_t), cudaMemcpyHostToDevice), "H2D");
    }
    DeviceWords(DeviceWords&& o) noexcept : d_(o.d_), n_(o.n_) { o.d_ = nullptr; }
    DeviceWords(const DeviceWords&) = delete;
    DeviceWords& operator=(const DeviceWords&) = delete;
    ~DeviceWords() {
        if (d_) cudaFree(d_);
    }
    const uint64_t* get() const { return d_; }

   private:
    uint64_t* d_ = nullptr;
    size_t n_;
};

class Polynomial {
   public:
    explicit Polynomial(const Context& ctx) : ctx_(&ctx), host_((size_t)ctx.n() * ctx.limbs(), 0) {}
    Polynomial(const Polynomial& o) : ctx_(o.ctx_) { copy_from(o); }
    Polynomial& operator=(const Polynomial& o) {
        if (this != &o) {
            ctx_ = o.ctx_;
            copy_from(o);
        }
        return *this;
    }
    Polynomial(Polynomial&& o) noexcept { swap(o); }
    Polynomial& operator=(Polynomial&& o) noexcept {
        swap(o);
        return *this;
    }
    virtual ~Polynomial() {
        if (dev_) cudaFree(dev_);
    }

    const Context& context() const { return *ctx_; }
    int n() const { return ctx_->n(); }

    // -- coefficients (src/polynomial.h:765-870) ------------------------------
    void set_coeff(int i, const ZZ& v) {
        host_sync();
        (v % ctx_->q()).to_limbs64(&host_[(size_t)i * ctx_->limbs()], ctx_->limbs());
        dev_ok_ = false;
    }
    void set_coeff(int i, uint64_t v) { set_coeff(i, ZZ(v)); }
    ZZ get_coeff(int i) const {
        host_sync();
        return ZZ::from_limbs64(&host_[(size_t)i * ctx_->limbs()], ctx_->limbs());
    }
    std::vector<ZZ> get_coeffs() const {
        std::vector<ZZ> v(n());
        for (int i = 0; i < n(); i++) v[i] = get_coeff(i);
        return v;
    }
    // zero every coefficient (the reference's set_coeffs() / set_coeffs(size))
    void set_coeffs(int = 0) {
        host_.assign(host_.size(), 0);
        host_ok_ = true;
        dev_ok_ = false;
    }
    int deg() const {
        for (int i = n() - 1; i >= 0; i--)
            if (!get_coeff(i).is_zero()) return i;
        return -1;
    }
    // uniform coefficients below q for degree + 1 terms (Polynomial::random,
    // src/polynomial.h:1370-1380), from a seeded splitmix64 stream
    static void random(Polynomial* a, int degree, uint64_t seed = 36251) {
        a->set_coeffs();
        uint64_t s = seed;
        auto next = [&s] {
            uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
            return z ^ (z >> 31);
        };
        for (int i = 0; i <= degree && i < a->n(); i++) {
            ZZ v;
            for (int w = 0; w < a->context().limbs() + 1; w++) v = v.shl(64) + ZZ(next());
            a->set_coeff(i, v);
        }
    }

    // -- arithmetic on the GPU -----------------------------------------------
    // c = a*b mod (x^N+1, q): the reference's `Polynomial c = a*b; c.reduce();`
    Polynomial operator*(const Polynomial& b) const {
        same_ring(b);
        Polynomial c(*ctx_);
        c.alloc_dev();
        check(cy_polymul(ctx_->ring(), device_data(), b.device_data(), c.dev_, 1, nullptr), "cy_polymul");
        c.dev_written();
        return c;
    }
    Polynomial operator+(const Polynomial& b) const {
        same_ring(b);
        Polynomial c(*ctx_);
        c.alloc_dev();
        check(cy_polyadd(ctx_->ring(), device_data(), b.device_data(), c.dev_, 1, nullptr), "cy_polyadd");
        c.dev_written();
        return c;
    }
    Polynomial operator-(const Polynomial& b) const {
        same_ring(b);
        Polynomial c(*ctx_);
        c.alloc_dev();
        check(cy_polysub(ctx_->ring(), device_data(), b.device_data(), c.dev_, 1, nullptr), "cy_polysub");
        c.dev_written();
        return c;
    }
    Polynomial operator*(const ZZ& s) const {
        Polynomial c(*ctx_);
        c.alloc_dev();
        std::vector<uint64_t> sl(ctx_->limbs());
        (s % ctx_->q()).to_limbs64(sl.data(), ctx_->limbs());
        check(cy_poly_scalar_mul(ctx_->ring(), device_data(), sl.data(), c.dev_, 1, nullptr), "cy_poly_scalar_mul");
        c.dev_written();
        return c;
    }
    Polynomial& operator*=(const Polynomial& b) { return *this = *this * b; }
    Polynomial& operator+=(const Polynomial& b) { return *this = *this + b; }
    Polynomial& operator-=(const Polynomial& b) { return *this = *this - b; }
    Polynomial& operator*=(const ZZ& s) { return *this = *this * s; }
    // every coefficient reduced mod the modulus of `target` (the reference's
    // `Polynomial % ZZ`, src/polynomial.h:574-592), as a polynomial of `target`
    Polynomial mod_to(const Context& target) const {
        Polynomial r(target);
        for (int i = 0; i < n(); i++) r.set_coeff(i, get_coeff(i) % target.q());
        return r;
    }
    // The reference folds by x^N+1 and reduces mod q here (src/cuda_functions.cu:
    // 1040-1077); every result of this API is already reduced.
    void reduce() {}
    bool operator==(const Polynomial& b) const {
        host_sync();
        b.host_sync();
        return ctx_ == b.ctx_ && host_ == b.host_;
    }
    bool operator!=(const Polynomial& b) const { return !(*this == b); }

    // -- host/device state (src/polynomial.cpp:265-417) ----------------------
    void update_device_data() const { (void)device_data(); }
    void update_host_data() const { host_sync(); }
    const uint64_t* device_data() const {
        if (!dev_ok_) {
            alloc_dev();
            check_cuda(cudaMemcpy(dev_, host_.data(), bytes(), cudaMemcpyHostToDevice), "update_device_data");
            dev_ok_ = true;
        }
        return dev_;
    }
    // raw host limbs [N][L] (synchronised)
    const std::vector<uint64_t>& limbs() const {
        host_sync();
        return host_;
    }
    void set_limbs(const uint64_t* src) {
        std::copy(src, src + host_.size(), host_.begin());
        host_ok_ = true;
        dev_ok_ = false;
    }
    std::string to_string() const {
        std::string s;
        for (int i = 0; i < n(); i++) s += get_coeff(i).to_dec() + (i + 1 < n() ? ", " : "");
        return s;
    }

   protected:
    uint64_t* mutable_device() {
        alloc_dev();
        return dev_;
    }
    void dev_written() {
        dev_ok_ = true;
        host_ok_ = false;
    }

   private:
    void same_ring(const Polynomial& b) const {
        if (b.ctx_ != ctx_) throw Error(CY_ERR_INVALID_ARGUMENT, "operands belong to different rings");
    }
    size_t bytes() const { return host_.size() * sizeof(uint64_t); }
    void alloc_dev() const {
        if (!dev_) check_cuda(cudaMalloc(&dev_, bytes()), "cudaMalloc");
    }
    void host_sync() const {
        if (!host_ok_) {
            check_cuda(cudaMemcpy(host_.data(), dev_, bytes(), cudaMemcpyDeviceToHost), "update_host_data");
            host_ok_ = true;
        }
    }
    void copy_from(const Polynomial& o) {
        o.host_sync();
        host_ = o.host_;
        host_ok_ = true;
        dev_ok_ = false;
    }
    void swap(Polynomial& o) {
        std::swap(ctx_, o.ctx_);
        std::swap(host_, o.host_);
        std::swap(dev_, o.dev_);
        std::swap(host_ok_, o.host_ok_);
        std::swap(dev_ok_, o.dev_ok_);
    }

    const Context* ctx_ = nullptr;
    mutable std::vector<uint64_t> host_;
    mutable uint64_t* dev_ = nullptr;
    mutable bool host_ok_ = true, dev_ok_ = false;
    friend class Ciphertext;
    friend class Yashe;
};

class Yashe;

// A YASHE ciphertext: src/ciphertext.h. `aftermul` marks a product that is not
// relinearised yet (decrypts with f^2); operator* relinearises such operands
// first, as the reference does (src/ciphertext.cpp:38-48).
class Ciphertext : public Polynomial {
   public:
    Ciphertext(Yashe& y);
    Ciphertext operator*(Ciphertext& b);
    Ciphertext operator+(Ciphertext& b);
    // plaintext operand m in R_t: c + Delta*m, and c * m (m centred mod t)
    Ciphertext operator+(const Polynomial& m);
    Ciphertext operator*(const Polynomial& m);
    void convert();
    int level = 0;
    bool aftermul = false;

   private:
    Yashe* y_;
};

// The scheme: src/yashe.h. Replaces the statics Yashe::{d, q, t, w, lwq, f, h,
// gamma} with an object that owns a cy_yashe (keys and evaluation key stay on
// the GPU).
class Yashe {
   public:
    Yashe(int n, const ZZ& q, uint64_t t, int w_bits = 32, double sigma = 8.0) : n_(n), q_(q), t_(t) {
        const int L = (q.bits() + 63) / 64;
        std::vector<uint64_t> ql(L);
        q.to_limbs64(ql.data(), L);
        cy_yashe_params p{n, ql.data(), L, t, w_bits, sigma};
        check(cy_yashe_create(&p, &y_), "cy_yashe_create");
        cy_ring* ring = nullptr;
        check(cy_yashe_get_ring(y_, &ring), "cy_yashe_get_ring");
        ctx_.reset(new Context(ring, n, q));
        pt_.reset(new Context(n, ZZ(t)));
    }
    Yashe(const Yashe&) = delete;
    Yashe& operator=(const Yashe&) = delete;
    ~Yashe() {
        pt_.reset();
        ctx_.reset();
        cy_yashe_destroy(y_);
    }
    const Context& context() const { return *ctx_; }            // R_q (ciphertexts)
    const Context& plaintext_context() const { return *pt_; }   // R_t (plaintexts)
    cy_yashe* handle() const { return y_; }
    uint64_t t() const { return t_; }

    void generate_keys(uint64_t seed = 1234) { check(cy_yashe_keygen(y_, seed), "cy_yashe_keygen"); }

    // c = [Delta*m + e + h*s]_q with s, e drawn on the GPU; m in R_t
    // (src/yashe.cpp:104-142)
    Ciphertext encrypt(const Polynomial& m, uint64_t seed = 1);

    // plaintext coefficients as one word each, on the device
    DeviceWords plaintext_words(const Polynomial& m) const {
        std::vector<uint64_t> mv(n_);
        for (int i = 0; i < n_; i++) {
            const ZZ v = m.get_coeff(i);
            if (v >= ZZ(t_)) throw Error(CY_ERR_INVALID_ARGUMENT, "plaintext coefficient >= t");
            mv[i] = v.low64();
        }
        return DeviceWords(mv);
    }

    // m = [round(t/q [key*c]_q)]_t for every coefficient (src/yashe.cpp:143-201)
    Polynomial decrypt(const Ciphertext& c) {
        uint64_t* dm = nullptr;
        check_cuda(cudaMalloc(&dm, sizeof(uint64_t) * n_), "cudaMalloc");
        cy_status st = cy_yashe_decrypt(y_, c.device_data(), dm, 1, c.aftermul ? 1 : 0, nullptr);
        std::vector<uint64_t> mv(n_);
        if (st == CY_OK) check_cuda(cudaMemcpy(mv.data(), dm, sizeof(uint64_t) * n_, cudaMemcpyDeviceToHost), "D2H");
        cudaFree(dm);
        check(st, "cy_yashe_decrypt");
        Polynomial m(*pt_);
        for (int i = 0; i < n_; i++) m.set_coeff(i, mv[i]);
        return m;
    }

   private:
    int n_;
    ZZ q_;
    uint64_t t_;
    cy_yashe* y_ = nullptr;
    std::unique_ptr<Context> ctx_, pt_;
};

inline Ciphertext::Ciphertext(Yashe& y) : Polynomial(y.context()), y_(&y) {}

inline Ciphertext Yashe::encrypt(const Polynomial& m, uint64_t seed) {
    const DeviceWords dm = plaintext_words(m);
    Ciphertext c(*this);
    check(cy_yashe_encrypt(y_, dm.get(), c.mutable_device(), 1, seed, nullptr), "cy_yashe_encrypt");
    c.dev_written();
    return c;
}

inline Ciphertext Ciphertext::operator+(const Polynomial& m) {
    const DeviceWords dm = y_->plaintext_words(m);
    Ciphertext c(*y_);
    check(cy_yashe_add_plain(y_->handle(), device_data(), dm.get(), c.mutable_device(), 1, nullptr),
          "cy_yashe_add_plain");
    c.dev_written();
    c.level = level;
    c.aftermul = aftermul;
    return c;
}

inline Ciphertext Ciphertext::operator*(const Polynomial& m) {
    const DeviceWords dm = y_->plaintext_words(m);
    Ciphertext c(*y_);
    check(cy_yashe_mul_plain(y_->handle(), device_data(), dm.get(), c.mutable_device(), 1, nullptr),
          "cy_yashe_mul_plain");
    c.dev_written();
    c.level = level;
    c.aftermul = aftermul;
    return c;
}

inline Ciphertext Ciphertext::operator*(Ciphertext& b) {
    if (b.y_ != y_) throw Error(CY_ERR_INVALID_ARGUMENT, "ciphertexts of different schemes");
    if (aftermul) convert();
    if (b.aftermul) b.convert();
    Ciphertext c(*y_);
    check(cy_yashe_mul(y_->handle(), device_data(), b.device_data(), c.mutable_device(), 1, 0, nullptr),
          "cy_yashe_mul");
    c.dev_written();
    c.aftermul = true;
    c.level = (level > b.level ? level : b.level) + 1;
    return c;
}

inline Ciphertext Ciphertext::operator+(Ciphertext& b) {
    if (b.y_ != y_) throw Error(CY_ERR_INVALID_ARGUMENT, "ciphertexts of different schemes");
    Ciphertext c(*y_);
    check(cy_yashe_add(y_->handle(), device_data(), b.device_data(), c.mutable_device(), 1, nullptr), "cy_yashe_add");
    c.dev_written();
    c.level = level > b.level ? level : b.level;
    c.aftermul = aftermul || b.aftermul;
    return c;
}

// relinearisation: [sum_d D_d(c) evk_d]_q (Ciphertext::convert / keyswitch,
// src/ciphertext.cpp:75-107)
inline void Ciphertext::convert() {
    Ciphertext c(*y_);
    check(cy_yashe_keyswitch(y_->handle(), device_data(), c.mutable_device(), 1, nullptr), "cy_yashe_keyswitch");
    c.dev_written();
    const int lv = level;
    *this = std::move(c);
    level = lv;
    aftermul = false;
}

}  // namespace cuyashe
