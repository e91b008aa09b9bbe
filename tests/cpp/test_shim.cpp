// test_shim.cpp -- the reference's PolySuite / YasheSuite cases (src/test.cu)
// written against the C++ API of cuyashe.hpp.
//
// Every GPU result is compared with host arithmetic on cuyashe::ZZ: sums and
// scalar products coefficient by coefficient, ring products by a negacyclic
// schoolbook product, decryptions with the plaintext computed in R_t. The
// YASHE cases check every coefficient (the reference's encrypt*/decrypt tests
// look at coefficient 0 only). Exit status = number of failed cases.
#include <cstdio>
#include <functional>
#include <string>
#include <vector>

#include "cuyashe.hpp"

using cuyashe::Ciphertext;
using cuyashe::Context;
using cuyashe::Polynomial;
using cuyashe::Yashe;
using cuyashe::ZZ;

namespace {

int failures = 0;
const int NTESTS = 10;  // src/test.cu:15

struct Fail {
    std::string what;
};

#define REQUIRE(cond)                                                              \
    do {                                                                           \
        if (!(cond)) throw Fail{std::string(#cond) + " at line " + std::to_string(__LINE__)}; \
    } while (0)

void run(const char* name, const std::function<void()>& body) {
    try {
        body();
        std::printf("ok   %s\n", name);
    } catch (const Fail& f) {
        failures++;
        std::printf("FAIL %s: %s\n", name, f.what.c_str());
    } catch (const std::exception& e) {
        failures++;
        std::printf("FAIL %s: exception %s\n", name, e.what());
    }
    std::fflush(stdout);
}

// deterministic test stream (splitmix64)
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed) {}
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        return z ^ (z >> 31);
    }
    ZZ below(const ZZ& m) {
        ZZ v;
        for (int i = 0; i < m.bits() / 64 + 2; i++) v = v.shl(64) + ZZ(next());
        return v % m;
    }
};

Polynomial random_poly(const Context& ctx, Rng& rng, int degree = -1) {
    Polynomial p(ctx);
    const int d = degree < 0 ? ctx.n() - 1 : degree;
    for (int i = 0; i <= d; i++) p.set_coeff(i, rng.below(ctx.q()));
    return p;
}

// [a*b mod x^N+1]_q on the host
std::vector<ZZ> schoolbook(const std::vector<ZZ>& a, const std::vector<ZZ>& b, const ZZ& q) {
    const int n = (int)a.size();
    std::vector<ZZ> pos(n), neg(n);
    for (int i = 0; i < n; i++) {
        if (a[i].is_zero()) continue;
        for (int j = 0; j < n; j++) {
            const ZZ p = a[i] * b[j];
            if (i + j < n)
                pos[i + j] = pos[i + j] + p;
            else
                neg[i + j - n] = neg[i + j - n] + p;
        }
    }
    std::vector<ZZ> c(n);
    for (int k = 0; k < n; k++) c[k] = (pos[k] % q + q - neg[k] % q) % q;
    return c;
}

void poly_suite() {
    // PolySuite: N = 8, the 96-bit modulus, srand(36251) (src/test.cu:39-63)
    const ZZ q = ZZ::from_dec("77287149995192912462927307869");
    Context ctx(8, q);
    Rng rng(36251);

    run("PolySuite/simpleAdd", [&] {
        Polynomial a = random_poly(ctx, rng), b = random_poly(ctx, rng);
        Polynomial c = a + b;
        for (int i = 0; i < ctx.n(); i++) REQUIRE(c.get_coeff(i) == (a.get_coeff(i) + b.get_coeff(i)) % q);
    });
    run("PolySuite/multipleAdds", [&] {
        Polynomial a = random_poly(ctx, rng), b(ctx);
        for (int count = 0; count < NTESTS; count++) b += a;
        REQUIRE(b == a * ZZ(NTESTS));
        for (int i = 0; i < ctx.n(); i++) REQUIRE(b.get_coeff(i) == a.get_coeff(i) * ZZ(NTESTS) % q);
    });
    run("PolySuite/multipleAddsWithDifferentDegrees", [&] {
        Polynomial b(ctx);
        std::vector<ZZ> want(ctx.n());
        for (int count = 0; count < NTESTS; count++) {
            Polynomial a = random_poly(ctx, rng, (int)(rng.next() % ctx.n()));
            b += a;
            for (int i = 0; i < ctx.n(); i++) want[i] = (want[i] + a.get_coeff(i)) % q;
        }
        REQUIRE(b.get_coeffs() == want);
    });
    run("PolySuite/zeroAdd", [&] {
        Polynomial a = random_poly(ctx, rng), z(ctx);
        REQUIRE(a + z == a);
        REQUIRE(z + a == a);
    });
    run("PolySuite/subtract", [&] {
        Polynomial a = random_poly(ctx, rng), b = random_poly(ctx, rng);
        Polynomial c = a - b;
        for (int i = 0; i < ctx.n(); i++) REQUIRE(c.get_coeff(i) == (a.get_coeff(i) + q - b.get_coeff(i)) % q);
        REQUIRE(c + b == a);
    });
    run("PolySuite/getDegreeHost", [&] {
        for (int i = 0; i < NTESTS; i++) {
            const int degree = (int)(rng.next() % ctx.n());
            Polynomial a = random_poly(ctx, rng, degree);
            a.set_coeff(degree, ZZ(1 + rng.next() % 1000));
            REQUIRE(a.deg() == degree);
        }
        REQUIRE(Polynomial(ctx).deg() == -1);
    });
    run("PolySuite/multiplyByZZOnGPU", [&] {
        for (int count = 0; count < NTESTS; count++) {
            Polynomial a = random_poly(ctx, rng);
            const ZZ s = rng.below(q);
            Polynomial c = a * s;
            for (int i = 0; i < ctx.n(); i++) REQUIRE(c.get_coeff(i) == a.get_coeff(i) * s % q);
        }
    });
    run("PolySuite/simpleMultiplyByPolynomial", [&] {
        // (1 + x) * x^(N-1) = x^(N-1) - 1 in Z_q[x]/(x^N+1)
        Polynomial a(ctx), b(ctx);
        a.set_coeff(0, 1);
        a.set_coeff(1, 1);
        b.set_coeff(ctx.n() - 1, 1);
        Polynomial c = a * b;
        c.reduce();
        REQUIRE(c.get_coeff(0) == q - ZZ(1));
        REQUIRE(c.get_coeff(ctx.n() - 1) == ZZ(1));
        for (int i = 1; i < ctx.n() - 1; i++) REQUIRE(c.get_coeff(i).is_zero());
    });
    run("PolySuite/multiplyByPolynomial", [&] {
        for (int count = 0; count < NTESTS; count++) {
            Polynomial a = random_poly(ctx, rng), b = random_poly(ctx, rng);
            Polynomial c = a * b;
            REQUIRE(c.get_coeffs() == schoolbook(a.get_coeffs(), b.get_coeffs(), q));
        }
    });
    run("PolySuite/severalMultiplications", [&] {
        Polynomial a = random_poly(ctx, rng);
        std::vector<ZZ> want = a.get_coeffs();
        Polynomial acc = a;
        for (int count = 0; count < NTESTS; count++) {
            Polynomial b = random_poly(ctx, rng);
            acc = acc * b;
            want = schoolbook(want, b.get_coeffs(), q);
        }
        REQUIRE(acc.get_coeffs() == want);
    });
    run("PolySuite/phiReduceGPU", [&] {
        // products are reduced by x^N+1 and q: a*b equals the schoolbook
        // product and reduce() leaves it unchanged
        Polynomial a = random_poly(ctx, rng), b = random_poly(ctx, rng);
        Polynomial c = a * b, d = c;
        d.reduce();
        REQUIRE(c == d);
        REQUIRE(c.deg() < ctx.n());
    });
    run("PolySuite/differentRingsRejected", [&] {
        Context other(16, q);
        Polynomial a = random_poly(ctx, rng), b = random_poly(other, rng);
        bool threw = false;
        try {
            Polynomial c = a * b;
        } catch (const cuyashe::Error& e) {
            threw = e.status == CY_ERR_INVALID_ARGUMENT;
        }
        REQUIRE(threw);
    });

    // the benchmark ring: N = 1024, q = 2^127 - 1 (src/benchmark_polynomial.cpp)
    const ZZ q127 = ZZ::pow2(127) - ZZ(1);
    Context big(1024, q127);
    run("PolySuite/multiplyByPolynomialN1024Q127", [&] {
        Polynomial a = random_poly(big, rng), b = random_poly(big, rng);
        Polynomial c = a * b;
        REQUIRE(c.get_coeffs() == schoolbook(a.get_coeffs(), b.get_coeffs(), q127));
        REQUIRE(a * b == b * a);
    });
}

void yashe_case(const char* suite, int n, const ZZ& q, uint64_t t, uint64_t seed, bool depth2) {
    Yashe cipher(n, q, t);
    cipher.generate_keys(seed);
    const Context& pt = cipher.plaintext_context();
    Rng rng(seed);
    auto plain = [&] { return random_poly(pt, rng); };
    auto name = [&](const char* c) { return std::string(suite) + "/" + c; };

    run(name("encryptDecrypt").c_str(), [&] {
        for (int i = 0; i < NTESTS; i++) {
            Polynomial a = plain();
            Ciphertext c = cipher.encrypt(a, rng.next());
            REQUIRE(cipher.decrypt(c) == a);
        }
    });
    run(name("encryptandAdd").c_str(), [&] {
        for (int i = 0; i < NTESTS; i++) {
            Polynomial a = plain();
            Ciphertext c = cipher.encrypt(a, rng.next());
            c = c + c;
            REQUIRE(cipher.decrypt(c) == (a + a));
        }
    });
    run(name("encryptandMul").c_str(), [&] {
        for (int i = 0; i < NTESTS; i++) {
            Polynomial a = plain(), b = plain();
            Ciphertext c1 = cipher.encrypt(a, rng.next());
            Ciphertext c2 = cipher.encrypt(b, rng.next());
            Ciphertext c = c1 * c2;
            REQUIRE(c.aftermul);
            Polynomial want = a * b;  // in R_t
            REQUIRE(want.get_coeffs() == schoolbook(a.get_coeffs(), b.get_coeffs(), ZZ(t)));
            REQUIRE(cipher.decrypt(c) == want);
            c.convert();  // relinearise: decrypts with f again
            REQUIRE(!c.aftermul);
            REQUIRE(cipher.decrypt(c) == want);
        }
    });
    if (depth2) run(name("encryptandMulDepth2").c_str(), [&] {
        Polynomial a = plain(), b = plain(), d = plain();
        Ciphertext c1 = cipher.encrypt(a, rng.next());
        Ciphertext c2 = cipher.encrypt(b, rng.next());
        Ciphertext c3 = cipher.encrypt(d, rng.next());
        Ciphertext c12 = c1 * c2;
        Ciphertext c = c12 * c3;  // relinearises c12 first
        REQUIRE(!c12.aftermul);
        REQUIRE(c.level == 2);
        REQUIRE(cipher.decrypt(c) == (a * b) * d);
    });
    run(name("encryptandAddPlain").c_str(), [&] {
        Polynomial a = plain(), b = plain();
        Ciphertext c = cipher.encrypt(a, rng.next());
        REQUIRE(cipher.decrypt(c + b) == (a + b));
    });
    run(name("encryptandMulPlain").c_str(), [&] {
        Polynomial a = plain(), b = plain();
        Ciphertext c = cipher.encrypt(a, rng.next());
        REQUIRE(cipher.decrypt(c * b) == (a * b));
    });
    run(name("encryptRejectsLargeCoefficients").c_str(), [&] {
        Polynomial a(cipher.context());
        a.set_coeff(0, ZZ(t));
        bool threw = false;
        try {
            cipher.encrypt(a);
        } catch (const cuyashe::Error& e) {
            threw = e.status == CY_ERR_INVALID_ARGUMENT;
        }
        REQUIRE(threw);
    });
}

}  // namespace

int main() {
    try {
        poly_suite();
        // YasheSuite: N = 4, t = 35951, the 96-bit modulus (src/test.cu:73-133).
        // Depth 1 only: after two products the noise is about 2^88 against
        // q/t = 2^81, so no implementation decrypts a depth-2 product here.
        yashe_case("YasheSuite", 4, ZZ::from_dec("77287149995192912462927307869"), 35951, 36251, false);
        // the HE multiply benchmark's modulus (the largest prime below 2^127 that
        // is 1 mod 2^16) and t = 1024, at N = 1024
        yashe_case("YasheN1024", 1024, ZZ::from_dec("170141183460469231731687303715883253761"), 1024, 7, true);
    } catch (const std::exception& e) {
        std::printf("FAIL setup: %s\n", e.what());
        return 100;
    }
    std::printf("%d failure(s)\n", failures);
    return failures;
}
