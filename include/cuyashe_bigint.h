// cuyashe_bigint.h -- small arbitrary-precision unsigned integer (host only).
//
// The reference keeps every wide value in NTL::ZZ on the host (src/polynomial.h,
// src/integer.h) and in its own bn_t on the device (src/cuda_bn.h:18-23). Here
// host-side wide arithmetic is needed for set-up (CRT products M, M/p_i, their
// residues mod q, Barrett constants, keygen) and as the coefficient type of the
// C++ API in cuyashe.hpp. Little-endian 32-bit words, schoolbook multiplication
// and Knuth's algorithm D for division.
#pragma once

#include <stdint.h>

#include <algorithm>
#include <string>
#include <vector>

namespace cy {

struct BigUInt {
    std::vector<uint32_t> w;  // little endian, no leading zero words

    BigUInt() {}
    BigUInt(uint64_t v) {  // NOLINT(google-explicit-constructor)
        if (v) w.push_back((uint32_t)v);
        if (v >> 32) w.push_back((uint32_t)(v >> 32));
    }
    static BigUInt from_limbs64(const uint64_t* p, int n) {
        BigUInt r;
        r.w.resize(2 * (size_t)n);
        for (int i = 0; i < n; i++) {
            r.w[2 * i] = (uint32_t)p[i];
            r.w[2 * i + 1] = (uint32_t)(p[i] >> 32);
        }
        r.trim();
        return r;
    }
    void to_limbs64(uint64_t* p, int n) const {
        for (int i = 0; i < n; i++) {
            uint64_t lo = (size_t)(2 * i) < w.size() ? w[2 * i] : 0;
            uint64_t hi = (size_t)(2 * i + 1) < w.size() ? w[2 * i + 1] : 0;
            p[i] = lo | (hi << 32);
        }
    }
    void to_words32(uint32_t* p, int n) const {
        for (int i = 0; i < n; i++) p[i] = (size_t)i < w.size() ? w[i] : 0;
    }
    uint64_t low64() const {
        uint64_t lo = w.size() > 0 ? w[0] : 0, hi = w.size() > 1 ? w[1] : 0;
        return lo | (hi << 32);
    }
    void trim() {
        while (!w.empty() && w.back() == 0) w.pop_back();
    }
    bool is_zero() const { return w.empty(); }
    int bits() const {
        if (w.empty()) return 0;
        return 32 * (int)(w.size() - 1) + (32 - __builtin_clz(w.back()));
    }
    bool bit(int i) const {
        size_t k = (size_t)i / 32;
        return k < w.size() && ((w[k] >> (i % 32)) & 1);
    }

    static int cmp(const BigUInt& a, const BigUInt& b) {
        if (a.w.size() != b.w.size()) return a.w.size() < b.w.size() ? -1 : 1;
        for (size_t i = a.w.size(); i-- > 0;)
            if (a.w[i] != b.w[i]) return a.w[i] < b.w[i] ? -1 : 1;
        return 0;
    }
    friend bool operator<(const BigUInt& a, const BigUInt& b) { return cmp(a, b) < 0; }
    friend bool operator<=(const BigUInt& a, const BigUInt& b) { return cmp(a, b) <= 0; }
    friend bool operator>(const BigUInt& a, const BigUInt& b) { return cmp(a, b) > 0; }
    friend bool operator>=(const BigUInt& a, const BigUInt& b) { return cmp(a, b) >= 0; }
    friend bool operator==(const BigUInt& a, const BigUInt& b) { return cmp(a, b) == 0; }
    friend bool operator!=(const BigUInt& a, const BigUInt& b) { return cmp(a, b) != 0; }

    friend BigUInt operator+(const BigUInt& a, const BigUInt& b) {
        BigUInt r;
        size_t n = std::max(a.w.size(), b.w.size());
        r.w.resize(n + 1);
        uint64_t c = 0;
        for (size_t i = 0; i < n; i++) {
            c += (uint64_t)(i < a.w.size() ? a.w[i] : 0) + (i < b.w.size() ? b.w[i] : 0);
            r.w[i] = (uint32_t)c;
            c >>= 32;
        }
        r.w[n] = (uint32_t)c;
        r.trim();
        return r;
    }
    // requires a >= b
    friend BigUInt operator-(const BigUInt& a, const BigUInt& b) {
        BigUInt r;
        r.w.resize(a.w.size());
        int64_t br = 0;
        for (size_t i = 0; i < a.w.size(); i++) {
            int64_t d = (int64_t)a.w[i] - (i < b.w.size() ? b.w[i] : 0) - br;
            br = d < 0;
            r.w[i] = (uint32_t)(d + (br << 32));
        }
        r.trim();
        return r;
    }
    friend BigUInt operator*(const BigUInt& a, const BigUInt& b) {
        BigUInt r;
        if (a.is_zero() || b.is_zero()) return r;
        r.w.assign(a.w.size() + b.w.size(), 0);
        for (size_t i = 0; i < a.w.size(); i++) {
            uint64_t c = 0;
            for (size_t j = 0; j < b.w.size(); j++) {
                c += (uint64_t)a.w[i] * b.w[j] + r.w[i + j];
                r.w[i + j] = (uint32_t)c;
                c >>= 32;
            }
            r.w[i + b.w.size()] = (uint32_t)c;
        }
        r.trim();
        return r;
    }
    BigUInt shl(int s) const {
        if (is_zero()) return *this;
        BigUInt r;
        int ws = s / 32, bs = s % 32;
        r.w.assign(w.size() + ws + 1, 0);
        for (size_t i = 0; i < w.size(); i++) {
            uint64_t v = (uint64_t)w[i] << bs;
            r.w[i + ws] |= (uint32_t)v;
            r.w[i + ws + 1] |= (uint32_t)(v >> 32);
        }
        r.trim();
        return r;
    }
    BigUInt shr(int s) const {
        int ws = s / 32, bs = s % 32;
        if ((size_t)ws >= w.size()) return BigUInt();
        BigUInt r;
        r.w.assign(w.size() - ws, 0);
        for (size_t i = 0; i < r.w.size(); i++) {
            uint64_t lo = w[i + ws];
            uint64_t hi = (i + ws + 1) < w.size() ? w[i + ws + 1] : 0;
            r.w[i] = (uint32_t)(((hi << 32) | lo) >> bs);
        }
        r.trim();
        return r;
    }
    static BigUInt pow2(int e) { return BigUInt(1).shl(e); }

    uint32_t mod_u32(uint32_t m) const {
        uint64_t r = 0;
        for (size_t i = w.size(); i-- > 0;) r = ((r << 32) | w[i]) % m;
        return (uint32_t)r;
    }

    // Knuth algorithm D: q = a / b, r = a % b (b != 0).
    static void divmod(const BigUInt& a, const BigUInt& b, BigUInt* q, BigUInt* r) {
        if (cmp(a, b) < 0) {
            if (q) *q = BigUInt();
            if (r) *r = a;
            return;
        }
        size_t n = b.w.size(), m = a.w.size() - n;
        if (n == 1) {
            BigUInt qq;
            qq.w.assign(a.w.size(), 0);
            uint64_t rem = 0;
            for (size_t i = a.w.size(); i-- > 0;) {
                uint64_t cur = (rem << 32) | a.w[i];
                qq.w[i] = (uint32_t)(cur / b.w[0]);
                rem = cur % b.w[0];
            }
            qq.trim();
            if (q) *q = qq;
            if (r) *r = BigUInt(rem);
            return;
        }
        int s = __builtin_clz(b.w.back());
        std::vector<uint32_t> vn(n), un(a.w.size() + 1);
        for (size_t i = n - 1; i > 0; i--)
            vn[i] = (b.w[i] << s) | (s ? (uint32_t)((uint64_t)b.w[i - 1] >> (32 - s)) : 0);
        vn[0] = b.w[0] << s;
        un[a.w.size()] = s ? (uint32_t)((uint64_t)a.w.back() >> (32 - s)) : 0;
        for (size_t i = a.w.size() - 1; i > 0; i--)
            un[i] = (a.w[i] << s) | (s ? (uint32_t)((uint64_t)a.w[i - 1] >> (32 - s)) : 0);
        un[0] = a.w[0] << s;
        BigUInt qq;
        qq.w.assign(m + 1, 0);
        for (size_t jj = m + 1; jj-- > 0;) {
            size_t j = jj;
            uint64_t num = ((uint64_t)un[j + n] << 32) | un[j + n - 1];
            uint64_t qhat = num / vn[n - 1], rhat = num % vn[n - 1];
            while (qhat >= (1ULL << 32) || qhat * vn[n - 2] > ((rhat << 32) | un[j + n - 2])) {
                qhat--;
                rhat += vn[n - 1];
                if (rhat >= (1ULL << 32)) break;
            }
            int64_t t = 0, k = 0;
            for (size_t i = 0; i < n; i++) {
                uint64_t p = qhat * vn[i];
                t = (int64_t)un[i + j] - k - (int64_t)(p & 0xFFFFFFFFULL);
                un[i + j] = (uint32_t)t;
                k = (int64_t)(p >> 32) - (t >> 32);
            }
            t = (int64_t)un[j + n] - k;
            un[j + n] = (uint32_t)t;
            if (t < 0) {
                qhat--;
                uint64_t c = 0;
                for (size_t i = 0; i < n; i++) {
                    c += (uint64_t)un[i + j] + vn[i];
                    un[i + j] = (uint32_t)c;
                    c >>= 32;
                }
                un[j + n] += (uint32_t)c;
            }
            qq.w[j] = (uint32_t)qhat;
        }
        qq.trim();
        if (q) *q = qq;
        if (r) {
            BigUInt rr;
            rr.w.assign(n, 0);
            for (size_t i = 0; i < n; i++)
                rr.w[i] = (un[i] >> s) | (s ? (uint32_t)((uint64_t)un[i + 1] << (32 - s)) : 0);
            rr.trim();
            *r = rr;
        }
    }
    friend BigUInt operator/(const BigUInt& a, const BigUInt& b) {
        BigUInt q;
        divmod(a, b, &q, nullptr);
        return q;
    }
    friend BigUInt operator%(const BigUInt& a, const BigUInt& b) {
        BigUInt r;
        divmod(a, b, nullptr, &r);
        return r;
    }

    static BigUInt powmod(BigUInt b, BigUInt e, const BigUInt& m) {
        BigUInt r(1);
        r = r % m;
        b = b % m;
        int nb = e.bits();
        for (int i = nb - 1; i >= 0; i--) {
            r = (r * r) % m;
            if (e.bit(i)) r = (r * b) % m;
        }
        return r;
    }

    static BigUInt from_dec(const char* s) {
        BigUInt r;
        for (; *s; s++)
            if (*s >= '0' && *s <= '9') r = r * BigUInt(10u) + BigUInt((uint64_t)(*s - '0'));
        return r;
    }

    std::string to_dec() const {
        if (is_zero()) return "0";
        std::string s;
        BigUInt x = *this;
        while (!x.is_zero()) {
            BigUInt q;
            BigUInt r;
            divmod(x, BigUInt(1000000000u), &q, &r);
            uint32_t d = r.is_zero() ? 0 : r.w[0];
            for (int i = 0; i < 9; i++) {
                s.push_back((char)('0' + d % 10));
                d /= 10;
            }
            x = q;
        }
        while (s.size() > 1 && s.back() == '0') s.pop_back();
        std::reverse(s.begin(), s.end());
        return s;
    }
};

}  // namespace cy
