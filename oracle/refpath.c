/*
 * refpath.c -- C restatement of the reference's own polynomial multiply
 * (test infrastructure and the timed CPU baseline; never linked into the product).
 *
 * The reference (cuYASHE) multiplies in Z_q[x]/(x^N+1) as follows; each step
 * below cites the file:line it restates.
 *
 *  1. CRT basis: primes are taken in order from PRIMES_BUCKET (the 100 largest
 *     primes below 2^29, src/polynomial.cpp:22) until M >= 2*degree*q^2
 *     (Polynomial::gen_crt_primes, src/polynomial.h:898-955). M/p_i and
 *     (M/p_i)^-1 mod p_i are kept (lines 930-935).
 *  2. CRT split: x mod p_i with bn_mod1_low (src/cuda_bn.cu:290-317), which walks
 *     the 64-bit words from the top in 32-bit halves. Its quirk is kept: when
 *     the upper half of a word is zero the running remainder is not shifted
 *     (line 301), which differs from x mod p only for multi-word x with a zero
 *     upper half below a non-zero word.
 *  3. Cyclic NTT of length n = 2^ceil(log2(deg a + deg b)) (src/common.h:139)
 *     over the Goldilocks prime P = 2^64 - 2^32 + 1 with root 7
 *     (src/cuda_functions.cu:18-19): W[j] = w^j, WInv[j] = w^-j with
 *     w = 7^((P-1)/n) (CUDAFunctions::init, lines 878-930).
 *     Radix-2 Stockham stages (NTTIteration / NTT / expand, lines 385-445),
 *     forward on both operands, pointwise s_mul (polynomialNTTMul, 460-474),
 *     inverse stages with WInv, then NTTScale: integer division by n
 *     (lines 397-402), exact only while n*c < P for every convolution value c.
 *  4. ICRT: x = sum_i M/p_i * [x_i * (M/p_i)^-1]_{p_i} mod M
 *     (cuPreICRT / cuICRT, src/cuda_bn.cu:854-968). The reference reduces with
 *     Barrett (bn_mod_barrt); the restatement reduces exactly.
 *  5. reduce(): c_i -= c_{i+N}, then %= q (non-negative), host loop
 *     src/cuda_functions.cu:1061-1076.
 *
 * The reference's own YASHE multiply (src/ciphertext.cpp:38-73) and keyswitch
 * (81-130) are defective by reading; rp_yashe_mul restates the intended
 * computation on top of steps 1-5 for timing: tensor over Z (fold without the
 * mod q), x t, round(./q), mod q, then base-2^w digits times gamma_d through
 * the same multiply, summed, folded and reduced mod q.
 *
 * Build: make -C oracle (gcc -O3 -fopenmp, portable C, no intrinsics).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef unsigned __int128 u128;

#define RP_P 0xFFFFFFFF00000001ULL
#define RP_ROOT 7ULL
#define RP_MAXW 40 /* 64-bit words of the widest intermediate (2560 bits) */

/* ------------------------------------------------------------------------ */
/* Goldilocks arithmetic (src/cuda_functions.cu:276-391)                     */
/* ------------------------------------------------------------------------ */

/* s_rem (lines 282-308): one conditional subtraction of P. */
static inline uint64_t s_rem(uint64_t a) {
    uint64_t x1 = a >> 32, x0 = a & 0xFFFFFFFFULL;
    uint64_t res = (x1 << 32) + x0;
    if (res >= RP_P) res -= RP_P;
    return res;
}

/* s_mul host branch (line 351): 128-bit product reduced with %. */
uint64_t rp_s_mul(uint64_t a, uint64_t b) { return (uint64_t)(((u128)a * (u128)b) % RP_P); }

static inline int ovf(uint64_t a, uint64_t b) { return (a + b) < a; }

/* s_mul device branch (lines 310-349): 2^96 = -1 and 2^64 = 2^32 - 1 (mod P)
 * with the reference's three-case branch-free fix-up. */
uint64_t rp_s_mul_device_formula(uint64_t a, uint64_t b) {
    const uint64_t GAP = (UINT64_MAX - RP_P + 1);
    u128 c = (u128)a * (u128)b;
    uint64_t cHi = (uint64_t)(c >> 64), cLo = (uint64_t)c;
    uint64_t x3 = cHi >> 32, x2 = cHi & 0xFFFFFFFFULL, x1 = cLo >> 32, x0 = cLo & 0xFFFFFFFFULL;
    uint64_t X1 = x1 << 32, X2 = x2 << 32;
    uint64_t res = X1 + X2 + x0 - x2 - x3;
    int testA = (x2 + x3 > X1 + X2 + x0) && !(ovf(X1, X2) || ovf(X1 + X2, x0));
    int testB = (res >= RP_P);
    int testC = (ovf(X1, X2) || ovf(X1 + X2, x0)) && (X1 + X2 + x0 > x2 + x3);
    res = (RP_P - res) * (uint64_t)(testA) + (res - RP_P) * (uint64_t)(!testA && testB) +
          (res + GAP) * (uint64_t)(!testA && !testB && testC) + res * (uint64_t)(!testA && !testB && !testC);
    return res;
}

/* s_add / s_sub (lines 355-383). */
static inline uint64_t s_add(uint64_t a, uint64_t b) {
    uint64_t res = a + b;
    res += (uint64_t)(res < a) * 4294967295ULL;
    return s_rem(res);
}
static inline uint64_t s_sub(uint64_t a, uint64_t b) { return (a - b) + (uint64_t)(b > a) * RP_P; }

static uint64_t pow_p(uint64_t b, uint64_t e) {
    uint64_t r = 1;
    while (e) {
        if (e & 1) r = rp_s_mul(r, b);
        b = rp_s_mul(b, b);
        e >>= 1;
    }
    return r;
}

uint64_t rp_omega(int n) { return pow_p(RP_ROOT, (RP_P - 1) / (uint64_t)n); }

/* CUDAFunctions::init: W[j] = w^j, WInv[j] = (w^j)^-1. */
void rp_twiddles(int n, uint64_t *W, uint64_t *WInv) {
    uint64_t w = rp_omega(n), acc = 1;
    for (int j = 0; j < n; j++) {
        W[j] = acc;
        acc = rp_s_mul(acc, w);
    }
    WInv[0] = 1;
    for (int j = 1; j < n; j++) WInv[j] = W[n - j];
}

/* One Stockham radix-2 stage (NTTIteration + expand, lines 385-433) over one residue. */
static void ntt_stage(const uint64_t *W, int n, int Ns, const uint64_t *in, uint64_t *out) {
    const int R = 2;
    for (int j = 0; j < n / R; j++) {
        int w_index = ((j % Ns) * n) / (Ns * R);
        uint64_t v0 = rp_s_mul(in[j], W[0]);
        uint64_t v1 = rp_s_mul(in[j + n / R], W[w_index]);
        v0 = s_rem(v0);
        v1 = s_rem(v1);
        uint64_t b0 = s_add(v0, v1), b1 = s_sub(v0, v1);
        int idxD = (j / Ns) * Ns * R + (j % Ns);
        out[idxD] = b0;
        out[idxD + Ns] = b1;
    }
}

/* log2(n) stages ping-ponging between x and tmp; result left in x. */
static void ntt(const uint64_t *W, int n, uint64_t *x, uint64_t *tmp) {
    uint64_t *a = x, *b = tmp;
    for (int Ns = 1; Ns < n; Ns *= 2) {
        ntt_stage(W, n, Ns, a, b);
        uint64_t *s = a; a = b; b = s;
    }
    if (a != x) memcpy(x, a, sizeof(uint64_t) * (size_t)n);
}

/* ------------------------------------------------------------------------ */
/* bignum helpers (64-bit words, little endian)                              */
/* ------------------------------------------------------------------------ */

/* bn_mod1_low (src/cuda_bn.cu:290-317), quirk included. */
uint64_t rp_mod1_low(const uint64_t *a, int size, uint32_t b) {
    uint64_t w = 0;
    for (int i = size - 1; i >= 0; i--) {
        uint32_t hi = (uint32_t)(a[i] >> 32);
        if (hi > 0) w = (w << 32) | (uint64_t)hi;
        if (w >= b || hi > 0) w %= b;
        uint32_t lo = (uint32_t)(a[i] & 0xFFFFFFFFULL);
        w = (w << 32) | (uint64_t)lo;
        w %= b;
    }
    return w;
}

static int bn_used(const uint64_t *a, int n) {
    while (n > 0 && a[n - 1] == 0) n--;
    return n;
}

static int bn_cmp(const uint64_t *a, const uint64_t *b, int n) {
    for (int i = n - 1; i >= 0; i--) {
        if (a[i] != b[i]) return a[i] > b[i] ? 1 : -1;
    }
    return 0;
}

static uint64_t bn_sub_n(uint64_t *c, const uint64_t *a, const uint64_t *b, int n) {
    uint64_t borrow = 0;
    for (int i = 0; i < n; i++) {
        uint64_t d = a[i] - b[i];
        uint64_t b1 = a[i] < b[i];
        uint64_t d2 = d - borrow;
        uint64_t b2 = d < borrow;
        c[i] = d2;
        borrow = b1 | b2;
    }
    return borrow;
}

static uint64_t bn_add_n(uint64_t *c, const uint64_t *a, const uint64_t *b, int n) {
    u128 carry = 0;
    for (int i = 0; i < n; i++) {
        carry += (u128)a[i] + b[i];
        c[i] = (uint64_t)carry;
        carry >>= 64;
    }
    return (uint64_t)carry;
}

/* c[0..n] += a[0..n-1] * d (c has n+1 valid words) */
static void bn_mac1(uint64_t *c, const uint64_t *a, uint64_t d, int n) {
    u128 carry = 0;
    for (int i = 0; i < n; i++) {
        carry += (u128)a[i] * d + c[i];
        c[i] = (uint64_t)carry;
        carry >>= 64;
    }
    u128 s = (u128)c[n] + carry;
    c[n] = (uint64_t)s;
}

/* quot = floor(x / m), r = x mod m (Knuth algorithm D, 32-bit digits).
 * x has nx words, m has nm words (m != 0); quot (if not NULL) gets nx words. */
static void bn_divmod(uint64_t *quot, uint64_t *r, const uint64_t *x, int nx, const uint64_t *m, int nm) {
    uint32_t u[2 * RP_MAXW + 2], v[2 * RP_MAXW], qd[2 * RP_MAXW + 2];
    int n, mlen, nx0 = nx, nm0 = nm;
    nx = bn_used(x, nx);
    nm = bn_used(m, nm);
    for (int i = 0; i < nm; i++) { v[2 * i] = (uint32_t)m[i]; v[2 * i + 1] = (uint32_t)(m[i] >> 32); }
    n = 2 * nm;
    while (n > 0 && v[n - 1] == 0) n--;
    for (int i = 0; i < nx; i++) { u[2 * i] = (uint32_t)x[i]; u[2 * i + 1] = (uint32_t)(x[i] >> 32); }
    mlen = 2 * nx;
    while (mlen > 0 && u[mlen - 1] == 0) mlen--;
    memset(r, 0, sizeof(uint64_t) * (size_t)nm0);
    if (quot) memset(quot, 0, sizeof(uint64_t) * (size_t)nx0);
    memset(qd, 0, sizeof(qd));
    if (mlen < n) {
        for (int i = 0; i < mlen; i++) r[i / 2] |= (uint64_t)u[i] << (32 * (i % 2));
        return;
    }
    if (n == 1) {
        uint64_t rem = 0;
        for (int i = mlen - 1; i >= 0; i--) {
            uint64_t cur = (rem << 32) | u[i];
            qd[i] = (uint32_t)(cur / v[0]);
            rem = cur % v[0];
        }
        r[0] = rem;
    } else {
        int s = __builtin_clz(v[n - 1]);
        uint32_t vn[2 * RP_MAXW], un[2 * RP_MAXW + 2];
        for (int i = n - 1; i > 0; i--) vn[i] = (v[i] << s) | (s ? (uint32_t)((uint64_t)v[i - 1] >> (32 - s)) : 0);
        vn[0] = v[0] << s;
        un[mlen] = s ? (uint32_t)((uint64_t)u[mlen - 1] >> (32 - s)) : 0;
        for (int i = mlen - 1; i > 0; i--) un[i] = (u[i] << s) | (s ? (uint32_t)((uint64_t)u[i - 1] >> (32 - s)) : 0);
        un[0] = u[0] << s;
        for (int j = mlen - n; j >= 0; j--) {
            uint64_t num = ((uint64_t)un[j + n] << 32) | un[j + n - 1];
            uint64_t qhat = num / vn[n - 1], rhat = num % vn[n - 1];
            while (qhat >= (1ULL << 32) || qhat * vn[n - 2] > ((rhat << 32) | un[j + n - 2])) {
                qhat--;
                rhat += vn[n - 1];
                if (rhat >= (1ULL << 32)) break;
            }
            int64_t t = 0, k = 0;
            for (int i = 0; i < n; i++) {
                uint64_t p = qhat * vn[i];
                t = (int64_t)un[i + j] - k - (int64_t)(p & 0xFFFFFFFFULL);
                un[i + j] = (uint32_t)t;
                k = (int64_t)(p >> 32) - (t >> 32);
            }
            t = (int64_t)un[j + n] - k;
            un[j + n] = (uint32_t)t;
            if (t < 0) {
                qhat--;
                uint64_t cc = 0;
                for (int i = 0; i < n; i++) {
                    cc += (uint64_t)un[i + j] + vn[i];
                    un[i + j] = (uint32_t)cc;
                    cc >>= 32;
                }
                un[j + n] += (uint32_t)cc;
            }
            qd[j] = (uint32_t)qhat;
        }
        for (int i = 0; i < n; i++) {
            uint32_t d = (un[i] >> s) | (s ? (uint32_t)((uint64_t)un[i + 1] << (32 - s)) : 0);
            r[i / 2] |= (uint64_t)d << (32 * (i % 2));
        }
    }
    if (quot)
        for (int i = 0; i < mlen && i / 2 < nx0; i++) quot[i / 2] |= (uint64_t)qd[i] << (32 * (i % 2));
}

static void bn_mod(uint64_t *r, const uint64_t *x, int nx, const uint64_t *m, int nm) {
    bn_divmod(NULL, r, x, nx, m, nm);
}

/* ------------------------------------------------------------------------ */
/* context: CRT basis (gen_crt_primes) and constants                         */
/* ------------------------------------------------------------------------ */

static int is_prime_u32(uint32_t n) {
    if (n < 2) return 0;
    for (uint32_t d = 2; (uint64_t)d * d <= n; d++)
        if (n % d == 0) return 0;
    return 1;
}

typedef struct rp_ctx {
    int k;                   /* number of CRT primes */
    uint32_t p[128];
    uint64_t invMpi[128];    /* (M/p_i)^-1 mod p_i */
    uint64_t *Mpi;           /* [k][mw] */
    uint64_t M[RP_MAXW];
    int mw;                  /* words of M (+1 slack) */
    uint64_t q[RP_MAXW];
    int qw;
} rp_ctx;

void rp_bucket(uint32_t *out, int count) {
    uint32_t n = (1u << 29) - 1;
    int c = 0;
    while (c < count) {
        if (is_prime_u32(n)) out[c++] = n;
        n--;
    }
}

static uint64_t inv_mod_u64(uint64_t a, uint64_t m) {
    int64_t t = 0, nt = 1;
    int64_t r = (int64_t)m, nr = (int64_t)(a % m);
    while (nr) {
        int64_t qq = r / nr, tmp;
        tmp = t - qq * nt; t = nt; nt = tmp;
        tmp = r - qq * nr; r = nr; nr = tmp;
    }
    if (t < 0) t += (int64_t)m;
    return (uint64_t)t;
}

/* gen_crt_primes(q, degree): primes until M >= 2*degree*q^2. */
rp_ctx *rp_create(const uint64_t *q, int qw, int degree) {
    rp_ctx *c = (rp_ctx *)calloc(1, sizeof(rp_ctx));
    uint32_t bucket[128];
    rp_bucket(bucket, 100);
    qw = bn_used(q, qw);
    memcpy(c->q, q, sizeof(uint64_t) * (size_t)qw);
    c->qw = qw;
    /* bound = 2*degree*q*q */
    uint64_t bound[RP_MAXW] = {0};
    uint64_t qq[RP_MAXW] = {0};
    for (int i = 0; i < qw; i++) bn_mac1(qq + i, q, q[i], qw);
    bn_mac1(bound, qq, (uint64_t)(2 * degree), 2 * qw);
    uint64_t M[RP_MAXW] = {0};
    M[0] = 1;
    int k = 0;
    while (bn_cmp(M, bound, RP_MAXW) < 0 && k < 100) {
        uint64_t nm[RP_MAXW] = {0};
        bn_mac1(nm, M, bucket[k], RP_MAXW - 1);
        memcpy(M, nm, sizeof(M));
        c->p[k] = bucket[k];
        k++;
    }
    c->k = k;
    memcpy(c->M, M, sizeof(M));
    c->mw = bn_used(M, RP_MAXW) + 1;
    c->Mpi = (uint64_t *)calloc((size_t)k * (size_t)c->mw, sizeof(uint64_t));
    for (int i = 0; i < k; i++) {
        /* M/p_i = product of the other primes */
        uint64_t acc[RP_MAXW] = {0};
        acc[0] = 1;
        for (int j = 0; j < k; j++) {
            if (j == i) continue;
            uint64_t nm[RP_MAXW] = {0};
            bn_mac1(nm, acc, c->p[j], RP_MAXW - 1);
            memcpy(acc, nm, sizeof(acc));
        }
        memcpy(c->Mpi + (size_t)i * c->mw, acc, sizeof(uint64_t) * (size_t)c->mw);
        uint64_t r = rp_mod1_low(acc, c->mw, c->p[i]);
        c->invMpi[i] = inv_mod_u64(r, c->p[i]);
    }
    return c;
}

void rp_destroy(rp_ctx *c) {
    if (!c) return;
    free(c->Mpi);
    free(c);
}

int rp_nprimes(const rp_ctx *c) { return c->k; }
void rp_primes(const rp_ctx *c, uint64_t *out) { for (int i = 0; i < c->k; i++) out[i] = c->p[i]; }
int rp_mwords(const rp_ctx *c) { return c->mw; }

/* ------------------------------------------------------------------------ */
/* multiply: operator* (CRT -> NTT -> pointwise -> INTT -> NTTScale -> ICRT)  */
/* ------------------------------------------------------------------------ */

static int spacing_for(int na, int nb) {
    int degs = (na - 1) + (nb - 1);
    int n = 1;
    while (n < degs) n <<= 1;
    if (n < 2) n = 2;
    return n;
}

/* Product over Z of one pair: out[n][mw] = a*b mod M for coefficients 0..n-1. */
static void mul_plain_one(const rp_ctx *c, const uint64_t *W, const uint64_t *WInv, int n,
                          const uint64_t *a, int na, int la, const uint64_t *b, int nb, int lb,
                          uint64_t *out, int inner_threads) {
    const int k = c->k, mw = c->mw;
    uint64_t *res = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)k * (size_t)n);
    (void)inner_threads;
#pragma omp parallel for schedule(static) num_threads(inner_threads) if (inner_threads > 1)
    for (int i = 0; i < k; i++) {
        uint64_t *da = (uint64_t *)calloc((size_t)n, sizeof(uint64_t));
        uint64_t *db = (uint64_t *)calloc((size_t)n, sizeof(uint64_t));
        uint64_t *tmp = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)n);
        for (int j = 0; j < na; j++) da[j] = rp_mod1_low(a + (size_t)j * la, la, c->p[i]);
        for (int j = 0; j < nb; j++) db[j] = rp_mod1_low(b + (size_t)j * lb, lb, c->p[i]);
        ntt(W, n, da, tmp);
        ntt(W, n, db, tmp);
        for (int j = 0; j < n; j++) da[j] = rp_s_mul(da[j], db[j]);
        ntt(WInv, n, da, tmp);
        for (int j = 0; j < n; j++) res[(size_t)i * n + j] = da[j] / (uint64_t)n; /* NTTScale */
        free(da); free(db); free(tmp);
    }
#pragma omp parallel for schedule(static) num_threads(inner_threads) if (inner_threads > 1)
    for (int j = 0; j < n; j++) {
        uint64_t acc[RP_MAXW] = {0};
        for (int i = 0; i < k; i++) {
            uint64_t x = (uint64_t)(((u128)(res[(size_t)i * n + j] % c->p[i]) * c->invMpi[i]) % c->p[i]);
            bn_mac1(acc, c->Mpi + (size_t)i * mw, x, mw - 1);
        }
        /* mod M: subtract M while acc >= M (acc < k*M) */
        uint64_t Mext[RP_MAXW] = {0};
        memcpy(Mext, c->M, sizeof(uint64_t) * (size_t)mw);
        if (bn_cmp(acc, Mext, mw) >= 0) {
            uint64_t r[RP_MAXW] = {0};
            bn_mod(r, acc, mw, Mext, mw);
            memset(acc, 0, sizeof(acc));
            memcpy(acc, r, sizeof(uint64_t) * (size_t)mw);
        }
        memcpy(out + (size_t)j * mw, acc, sizeof(uint64_t) * (size_t)mw);
    }
    free(res);
}

/* operator*: returns the spacing n; out holds n coefficients of mw words (mod M). */
int rp_mul_plain(const rp_ctx *c, const uint64_t *a, int na, int la, const uint64_t *b, int nb, int lb,
                 uint64_t *out) {
    int n = spacing_for(na, nb);
    uint64_t *W = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)n);
    uint64_t *WInv = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)n);
    rp_twiddles(n, W, WInv);
    mul_plain_one(c, W, WInv, n, a, na, la, b, nb, lb, out, 1);
    free(W); free(WInv);
    return n;
}

/* reduce(): fold by x^N+1, then % q. prod holds 2N coefficients (mw words each). */
static void reduce_fold_modq(const rp_ctx *c, const uint64_t *prod, int N, uint64_t *out) {
    const int mw = c->mw, qw = c->qw;
    for (int j = 0; j < N; j++) {
        uint64_t lo[RP_MAXW] = {0}, hi[RP_MAXW] = {0};
        bn_mod(lo, prod + (size_t)j * mw, mw, c->q, qw);
        bn_mod(hi, prod + (size_t)(j + N) * mw, mw, c->q, qw);
        uint64_t r[RP_MAXW] = {0};
        if (bn_sub_n(r, lo, hi, qw)) bn_add_n(r, r, c->q, qw);
        memcpy(out + (size_t)j * qw, r, sizeof(uint64_t) * (size_t)qw);
    }
}

/* Polynomial c = a*b; c.reduce(); over a batch. a, b, out: [batch][N][qw]. */
int rp_polymul(const rp_ctx *c, const uint64_t *a, const uint64_t *b, int N, int batch, uint64_t *out,
               int nthreads) {
    const int qw = c->qw, mw = c->mw;
    int n = spacing_for(N, N);
    uint64_t *W = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)n);
    uint64_t *WInv = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)n);
    rp_twiddles(n, W, WInv);
    if (nthreads < 1) nthreads = 1;
    int outer = batch < nthreads ? batch : nthreads;
    int inner = nthreads / (outer > 0 ? outer : 1);
    if (inner < 1) inner = 1;
#ifdef _OPENMP
    omp_set_max_active_levels(2);
#endif
#pragma omp parallel for schedule(dynamic) num_threads(outer) if (outer > 1)
    for (int s = 0; s < batch; s++) {
        uint64_t *prod = (uint64_t *)calloc((size_t)n * (size_t)mw, sizeof(uint64_t));
        mul_plain_one(c, W, WInv, n, a + (size_t)s * N * qw, N, qw, b + (size_t)s * N * qw, N, qw, prod, inner);
        reduce_fold_modq(c, prod, N, out + (size_t)s * N * qw);
        free(prod);
    }
    free(W); free(WInv);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* YASHE multiply (+ keyswitch) restated on the multiply above (timing)       */
/* ------------------------------------------------------------------------ */

/* signed fold of the plain product over Z (values are non-negative < M), then
 * x t, round(./q), mod q. Coefficients of the inputs are in [0, q). */
static void tensor_round(const rp_ctx *c, const uint64_t *prod, int N, uint64_t t, uint64_t *out) {
    const int mw = c->mw, qw = c->qw;
    if (qw <= 0 || mw <= 0) return;
    for (int j = 0; j < N; j++) {
        /* g = prod[j] - prod[j+N] over Z, as sign and magnitude */
        uint64_t g[RP_MAXW] = {0}, tg[RP_MAXW] = {0};
        int neg = bn_cmp(prod + (size_t)j * mw, prod + (size_t)(j + N) * mw, mw) < 0;
        if (!neg) bn_sub_n(g, prod + (size_t)j * mw, prod + (size_t)(j + N) * mw, mw);
        else bn_sub_n(g, prod + (size_t)(j + N) * mw, prod + (size_t)j * mw, mw);
        bn_mac1(tg, g, t, mw);
        /* |g| t = quot q + rem; round(|g| t / q) = quot + (2 rem > q) (src/ciphertext.cpp:55-63) */
        uint64_t quot[RP_MAXW] = {0}, rem[RP_MAXW] = {0};
        bn_divmod(quot, rem, tg, mw + 1, c->q, qw);
        uint64_t twice[RP_MAXW] = {0}, qx[RP_MAXW] = {0};
        bn_add_n(twice, rem, rem, qw + 1);
        memcpy(qx, c->q, sizeof(uint64_t) * (size_t)qw);
        if (bn_cmp(twice, qx, qw + 1) > 0) {
            uint64_t one[RP_MAXW] = {0};
            one[0] = 1;
            bn_add_n(quot, quot, one, mw + 1);
        }
        uint64_t qm[RP_MAXW] = {0};
        bn_mod(qm, quot, mw + 1, c->q, qw);
        if (neg && bn_used(qm, qw)) bn_sub_n(qm, c->q, qm, qw);
        memcpy(out + (size_t)j * qw, qm, sizeof(uint64_t) * (size_t)qw);
    }
}

int rp_yashe_mul(const rp_ctx *c, const uint64_t *c1, const uint64_t *c2, int N, uint64_t t, int w_bits,
                 const uint64_t *evk, int ell, int batch, uint64_t *out, int nthreads) {
    const int qw = c->qw, mw = c->mw;
    int n = spacing_for(N, N);
    uint64_t *W = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)n);
    uint64_t *WInv = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)n);
    rp_twiddles(n, W, WInv);
    if (nthreads < 1) nthreads = 1;
    int outer = batch < nthreads ? batch : nthreads;
    int inner = nthreads / (outer > 0 ? outer : 1);
    if (inner < 1) inner = 1;
#ifdef _OPENMP
    omp_set_max_active_levels(2);
#endif
#pragma omp parallel for schedule(dynamic) num_threads(outer) if (outer > 1)
    for (int s = 0; s < batch; s++) {
        uint64_t *prod = (uint64_t *)calloc((size_t)n * (size_t)mw, sizeof(uint64_t));
        uint64_t *g = (uint64_t *)calloc((size_t)N * (size_t)qw, sizeof(uint64_t));
        mul_plain_one(c, W, WInv, n, c1 + (size_t)s * N * qw, N, qw, c2 + (size_t)s * N * qw, N, qw, prod, inner);
        tensor_round(c, prod, N, t, g);
        uint64_t *o = out + (size_t)s * N * qw;
        if (evk == NULL || ell <= 0) {
            memcpy(o, g, sizeof(uint64_t) * (size_t)N * (size_t)qw);
        } else {
            uint64_t *acc = (uint64_t *)calloc((size_t)N * (size_t)qw, sizeof(uint64_t));
            uint64_t *dig = (uint64_t *)calloc((size_t)N, sizeof(uint64_t));
            uint64_t *part = (uint64_t *)calloc((size_t)N * (size_t)qw, sizeof(uint64_t));
            for (int d = 0; d < ell; d++) {
                for (int j = 0; j < N; j++) {
                    int bit = d * w_bits;
                    const uint64_t *x = g + (size_t)j * qw;
                    uint64_t v = x[bit / 64] >> (bit % 64);
                    if ((bit % 64) + w_bits > 64 && bit / 64 + 1 < qw) v |= x[bit / 64 + 1] << (64 - bit % 64);
                    dig[j] = w_bits >= 64 ? v : (v & ((1ULL << w_bits) - 1));
                }
                memset(prod, 0, sizeof(uint64_t) * (size_t)n * (size_t)mw);
                mul_plain_one(c, W, WInv, n, dig, N, 1, evk + (size_t)d * N * qw, N, qw, prod, inner);
                reduce_fold_modq(c, prod, N, part);
                for (int j = 0; j < N; j++) {
                    uint64_t *a = acc + (size_t)j * qw;
                    uint64_t tmp[RP_MAXW] = {0}, qx[RP_MAXW] = {0};
                    uint64_t carry = bn_add_n(tmp, a, part + (size_t)j * qw, qw);
                    tmp[qw] = carry;
                    memcpy(qx, c->q, sizeof(uint64_t) * (size_t)qw);
                    if (bn_cmp(tmp, qx, qw + 1) >= 0) bn_sub_n(tmp, tmp, qx, qw + 1);
                    memcpy(a, tmp, sizeof(uint64_t) * (size_t)qw);
                }
            }
            memcpy(o, acc, sizeof(uint64_t) * (size_t)N * (size_t)qw);
            free(acc); free(dig); free(part);
        }
        free(prod); free(g);
    }
    free(W); free(WInv);
    return 0;
}
