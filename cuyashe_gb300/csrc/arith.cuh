// arith.cuh -- 32-bit modular arithmetic for word-sized NTT primes p < 2^30.
//
// The reference reduces modulo one 64-bit Goldilocks prime with __umul64hi and a
// three-case fix-up (s_mul, src/cuda_functions.cu:310-349), i.e. emulated
// 64x64-bit products on every butterfly. Here every residue is a 32-bit word
// and products are 32x32-bit:
//   * Shoup multiplication by a precomputed constant (twiddles, CRT factors):
//     one mul.hi and two mul.lo, result in [0, 2p) for any 32-bit input;
//   * Montgomery multiplication for the pointwise product of two variables;
//   * lazy reduction with the unsigned-min trick min(x, x - m), written with the
//     add-then-min intrinsic __viaddmin_u32 so that it is one instruction.
#pragma once

#include <stdint.h>

namespace cy {

// x in [0, 2m) -> [0, m)   (x - m wraps above x when x < m)
__device__ __forceinline__ uint32_t red(uint32_t x, uint32_t m) { return __viaddmin_u32(x, 0u - m, x); }

// x * w mod p in [0, 2p), any 32-bit x; w < p, ws = floor(w * 2^32 / p), p < 2^31.
__device__ __forceinline__ uint32_t shoup(uint32_t x, uint32_t w, uint32_t ws, uint32_t p) {
    const uint32_t q = __umulhi(x, ws);
    return x * w - q * p;
}

// a * b * 2^-32 mod p in [0, 2p) for a, b in [0, 2p), p < 2^30; pinv = -p^-1 mod 2^32.
__device__ __forceinline__ uint32_t mont(uint32_t a, uint32_t b, uint32_t p, uint32_t pinv) {
    const uint64_t T = (uint64_t)a * b;
    const uint32_t m = (uint32_t)T * pinv;
    const uint64_t u = T + (uint64_t)m * p;  // low word is zero
    return (uint32_t)(u >> 32);
}

// The modulus with the constants derived from it. Each field is loaded from
// memory on its own (BasisDev::p, p2, np, np2), so that the compiler cannot
// relate them: it then emits the lazy reduction min(x, x - 2p) as one
// add-then-min and x w - q p as one multiply-add with -p. Constants it can
// derive from p were measured to cost two more integer instructions per
// butterfly (8 instead of 6).
struct Mod {
    uint32_t p, p2, np, np2;  // p, 2p, -p, -2p (mod 2^32)
};

// The same constants computed from p in registers: the compiler folds them
// (fewer live registers, two more instructions per butterfly), for kernels that
// are short of registers.
__device__ __forceinline__ Mod mod_of(uint32_t p) { return Mod{p, 2 * p, 0u - p, 0u - 2 * p}; }

// x * w mod p in [0, 2p), any 32-bit x (Shoup, with -p from m)
__device__ __forceinline__ uint32_t shoup_m(uint32_t x, uint32_t w, uint32_t ws, const Mod& m) {
    return __umulhi(x, ws) * m.np + x * w;
}

// Cooley-Tukey butterfly (Harvey's lazy form): X, Y in [0, 4p) -> X + wY, X - wY in [0, 4p).
// Six integer instructions: add-then-min, mul.hi, two multiply-adds, two adds.
__device__ __forceinline__ void ct_bfly(uint32_t& X, uint32_t& Y, uint32_t w, uint32_t ws, const Mod& m) {
    const uint32_t x = __viaddmin_u32(X, m.np2, X);  // [0, 2p)
    const uint32_t t = shoup_m(Y, w, ws, m);        // [0, 2p)
    Y = x - t + m.p2;
    X = x + t;
}

// Gentleman-Sande butterfly: X, Y in [0, 2p) -> X + Y, (X - Y) w in [0, 2p).
__device__ __forceinline__ void gs_bfly(uint32_t& X, uint32_t& Y, uint32_t w, uint32_t ws, const Mod& m) {
    const uint32_t s = __viaddmin_u32(X, Y, X + Y + m.np2);  // min(X + Y, X + Y - 2p)
    const uint32_t d = X - Y + m.p2;
    Y = shoup_m(d, w, ws, m);
    X = s;
}

}  // namespace cy
