// pcg_ieee.cuh -- correctly rounded FP64 divide and square root on the
// integer pipes.
//
// On GB300 the FP64 pipe issues about two DFMA per clock per SM and a
// hardware FP64 divide or square root occupies it for about ten DFMA slots.
// These routines produce the IEEE-754 round-to-nearest-even result bit for
// bit (the same value as the `/` operator and sqrt()), using 64-bit integer
// arithmetic plus one FP32 seed, so the FP64 pipe stays free for the adds,
// multiplies and FMAs of the f-wave solve.
//
// Method (written from the mathematics, see Muller et al., Handbook of
// Floating-Point Arithmetic, 2nd ed., ch. 9 and 10, and Moller & Granlund,
// "Improved division by invariant integers", IEEE TC 60(2), 2011):
//   * significands as 53-bit integers;
//   * a fixed-point reciprocal (or reciprocal square root) is seeded from the
//     FP32 approximation of the leading 24 bits and refined by two
//     Newton-Raphson steps in 64-bit fixed point;
//   * the candidate quotient (root) comes from one high 64x64 product; its
//     exact remainder, computed modulo 2^64, corrects it to the truncated
//     result and decides the rounding (ties to even for the quotient; a
//     square root of a double is never exactly half way).
// Operands outside the fast path (zero, subnormal, infinite, NaN, results
// that would leave the normal range) are handed to the hardware operation,
// so the functions are exact for every input.
#pragma once

#include <cstdint>
#include <cstring>
#include <cmath>

#if defined(__CUDACC__)
#define PCG_HD __host__ __device__ __forceinline__
#else
#define PCG_HD inline
#endif

namespace pcg {
namespace ieee {

constexpr uint64_t kSign = 0x8000000000000000ull;
constexpr uint64_t kFrac = 0x000FFFFFFFFFFFFFull;
constexpr uint64_t kHidden = 0x0010000000000000ull;

PCG_HD uint64_t mulhi(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

PCG_HD uint64_t bits(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  std::memcpy(&u, &x, 8);
  return u;
#endif
}

PCG_HD double from_bits(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double x;
  std::memcpy(&x, &u, 8);
  return x;
#endif
}

PCG_HD float bits_float(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f;
  std::memcpy(&f, &u, 4);
  return f;
#endif
}

PCG_HD uint32_t float_bits(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
#endif
}

// FP32 seeds: only their accuracy matters (the integer refinement corrects
// any seed within a few units of 2^-22), not their exact value.
PCG_HD float rcp_seed(float d) {
#if defined(__CUDA_ARCH__)
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(d));
  return r;
#else
  return 1.0f / d;
#endif
}

PCG_HD float rsqrt_seed(float d) {
#if defined(__CUDA_ARCH__)
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(d));
  return r;
#else
  return 1.0f / std::sqrt(d);
#endif
}

// Fallbacks for operands outside the fast path.  Kept out of line on the
// device so the compiler cannot evaluate them speculatively next to the fast
// path (that would put the FP64 divide / square root back on the FP64 pipe).
#if defined(__CUDACC__)
static __host__ __device__ __noinline__ double hw_div(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __ddiv_rn(a, b);
#else
  return a / b;
#endif
}

static __host__ __device__ __noinline__ double hw_sqrt(double a) {
#if defined(__CUDA_ARCH__)
  return __dsqrt_rn(a);
#else
  return std::sqrt(a);
#endif
}
#else
inline double hw_div(double a, double b) { return a / b; }
inline double hw_sqrt(double a) { return std::sqrt(a); }
#endif

// One Newton-Raphson step for V ~ 2^116 / m  (m in [2^52, 2^53), V in (2^63, 2^64)).
PCG_HD uint64_t recip_step(uint64_t m, uint64_t V) {
  uint64_t hi = mulhi(m, V), lo = m * V;
  // E = 2^116 - m*V as a signed 128-bit number (hi part small), then E / 2^52
  int64_t ehi = (int64_t)(kHidden - hi) - (lo != 0 ? 1 : 0);
  uint64_t elo = (uint64_t)0 - lo;
  int64_t e = (int64_t)((uint64_t)ehi << 12) | (int64_t)(elo >> 52);
  uint64_t ae = e < 0 ? (uint64_t)(-e) : (uint64_t)e;
  uint64_t d = mulhi(V, ae);
  return e < 0 ? V - d : V + d;
}

// Correctly rounded a / b.
PCG_HD double div_rn(double a, double b) {
  uint64_t A = bits(a), B = bits(b);
  uint32_t ea = (uint32_t)(A >> 52) & 0x7FFu, eb = (uint32_t)(B >> 52) & 0x7FFu;
  uint64_t sign = (A ^ B) & kSign;
  if (eb - 1u >= 2046u) return hw_div(a, b);
  if ((A & ~kSign) == 0) return from_bits(sign);  // +-0 / normal
  if (ea - 1u >= 2046u) return hw_div(a, b);
  uint64_t ma = (A & kFrac) | kHidden, mb = (B & kFrac) | kHidden;
  int e = (int)ea - (int)eb + 1023;
  uint64_t x = ma;
  if (ma < mb) {
    x = ma << 1;
    e -= 1;
  }
  if (e <= 0 || e >= 2047) return hw_div(a, b);
  uint64_t q;
  if ((B & kFrac) == 0) {
    q = x;  // divisor is a power of two: exact
  } else {
    // leading 23 fraction bits of the divisor as a float in [1, 2); its
    // reciprocal r in (0.5, 1] gives V0 = r * 2^64 straight from r's bits
    float d = bits_float(0x3F800000u | (uint32_t)((mb >> 29) & 0x7FFFFFu));
    uint32_t rb = float_bits(rcp_seed(d));
    uint64_t V = ((uint64_t)((rb & 0x7FFFFFu) | 0x800000u)) << ((int)((rb >> 23) & 0xFFu) - 86);
    if (((rb >> 23) & 0xFFu) >= 127u) V = 0xFFFFFFFFFFFFFFFFull;  // r == 1: clamp below 2^64
    V = recip_step(mb, V);
    V = recip_step(mb, V);
    q = mulhi(x, V);
    int64_t rem = (int64_t)((x << 52) - q * mb);
    if (rem < 0) { q -= 1; rem += (int64_t)mb; }
    if (rem < 0) { q -= 1; rem += (int64_t)mb; }
    if (rem >= (int64_t)mb) { q += 1; rem -= (int64_t)mb; }
    if (rem >= (int64_t)mb) { q += 1; rem -= (int64_t)mb; }
    uint64_t twice = (uint64_t)rem << 1;
    if (twice > mb || (twice == mb && (q & 1))) q += 1;
  }
  return from_bits(sign | ((uint64_t)e << 52) | (q - kHidden));
}

// One Newton-Raphson step for Y ~ 2^90 / sqrt(M)  (M in [2^52, 2^54), Y in (2^63, 2^64)).
PCG_HD uint64_t rsqrt_step(uint64_t M, uint64_t Y) {
  uint64_t y2 = mulhi(Y, Y);  // Y^2 / 2^64 ~ 2^116 / M
  uint64_t hi = mulhi(M, y2), lo = M * y2;
  int64_t ehi = (int64_t)(kHidden - hi) - (lo != 0 ? 1 : 0);
  uint64_t elo = (uint64_t)0 - lo;
  // Y' = Y + Y * E / 2^117 with E = 2^116 - M*y2; E / 2^53 first
  int64_t e = (int64_t)((uint64_t)ehi << 11) | (int64_t)(elo >> 53);
  uint64_t ae = e < 0 ? (uint64_t)(-e) : (uint64_t)e;
  uint64_t d = mulhi(Y, ae);
  return e < 0 ? Y - d : Y + d;
}

// Correctly rounded sqrt(a).
PCG_HD double sqrt_rn(double a) {
  uint64_t A = bits(a);
  uint32_t ea = (uint32_t)(A >> 52) & 0x7FFu;
  if ((A & kSign) || ea - 1u >= 2046u) return hw_sqrt(a);
  int k = (int)ea - 1023;
  uint64_t M = (A & kFrac) | kHidden;
  if (k & 1) {
    M <<= 1;
    k -= 1;
  }
  uint64_t s;
  if (M == kHidden) {
    s = kHidden;  // power of four: exact
  } else {
    // M / 2^52 in [1, 4) as a float (leading 24 bits); its reciprocal square
    // root r in (0.5, 1] gives Y0 = r * 2^64 straight from r's bits
    float f = bits_float(((M >> 53) ? 0x40000000u : 0x3F800000u) |
                         (uint32_t)((M >> ((M >> 53) ? 30 : 29)) & 0x7FFFFFu));
    uint32_t rb = float_bits(rsqrt_seed(f));
    uint64_t Y = ((uint64_t)((rb & 0x7FFFFFu) | 0x800000u)) << ((int)((rb >> 23) & 0xFFu) - 86);
    if (((rb >> 23) & 0xFFu) >= 127u) Y = 0xFFFFFFFFFFFFFFFFull;  // r == 1: clamp below 2^64
    Y = rsqrt_step(M, Y);
    Y = rsqrt_step(M, Y);
    s = mulhi(M, Y);
    int64_t rem = (int64_t)((M << 52) - s * s);
    if (rem < 0) { s -= 1; rem += (int64_t)(2 * s + 1); }
    if (rem < 0) { s -= 1; rem += (int64_t)(2 * s + 1); }
    if (rem > (int64_t)(2 * s)) { rem -= (int64_t)(2 * s + 1); s += 1; }
    if (rem > (int64_t)(2 * s)) { rem -= (int64_t)(2 * s + 1); s += 1; }
    if (rem > (int64_t)s) s += 1;
  }
  return from_bits(((uint64_t)(k / 2 + 1023) << 52) | (s - kHidden));
}

}  // namespace ieee
}  // namespace pcg
