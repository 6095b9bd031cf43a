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
//   * a 64-bit fixed-point reciprocal (or reciprocal square root) from an
//     FP32 seed of the leading 24 bits, one FP32 Newton step and a
//     second-order correction computed in FP32 on a two-float split of the
//     operand (about 46 correct bits);
//   * the candidate quotient (root) from one high 64x64 product, its exact
//     remainder modulo 2^64, one FP32 correction step of the remainder and
//     one fix-up give the truncated result, and the remainder decides the
//     rounding (ties to even for the quotient; a square root of a double is
//     never exactly half way).
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

// On the device the bits move through an opaque register copy, so that the
// compiler does not turn integer tests on them back into FP64 instructions.
PCG_HD uint64_t bits(double x) {
#if defined(__CUDA_ARCH__)
  uint64_t u;
  asm("mov.b64 %0, %1;" : "=l"(u) : "d"(x));
  return u;
#else
  uint64_t u;
  std::memcpy(&u, &x, 8);
  return u;
#endif
}

PCG_HD double from_bits(uint64_t u) {
#if defined(__CUDA_ARCH__)
  double x;
  asm("mov.b64 %0, %1;" : "=d"(x) : "l"(u));
  return x;
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

PCG_HD float fma_f(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  return __fmaf_rn(a, b, c);
#else
  return std::fmaf(a, b, c);
#endif
}

PCG_HD float mul_f(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}

PCG_HD int32_t rint_f(float a) {
#if defined(__CUDA_ARCH__)
  return __float2int_rn(a);
#else
  return (int32_t)std::lrintf(a);
#endif
}

// FP32 seeds: only their accuracy matters, not their exact value (one FP32
// Newton step squares the seed's error; any seed within 2^-12 of the
// reciprocal (square root) gives exact results).
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

// 2^64 / D for D = mb / 2^52 in (1, 2), accurate to about 2^-46 relative and
// below 2^64, plus the FP32 reciprocal r0 of D's leading 24 bits.
// r0 = 1 / d_hi to float precision (one FP32 Newton step on the seed), then
// 1/D = r0 (1 + e + e^2 + ...) with e = 1 - D r0 computed from the two-float
// split D = d_hi + d_lo.  r0 lies in (0.5, 1]: its significand shifted by 40
// is r0 * 2^64 (r0 == 1, for d_hi == 1, is clamped to 2^64 - 1; its
// correction is then <= 0).  The correction r0 (e + e^2) (|.| < 2^-22) is
// added as a multiple of 2^-50.
PCG_HD uint64_t recip64(uint64_t mb, float &r0) {
  const float d_hi = bits_float(0x3F800000u | (uint32_t)((mb >> 29) & 0x7FFFFFu));
  const float d_lo = mul_f((float)(uint32_t)(mb & 0x1FFFFFFFull), 2.220446049250313e-16f);  // * 2^-52
  r0 = rcp_seed(d_hi);
  r0 = fma_f(r0, fma_f(-d_hi, r0, 1.0f), r0);
  float er = fma_f(-d_hi, r0, 1.0f);
  er = fma_f(-d_lo, r0, er);
  const float corr = mul_f(r0, fma_f(er, er, er));
  const uint32_t rb = float_bits(r0);
  uint64_t V = rb >= 0x3F800000u ? 0xFFFFFFFFFFFFFFFFull
                                 : ((uint64_t)((rb & 0x7FFFFFu) | 0x800000u) << 40);
  return V + ((uint64_t)(int64_t)rint_f(mul_f(corr, 1.125899906842624e15f)) << 14);  // corr * 2^50
}

// Quotient significand q = x * 2^52 / mb (x in [mb, 2 mb)) rounded to nearest
// even, from the estimate q0 (within a few hundred units) and
// rem = x * 2^52 - q0 * mb (exact modulo 2^64; its true value is small).
// One FP32 step rem / mb (error < 2^-14) brings the remainder into
// (-(1/2 + 2^-14) mb, (1/2 + 2^-14) mb); one fix-up makes it the remainder
// of the truncated quotient.
PCG_HD uint64_t quot_round(uint64_t q, int64_t rem, uint64_t mb, float r0) {
  const float dq = mul_f(mul_f((float)(int32_t)(rem >> 32), r0), 9.5367431640625e-07f);  // * 2^-20
  const int64_t di = (int64_t)rint_f(dq);
  q = (uint64_t)((int64_t)q + di);
  rem -= di * (int64_t)mb;
  if (rem < 0) {
    q -= 1;
    rem += (int64_t)mb;
  }
  const uint64_t twice = (uint64_t)rem << 1;
  if (twice > mb || (twice == mb && (q & 1))) q += 1;
  return q;
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
    float r0;
    const uint64_t V = recip64(mb, r0);
    const uint64_t q0 = mulhi(x, V);
    q = quot_round(q0, (int64_t)((x << 52) - q0 * mb), mb, r0);
  }
  return from_bits(sign | ((uint64_t)e << 52) | (q - kHidden));
}

// Correctly rounded 1 / b (div_rn(1.0, b) with the dividend's work folded in).
PCG_HD double rcp_rn(double b) {
  const uint64_t B = bits(b);
  const uint32_t eb = (uint32_t)(B >> 52) & 0x7FFu;
  if (eb - 1u >= 2044u) return hw_div(1.0, b);  // zero, subnormal, huge, inf, NaN
  const uint64_t sign = B & kSign;
  if ((B & kFrac) == 0) return from_bits(sign | ((uint64_t)(2046u - eb) << 52));  // 2^-k
  const uint64_t mb = (B & kFrac) | kHidden;
  float r0;
  const uint64_t V = recip64(mb, r0);
  // x = 2^53 (1 < mb / 2^52): q0 = 2^53 V / 2^64, and x * 2^52 = 2^105 is 0 mod 2^64
  const uint64_t q0 = V >> 11;
  const uint64_t q = quot_round(q0, (int64_t)(0ull - q0 * mb), mb, r0);
  return from_bits(sign | ((uint64_t)(2045u - eb) << 52) | (q - kHidden));
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
    // 1/sqrt(F) for F = M / 2^52 in [1, 4): r0 = 1/sqrt(f_hi) to float
    // precision (one FP32 Newton step on the seed), refined with the
    // two-float split F = f_hi + f_lo: 1/sqrt(F) ~ r0 (1 + e/2 + 3e^2/8),
    // e = 1 - F r0^2.  r0 lies in (0.5, 1]: Y = r0 * 2^64 is its significand
    // shifted by 40 (r0 == 1 clamped to 2^64 - 1), the correction is added as
    // a multiple of 2^-50.
    const bool hi = (M >> 53) != 0;
    const int sh = hi ? 30 : 29;
    const float f_hi = bits_float((hi ? 0x40000000u : 0x3F800000u) | (uint32_t)((M >> sh) & 0x7FFFFFu));
    const float f_lo = mul_f((float)(uint32_t)(M & ((1ull << sh) - 1)), 2.220446049250313e-16f);  // * 2^-52
    float r0 = rsqrt_seed(f_hi);
    r0 = fma_f(mul_f(r0, 0.5f), fma_f(-mul_f(f_hi, r0), r0, 1.0f), r0);
    const float s0 = mul_f(f_hi, r0);
    const float s0e = fma_f(f_hi, r0, -s0);  // f_hi * r0 = s0 + s0e exactly
    float er = fma_f(-s0, r0, 1.0f);
    er = fma_f(-s0e, r0, er);
    er = fma_f(-mul_f(f_lo, r0), r0, er);
    const float corr = mul_f(r0, fma_f(mul_f(er, 0.375f), er, mul_f(er, 0.5f)));
    const uint32_t rb = float_bits(r0);
    uint64_t Y = rb >= 0x3F800000u ? 0xFFFFFFFFFFFFFFFFull
                                   : ((uint64_t)((rb & 0x7FFFFFu) | 0x800000u) << 40);
    Y += (uint64_t)(int64_t)rint_f(mul_f(corr, 1.125899906842624e15f)) << 14;  // corr * 2^50
    s = mulhi(M, Y);  // within a few hundred units of floor(sqrt(M * 2^52))
    int64_t rem = (int64_t)((M << 52) - s * s);
    // one FP32 step delta = rem / (2 s), 1/(2 s) ~ r0 * 2^-53 (error < 2^-14),
    // then one fix-up gives floor(sqrt) and its remainder
    const float ds = mul_f(mul_f((float)(int32_t)(rem >> 32), r0), 4.76837158203125e-07f);  // * 2^-21
    const int64_t di = (int64_t)rint_f(ds);
    rem -= di * (int64_t)(2 * s) + di * di;
    s = (uint64_t)((int64_t)s + di);
    if (rem < 0) {
      s -= 1;
      rem += (int64_t)(2 * s + 1);
    }
    if (rem > (int64_t)s) s += 1;  // never a tie
  }
  return from_bits(((uint64_t)(k / 2 + 1023) << 52) | (s - kHidden));
}

}  // namespace ieee
}  // namespace pcg
