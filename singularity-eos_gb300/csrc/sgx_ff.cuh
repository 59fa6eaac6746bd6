// Float-float ("ff") arithmetic: a value carried as an unevaluated sum
// hi + lo of two floats, |lo| <= ulp(hi) / 2, about 48 significant bits.
// On GB300 the FP32 pipe issues 64 times the FP64 pipe's operations, so a
// kernel that needs ~1e-14 relative accuracy runs faster in ff than in FP64
// even at 10-20 FP32 operations per ff operation.
//
// The building blocks are the error-free transformations of Knuth (two-sum)
// and Dekker (quick two-sum), with the exact product error from fmaf; the
// composite operations follow the classical double-word algorithms (Dekker
// 1971; Bailey's double-double, restated for floats). Conversions between
// double and ff go through the IEEE bit patterns with integer operations
// only, so they never occupy the FP64 pipe; they are exact for normal values
// whose exponents the callers check (ff_from_double_ok).
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

namespace sgx {

struct ff {
  float hi, lo;
};

__device__ __forceinline__ ff ff_make(const float hi, const float lo = 0.0f) { return {hi, lo}; }

// Every rounding the transformations below rely on is written with the _rn
// intrinsics, which the compiler never fuses into an FMA: a fused
// multiply-add in place of a separate product and sum would change s and
// break the exactness of the error terms.
#define FADD __fadd_rn
#define FSUB __fsub_rn
#define FMUL __fmul_rn

// s + e == a + b exactly (Knuth).
__device__ __forceinline__ ff two_sum(const float a, const float b) {
  const float s = FADD(a, b);
  const float bb = FSUB(s, a);
  const float e = FADD(FSUB(a, FSUB(s, bb)), FSUB(b, bb));
  return {s, e};
}
// Same when |a| >= |b| (Dekker).
__device__ __forceinline__ ff quick_two_sum(const float a, const float b) {
  const float s = FADD(a, b);
  return {s, FSUB(b, FSUB(s, a))};
}
// p + e == a * b exactly.
__device__ __forceinline__ ff two_prod(const float a, const float b) {
  const float p = FMUL(a, b);
  return {p, fmaf(a, b, -p)};
}

__device__ __forceinline__ ff ff_add(const ff x, const ff y) {
  ff s = two_sum(x.hi, y.hi);
  const ff t = two_sum(x.lo, y.lo);
  s.lo = FADD(s.lo, t.hi);
  s = quick_two_sum(s.hi, s.lo);
  s.lo = FADD(s.lo, t.lo);
  return quick_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ ff ff_neg(const ff x) { return {-x.hi, -x.lo}; }
__device__ __forceinline__ ff ff_sub(const ff x, const ff y) { return ff_add(x, ff_neg(y)); }

__device__ __forceinline__ ff ff_mul(const ff x, const ff y) {
  ff p = two_prod(x.hi, y.hi);
  p.lo = fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, p.lo));
  return quick_two_sum(p.hi, p.lo);
}
// x y without the final renormalisation (for sums that accept an
// unnormalised low part, such as ff_sum4).
__device__ __forceinline__ ff ff_mul_nn(const ff x, const ff y) {
  ff p = two_prod(x.hi, y.hi);
  p.lo = fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, p.lo));
  return p;
}
__device__ __forceinline__ ff ff_mul_f(const ff x, const float y) {
  ff p = two_prod(x.hi, y);
  p.lo = fmaf(x.lo, y, p.lo);
  return quick_two_sum(p.hi, p.lo);
}

// x / y: a float quotient refined twice with exact residuals.
__device__ __forceinline__ ff ff_div(const ff x, const ff y) {
  const float r = 1.0f / y.hi;
  const float q1 = FMUL(x.hi, r);
  ff rem = ff_sub(x, ff_mul_f(y, q1));
  const float q2 = FMUL(rem.hi, r);
  rem = ff_sub(rem, ff_mul_f(y, q2));
  const float q3 = FMUL(rem.hi, r);
  const ff q = quick_two_sum(q1, q2);
  return ff_add(q, ff_make(q3));
}

// sqrt(x) for x > 0: a float root refined by one Newton step in ff.
__device__ __forceinline__ ff ff_sqrt(const ff x) {
  const float s = sqrtf(x.hi);
  const ff s2 = two_prod(s, s);
  const ff d = ff_sub(x, s2);
  return ff_add(ff_make(s), ff_make(FMUL(d.hi, 0.5f / s)));
}

// ---- cheaper forms for the ~1e-14 a lookup needs (ff carries ~1e-14.5) ----

// 1/x and 1/sqrt(x) to about one float ulp: the MUFU approximations, whose
// error the one correction step of each caller below squares away.
__device__ __forceinline__ float rcp_approx(const float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float rsqrt_approx(const float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// x / y (y.hi normal, non-zero): q1 = x.hi / y.hi from the approximate
// reciprocal, then one correction q2 = (x - q1 y) / y with the residual
// formed exactly in its leading part (x.hi - q1 y.hi cancels by Sterbenz).
// Relative error about 2^-45.
__device__ __forceinline__ ff ff_div_fast(const ff x, const ff y) {
  const float r = rcp_approx(y.hi);
  const float q1 = FMUL(x.hi, r);
  const float ph = FMUL(y.hi, q1);
  float pl = fmaf(y.hi, q1, -ph); // y.hi q1 = ph + pl exactly
  pl = fmaf(y.lo, q1, pl);
  const float rem = FADD(FSUB(x.hi, ph), FSUB(x.lo, pl));
  return quick_two_sum(q1, FMUL(rem, r));
}

// sqrt(x), x.hi > 0 normal: s = sqrtf(x.hi) (correctly rounded) and one
// Newton correction with the residual x - s^2 exact in its leading part.
// Relative error about 2^-47.
__device__ __forceinline__ ff ff_sqrt_fast(const ff x) {
  const float s = sqrtf(x.hi);
  const float sq = FMUL(s, s);
  const float sqe = fmaf(s, s, -sq); // s^2 = sq + sqe exactly
  const float d = FADD(FSUB(x.hi, sq), FSUB(x.lo, sqe));
  return quick_two_sum(s, FMUL(d, FMUL(0.5f, rcp_approx(s))));
}

// sqrt(b / r) for b, r > 0 normal, as b (b r)^(-1/2): y0 = rsqrt(p.hi) for
// p = b r, one Newton step y1 = y0 (1 + h / 2) with h = 1 - p y0^2 formed
// exactly in its leading part, then b y1. Relative error about 2^-44.
__device__ __forceinline__ ff ff_sqrt_ratio(const ff b, const ff r) {
  const ff p = ff_mul(b, r);
  const float y0 = rsqrt_approx(p.hi);
  const float s = FMUL(y0, y0);
  const float se = fmaf(y0, y0, -s); // y0^2 = s + se exactly
  const float th = FMUL(p.hi, s);
  float tl = fmaf(p.hi, s, -th); // p.hi s = th + tl exactly
  tl = fmaf(p.hi, se, fmaf(p.lo, s, tl));
  const float h = FSUB(FSUB(1.0f, th), tl);
  const ff y1 = quick_two_sum(y0, FMUL(FMUL(0.5f, y0), h));
  return ff_mul(b, y1);
}

// x + y0 + y1 + y2 for the lookup's bilinear forms: the four leading parts
// summed by exact two-sums, every low part and rounding error added once in
// float. The result's low part is not renormalised (ff2d accepts that).
__device__ __forceinline__ ff ff_sum4(const ff x, const ff y0, const ff y1, const ff y2) {
  const ff s0 = two_sum(x.hi, y0.hi);
  const ff s1 = two_sum(s0.hi, y1.hi);
  const ff s2 = two_sum(s1.hi, y2.hi);
  const float lo = FADD(FADD(FADD(x.lo, y0.lo), FADD(y1.lo, y2.lo)),
                        FADD(FADD(s0.lo, s1.lo), s2.lo));
  return {s2.hi, lo};
}

__device__ __forceinline__ bool ff_gt(const ff a, const ff b) {
  return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo);
}
__device__ __forceinline__ bool ff_lt(const ff a, const ff b) {
  return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}

// ---- conversions through the bit patterns ----

// The two 32-bit words of a double's bit pattern, through a move the
// compiler cannot see into: tests of the pattern then stay integer
// instructions. (A test of the 64-bit pattern with the sign masked off
// against zero is otherwise folded into a floating-point compare with 0.0,
// which issues on the FP64 pipe.)
__device__ __forceinline__ void d_words(const double x, unsigned &lo, unsigned &hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "d"(x));
}
// x == +-0, as an integer test
__device__ __forceinline__ bool d_zero_bits(const double x) {
  unsigned lo, hi;
  d_words(x, lo, hi);
  return ((hi & 0x7fffffffu) | lo) == 0u;
}
// x == +-0, or its unbiased binary exponent in [emin, emax]
__device__ __forceinline__ bool d_zero_or_exp_in(const double x, const int emin, const int emax) {
  unsigned lo, hi;
  d_words(x, lo, hi);
  const int e = static_cast<int>((hi >> 20) & 0x7ffu) - 1023;
  return ((hi & 0x7fffffffu) | lo) == 0u || (e >= emin && e <= emax);
}

// Whether d2ff below represents x to ~48 bits: x == 0, or its binary
// exponent in [-74, 127] (then hi is a normal float and lo does not
// underflow).
__device__ __forceinline__ bool ff_from_double_ok(const double x) {
  return d_zero_or_exp_in(x, -74, 127);
}

// hi: x truncated to 24 significant bits; lo: the remaining 29 bits,
// rounded to 24. Integer and FP32 operations only.
__device__ __forceinline__ ff d2ff(const double x) {
  const long long b = __double_as_longlong(x);
  const int ex = static_cast<int>((b >> 52) & 0x7ff);
  if (ex == 0) return {0.0f, 0.0f};
  const int e = ex - 1023;
  const unsigned sign = static_cast<unsigned>((b >> 32) & 0x80000000u);
  const long long mant = b & ((1LL << 52) - 1);
  const float hi = __uint_as_float(sign | (static_cast<unsigned>(e + 127) << 23) |
                                   static_cast<unsigned>(mant >> 29));
  const unsigned rest = static_cast<unsigned>(mant & ((1LL << 29) - 1));
  // rest * 2^(e - 52), with the sign of x; e - 52 + 127 >= 1 under the
  // ff_from_double_ok range
  const float scale = __uint_as_float(static_cast<unsigned>(e - 52 + 127) << 23);
  const float lo = __uint_as_float(__float_as_uint(static_cast<float>(rest) * scale) | sign);
  return {hi, lo};
}

// The double with the value of a float (normal floats, zero, inf, NaN;
// subnormal floats become zero), by moving the fields.
__device__ __forceinline__ double f2d_bits(const float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned long long sign = static_cast<unsigned long long>(u & 0x80000000u) << 32;
  const unsigned ex = (u >> 23) & 0xff;
  const unsigned long long mant = static_cast<unsigned long long>(u & 0x7fffff) << 29;
  if (ex == 0) return __longlong_as_double(static_cast<long long>(sign));
  const unsigned long long e64 = ex == 0xff ? 0x7ffULL : static_cast<unsigned long long>(ex + 896);
  return __longlong_as_double(static_cast<long long>(sign | (e64 << 52) | mant));
}

// hi + lo as a double, by 32-bit integer operations. The pair is first
// renormalised (two_sum, exact), so |lo| <= ulp(hi) / 2; hi as a double then
// has 29 zero bits below its float significand, and lo's significand
// (subnormal ones included), aligned to hi's 2^(e-52) grid (bits below it
// dropped: an error below 2^-52 relative), is at most 2^28 units of that
// grid. It is added to or subtracted from the low word of hi's bit pattern:
// an addition cannot carry out of it, a subtraction borrows from the high
// word, and when hi is a power of two that borrow moves the result into the
// binade below, so the amount is aligned to that binade's grid, twice as
// fine, instead. hi must be a normal float or zero after the
// renormalisation (lo may be anything); zero, inf and NaN come out as
// f2d_bits of hi.
__device__ __forceinline__ double ff2d(const ff x0) {
  const ff x = two_sum(x0.hi, x0.lo);
  const unsigned uh = __float_as_uint(x.hi), ul = __float_as_uint(x.lo);
  const unsigned eh = (uh >> 23) & 0xffu, el = (ul >> 23) & 0xffu;
  if (eh == 0u || eh == 0xffu) return f2d_bits(x.hi);
  // hi as a double: high word sign | exponent | top 20 significand bits,
  // low word the other 3 bits
  int H = static_cast<int>((uh & 0x80000000u) | ((eh + 896u) << 20) | ((uh & 0x7fffffu) >> 3));
  unsigned L = uh << 29;
  if ((ul & 0x7fffffffu) != 0u) {
    // lo = ml 2^(el - 150), el = 1 for a subnormal lo
    const unsigned ml = el != 0u ? ((ul & 0x7fffffu) | 0x800000u) : (ul & 0x7fffffu);
    const bool down = ((uh ^ ul) & 0x80000000u) && (uh & 0x7fffffu) == 0u;
    // the grid 2^(eh - 179 - down) in units of which lo is counted
    const unsigned sh = eh - (el != 0u ? el : 1u) - (down ? 1u : 0u); // >= 23
    const unsigned add = sh <= 29u ? ml << (29u - sh) : (sh < 61u ? ml >> (sh - 29u) : 0u);
    if ((uh ^ ul) & 0x80000000u) {
      H -= L < add ? 1 : 0;
      L -= add;
    } else {
      L += add;
    }
  }
  return __hiloint2double(H, static_cast<int>(L));
}

// hi + lo as a double, correctly rounded, by one FP64 addition of the two
// parts widened exactly by moving their fields (subnormal parts count as
// zero). Fewer instructions than ff2d for one FP64-pipe instruction, which
// pays where the FP64 pipe has room and instruction issue binds; lo need
// not be normalised.
__device__ __forceinline__ double ff2d_add(const ff x) {
  return __dadd_rn(f2d_bits(x.hi), f2d_bits(x.lo));
}

// A float that holds an integer of magnitude < 2^62, as int64 (shift of the
// significand by the exponent); values below 1 give 0.
__device__ __forceinline__ long long f2ll_bits(const float f) {
  const unsigned u = __float_as_uint(f);
  const int ex = static_cast<int>((u >> 23) & 0xff) - 127;
  if (ex < 0) return 0;
  const long long m = static_cast<long long>((u & 0x7fffff) | 0x800000);
  const long long v = ex >= 23 ? (m << (ex - 23)) : (m >> (23 - ex));
  return (u & 0x80000000u) ? -v : v;
}

#undef FADD
#undef FSUB
#undef FMUL

} // namespace sgx
