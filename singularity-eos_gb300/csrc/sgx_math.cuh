// Scalar numerics shared by every kernel: robust division, NaN-propagating
// min/max with the C++ standard library's semantics, compensated sums, the
// NQT "fast log" grid transform and the 1-D root finders.
//
// Everything here is __host__ __device__ and templated on the arithmetic type
// so the same source serves the FP64 parity path (compiled with --fmad=false,
// bit-identical to the reference compiled with -ffp-contract=off) and the
// FP32 iteration path.
#pragma once

#include <cstdint>
#include <cfloat>

#if defined(__CUDACC__)
#define SGX_HD __host__ __device__ __forceinline__
#define SGX_HDI __host__ __device__ inline
// Out-of-line helpers (root finds, table lookups) that would otherwise be
// inlined at dozens of call sites inside the PTE solver.
#define SGX_HDN static __host__ __device__ __noinline__
#else
#define SGX_HD inline
#define SGX_HDI inline
#define SGX_HDN static __attribute__((noinline))
#endif

namespace sgx {

template <typename T> struct lim;
template <> struct lim<double> {
  // robust::SMALL / EPS (base/robust_utils.hpp:26-34): 10 * min, 10 * epsilon
  static constexpr double small = 10 * DBL_MIN;
  static constexpr double eps = 10 * DBL_EPSILON;
};
template <> struct lim<float> {
  static constexpr float small = 10 * FLT_MIN;
  static constexpr float eps = 10 * FLT_EPSILON;
};

// std::max / std::min semantics (first argument returned on NaN ties), which
// differ from fmax/fmin; the reference relies on them.
template <typename T> SGX_HD T smax(T a, T b) { return (a < b) ? b : a; }
template <typename T> SGX_HD T smin(T a, T b) { return (b < a) ? b : a; }
// The reference's MYMAX macro (eos_ideal.hpp:32): a > b ? a : b.
template <typename T> SGX_HD T mymax(T a, T b) { return a > b ? a : b; }
// std::abs on floating point: clears the sign bit (also of NaN and -0).
SGX_HD double sabs(double a) {
#if defined(__CUDA_ARCH__)
  return fabs(a);
#else
  return __builtin_fabs(a);
#endif
}
SGX_HD float sabs(float a) {
#if defined(__CUDA_ARCH__)
  return fabsf(a);
#else
  return __builtin_fabsf(a);
#endif
}

// std::sqrt (correctly rounded on both sides).
SGX_HD double ssqrt(double a) {
#if defined(__CUDA_ARCH__)
  return sqrt(a);
#else
  return __builtin_sqrt(a);
#endif
}
SGX_HD float ssqrt(float a) {
#if defined(__CUDA_ARCH__)
  return sqrtf(a);
#else
  return __builtin_sqrtf(a);
#endif
}

// robust::sgn (robust_utils.hpp:50-56): sgn(0) = +1.
template <typename T> SGX_HD int rsgn(T v) { return (T(0) <= v) - (v < T(0)); }
// robust::ratio (robust_utils.hpp:58-61): a / (b + sgn(b) * SMALL).
template <typename T> SGX_HD T ratio(T a, T b) {
  return a / (b + rsgn(b) * lim<T>::small);
}

// error_utils::bad_value (error_utils.hpp:29-36,71-75): true unless the value
// is zero or both it and 1e10 times it are normal numbers.
SGX_HD bool is_normal_d(double v) {
  const double a = v < 0 ? -v : v;
  return a >= DBL_MIN && a <= DBL_MAX;
}
SGX_HD bool bad_value(double v) {
  return !((v == 0.0) || (is_normal_d(1.0e10 * v) && is_normal_d(v)));
}
// bad_value(double(v)) for a float v, without the conversion: only an
// infinite or NaN float is bad once widened.
SGX_HD bool mix_bad_f(float v) { return !(v - v == 0.0f); }

// ---------------------------------------------------------------------------
// NQT order-2 transforms (base/fast-math/logs.hpp:188-214, 282-292): an
// integer-aliased quadratic approximation of log2 and its exact inverse.
// Bit-exact on host and device.
SGX_HD int64_t as_i64(double x) {
#if defined(__CUDA_ARCH__)
  return __double_as_longlong(x);
#else
  int64_t i;
  __builtin_memcpy(&i, &x, 8);
  return i;
#endif
}
SGX_HD double as_f64(int64_t i) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double(i);
#else
  double x;
  __builtin_memcpy(&x, &i, 8);
  return x;
#endif
}

namespace nqt {
constexpr int64_t one = 1;
constexpr int64_t one_as_int = (one << 62) - (one << 52);
constexpr double scale_down = 2.22044604925031e-16;
constexpr double scale_up = static_cast<double>(one << 52);
constexpr int64_t mantissa_mask = (one << 52) - one;
constexpr int64_t low_mask = (one << 26) - 1;
constexpr double log2_over_log10 = 0.301029995663981195;
constexpr double log10_over_log2 = 3.321928094887362626;
} // namespace nqt

SGX_HD double lg_nqt(double x) {
  using namespace nqt;
  const int64_t x_as_int = as_i64(x) - one_as_int;
  const int64_t frac_as_int = x_as_int & mantissa_mask;
  const int64_t frac_high = frac_as_int >> 26;
  const int64_t frac_low = frac_as_int & low_mask;
  const int64_t frac_squared = frac_high * frac_high + ((frac_high * frac_low) >> 25);
  return static_cast<double>(x_as_int + ((frac_as_int - frac_squared) / 3)) * scale_down;
}
SGX_HD double pow2_nqt(double x) {
  using namespace nqt;
  constexpr int64_t a = 9007199254740992;
  constexpr double b = 67108864;
  constexpr int64_t c = 18014398509481984;
  const int64_t x_as_int = static_cast<int64_t>(x * scale_up);
  const int64_t frac_as_int = x_as_int & mantissa_mask;
#if defined(__CUDA_ARCH__)
  const double sq = __dsqrt_rn(static_cast<double>(c - 3 * frac_as_int));
#else
  const double sq = __builtin_sqrt(static_cast<double>(c - 3 * frac_as_int));
#endif
  const int64_t frac_sqrt = static_cast<int64_t>(b * sq);
  return as_f64(x_as_int + a - frac_sqrt - frac_as_int + one_as_int);
}
// lg_nqt's integer x_as_int + (frac - frac_squared) / 3 on the bits of x,
// bit for bit, in 32-bit pieces: frac_high and frac_low are below 2^26,
// and frac - frac_squared lies in [0, 2^52) (frac_squared <= frac^2 2^-52
// <= frac), so the signed division is a floor, taken on the two 26-bit
// halves by floor(n / 3) = (n * 0xAAAAAAAB) >> 33 (exact for every 32-bit
// n). lg_nqt(x) is this value times scale_down.
SGX_HD int64_t lg_nqt_int(const double x) {
  using namespace nqt;
  const int64_t x_as_int = as_i64(x) - one_as_int;
  const uint64_t frac = static_cast<uint64_t>(x_as_int & mantissa_mask);
  const uint32_t fh = static_cast<uint32_t>(frac >> 26);
  const uint32_t fl = static_cast<uint32_t>(frac) & 0x3ffffffu;
  const uint64_t fsq = static_cast<uint64_t>(fh) * fh + ((static_cast<uint64_t>(fh) * fl) >> 25);
  const uint64_t d = frac - fsq;
  const uint32_t dh = static_cast<uint32_t>(d >> 26);
  const uint32_t qh = static_cast<uint32_t>((static_cast<uint64_t>(dh) * 0xAAAAAAABu) >> 33);
  const uint32_t rl = ((dh - 3u * qh) << 26) | (static_cast<uint32_t>(d) & 0x3ffffffu);
  const uint32_t ql = static_cast<uint32_t>((static_cast<uint64_t>(rl) * 0xAAAAAAABu) >> 33);
  return x_as_int + static_cast<int64_t>((static_cast<uint64_t>(qh) << 26) + ql);
}
SGX_HD double log10_nqt(double x) { return nqt::log2_over_log10 * lg_nqt(x); }
SGX_HD double pow10_nqt(double x) { return pow2_nqt(nqt::log10_over_log2 * x); }

// spiner_common::to_log / from_log (eos_spiner_common.hpp:52-57).
SGX_HD double to_log(double x, double offset) {
  return log10_nqt(sabs(smax(x, -offset) + offset) + lim<double>::eps);
}
SGX_HD double from_log(double lx, double offset) { return pow10_nqt(lx) - offset; }

// ---------------------------------------------------------------------------
// Kahan-Neumaier sum over a register array, skipping index `iskip`
// (mix_impl::sum_neumaier, mixed_cell_models.hpp:287-305).
template <typename T, int N>
SGX_HD T sum_neumaier(const T (&d)[N], int n, int offset = 0, int iskip = -1) {
  T sum = 0, c = 0;
  for (int i = 0; i < n; ++i) {
    if (iskip >= 0 && i == iskip) continue;
    const T x = d[i + offset];
    const T t = sum + x;
    if (sabs(sum) >= sabs(x))
      c += (sum - t) + x;
    else
      c += (x - t) + sum;
    sum = t;
  }
  return sum + c;
}
// Same, summing squares.
template <typename T, int N>
SGX_HD T sum_neumaier_sq(const T (&d)[N], int n, int offset = 0) {
  T sum = 0, c = 0;
  for (int i = 0; i < n; ++i) {
    const T x = d[i + offset] * d[i + offset];
    const T t = sum + x;
    if (sabs(sum) >= sabs(x))
      c += (sum - t) + x;
    else
      c += (x - t) + sum;
    sum = t;
  }
  return sum + c;
}

// ---------------------------------------------------------------------------
// Root finding (base/root-finding-1d/root_finding.hpp).
enum class RootStatus : int { SUCCESS = 0, FAIL = 1 };

SGX_HD bool check_bracket(double ya, double yb) { return ya * yb <= 0.0; }

// set_bracket (root_finding.hpp:118-151): scans 1,2,4,...,32 midpoints.
template <typename F>
SGX_HD bool set_bracket(const F &f, double &a, const double guess, double &b, double &ya,
                        const double yg, double &yb) {
  const double dx = b - a;
  for (int level = 0; level < 6; level++) {
    const int nlev = 1 << level;
    for (int i = 0; i < nlev; i++) {
      const double x = a + (i + 0.5) * dx;
      const double yx = f(x);
      if (check_bracket(yx, yg)) {
        if (x < guess) {
          a = x;
          ya = yx;
          b = guess;
          yb = yg;
        } else {
          a = guess;
          ya = yg;
          b = x;
          yb = yx;
        }
        return true;
      }
    }
  }
  return false;
}

// regula_falsi with Illinois halving (root_finding.hpp:154-240). Solves
// f(x) = ytarget; on exit xroot = (a + b) / 2 of the final bracket.
// max_iter is the reference's SECANT_NITER_MAX (1000); `iters` receives the
// iteration count.
template <typename F>
SGX_HD RootStatus regula_falsi(const F &f, const double ytarget, const double guess,
                               double a, double b, const double xtol, const double ytol,
                               double &xroot, int *iters = nullptr) {
  constexpr int max_iter = 1000;
  auto func = [&](const double x) { return f(x) - ytarget; };
  double ya = func(a);
  double yg = func(guess);
  double yb;
  if (check_bracket(ya, yg)) {
    b = guess;
    yb = yg;
  } else {
    yb = func(b);
    if (check_bracket(yg, yb)) {
      a = guess;
      ya = yg;
    } else {
      if (!set_bracket(func, a, guess, b, ya, yg, yb)) {
        if (iters) *iters = 0;
        return RootStatus::FAIL;
      }
    }
  }
  const double sign = (ya < 0 ? 1.0 : -1.0);
  ya *= sign;
  yb *= sign;
  int b1 = 0, b2 = 0, iteration_count = 0;
  while (b - a > 2.0 * xtol && (sabs(ya) > ytol || sabs(yb) > ytol) &&
         iteration_count < max_iter) {
    const double c = (a * yb - b * ya) / (yb - ya);
    if (c == a) {
      b = a;
      continue;
    } else if (c == b) {
      a = b;
      continue;
    }
    const double yc = sign * func(c);
    if (yc > 0.0) {
      b = c;
      yb = yc;
      b1++;
      ya *= (b1 > 1 ? 0.5 : 1.0);
      b2 = 0;
    } else if (yc < 0.0) {
      a = c;
      ya = yc;
      b2++;
      yb *= (b2 > 1 ? 0.5 : 1.0);
      b1 = 0;
    } else {
      a = c;
      b = c;
    }
    iteration_count++;
  }
  if (iters) *iters = iteration_count;
  xroot = 0.5 * (a + b);
  return iteration_count == max_iter ? RootStatus::FAIL : RootStatus::SUCCESS;
}

SGX_HD bool nan_or_inf(const double x) { return x != x || sabs(x) > DBL_MAX; }

// secant (root_finding.hpp:379-472): central-difference Newton steps,
// clamped to [xmin, xmax], up to SECANT_NITER_MAX (1000) iterations.
template <typename F>
SGX_HD RootStatus secant(const F &f, const double ytarget, const double xguess,
                         const double xmin, const double xmax, const double xtol,
                         const double ytol, double &xroot) {
  double x = xguess, x_last = xguess;
  for (int iter = 0; iter < 1000; ++iter) {
    x_last = x;
    const double dx = sabs(1.e-7 * x) + xtol;
    const double y = f(x) - ytarget;
    const double yp = f(x + dx);
    const double ym = f(x - dx);
    const double dyNum = yp - ym;
    const double dyDen = (2. * dx);
    const double dy = dyNum / dyDen;
    x -= y / dy;
    if (x < xmin) x = xmin;
    if (x > xmax) x = xmax;
    if (nan_or_inf(x)) return RootStatus::FAIL;
    if (sabs(x - x_last) / (sabs(x) + xtol) < xtol) break;
  }
  xroot = x;
  const double y = f(x);
  const double frac_error = sabs(y - ytarget) / (sabs(y) + ytol);
  const bool failed =
      sabs(x - x_last) > xtol || sabs(frac_error) > ytol || nan_or_inf(x);
  return failed ? RootStatus::FAIL : RootStatus::SUCCESS;
}

// bisect (root_finding.hpp:474-596): grows a bracket around the guess by
// 1 % steps (x1.1 each, up to BISECT_REG_MAX = 1000), then halves it up to
// BISECT_NITER_MAX (1000) times.
template <typename F>
SGX_HD RootStatus bisect(const F &f, const double ytarget, const double xguess,
                         const double xmin, const double xmax, const double xtol,
                         const double ytol, double &xroot) {
  double xl = 0, xr = 0, fl = 0, fr = 0;
  double grow = 0.01;
  double x = xguess;
  if (sabs(x) < xtol) x += 2. * xtol;
  for (int i = 0; i < 1000; ++i) {
    const double dx = sabs(grow * x);
    xl = x - dx;
    xr = x + dx;
    fl = f(xl) - ytarget;
    fr = f(xr) - ytarget;
    grow *= 1.1;
    if (fl * fr < 0.0 || xl < xmin || xr > xmax) break;
    if (i > 1000 - 2) return RootStatus::FAIL;
  }
  if (xr > xmax) {
    xr = xmax;
    fr = f(xr) - ytarget;
  }
  if (xl < xmin) {
    xl = xmin;
    fl = f(xl) - ytarget;
  }
  if (fl * fr > 0) {
    xl = xmin;
    fl = f(xl) - ytarget;
    if (fl * fr > 0) {
      xr = xmax;
      fr = f(xr) - ytarget;
      if (fl * fr > 0) return RootStatus::FAIL;
    }
  }
  for (int i = 0; i < 1000; ++i) {
    const double xm = 0.5 * (xl + xr);
    const double fm = f(xm) - ytarget;
    if (fl * fm <= 0) {
      xr = xm;
      fr = fm;
    } else {
      xl = xm;
      fl = fm;
    }
    if (xr - xl < xtol) {
      xroot = 0.5 * (xl + xr);
      return RootStatus::SUCCESS;
    }
  }
  xroot = 0.5 * (xl + xr);
  return RootStatus::FAIL;
}

// findRoot (root_finding.hpp:312-372): the ends first, then secant from the
// guess, then bisection. xroot keeps its value where no stage writes it.
template <typename F>
SGX_HD RootStatus find_root(const F &f, const double ytarget, double xguess, const double xmin,
                            const double xmax, const double xtol, const double ytol,
                            double &xroot) {
  const double fmax = f(xmax);
  const double errmax = sabs(fmax - ytarget) / (sabs(fmax) + ytol);
  if (errmax < ytol) {
    xroot = xmax;
    return RootStatus::SUCCESS;
  }
  const double fmin = f(xmin);
  const double errmin = sabs(fmin - ytarget) / (sabs(fmin) + ytol);
  if (errmin < ytol) {
    xroot = xmin;
    return RootStatus::SUCCESS;
  }
  if (xguess >= xmax) xguess = xmax - xtol;
  if (xguess <= xmin) xguess = xmin + xtol;
  RootStatus status = secant(f, ytarget, xguess, xmin, xmax, xtol, ytol, xroot);
  if (status == RootStatus::SUCCESS) return status;
  status = bisect(f, ytarget, xguess, xmin, xmax, xtol, ytol, xroot);
  if (nan_or_inf(xroot)) return RootStatus::FAIL;
  if (xroot < xmin) return RootStatus::FAIL;
  if (xroot > xmax) return RootStatus::FAIL;
  return status;
}

} // namespace sgx
