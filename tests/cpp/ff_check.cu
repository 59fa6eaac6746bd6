// Device check of sgx_ff.cuh's conversions between float-float and double:
// ff2d(hi, lo) against the FP64 sum (double)hi + (double)lo over seeded
// pairs of every magnitude, unnormalised pairs, exact powers of two with a
// low part of the opposite sign, zero and subnormal low parts; ff2d_add
// bit for bit against the correctly rounded FP64 sum; d2ff round trips; the
// NQT log's integer core in 32-bit pieces (lg_nqt_int) against
// the reference's 64-bit formula (logs.hpp:188-200), bit for bit. Prints
// "bad=<count>"; run by tests/test_gpu_ff.py.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include <cuda_runtime.h>

#include "sgx_ff.cuh"
#include "sgx_math.cuh"

__global__ void conv(const float *hi, const float *lo, const double *d, double *out, double *rt,
                     double *add, const int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = sgx::ff2d(sgx::ff_make(hi[i], lo[i]));
  rt[i] = sgx::ff2d(sgx::d2ff(d[i]));
  add[i] = sgx::ff2d_add(sgx::ff_make(hi[i], lo[i]));
}

__global__ void lgint(const double *x, long long *out, const int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = sgx::lg_nqt_int(x[i]);
}

static double ulp(const double x) {
  return std::nextafter(std::fabs(x), INFINITY) - std::fabs(x);
}

int main() {
  const int n = 1 << 20;
  std::mt19937_64 g(7);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  std::vector<float> hi(n), lo(n);
  std::vector<double> d(n);
  for (int i = 0; i < n; ++i) {
    const int kind = i % 8;
    const int e = static_cast<int>(g() % 200) - 100;
    float h = static_cast<float>(std::ldexp(1.0 + std::fabs(u(g)), e)) * (u(g) < 0 ? -1.f : 1.f);
    float l;
    if (kind == 0) l = 0.0f;
    else if (kind == 1) { h = std::ldexp(1.0f, e) * (u(g) < 0 ? -1.f : 1.f); l = -h * static_cast<float>(std::fabs(u(g))) * 5.9604645e-8f; }
    else if (kind == 2) l = h * static_cast<float>(u(g)) * 1e-3f; // unnormalised
    else if (kind == 3) l = std::ldexp(1.0f, -140) * static_cast<float>(u(g)); // subnormal low part
    else l = h * static_cast<float>(u(g)) * 5.9604645e-8f;
    hi[i] = h;
    lo[i] = l;
    // inside d2ff's range (binary exponents -74..127)
    d[i] = std::ldexp(0.5 + 0.5 * std::fabs(u(g)), static_cast<int>(g() % 190) - 70) *
           (u(g) < 0 ? -1.0 : 1.0);
  }
  float *dh, *dl;
  double *dd, *dout, *drt, *dadd;
  cudaMalloc(&dh, n * 4);
  cudaMalloc(&dl, n * 4);
  cudaMalloc(&dd, n * 8);
  cudaMalloc(&dout, n * 8);
  cudaMalloc(&drt, n * 8);
  cudaMalloc(&dadd, n * 8);
  cudaMemcpy(dh, hi.data(), n * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(dl, lo.data(), n * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(dd, d.data(), n * 8, cudaMemcpyHostToDevice);
  conv<<<(n + 255) / 256, 256>>>(dh, dl, dd, dout, drt, dadd, n);
  std::vector<double> out(n), rt(n), add(n);
  if (cudaMemcpy(out.data(), dout, n * 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(rt.data(), drt, n * 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(add.data(), dadd, n * 8, cudaMemcpyDeviceToHost) != cudaSuccess) {
    std::printf("cuda error\n");
    return 2;
  }
  long bad = 0;
  for (int i = 0; i < n; ++i) {
    const double want = double(hi[i]) + double(lo[i]);
    // ff2d_add: the correctly rounded sum, a subnormal part counting as 0
    const double want_add = (std::fpclassify(lo[i]) == FP_SUBNORMAL ? 0.0 : double(lo[i])) +
                            (std::fpclassify(hi[i]) == FP_SUBNORMAL ? 0.0 : double(hi[i]));
    if (std::memcmp(&want_add, &add[i], 8) != 0) {
      if (bad < 5) std::printf("ff2d_add %a %a -> %a want %a\n", hi[i], lo[i], add[i], want_add);
      ++bad;
    }
    if (!(std::fabs(out[i] - want) <= ulp(want))) {
      if (bad < 5) std::printf("ff2d %a %a -> %a want %a\n", hi[i], lo[i], out[i], want);
      ++bad;
    }
    // d2ff keeps ~48 bits: the round trip within 2^-47 relative
    if (!(std::fabs(rt[i] - d[i]) <= std::ldexp(std::fabs(d[i]), -47))) {
      if (bad < 5) std::printf("round trip %a -> %a\n", d[i], rt[i]);
      ++bad;
    }
  }
  // lg_nqt_int over positive normal doubles of every exponent
  for (int i = 0; i < n; ++i) {
    uint64_t b = g() & 0x7fefffffffffffffULL;
    if ((b >> 52) == 0) b |= 1ULL << 52;
    std::memcpy(&d[i], &b, 8);
  }
  long long *dl_out;
  cudaMalloc(&dl_out, n * 8);
  cudaMemcpy(dd, d.data(), n * 8, cudaMemcpyHostToDevice);
  lgint<<<(n + 255) / 256, 256>>>(dd, dl_out, n);
  std::vector<long long> li(n);
  if (cudaMemcpy(li.data(), dl_out, n * 8, cudaMemcpyDeviceToHost) != cudaSuccess) {
    std::printf("cuda error\n");
    return 2;
  }
  for (int i = 0; i < n; ++i) {
    int64_t xb;
    std::memcpy(&xb, &d[i], 8);
    const int64_t x_as_int = xb - sgx::nqt::one_as_int;
    const int64_t frac = x_as_int & sgx::nqt::mantissa_mask;
    const int64_t fh = frac >> 26, fl = frac & sgx::nqt::low_mask;
    const int64_t want = x_as_int + (frac - (fh * fh + ((fh * fl) >> 25))) / 3;
    if (li[i] != want) {
      if (bad < 5) std::printf("lg_nqt_int %a -> %lld want %lld\n", d[i], li[i], (long long)want);
      ++bad;
    }
  }
  std::printf("bad=%ld\n", bad);
  return bad != 0;
}
