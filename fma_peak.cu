// fma_peak: measures the FP64 and FP32 FMA throughput of the current
// device (a benchmark probe beside bench.py, not part of the library): the
// denominators of the pipe fractions bench.py reports for the
// FP64-bound closure kernels (HBM bandwidth comes from a copy measurement).
//
// Each thread runs 8 independent FMA chains for `iters` rounds; a grid of
// 8 blocks of 256 threads per SM keeps every scheduler issuing. Timed with
// CUDA events after one warm-up launch; prints one JSON line:
//   {"fp64_tflops": .., "fp32_tflops": .., "sms": .., "sm_clock_mhz": ..}
#include <cstdio>

#include <cuda_runtime.h>

namespace {

template <typename T>
__global__ void __launch_bounds__(256) fma_chains(T *out, const int iters, const T a,
                                                  const T b) {
  T x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k)
    x[k] = static_cast<T>(threadIdx.x + k);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k)
      x[k] = fma(x[k], a, b);
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k)
    s += x[k];
  // a = 1, b = 0 at run time: the value is unchanged, but the compiler
  // cannot know that, and the store below is never taken
  if (s == static_cast<T>(-1.2345)) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T> double measure(const int sms, const int iters) {
  const int blocks = sms * 8, threads = 256;
  T *out = nullptr;
  if (cudaMalloc(&out, sizeof(T) * blocks * threads) != cudaSuccess) return -1;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fma_chains<T><<<blocks, threads>>>(out, iters, T(1), T(0));
  cudaEventRecord(e0);
  fma_chains<T><<<blocks, threads>>>(out, iters, T(1), T(0));
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  const cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess || ms <= 0) return -1;
  const double flops = 2.0 * 8.0 * iters * static_cast<double>(blocks) * threads;
  return flops / (ms * 1e-3) / 1e12;
}

} // namespace

int main() {
  int dev = 0, sms = 0, clk_khz = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&clk_khz, cudaDevAttrClockRate, dev);
  // about 0.1-0.3 s per measurement on a GB300
  const double fp64 = measure<double>(sms, 1 << 14);
  const double fp32 = measure<float>(sms, 1 << 18);
  if (fp64 <= 0 || fp32 <= 0) return 2;
  std::printf("{\"fp64_tflops\": %.4f, \"fp32_tflops\": %.4f, \"sms\": %d, "
              "\"sm_clock_mhz\": %.0f}\n",
              fp64, fp32, sms, clk_khz / 1e3);
  return 0;
}
