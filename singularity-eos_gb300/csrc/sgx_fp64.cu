// FP64 kernels of the plain path: the vector EOS lookups and the dispatch of
// the per-cell PTE kernels (one instantiation per material count, built from
// sgx_pte_fp64_n.cu). Compiled with --fmad=false so that every expression
// rounds exactly as the reference does when built without FP contraction.
//
//   eval_kernel      the EosBase vector overloads (eos/eos_base.hpp:169-230)
//   fill_kernel      vector FillEos (eos/eos_base.hpp:503-531)
//   pt_derivs_kernel PTDerivativesFromPreferred per element (eos_base.hpp:410-419)
//   spiner_fill_ref  tabulated FillEos for the elements the mixed-precision
//                    lookup (sgx_lookup_mixed.cu) leaves to FP64
#include <cuda_runtime.h>

#include "sgx_internal.h"
#include "sgx_dispatch.cuh"

namespace sgx {

template <int N> cudaError_t launch_pte_fp64_n(const PteArgs &a, cudaStream_t stream);
template <int N> cudaError_t launch_pte_fp64_n_bare(const PteArgs &a, cudaStream_t stream);
template <int N> cudaError_t launch_pte_ext_n(const PteArgs &a, cudaStream_t stream);

namespace {

using PteLauncher = cudaError_t (*)(const PteArgs &, cudaStream_t);

template <int N> PteLauncher pte_launcher_n(const bool ext, const bool mods) {
  if (ext) return launch_pte_ext_n<N>;
  return mods ? launch_pte_fp64_n<N> : launch_pte_fp64_n_bare<N>;
}
PteLauncher pte_launcher(const int n, const bool ext, const bool mods) {
  switch (n) {
  case 1: return pte_launcher_n<1>(ext, mods);
  case 2: return pte_launcher_n<2>(ext, mods);
  case 3: return pte_launcher_n<3>(ext, mods);
  case 4: return pte_launcher_n<4>(ext, mods);
  case 5: return pte_launcher_n<5>(ext, mods);
  default: return pte_launcher_n<6>(ext, mods);
  }
}

__global__ void eval_kernel(const EvalArgs a) {
  const sgx_eos e = a.eos;
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < a.n;
       i += stride) {
    double *lam = a.lambda ? a.lambda + i * a.lambda_stride : nullptr;
    const double b = a.in2 ? a.in2[i] : 0.0;
    a.out[i] = ev_eval(e, a.fn, a.in1[i], b, lam);
  }
}

// The bounds introspection members (eos_base.hpp:533-560 and the models'
// overrides), one value per element; x is the temperature of
// MaximumPressureAtTemperature and RhoPmin, unused by the others.
__global__ void bounds_kernel(const sgx_eos e, const int what, const long long n,
                              const double *x, double *out) {
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += stride) {
    int err = 0;
    double v = 0.0;
    switch (what) {
    case SGX_BOUND_MIN_DENSITY: v = ev_min_density(e); break;
    case SGX_BOUND_MIN_TEMPERATURE: v = ev_min_temperature(e); break;
    case SGX_BOUND_MAX_DENSITY: v = ev_max_density(e); break;
    case SGX_BOUND_MIN_PRESSURE: v = ev_min_pressure(e); break;
    case SGX_BOUND_MAX_PRESSURE_AT_T: v = ev_max_pressure_at_T(e, x[i], &err); break;
    default: v = ev_rho_pmin(e, x[i]); break;
    }
    out[i] = v;
  }
}

__global__ void fill_kernel(const FillArgs a) {
  const sgx_eos e = a.eos;
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  int bad = 0;
  for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < a.n;
       i += stride) {
    double rho = a.rho ? a.rho[i] : 0.0;
    double temp = a.temp ? a.temp[i] : 0.0;
    double sie = a.sie ? a.sie[i] : 0.0;
    double press = a.press ? a.press[i] : 0.0;
    double cv = 0.0, bmod = 0.0;
    if (e.mods) {
      cv = a.cv ? a.cv[i] : 0.0;
      bmod = a.bmod ? a.bmod[i] : 0.0;
    }
    double *lam = a.lambda ? a.lambda + i * a.lambda_stride : nullptr;
    int err = 0;
    ev_fill(e, rho, temp, sie, press, cv, bmod, a.output | (a.cs ? Q_BMOD : 0u), lam, &err);
    bad |= err;
    if (a.cs) a.cs[i] = sqrt(bmod / rho);
    // The reference's FillEos takes every quantity by reference; a modifier
    // can write one that is not an output (ShiftedEOS adds its shift to an
    // input sie of a rho-T model, BilinearRampEOS always rewrites bmod), so
    // a modified EOS writes back every array it was given.
    const unsigned wb = e.mods ? ~0u : a.output;
    if ((wb & Q_DENSITY) && a.rho) a.rho[i] = rho;
    if ((wb & Q_TEMPERATURE) && a.temp) a.temp[i] = temp;
    if ((wb & Q_SIE) && a.sie) a.sie[i] = sie;
    if ((wb & Q_PRESSURE) && a.press) a.press[i] = press;
    if ((wb & Q_CV) && a.cv) a.cv[i] = cv;
    if ((wb & Q_BMOD) && a.bmod) a.bmod[i] = bmod;
  }
  if (bad && a.err) atomicOr(a.err, 1);
}

__global__ void pt_derivs_kernel(const PtDerivArgs a) {
  const sgx_eos e = a.eos;
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < a.n;
       i += stride) {
    double *lam = a.lambda ? a.lambda + i * a.lambda_stride : nullptr;
    double d0, d1, d2, d3;
    int err = 0;
    ev_pt_derivs(e, a.rho[i], a.sie[i], a.press[i], a.temp[i], lam, d0, d1, d2, d3, &err);
    a.d[0][i] = d0;
    a.d[1][i] = d1;
    a.d[2][i] = d2;
    a.d[3][i] = d3;
  }
}

// The reference's FP64 path (eos_spiner_rho_temp.hpp:1052-1101) for the
// elements whose bit in `left` is set.
__device__ void ref_element(const SpinerTable &t, const FillArgs &a, const long long e) {
  const unsigned out = a.output;
  const double rho = a.rho[e], sie = a.sie[e];
  double *lam = a.lambda ? a.lambda + e * a.lambda_stride : nullptr;
  const double lRho = sp_lRho(t, rho);
  TableStatus ws;
  const double lT = sp_lT_from_lRho_sie(t, lRho, sie, ws, lam);
  const double temp = sp_T(t, lT);
  ws = sp_loc_rho_T(t, lRho, lT);
  if ((out & Q_TEMPERATURE) && a.temp) a.temp[e] = temp;
  if ((out & Q_PRESSURE) && a.press) a.press[e] = sp_P_from(t, rho, lRho, temp, lT, ws);
  if ((out & Q_CV) && a.cv) a.cv[e] = sp_cv_from(t, lRho, lT, ws);
  if ((out & Q_BMOD) || a.cs) {
    const double bmod = sp_bmod_from(t, rho, lRho, temp, lT, ws);
    if ((out & Q_BMOD) && a.bmod) a.bmod[e] = bmod;
    if (a.cs) a.cs[e] = sqrt(bmod / rho);
  }
  if (lam) {
    lam[0] = lRho;
    lam[1] = lT;
  }
}

// Each block takes REF_WORDS consecutive mask words per round (REF_WORDS
// x 32 elements), lists their set bits in shared memory and then runs the
// list with all its threads, so that a sparse mask still fills the lanes.
constexpr int REF_BLOCK = 256;
constexpr int REF_WPT = 2; // mask words per thread per round
constexpr int REF_WORDS = REF_BLOCK * REF_WPT;

__global__ void __launch_bounds__(REF_BLOCK)
    spiner_fill_ref(const FillArgs a, const unsigned *__restrict__ left) {
  __shared__ SpinerTable st;
  __shared__ unsigned count;
  __shared__ unsigned short list[REF_WORDS * 32]; // element offsets within the round
  if (threadIdx.x == 0) st = sp_table(a.eos);
  const long long nwords = (a.n + 31) >> 5;
  for (long long base = static_cast<long long>(blockIdx.x) * REF_WORDS; base < nwords;
       base += static_cast<long long>(gridDim.x) * REF_WORDS) {
    if (threadIdx.x == 0) count = 0;
    __syncthreads();
    for (int q = 0; q < REF_WPT; ++q) {
      const int wi = q * REF_BLOCK + threadIdx.x;
      const long long w = base + wi;
      unsigned m = w < nwords ? left[w] : 0u;
      if (m) {
        unsigned pos = atomicAdd(&count, static_cast<unsigned>(__popc(m)));
        while (m) {
          const int b = __ffs(m) - 1;
          m &= m - 1;
          list[pos++] = static_cast<unsigned short>(wi * 32 + b);
        }
      }
    }
    __syncthreads();
    const unsigned total = count;
    for (unsigned k = threadIdx.x; k < total; k += REF_BLOCK)
      ref_element(st, a, (base << 5) + list[k]);
    __syncthreads();
  }
}

int grid_for(long long n, int block) {
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long want = (n + block - 1) / block;
  const long long cap = static_cast<long long>(sms) * 16;
  return static_cast<int>(want < cap ? (want > 0 ? want : 1) : cap);
}

} // namespace

cudaError_t launch_pte_fp64_with(const PteArgs &args, unsigned *bins, int *perm,
                                 cudaStream_t stream) {
  if (args.ncell <= 0) return cudaSuccess;
  PteArgs a = args;
  a.perm = nullptr;
  // Without an index map every cell holds exactly nmat materials; with one,
  // the cells are binned by count and EOS-kind signature first
  // (sgx_mixed.cu), so that each per-count kernel runs full warps.
  cudaError_t e = cudaSuccess;
  if (a.eos_idx) {
    a.bins = bins;
    e = cudaMemsetAsync(a.bins, 0, PTE_BINS_BYTES, stream);
    if (e == cudaSuccess) e = launch_pte_binning(a, perm, stream);
    if (e != cudaSuccess) return e;
    a.perm = perm;
  }
  const int lo = a.eos_idx ? 1 : a.nmat;
  const int hi = a.nmat < PTE_MAX_N ? a.nmat : PTE_MAX_N;
  const bool ext = a.solver != SGX_PTE_RHOT && a.solver != SGX_PTE_PT;
  // RhoT and PT over bare models run the build without modifier code
  bool mods = false;
  for (int k = 0; k < a.neos; ++k)
    mods = mods || a.eos[k].mods != 0;
  for (int n = lo; n <= hi && e == cudaSuccess; ++n)
    e = pte_launcher(n, ext, mods)(a, stream);
  return e;
}

cudaError_t launch_pte_fp64(const PteArgs &a, cudaStream_t stream) {
  if (a.ncell <= 0) return cudaSuccess;
  if (!a.eos_idx) return launch_pte_fp64_with(a, nullptr, nullptr, stream);
  if (a.ncell > 0x7fffffffLL) return cudaErrorInvalidValue; // int32 cell ids in perm
  const size_t nb = (PTE_BINS_BYTES + 255) / 256 * 256;
  void *scratch = nullptr;
  cudaError_t e = scratch_alloc(&scratch, nb + static_cast<size_t>(a.ncell) * sizeof(int), stream);
  if (e != cudaSuccess) return e;
  e = launch_pte_fp64_with(a, static_cast<unsigned *>(scratch),
                           reinterpret_cast<int *>(static_cast<char *>(scratch) + nb), stream);
  const cudaError_t f = scratch_free(scratch, stream);
  return e != cudaSuccess ? e : f;
}

cudaError_t launch_bounds_fp64(const sgx_eos &e, const int what, const long long n,
                               const double *x, double *out, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  bounds_kernel<<<grid_for(n, 256), 256, 0, stream>>>(e, what, n, x, out);
  return cudaGetLastError();
}

cudaError_t launch_eval_fp64(const EvalArgs &a, cudaStream_t stream) {
  if (a.n <= 0) return cudaSuccess;
  eval_kernel<<<grid_for(a.n, 256), 256, 0, stream>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_fill_ref(const FillArgs &a, const unsigned *left, cudaStream_t stream) {
  if (a.n <= 0) return cudaSuccess;
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long words = (a.n + 31) >> 5;
  const long long blocks = (words + REF_WORDS - 1) / REF_WORDS;
  const long long cap = static_cast<long long>(sms) * 4;
  spiner_fill_ref<<<static_cast<int>(blocks < cap ? blocks : cap), REF_BLOCK, 0, stream>>>(a,
                                                                                        left);
  return cudaGetLastError();
}

cudaError_t launch_pt_derivs(const PtDerivArgs &a, cudaStream_t stream) {
  if (a.n <= 0) return cudaSuccess;
  pt_derivs_kernel<<<grid_for(a.n, 256), 256, 0, stream>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_fill_fp64(const FillArgs &a, cudaStream_t stream) {
  if (a.n <= 0) return cudaSuccess;
  fill_kernel<<<grid_for(a.n, 256), 256, 0, stream>>>(a);
  return cudaGetLastError();
}

} // namespace sgx
