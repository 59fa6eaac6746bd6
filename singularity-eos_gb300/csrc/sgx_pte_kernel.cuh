// The per-cell PTE kernel of the plain FP64 path, templated on the number of
// materials N present in a cell. One launch per N covers the cells that hold
// exactly N materials, taken from their segment of the binned cell ids (by
// count and EOS-kind signature, so a warp runs one system size and mostly
// one set of EOS branches); each instantiation is compiled in its own
// translation unit.
//
// One thread per cell: gather the cell's materials, run one of the solvers
// (PTESolverRhoT, PTESolverPT, PTESolverFixedT, PTESolverFixedP,
// PTESolverRhoU; closure/mixed_cell_models.hpp:884-2183) through PTESolver()
// (:2188-2291), scatter the equilibrium state. The per-cell target array
// carries the solver's scalar constructor argument: sie_tot for RhoT, PT and
// RhoU, T_true for FixedT, P for FixedP. get_sg_eos_rho_e.cpp:30-88 is
// the reference's per-cell loop.
#pragma once

#include <cuda_runtime.h>

#include "sgx_internal.h"
#include "sgx_pte.cuh"

// The plain FP64 path is built twice: for lists that hold a modified EOS
// (the modifier arithmetic of sgx_dispatch.cuh compiled in) and, with
// SGX_BARE_MODELS defined, for lists of bare models, whose kernels carry no
// modifier code (it costs the bare kernels registers and 5-9% of their
// speed). The kernels live in the dispatch's inline namespace; the
// launchers get a _bare suffix in the second build.
#ifdef SGX_BARE_MODELS
#define SGX_PTE_LAUNCHER(name) name##_bare
#else
#define SGX_PTE_LAUNCHER(name) name
#endif

namespace sgx {
SGX_DISPATCH_BEGIN

constexpr int PTE_BLOCK = 128;

// Collects the present materials of cell i; returns their count.
__device__ __forceinline__ int pte_gather(const PteArgs &a, long long i, int (&slot)[MAX_NMAT],
                                          int (&eidx)[MAX_NMAT]) {
  int n = 0;
  for (int m = 0; m < a.nmat; ++m) {
    const int ie = a.eos_idx ? a.eos_idx[static_cast<long long>(m) * a.ncell + i] : m;
    if (ie < 0 || ie >= a.neos) continue;
    slot[n] = m;
    eidx[n] = ie;
    ++n;
  }
  return n;
}

// Where the cells with N materials start in perm[] (and in retry_idx[]):
// the sum of the smaller counts (0 without an index map).
template <int N> __device__ __forceinline__ unsigned pte_bin_offset(const PteArgs &a) {
  if (!a.perm) return 0;
  unsigned off = 0;
#pragma unroll
  for (int n = 0; n < N; ++n)
    off += a.bins[n];
  return off;
}

// Cell id of the t-th cell with N materials (false past the bin's end).
template <int N> __device__ __forceinline__ bool pte_bin_cell(const PteArgs &a, long long t,
                                                              long long &i) {
  if (!a.perm) {
    i = t;
    return t < a.ncell;
  }
  if (t >= a.bins[N]) return false;
  i = a.perm[pte_bin_offset<N>(a) + t];
  return true;
}

// True for a whole block past the end of the N-bin: it leaves before
// staging the EOS list (launches are sized for every cell, the bin is not).
template <int N> __device__ __forceinline__ bool pte_block_idle(const PteArgs &a) {
  return a.perm && static_cast<long long>(blockIdx.x) * blockDim.x >= a.bins[N];
}

template <template <typename, int> class Solver, int N>
__global__ void __launch_bounds__(PTE_BLOCK) pte_cell_kernel(const PteArgs a) {
  if (pte_block_idle<N>(a)) return;
  __shared__ sgx_eos s_eos[MAX_EOS];
  for (int k = threadIdx.x; k < a.neos; k += blockDim.x)
    s_eos[k] = a.eos[k];
  __syncthreads();
  long long i;
  if (!pte_bin_cell<N>(a, static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x, i))
    return;
  int slot[MAX_NMAT], eidx[MAX_NMAT];
  if (pte_gather(a, i, slot, eidx) != N) return;
  const MixP<double> mp(a.params);
  const long long nc = a.ncell;
  Solver<double, N> s;
  double cache[N][3];
  s.P = &mp;
  s.vfrac_total = a.vfrac_tot[i];
  s.configure(a.sie_tot[i]);
  s.err_flags = 0;
  for (int q = 0; q < N; ++q) {
    const long long k = static_cast<long long>(slot[q]) * nc + i;
    s.eos[q] = &s_eos[eidx[q]];
    s.rho[q] = a.rho[k];
    s.vfrac[q] = a.vfrac[k];
    s.sie[q] = a.sie[k];
    s.temp[q] = a.temp[k];
    s.press[q] = a.press[k];
    for (int l = 0; l < 3; ++l)
      cache[q][l] = a.lambda ? a.lambda[(static_cast<long long>(slot[q]) * 3 + l) * nc + i] : 0.0;
    s.lam[q] = cache[q];
  }
  const PteStatusLocal st = pte_solve<Solver<double, N>, double>(s);
  for (int q = 0; q < N; ++q) {
    const long long k = static_cast<long long>(slot[q]) * nc + i;
    a.rho[k] = s.rho[q];
    a.vfrac[k] = s.vfrac[q];
    a.sie[k] = s.sie[q];
    a.temp[k] = s.temp[q];
    a.press[k] = s.press[q];
    if (a.lambda)
      for (int l = 0; l < 3; ++l)
        a.lambda[(static_cast<long long>(slot[q]) * 3 + l) * nc + i] = cache[q][l];
  }
  if (a.status) {
    sgx_pte_status o;
    o.residual = st.residual;
    o.niter = st.niter;
    o.converged = st.converged ? 1 : 0;
    o.slow_convergence_detected = st.slow ? 1 : 0;
    o.max_line_niter = static_cast<uint8_t>(st.max_line_niter);
    o.small_step_iters =
        static_cast<uint8_t>((st.small_step_iters & 0x3F) | (s.err_flags ? 0x80 : 0));
    a.status[i] = o;
  }
}

} // inline namespace

template <int N>
cudaError_t SGX_PTE_LAUNCHER(launch_pte_fp64_n)(const PteArgs &a, cudaStream_t stream) {
  const long long blocks = (a.ncell + PTE_BLOCK - 1) / PTE_BLOCK;
  if (a.solver == SGX_PTE_PT)
    pte_cell_kernel<PtePT, N><<<static_cast<unsigned>(blocks), PTE_BLOCK, 0, stream>>>(a);
  else
    pte_cell_kernel<PteRhoT, N><<<static_cast<unsigned>(blocks), PTE_BLOCK, 0, stream>>>(a);
  return cudaGetLastError();
}

// The three solvers beyond RhoT and PT, compiled in their own translation
// units (sgx_pte_ext_n.cu).
template <int N>
cudaError_t SGX_PTE_LAUNCHER(launch_pte_ext_n)(const PteArgs &a, cudaStream_t stream) {
  const long long blocks = (a.ncell + PTE_BLOCK - 1) / PTE_BLOCK;
  const unsigned g = static_cast<unsigned>(blocks);
  switch (a.solver) {
  case SGX_PTE_FIXED_T: pte_cell_kernel<PteFixedT, N><<<g, PTE_BLOCK, 0, stream>>>(a); break;
  case SGX_PTE_FIXED_P: pte_cell_kernel<PteFixedP, N><<<g, PTE_BLOCK, 0, stream>>>(a); break;
  case SGX_PTE_RHOU: pte_cell_kernel<PteRhoU, N><<<g, PTE_BLOCK, 0, stream>>>(a); break;
  default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

} // namespace sgx
