// A C++ caller of include/sgx.hpp, built by tests/test_cpp_layer.py: the
// reference's API used as a hydro code would use it, with its own indexer
// types and its own kernel around the per-cell PTE solver.
//
//   hpp_check <dir>
//
// reads <dir>/in_*.bin (raw little-endian arrays written by the test) and
// writes <dir>/out_*.bin:
//   1. StiffGas vector lookups T(rho, sie) and P(rho, sie) through raw device
//      pointers (the library's precompiled kernel) and through a strided
//      indexer type (a kernel instantiated from the header);
//   2. tabulated FillEos (T, P, bmod from rho, sie) with a type-indexed
//      lambda: one VariadicIndexer<LogTemperature, LogDensity> per element,
//      slots in the opposite order to the model's numbering;
//   3. a user kernel that builds PTESolverRhoT per cell over per-cell views of
//      the caller's [nmat][ncell] arrays and runs PTESolver.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "sgx.hpp"

namespace {

std::vector<double> read_f64(const std::string &path) {
  std::vector<double> v;
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f) {
    std::fprintf(stderr, "cannot open %s\n", path.c_str());
    std::exit(2);
  }
  double x;
  while (std::fread(&x, sizeof(x), 1, f) == 1)
    v.push_back(x);
  std::fclose(f);
  return v;
}
template <typename T> void write(const std::string &path, const std::vector<T> &v) {
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f || std::fwrite(v.data(), sizeof(T), v.size(), f) != v.size()) {
    std::fprintf(stderr, "cannot write %s\n", path.c_str());
    std::exit(2);
  }
  std::fclose(f);
}
#define CK(x)                                                                                  \
  do {                                                                                         \
    cudaError_t e_ = (x);                                                                      \
    if (e_ != cudaSuccess) {                                                                   \
      std::fprintf(stderr, "%s: %s\n", #x, cudaGetErrorString(e_));                            \
      std::exit(3);                                                                            \
    }                                                                                          \
  } while (0)

template <typename T> T *to_device(const std::vector<T> &h) {
  T *d = nullptr;
  CK(cudaMalloc(&d, h.size() * sizeof(T) + 8));
  CK(cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
  return d;
}
template <typename T> std::vector<T> to_host(const T *d, size_t n) {
  std::vector<T> h(n);
  CK(cudaMemcpy(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost));
  return h;
}

// A caller-side indexer: every s-th element of a device array.
struct Strided {
  double *p;
  int s;
  __host__ __device__ double &operator[](int i) const { return p[static_cast<long>(i) * s]; }
};

// Material m of cell i in a [nmat][ncell] (cell-fastest) array.
struct CellView {
  double *p;
  long ncell, i;
  __device__ double &operator[](int m) const { return p[m * ncell + i]; }
};

using Lam2 = sgx::IndexerUtils::VariadicIndexer<sgx::IndexableTypes::LogTemperature,
                                                sgx::IndexableTypes::LogDensity>;

__global__ void pte_cells(const sgx::EOS *eos, int nmat, long ncell, const double *vfrac_tot,
                          const double *sie_tot, double *rho, double *vfrac, double *sie,
                          double *temp, double *press, int *conv, int *niter) {
  const long i = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
  if (i >= ncell) return;
  CellView r{rho, ncell, i}, v{vfrac, ncell, i}, s{sie, ncell, i}, t{temp, ncell, i},
      p{press, ncell, i};
  sgx::NullIndexer lam;
  double scratch[sgx::PTESolverRhoTRequiredScratch(6)];
  sgx::PTESolverRhoT method(nmat, eos, vfrac_tot[i], sie_tot[i], r, v, s, t, p, lam, scratch);
  const sgx::SolverStatus st = sgx::PTESolver(method);
  conv[i] = st.converged ? 1 : 0;
  niter[i] = static_cast<int>(st.max_niter);
}

} // namespace

int main(int argc, char **argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: hpp_check <dir> <table.sp5>\n");
    return 1;
  }
  const std::string dir = argv[1];
  try {
    // ---- 1. analytic vector lookups ----
    const sgx::EOS stiff = sgx::EOS::StiffGas(3.4, 1.816e7, 6e9, 0.0);
    const std::vector<double> rho_h = read_f64(dir + "/in_vec_rho.bin");
    const std::vector<double> sie_h = read_f64(dir + "/in_vec_sie.bin");
    const int n = static_cast<int>(rho_h.size());
    double *rho = to_device(rho_h), *sie = to_device(sie_h);
    double *T1, *T2, *P1;
    CK(cudaMalloc(&T1, n * sizeof(double)));
    CK(cudaMalloc(&P1, n * sizeof(double)));
    CK(cudaMalloc(&T2, 2 * n * sizeof(double)));
    CK(cudaMemset(T2, 0, 2 * n * sizeof(double)));
    stiff.TemperatureFromDensityInternalEnergy(rho, sie, T1, n);
    stiff.PressureFromDensityInternalEnergy(rho, sie, P1, nullptr, n);
    stiff.TemperatureFromDensityInternalEnergy(Strided{rho, 1}, Strided{sie, 1},
                                               Strided{T2, 2}, n, sgx::NullIndexer());
    CK(cudaDeviceSynchronize());
    write(dir + "/out_vec_T.bin", to_host(T1, n));
    write(dir + "/out_vec_P.bin", to_host(P1, n));
    write(dir + "/out_vec_T_strided.bin", to_host(T2, 2 * n));

    // ---- 2. tabulated FillEos with type-indexed lambda rows ----
    sgx::EOS tab = sgx::EOS::SpinerEOSDependsRhoT(argv[2], 1);
    const std::vector<double> trho_h = read_f64(dir + "/in_tab_rho.bin");
    const std::vector<double> tsie_h = read_f64(dir + "/in_tab_sie.bin");
    const int nt = static_cast<int>(trho_h.size());
    double *trho = to_device(trho_h), *tsie = to_device(tsie_h);
    std::vector<double> zeros(nt, 0.0);
    double *tT = to_device(zeros), *tP = to_device(zeros), *tcv = to_device(zeros),
           *tB = to_device(zeros);
    std::vector<Lam2> lam_h(nt);
    for (auto &l : lam_h) {
      l[sgx::IndexableTypes::LogTemperature{}] = 1e300; // out of range: no guess
      l[sgx::IndexableTypes::LogDensity{}] = 0.0;
    }
    Lam2 *lam = to_device(lam_h);
    tab.FillEos(trho, tT, tsie, tP, tcv, tB, nt,
                SGX_Q_TEMPERATURE | SGX_Q_PRESSURE | SGX_Q_BULK_MODULUS, lam);
    CK(cudaDeviceSynchronize());
    write(dir + "/out_tab_T.bin", to_host(tT, nt));
    write(dir + "/out_tab_P.bin", to_host(tP, nt));
    write(dir + "/out_tab_B.bin", to_host(tB, nt));
    std::vector<Lam2> lam_out = to_host(lam, nt);
    std::vector<double> lrho(nt), lT(nt);
    for (int k = 0; k < nt; ++k) {
      lrho[k] = lam_out[k][sgx::IndexableTypes::LogDensity{}];
      lT[k] = lam_out[k][sgx::IndexableTypes::LogTemperature{}];
    }
    write(dir + "/out_tab_lrho.bin", lrho);
    write(dir + "/out_tab_lT.bin", lT);
    tab.Finalize();

    // ---- 3. per-cell PTE in the caller's kernel ----
    const std::vector<double> prho = read_f64(dir + "/in_pte_rho.bin");
    const std::vector<double> pvf = read_f64(dir + "/in_pte_vfrac.bin");
    const std::vector<double> pst = read_f64(dir + "/in_pte_sie_tot.bin");
    const std::vector<double> pvt = read_f64(dir + "/in_pte_vfrac_tot.bin");
    const long nc = static_cast<long>(pst.size());
    const int nmat = static_cast<int>(prho.size() / nc);
    std::vector<sgx::EOS> eos_h = {sgx::EOS::IdealGas(0.4, 0.718e7), stiff};
    sgx::EOS *eos = to_device(eos_h);
    std::vector<double> zc(nmat * nc, 0.0);
    double *d_rho = to_device(prho), *d_vf = to_device(pvf), *d_sie = to_device(zc),
           *d_T = to_device(zc), *d_P = to_device(zc), *d_st = to_device(pst),
           *d_vt = to_device(pvt);
    int *d_conv, *d_nit;
    CK(cudaMalloc(&d_conv, nc * sizeof(int)));
    CK(cudaMalloc(&d_nit, nc * sizeof(int)));
    pte_cells<<<static_cast<unsigned>((nc + 127) / 128), 128>>>(
        eos, nmat, nc, d_vt, d_st, d_rho, d_vf, d_sie, d_T, d_P, d_conv, d_nit);
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    write(dir + "/out_pte_rho.bin", to_host(d_rho, nmat * nc));
    write(dir + "/out_pte_vfrac.bin", to_host(d_vf, nmat * nc));
    write(dir + "/out_pte_sie.bin", to_host(d_sie, nmat * nc));
    write(dir + "/out_pte_temp.bin", to_host(d_T, nmat * nc));
    write(dir + "/out_pte_press.bin", to_host(d_P, nmat * nc));
    write(dir + "/out_pte_conv.bin", to_host(d_conv, nc));
    write(dir + "/out_pte_niter.bin", to_host(d_nit, nc));
  } catch (const std::exception &ex) {
    std::fprintf(stderr, "sgx: %s\n", ex.what());
    return 4;
  }
  std::printf("hpp_check: ok\n");
  return 0;
}
