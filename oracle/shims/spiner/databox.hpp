// spiner-lite: the DataBox / grid surface that singularity-eos's tabulated
// EOS headers use, restated for the host-only oracle build.
//
// TEST INFRASTRUCTURE ONLY. The upstream spiner library (pinned by the
// reference at spiner >= 1.6, cmake/singularity-eos/spiner.cmake:17) is not
// present, so its interpolation is restated here from its published
// behaviour: a uniform grid x_i = min + i*dx, the cell index clamped to
// [0, N-2] (linear extrapolation outside the table), and multilinear
// interpolation with weights w1 = (x - x_i)/dx, w0 = 1 - w1. The GB300
// product implements the same formula with the same operation order, so the
// two agree bit for bit; edge semantics of the real spiner are unpinned.
//
// Index convention (matching the reference's call sites,
// eos_spiner_rho_temp.hpp:603-612): operator()(j, i) is row-major with i
// fastest; range(0) is the grid of the fastest index, dim(1) its size.
#ifndef SGX_ORACLE_SHIM_SPINER_DATABOX_HPP
#define SGX_ORACLE_SHIM_SPINER_DATABOX_HPP

#include <array>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include <ports-of-call/portability.hpp>
#include <ports-of-call/portable_errors.hpp>
#include <spiner/spiner_types.hpp>

#include "../hdf5.h"

namespace Spiner {

template <typename T = Real>
class RegularGrid1D {
 public:
  RegularGrid1D() = default;
  RegularGrid1D(T min, T max, std::size_t N)
      : min_(min), max_(max), dx_((max - min) / static_cast<T>(N - 1)),
        inv_dx_(1 / dx_), N_(static_cast<int>(N)) {}
  inline T x(const int i) const { return min_ + i * dx_; }
  inline T min() const { return min_; }
  inline T max() const { return max_; }
  inline T dx() const { return dx_; }
  inline int nPoints() const { return N_; }
  // Cell index of x, clamped to [0, N-2]; NaN maps to cell 0.
  inline int index(const T x) const {
    const T u = (x - min_) * inv_dx_;
    if (!(u >= 0)) return 0;
    if (u > static_cast<T>(N_ - 2)) return N_ - 2;
    return static_cast<int>(u);
  }
  inline void weights(const T x, int &ix, T &w0, T &w1) const {
    ix = index(x);
    const T xl = min_ + ix * dx_;
    w1 = (x - xl) * inv_dx_;
    w0 = 1 - w1;
  }
  bool operator==(const RegularGrid1D &o) const {
    return min_ == o.min_ && max_ == o.max_ && N_ == o.N_;
  }

 private:
  T min_ = 0, max_ = 0, dx_ = 0, inv_dx_ = 0;
  int N_ = 0;
};

// Only the single-grid form is supported by this shim; a multi-grid
// construction aborts.
template <typename T = Real, int NGRIDSMAX = 5>
class PiecewiseGrid1D {
 public:
  PiecewiseGrid1D() = default;
  PiecewiseGrid1D(const std::vector<RegularGrid1D<T>> &grids) {
    PORTABLE_ALWAYS_REQUIRE(grids.size() == 1, "spiner-lite: single grid only");
    g_ = grids[0];
  }
  PiecewiseGrid1D(const RegularGrid1D<T> &g) : g_(g) {}
  inline T x(const int i) const { return g_.x(i); }
  inline T min() const { return g_.min(); }
  inline T max() const { return g_.max(); }
  inline int nPoints() const { return g_.nPoints(); }
  inline int nGrids() const { return 1; }
  inline int index(const T x) const { return g_.index(x); }
  inline void weights(const T x, int &ix, T &w0, T &w1) const { g_.weights(x, ix, w0, w1); }
  const RegularGrid1D<T> &grid() const { return g_; }

 private:
  RegularGrid1D<T> g_;
};

template <typename T = Real, typename Grid_t = RegularGrid1D<T>>
class DataBox {
 public:
  static constexpr int MAXRANK = 3;
  DataBox() = default;
  DataBox(T *data, int n1) : data_(data), rank_(1), owns_(false) {
    dims_[0] = n1;
  }
  DataBox(int n1) { resize(n1); }
  DataBox(int n2, int n1) { resize(n2, n1); }

  void resize(int n1) {
    setShape_(1, n1, 1, 1);
  }
  void resize(int n2, int n1) { setShape_(2, n1, n2, 1); }
  void resize(int n3, int n2, int n1) { setShape_(3, n1, n2, n3); }

  inline T &operator()(const int i) { return data_[i]; }
  inline const T &operator()(const int i) const { return data_[i]; }
  inline T &operator()(const int j, const int i) { return data_[j * dims_[0] + i]; }
  inline const T &operator()(const int j, const int i) const {
    return data_[j * dims_[0] + i];
  }
  inline T &operator()(const int k, const int j, const int i) {
    return data_[(k * dims_[1] + j) * dims_[0] + i];
  }
  inline const T &operator()(const int k, const int j, const int i) const {
    return data_[(k * dims_[1] + j) * dims_[0] + i];
  }

  // 1-based dimension query; dim(1) is the fastest index.
  inline int dim(const int d) const { return dims_[d - 1]; }
  inline int rank() const { return rank_; }
  inline const Grid_t &range(const int d) const { return grids_[d]; }
  inline void setRange(const int d, const Grid_t &g) { grids_[d] = g; }
  template <typename G>
  inline void setRange(const int d, const G &g) {
    grids_[d] = Grid_t(g);
  }
  inline void setRange(const int d, const T min, const T max, const int N) {
    grids_[d] = Grid_t(RegularGrid1D<T>(min, max, N));
  }

  void copyMetadata(const DataBox &src) {
    setShape_(src.rank_, src.dims_[0], src.dims_[1], src.dims_[2]);
    for (int d = 0; d < MAXRANK; ++d)
      grids_[d] = src.grids_[d];
  }

  inline T interpToReal(const T x1) const {
    int i;
    T w0, w1;
    grids_[0].weights(x1, i, w0, w1);
    return w0 * data_[i] + w1 * data_[i + 1];
  }
  inline T interpToReal(const T x2, const T x1) const {
    int i, j;
    T a0, a1, b0, b1;
    grids_[0].weights(x1, i, a0, a1);
    grids_[1].weights(x2, j, b0, b1);
    const int n1 = dims_[0];
    const T *r0 = data_ + j * n1 + i;
    const T *r1 = r0 + n1;
    return b0 * (a0 * r0[0] + a1 * r0[1]) + b1 * (a0 * r1[0] + a1 * r1[1]);
  }
  // 2-D interpolation in (x3, x2) at fixed fastest index idx.
  inline T interpToReal(const T x3, const T x2, const int idx) const {
    int j, k;
    T a0, a1, b0, b1;
    grids_[1].weights(x2, j, a0, a1);
    grids_[2].weights(x3, k, b0, b1);
    const int n1 = dims_[0], n2 = dims_[1];
    auto at = [&](int kk, int jj) { return data_[(kk * n2 + jj) * n1 + idx]; };
    return b0 * (a0 * at(k, j) + a1 * at(k, j + 1)) +
           b1 * (a0 * at(k + 1, j) + a1 * at(k + 1, j + 1));
  }
  // Index ix of the slowest dimension as a box of one rank lower that shares
  // this box's memory and keeps its remaining grids (spiner's
  // DataBox::slice, used by eos_spiner_rho_sie.hpp:520-521).
  DataBox slice(const int ix) const {
    DataBox out;
    out.rank_ = rank_ - 1;
    std::size_t stride = 1;
    for (int d = 0; d < out.rank_; ++d) {
      out.dims_[d] = dims_[d];
      out.grids_[d] = grids_[d];
      stride *= static_cast<std::size_t>(dims_[d]);
    }
    out.data_ = data_ + static_cast<std::size_t>(ix) * stride;
    out.owns_ = false;
    return out;
  }
  void interpFromDB(const DataBox &db, const T x3, const T x2) {
    for (int n = 0; n < dims_[0]; ++n)
      data_[n] = db.interpToReal(x3, x2, n);
  }

  herr_t loadHDF(hid_t loc, const char *name) {
    const sgx_h5lite::Dataset *ds = sgx_h5lite::find_dataset(loc, name);
    if (ds == nullptr) return -1;
    const int r = static_cast<int>(ds->n.size());
    setShape_(r, ds->n[0], r > 1 ? ds->n[1] : 1, r > 2 ? ds->n[2] : 1);
    for (int d = 0; d < r; ++d)
      grids_[d] = Grid_t(RegularGrid1D<T>(ds->min[d], ds->max[d], ds->n[d]));
    std::memcpy(data_, ds->data.data(), sizeBytes());
    return H5_SUCCESS;
  }

  DataBox getOnDevice() const {
    DataBox out;
    out.copyMetadata(*this);
    if (size() > 0) std::memcpy(out.data_, data_, sizeBytes());
    return out;
  }
  void finalize() {
    if (owns_ && data_ != nullptr) std::free(data_);
    data_ = nullptr;
    owns_ = false;
  }
  inline std::size_t size() const {
    std::size_t s = 1;
    for (int d = 0; d < rank_; ++d)
      s *= dims_[d];
    return rank_ == 0 ? 0 : s;
  }
  inline std::size_t sizeBytes() const { return size() * sizeof(T); }
  inline T *data() const { return data_; }
  template <typename P>
  std::size_t setPointer(P *src) {
    if (owns_ && data_ != nullptr) std::free(data_);
    data_ = reinterpret_cast<T *>(src);
    owns_ = false;
    return sizeBytes();
  }
  inline bool ownsAllocatedMemory() const { return owns_; }

 private:
  void setShape_(int rank, int n1, int n2, int n3) {
    rank_ = rank;
    dims_ = {n1, n2, n3};
    data_ = static_cast<T *>(std::calloc(size() > 0 ? size() : 1, sizeof(T)));
    owns_ = true;
  }
  T *data_ = nullptr;
  int rank_ = 0;
  std::array<int, MAXRANK> dims_{0, 0, 0};
  std::array<Grid_t, MAXRANK> grids_{};
  bool owns_ = false;
};

} // namespace Spiner

#endif // SGX_ORACLE_SHIM_SPINER_DATABOX_HPP
