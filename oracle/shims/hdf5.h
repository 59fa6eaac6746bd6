// hdf5-lite: the ~12 HDF5 calls that singularity-eos's Spiner table loader
// makes (eos_spiner_common.hpp:122-206, eos_spiner_rho_temp.hpp:373-424),
// restated over the "sp5-lite" flat binary image that this project writes
// instead of HDF5 (HDF5 is absent here).
//
// TEST INFRASTRUCTURE ONLY. The product has its own reader of the same
// image format (singularity-eos_gb300/csrc/sp5lite.cpp).
//
// sp5-lite layout (little endian):
//   char magic[8] = "SGXSP5L\0"; u32 version = 1; u32 nrecords;
//   record: u32 kind (1 attr f64, 2 attr i32, 3 dataset f64, 4 attr string);
//           u32 len, char path[len]; u32 len, char name[len];
//           kind 1: f64;  kind 2: i32;  kind 4: u32 len, bytes;
//           kind 3: u32 rank, then per dim (fastest first) i32 n, f64 min,
//                   f64 max; then f64 data[prod n], fastest index last in
//                   memory order (C order of [n_{rank-1}]...[n_0]).
#ifndef SGX_ORACLE_SHIM_HDF5_H
#define SGX_ORACLE_SHIM_HDF5_H

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

typedef std::int64_t hid_t;
typedef int herr_t;
typedef unsigned long long hsize_t;
typedef int htri_t;
enum H5T_class_t { H5T_NO_CLASS = -1, H5T_INTEGER = 0, H5T_FLOAT = 1, H5T_STRING = 3 };

#define H5_SUCCESS 0
#define H5E_DEFAULT 0
#define H5F_ACC_RDONLY 0u
#define H5P_DEFAULT 0

namespace sgx_h5lite {

struct Dataset {
  std::vector<int> n;
  std::vector<double> min, max;
  std::vector<double> data;
};
struct Registry {
  std::map<std::string, double> attr_f64;
  std::map<std::string, int> attr_i32;
  std::map<std::string, std::string> attr_str;
  std::map<std::string, Dataset> datasets;
  std::vector<std::string> handles; // hid_t -> path
};
inline Registry &reg() {
  static Registry r;
  return r;
}
inline std::string join(const std::string &a, const std::string &b) {
  if (b == "." || b.empty()) return a;
  if (!b.empty() && b[0] == '/') return b;
  if (a == "/") return "/" + b;
  return a + "/" + b;
}
inline const std::string &path_of(hid_t h) { return reg().handles.at(h); }
inline hid_t new_handle(const std::string &p) {
  reg().handles.push_back(p);
  return static_cast<hid_t>(reg().handles.size() - 1);
}
inline bool path_exists(const std::string &p) {
  const Registry &r = reg();
  const std::string pre = p + "/";
  auto has_prefix = [&](const auto &m) {
    for (const auto &kv : m)
      if (kv.first == p || kv.first.compare(0, pre.size(), pre) == 0) return true;
    return false;
  };
  return has_prefix(r.datasets) || has_prefix(r.attr_f64) || has_prefix(r.attr_i32) ||
         has_prefix(r.attr_str);
}
inline const Dataset *find_dataset(hid_t loc, const char *name) {
  auto it = reg().datasets.find(join(path_of(loc), name));
  return it == reg().datasets.end() ? nullptr : &it->second;
}
inline std::string attr_key(hid_t loc, const char *obj, const char *attr) {
  return join(path_of(loc), obj) + "@" + attr;
}

inline bool load_file(const char *fname) {
  FILE *f = std::fopen(fname, "rb");
  if (!f) return false;
  auto rd = [&](void *p, size_t n) { return std::fread(p, 1, n, f) == n; };
  auto rdstr = [&](std::string &s) {
    std::uint32_t len;
    if (!rd(&len, 4)) return false;
    s.resize(len);
    return len == 0 || rd(&s[0], len);
  };
  char magic[8];
  std::uint32_t version, nrec;
  bool ok = rd(magic, 8) && std::memcmp(magic, "SGXSP5L", 8) == 0 && rd(&version, 4) &&
            version == 1 && rd(&nrec, 4);
  Registry &r = reg();
  for (std::uint32_t k = 0; ok && k < nrec; ++k) {
    std::uint32_t kind;
    std::string path, name;
    ok = rd(&kind, 4) && rdstr(path) && rdstr(name);
    if (!ok) break;
    const std::string key = path + "@" + name;
    if (kind == 1) {
      double v;
      ok = rd(&v, 8);
      r.attr_f64[key] = v;
    } else if (kind == 2) {
      std::int32_t v;
      ok = rd(&v, 4);
      r.attr_i32[key] = v;
    } else if (kind == 4) {
      std::string s;
      ok = rdstr(s);
      r.attr_str[key] = s;
    } else if (kind == 3) {
      std::uint32_t rank;
      ok = rd(&rank, 4);
      Dataset ds;
      std::size_t total = 1;
      for (std::uint32_t d = 0; ok && d < rank; ++d) {
        std::int32_t n;
        double mn, mx;
        ok = rd(&n, 4) && rd(&mn, 8) && rd(&mx, 8);
        ds.n.push_back(n);
        ds.min.push_back(mn);
        ds.max.push_back(mx);
        total *= static_cast<std::size_t>(n);
      }
      ds.data.resize(total);
      ok = ok && rd(ds.data.data(), total * 8);
      r.datasets[path] = std::move(ds);
    } else {
      ok = false;
    }
  }
  std::fclose(f);
  return ok;
}

} // namespace sgx_h5lite

typedef herr_t (*H5E_auto2_t)(hid_t, void *);
inline herr_t H5Eset_auto(hid_t, H5E_auto2_t, void *) { return H5_SUCCESS; }
inline herr_t H5Eprint2(hid_t, FILE *) { return H5_SUCCESS; }
inline hid_t H5Fopen(const char *name, unsigned, hid_t) {
  if (!sgx_h5lite::load_file(name)) return -1;
  return sgx_h5lite::new_handle("/");
}
inline herr_t H5Fclose(hid_t) { return H5_SUCCESS; }
inline hid_t H5Gopen(hid_t loc, const char *name, hid_t) {
  return sgx_h5lite::new_handle(sgx_h5lite::join(sgx_h5lite::path_of(loc), name));
}
inline herr_t H5Gclose(hid_t) { return H5_SUCCESS; }
inline htri_t H5Lexists(hid_t loc, const char *name, hid_t) {
  return sgx_h5lite::path_exists(sgx_h5lite::join(sgx_h5lite::path_of(loc), name)) ? 1 : 0;
}

#endif // SGX_ORACLE_SHIM_HDF5_H
