// hdf5-lite high-level attribute calls over the sp5-lite image.
// TEST INFRASTRUCTURE ONLY (see hdf5.h in this folder).
#ifndef SGX_ORACLE_SHIM_HDF5_HL_H
#define SGX_ORACLE_SHIM_HDF5_HL_H

#include "hdf5.h"

inline herr_t H5LTget_attribute_double(hid_t loc, const char *obj, const char *attr,
                                       double *out) {
  auto &m = sgx_h5lite::reg().attr_f64;
  auto it = m.find(sgx_h5lite::attr_key(loc, obj, attr));
  if (it == m.end()) return -1;
  *out = it->second;
  return H5_SUCCESS;
}
inline herr_t H5LTget_attribute_int(hid_t loc, const char *obj, const char *attr,
                                    int *out) {
  auto &m = sgx_h5lite::reg().attr_i32;
  auto it = m.find(sgx_h5lite::attr_key(loc, obj, attr));
  if (it == m.end()) return -1;
  *out = it->second;
  return H5_SUCCESS;
}
inline herr_t H5LTget_attribute_char(hid_t loc, const char *obj, const char *attr,
                                     char *out) {
  auto &m = sgx_h5lite::reg().attr_str;
  auto it = m.find(sgx_h5lite::attr_key(loc, obj, attr));
  if (it == m.end()) return -1;
  *out = it->second.empty() ? '\0' : it->second[0];
  return H5_SUCCESS;
}
inline herr_t H5LTget_attribute_info(hid_t loc, const char *obj, const char *attr,
                                     hsize_t *dims, H5T_class_t *cls, std::size_t *len) {
  auto &m = sgx_h5lite::reg().attr_str;
  auto it = m.find(sgx_h5lite::attr_key(loc, obj, attr));
  if (it == m.end()) return -1;
  dims[0] = 1;
  *cls = H5T_STRING;
  *len = it->second.size();
  return H5_SUCCESS;
}
inline herr_t H5LTget_attribute_string(hid_t loc, const char *obj, const char *attr,
                                       char *out) {
  auto &m = sgx_h5lite::reg().attr_str;
  auto it = m.find(sgx_h5lite::attr_key(loc, obj, attr));
  if (it == m.end()) return -1;
  std::memcpy(out, it->second.data(), it->second.size());
  return H5_SUCCESS;
}

#endif // SGX_ORACLE_SHIM_HDF5_HL_H
