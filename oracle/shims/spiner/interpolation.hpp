// spiner-lite: interpolation lives in databox.hpp for this shim.
// TEST INFRASTRUCTURE ONLY.
#ifndef SGX_ORACLE_SHIM_SPINER_INTERPOLATION_HPP
#define SGX_ORACLE_SHIM_SPINER_INTERPOLATION_HPP
#include <spiner/databox.hpp>
#endif
