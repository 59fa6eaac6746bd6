// spiner-lite types. TEST INFRASTRUCTURE ONLY.
#ifndef SGX_ORACLE_SHIM_SPINER_TYPES_HPP
#define SGX_ORACLE_SHIM_SPINER_TYPES_HPP
#include <ports-of-call/portability.hpp>
#endif
