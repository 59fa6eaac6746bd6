// spiner-lite sp5 key names are not used by the hot path. TEST INFRASTRUCTURE ONLY.
#ifndef SGX_ORACLE_SHIM_SPINER_SP5_HPP
#define SGX_ORACLE_SHIM_SPINER_SP5_HPP
#endif
