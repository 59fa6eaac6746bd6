// Configured eos.hpp for the oracle build: the reference's own hook
// (eos/eos.hpp.in includes @SINGULARITY_VARIANT@, CMakeLists.txt:150-151)
// pointed at the oracle's variant header. TEST INFRASTRUCTURE ONLY.
#ifndef _SINGULARITY_EOS_EOS_EOS_HPP_
#define _SINGULARITY_EOS_EOS_EOS_HPP_
#include <sgx_oracle_variant.hpp>
#endif
