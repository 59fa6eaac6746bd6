// The EOS variant the oracle is built with: the hot-path models only, in
// the way the reference's tests define custom variants (test_pte.cpp:45).
// TEST INFRASTRUCTURE ONLY.
#ifndef SGX_ORACLE_VARIANT_HPP
#define SGX_ORACLE_VARIANT_HPP
#include <singularity-eos/base/eos_error.hpp>
#include <singularity-eos/eos/eos_variant.hpp>
#include <singularity-eos/eos/eos_gruneisen.hpp>
#include <singularity-eos/eos/eos_helmholtz.hpp>
#include <singularity-eos/eos/eos_ideal.hpp>
#include <singularity-eos/eos/eos_noble_abel.hpp>
#include <singularity-eos/eos/eos_spiner_rho_temp.hpp>
#include <singularity-eos/eos/eos_stiff.hpp>
namespace singularity {
using EOS = Variant<IdealGas, StiffGas, NobleAbel, Gruneisen, SpinerEOSDependsRhoT,
                    Helmholtz>;
} // namespace singularity
#endif
