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
#include <singularity-eos/eos/eos_spiner_rho_sie.hpp>
#include <singularity-eos/eos/eos_spiner_rho_temp.hpp>
#include <singularity-eos/eos/eos_stiff.hpp>
#include <singularity-eos/eos/modifiers/ramps_eos.hpp>
#include <singularity-eos/eos/modifiers/scaled_eos.hpp>
#include <singularity-eos/eos/modifiers/shifted_eos.hpp>
namespace singularity {
// Each hot-path model bare, shifted, scaled and scaled-shifted, and each of
// those under a bilinear ramp: the nestings of the reference's default
// variant (eos_type_lists.hpp:80-96). Helmholtz and SpinerEOSDependsRhoSie
// are carried bare.
#define SGX_ORACLE_MODS(M)                                                               \
  M, ShiftedEOS<M>, ScaledEOS<M>, ScaledEOS<ShiftedEOS<M>>, BilinearRampEOS<M>,          \
      BilinearRampEOS<ShiftedEOS<M>>, BilinearRampEOS<ScaledEOS<M>>,                     \
      BilinearRampEOS<ScaledEOS<ShiftedEOS<M>>>
using EOS = Variant<SGX_ORACLE_MODS(IdealGas), SGX_ORACLE_MODS(StiffGas),
                    SGX_ORACLE_MODS(NobleAbel), SGX_ORACLE_MODS(Gruneisen),
                    SGX_ORACLE_MODS(SpinerEOSDependsRhoT), Helmholtz,
                    SpinerEOSDependsRhoSie>;
#undef SGX_ORACLE_MODS
} // namespace singularity
#endif
