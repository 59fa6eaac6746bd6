// ports-of-call-lite variant: PortsOfCall::{variant,visit,get,holds_alternative}
// mapped onto std::variant for the host-only oracle build.
// TEST INFRASTRUCTURE ONLY.
#ifndef SGX_ORACLE_SHIM_VARIANT_HPP
#define SGX_ORACLE_SHIM_VARIANT_HPP

#include <variant>

namespace PortsOfCall {
using std::get;
using std::holds_alternative;
using std::variant;
using std::visit;
} // namespace PortsOfCall

#endif // SGX_ORACLE_SHIM_VARIANT_HPP
