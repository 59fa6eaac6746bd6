// ports-of-call-lite: the portability surface that the singularity-eos
// hot-path headers use, restated for a host-only (OpenMP) oracle build.
//
// TEST INFRASTRUCTURE ONLY. This shim exists so that the reference's own
// headers (mixed_cell_models.hpp, eos_*.hpp, root_finding.hpp, logs.hpp)
// compile unmodified into the CPU oracle under oracle/_ref. It is never
// linked into the product library.
//
// Written from the call sites in the reference (PORTABLE_* macros,
// portableFor(name, [space,] start, stop, f), PortsOfCall::Exec::*), not
// from the upstream ports-of-call sources, which are absent.
#ifndef SGX_ORACLE_SHIM_PORTABILITY_HPP
#define SGX_ORACLE_SHIM_PORTABILITY_HPP

#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>

using Real = double;

#define PORTABLE_FUNCTION
#define PORTABLE_INLINE_FUNCTION inline
#define PORTABLE_FORCEINLINE_FUNCTION inline __attribute__((always_inline))
#define PORTABLE_LAMBDA [=]

#define PORTABILITY_STRATEGY_NONE 1

namespace PortsOfCall {
namespace Exec {
struct Host {};
struct Device {};
} // namespace Exec
using std::printf;
} // namespace PortsOfCall

// The oracle runs cells in a plain loop; the harness parallelises over
// cells itself (one EOS copy per thread) where it needs threads.
template <typename Function>
inline void portableFor(const char * /*name*/, int start, int stop, Function function) {
  for (int i = start; i < stop; ++i)
    function(i);
}
template <typename Space, typename Function>
inline void portableFor(const char * /*name*/, const Space & /*s*/, int start, int stop,
                        Function function) {
  for (int i = start; i < stop; ++i)
    function(i);
}

#define PORTABLE_MALLOC(size) std::malloc(size)
#define PORTABLE_FREE(ptr) std::free(ptr)

template <typename T>
inline void portableCopyToDevice(T *const to, T const *const from, std::size_t size_bytes) {
  std::memcpy(to, from, size_bytes);
}
template <typename T>
inline void portableCopyToHost(T *const to, T const *const from, std::size_t size_bytes) {
  std::memcpy(to, from, size_bytes);
}

#endif // SGX_ORACLE_SHIM_PORTABILITY_HPP
