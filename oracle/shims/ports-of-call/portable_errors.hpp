// ports-of-call-lite error macros for the host-only oracle build.
// TEST INFRASTRUCTURE ONLY (see portability.hpp in this folder).
//
// PORTABLE_REQUIRE is a debug-only check (compiled out under NDEBUG, as the
// reference's release builds do); the ALWAYS variants abort with a message.
#ifndef SGX_ORACLE_SHIM_PORTABLE_ERRORS_HPP
#define SGX_ORACLE_SHIM_PORTABLE_ERRORS_HPP

#include <cstdio>
#include <cstdlib>
#include <sstream>
#include <stdexcept>
#include <string>

namespace sgx_oracle_shim {
inline void die(const char *msg, const char *file, int line) {
  std::fprintf(stderr, "oracle abort: %s (%s:%d)\n", msg, file, line);
  std::abort();
}
inline void die(const std::string &msg, const char *file, int line) {
  die(msg.c_str(), file, line);
}
inline std::string to_msg(const char *m) { return std::string(m); }
inline std::string to_msg(const std::string &m) { return m; }
inline std::string to_msg(const std::stringstream &m) { return m.str(); }
} // namespace sgx_oracle_shim

#ifdef NDEBUG
#define PORTABLE_REQUIRE(cond, msg) ((void)0)
#define PORTABLE_WARN(msg) ((void)0)
#else
#define PORTABLE_REQUIRE(cond, msg)                                                      \
  do {                                                                                   \
    if (!(cond)) sgx_oracle_shim::die(msg, __FILE__, __LINE__);                          \
  } while (0)
#define PORTABLE_WARN(msg) std::fprintf(stderr, "oracle warn: %s\n", msg)
#endif

#define PORTABLE_ALWAYS_REQUIRE(cond, msg)                                               \
  do {                                                                                   \
    if (!(cond)) sgx_oracle_shim::die(msg, __FILE__, __LINE__);                          \
  } while (0)
#define PORTABLE_ALWAYS_WARN(msg) ((void)0)
#define PORTABLE_ABORT(msg)                                                              \
  sgx_oracle_shim::die(sgx_oracle_shim::to_msg(msg), __FILE__, __LINE__)
#define PORTABLE_ALWAYS_ABORT(msg) PORTABLE_ABORT(msg)
#define PORTABLE_THROW_OR_ABORT(msg) throw std::runtime_error(sgx_oracle_shim::to_msg(msg))
#define PORTABLE_ALWAYS_THROW_OR_ABORT(msg) PORTABLE_THROW_OR_ABORT(msg)

#endif // SGX_ORACLE_SHIM_PORTABLE_ERRORS_HPP
