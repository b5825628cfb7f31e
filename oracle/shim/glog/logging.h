// Single-process stand-in for the glog API used by the reference engine
// (LOG/VLOG/DLOG streams, CHECK, InitGoogleLogging). Test infrastructure for
// building the reference as an oracle; not part of the product.
#pragma once
#include <ostream>
#include <stdexcept>
#include <string>

namespace oracle_shim {
struct NullLog {
    template <class T>
    NullLog& operator<<(const T&) { return *this; }
    NullLog& operator<<(std::ostream& (*)(std::ostream&)) { return *this; }
};
}  // namespace oracle_shim

#define LOG(severity) ::oracle_shim::NullLog()
#define VLOG(level) ::oracle_shim::NullLog()
#define DLOG(severity) ::oracle_shim::NullLog()
#define CHECK(cond)                                                         \
    if (!(cond))                                                            \
        throw std::runtime_error(std::string("CHECK failed: ") + #cond);    \
    else                                                                    \
        ::oracle_shim::NullLog()

namespace google {
inline void InitGoogleLogging(const char*) {}
inline void ShutdownGoogleLogging() {}
}  // namespace google
