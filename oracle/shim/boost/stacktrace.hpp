/* Minimal stand-in for boost::stacktrace so the reference's error header
 * compiles without Boost. The oracle never raises through it. */
#pragma once
#include <ostream>
namespace boost {
namespace stacktrace {
struct stacktrace {
    stacktrace() {}
    stacktrace(unsigned, unsigned) {}
    bool empty() const { return true; }
};
inline std::ostream &operator<<(std::ostream &os, const stacktrace &) { return os; }
}  // namespace stacktrace
}  // namespace boost
