// Stand-in for Boost.Stacktrace, which the reference's host error macro
// streams into a message (src/cochlea.cu:30,53-60).  Only the reference
// cubin build includes this file; the host code it serves is not compiled
// into the cubin.
#pragma once
#include <ostream>
namespace boost {
namespace stacktrace {
struct stacktrace {};
inline std::ostream& operator<<(std::ostream& o, const stacktrace&) { return o; }
}  // namespace stacktrace
}  // namespace boost
