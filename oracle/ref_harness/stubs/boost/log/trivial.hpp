// Stand-in for Boost.Log's trivial logger (Boost is not installed).
// BOOST_LOG_TRIVIAL(sev) << ... compiles to a discarded stream expression.
#pragma once
#include <ostream>
namespace risa_ref_stub {
struct NullStream {
   template <typename T> NullStream& operator<<(const T&) { return *this; }
   NullStream& operator<<(std::ostream& (*)(std::ostream&)) { return *this; }
};
inline NullStream& null_stream() { static NullStream s; return s; }
}
#define BOOST_LOG_TRIVIAL(sev) ::risa_ref_stub::null_stream()
