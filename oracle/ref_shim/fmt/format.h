// Minimal stand-in for the {fmt} header that the reference's serde.h includes.  TEST
// INFRASTRUCTURE ONLY: used when oracle/build_ref.sh compiles the reference's kernels for the CPU.
// It provides fmt::format with "{}" substitution, which is all serde.h uses.
#pragma once
#include <sstream>
#include <string>

namespace fmt {
inline void format_into(std::ostringstream &os, const char *f) { os << f; }
template <typename A, typename... R>
inline void format_into(std::ostringstream &os, const char *f, const A &a, const R &...r) {
    for (; *f; ++f) {
        if (f[0] == '{' && f[1] == '}') { os << a; format_into(os, f + 2, r...); return; }
        os << *f;
    }
}
template <typename... A>
inline std::string format(const char *f, const A &...a) {
    std::ostringstream os;
    format_into(os, f, a...);
    return os.str();
}
}  // namespace fmt
