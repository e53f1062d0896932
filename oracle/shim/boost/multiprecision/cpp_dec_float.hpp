// Stand-in for boost::multiprecision::cpp_dec_float_50, used ONLY to compile
// the reference's progress bar (src/utils/io.h:24-65) when cross-checking the
// oracle.  A long double carries the percentage it prints.
#pragma once
#include <ostream>
#include "cpp_int.hpp"

namespace boost {
namespace multiprecision {

class cpp_dec_float_50 {
public:
    long double v;
    cpp_dec_float_50() : v(0) {}
    cpp_dec_float_50(long double x) : v(x) {}
    explicit cpp_dec_float_50(const cpp_int& x) : v((long double)x.v) {}
    friend cpp_dec_float_50 operator/(const cpp_dec_float_50& a, const cpp_dec_float_50& b) { return a.v / b.v; }
    friend cpp_dec_float_50 operator*(const cpp_dec_float_50& a, int b) { return a.v * b; }
    friend std::ostream& operator<<(std::ostream& os, const cpp_dec_float_50& a) { return os << (double)a.v; }
};

}  // namespace multiprecision
}  // namespace boost
