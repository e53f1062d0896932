// Stand-in for boost::multiprecision::cpp_int, used ONLY to compile the
// reference's own sources for cross-checking the oracle (test
// infrastructure; never shipped).  Boost is not installed on this machine.
//
// The reference uses cpp_int for counters and necklace counts
// (src/utils/lyndon.cpp:38-45,100; src/core/generate/generate_hybrid.cpp:127-129;
// src/utils/io.h:24-65).  A signed 128-bit integer holds every value those
// paths reach for the orders exercised here (necklace counts < 2^100).
#pragma once
#include <cstdint>
#include <ostream>
#include <string>
#include <algorithm>

namespace boost {
namespace multiprecision {

class cpp_int {
public:
    __int128 v;
    cpp_int() : v(0) {}
    template <typename T, typename = std::enable_if_t<std::is_integral_v<T>>>
    cpp_int(T x) : v((__int128)x) {}
    static cpp_int raw(__int128 x) { cpp_int r; r.v = x; return r; }

    cpp_int& operator++() { ++v; return *this; }
    cpp_int operator++(int) { cpp_int t = *this; ++v; return t; }
    cpp_int& operator+=(const cpp_int& o) { v += o.v; return *this; }
    cpp_int& operator-=(const cpp_int& o) { v -= o.v; return *this; }
    cpp_int& operator*=(const cpp_int& o) { v *= o.v; return *this; }
    cpp_int& operator/=(const cpp_int& o) { v /= o.v; return *this; }

    friend cpp_int operator+(const cpp_int& a, const cpp_int& b) { return raw(a.v + b.v); }
    friend cpp_int operator-(const cpp_int& a, const cpp_int& b) { return raw(a.v - b.v); }
    friend cpp_int operator*(const cpp_int& a, const cpp_int& b) { return raw(a.v * b.v); }
    friend cpp_int operator/(const cpp_int& a, const cpp_int& b) { return raw(a.v / b.v); }
    friend cpp_int operator%(const cpp_int& a, const cpp_int& b) { return raw(a.v % b.v); }
    friend bool operator==(const cpp_int& a, const cpp_int& b) { return a.v == b.v; }
    friend bool operator!=(const cpp_int& a, const cpp_int& b) { return a.v != b.v; }
    friend bool operator<(const cpp_int& a, const cpp_int& b) { return a.v < b.v; }
    friend bool operator>(const cpp_int& a, const cpp_int& b) { return a.v > b.v; }
    friend bool operator<=(const cpp_int& a, const cpp_int& b) { return a.v <= b.v; }
    friend bool operator>=(const cpp_int& a, const cpp_int& b) { return a.v >= b.v; }

    template <typename T, typename = std::enable_if_t<std::is_integral_v<T>>>
    explicit operator T() const { return (T)v; }
    explicit operator long double() const { return (long double)v; }

    std::string str() const {
        if (v == 0) return "0";
        __int128 x = v < 0 ? -v : v;
        std::string s;
        while (x > 0) { s.push_back(char('0' + (int)(x % 10))); x /= 10; }
        if (v < 0) s.push_back('-');
        std::reverse(s.begin(), s.end());
        return s;
    }
    friend std::ostream& operator<<(std::ostream& os, const cpp_int& a) { return os << a.str(); }
};

inline cpp_int pow(const cpp_int& base, unsigned e) {
    cpp_int r(1);
    for (unsigned i = 0; i < e; ++i) r.v *= base.v;
    return r;
}

}  // namespace multiprecision
}  // namespace boost
