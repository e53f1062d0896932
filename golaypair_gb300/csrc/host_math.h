// host_math.h -- small host-side tables of the search (alphabet, two-square
// decompositions, necklace counts, prenecklaces, rank <-> packed words).
#pragma once
#include <cstdint>
#include <functional>
#include <numeric>
#include <vector>

namespace gp {

using u128 = unsigned __int128;

// src/utils/golay.cpp:60-75: even c -> {-c..c step 2}; odd c -> +-{1..c step 2}
inline std::vector<int> alphabet(int c) {
    std::vector<int> a;
    if (c % 2 == 0) {
        for (int v = -c; v <= c; v += 2) a.push_back(v);
    } else {
        for (int v = -c; v <= -1; v += 2) a.push_back(v);
        for (int v = 1; v <= c; v += 2) a.push_back(v);
    }
    return a;
}

// src/utils/decomps.cpp:6-17
inline std::vector<std::pair<int, int>> decomps(int k) {
    std::vector<std::pair<int, int>> out;
    for (int x = 0; x <= k; ++x)
        for (int y = x; y <= k; ++y)
            if (x * x + y * y == k) out.emplace_back(x, y);
    return out;
}

// src/core/generate/generate_hybrid.cpp:45-47
inline int sum_constant(int order, int paf) { return order * 2 + (order - 1) * paf; }

inline int bits_for(int k) {
    int b = 1;
    while ((1 << b) < k) ++b;
    return b;
}

// src/utils/lyndon.cpp:38-45 (saturating)
inline u128 necklace_count(int L, int k) {
    u128 sum = 0;
    const u128 cap = (u128)1 << 120;
    for (int i = 1; i <= L; ++i) {
        const int e = std::gcd(i, L);
        u128 p = 1;
        for (int t = 0; t < e; ++t) {
            p *= (u128)k;
            if (p > cap) return cap;
        }
        sum += p;
    }
    return sum / (u128)L;
}

inline u128 upow(int k, int e) {
    u128 p = 1;
    for (int i = 0; i < e; ++i) p *= (u128)k;
    return p;
}

// Packed word of the word with lexicographic rank r (base-k digits, digit 0
// most significant, b bits per digit).
inline u128 rank_to_word(u128 r, int k, int b, int L) {
    u128 w = 0;
    int j = L - 1;
    // 128-bit division is a library call: divide in 128 bits only while the
    // rank does not fit 64 bits
    for (; j >= 0 && (r >> 64) != 0; --j) {
        const int d = (int)(r % (u128)k);
        r /= (u128)k;
        w |= (u128)d << (b * (L - 1 - j));
    }
    uint64_t q = (uint64_t)r;
    for (; j >= 0; --j) {
        const int d = (int)(q % (uint64_t)k);
        q /= (uint64_t)k;
        w |= (u128)d << (b * (L - 1 - j));
    }
    return w;
}

// Words of the ranks r0, r0 + step, r0 + 2 step, ...: the rank's base-k
// digits are kept and the step's digits added with carry, so each word
// costs L small additions instead of L 128-bit divisions.
struct RankStepper {
    int k, b, L;
    std::vector<int> d, s;  // digit 0 most significant
    bool past_end = false;  // the rank reached k^L
    RankStepper(u128 r0, u128 step, int k_, int b_, int L_) : k(k_), b(b_), L(L_), d(L_), s(L_) {
        for (int j = L - 1; j >= 0; --j) {
            d[j] = (int)(r0 % (u128)k);
            r0 /= (u128)k;
            s[j] = (int)(step % (u128)k);
            step /= (u128)k;
        }
        past_end = r0 != 0 || step != 0;  // inputs of k^L or more
    }
    u128 word() const {
        u128 w = 0;
        for (int j = 0; j < L; ++j) w = (w << b) | (u128)d[j];
        return w;
    }
    void advance() {
        int carry = 0;
        for (int j = L - 1; j >= 0; --j) {
            int v = d[j] + s[j] + carry;
            carry = v >= k;
            d[j] = carry ? v - k : v;
        }
        if (carry) past_end = true;
    }
};

inline int word_digit_h(u128 w, int b, int L, int j) { return (int)((w >> (b * (L - 1 - j))) & (((u128)1 << b) - 1)); }

// Rank of a word (inverse of rank_to_word).  A bound past the last word
// (a digit >= k, or bits above digit 0's field) maps to k^L.
inline u128 word_to_rank(u128 w, int k, int b, int L) {
    if (b * L < 128 && (w >> (b * L)) != 0) return upow(k, L);
    u128 r = 0;
    for (int j = 0; j < L; ++j) {
        const int d = word_digit_h(w, b, L, j);
        if (d >= k) return upow(k, L);
        r = r * (u128)k + (u128)d;
    }
    return r;
}

// Every prenecklace of length n over digits 0..k-1 in lexicographic order
// with its period (the FKM recursion of src/utils/lyndon.cpp:47-85).
inline void prenecklaces(int n, int k, const std::function<void(const std::vector<int>&, int)>& cb) {
    std::vector<int> a(n + 1, 0);
    std::function<void(int, int)> rec = [&](int t, int p) {
        if (t > n) {
            cb(std::vector<int>(a.begin() + 1, a.end()), p);
            return;
        }
        a[t] = a[t - p];
        rec(t + 1, p);
        for (int j = a[t - p] + 1; j < k; ++j) {
            a[t] = j;
            rec(t + 1, t);
        }
    };
    for (int d = 0; d < k; ++d) {
        a[1] = d;
        rec(2, 1);
    }
}

}  // namespace gp
