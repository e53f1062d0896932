// host_par.h -- host-side helpers of the text stages: a block-parallel loop
// over up to 16 threads, cutting a text into line-aligned chunks, and a
// decimal integer reader/writer for the small entries of candidate lines.
#pragma once
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

namespace gp {

inline unsigned host_threads() { return std::max(1u, std::min(16u, std::thread::hardware_concurrency())); }

// fn(b) for b in [0, nblocks), blocks dealt round robin to the threads.
template <class F>
void par_for(size_t nblocks, F&& fn) {
    const unsigned nt = (unsigned)std::min<size_t>(host_threads(), std::max<size_t>(1, nblocks));
    if (nt <= 1) {
        for (size_t b = 0; b < nblocks; ++b) fn(b);
        return;
    }
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; ++t)
        th.emplace_back([&, t] {
            for (size_t b = t; b < nblocks; b += nt) fn(b);
        });
    for (auto& x : th) x.join();
}

// Start offsets of up to `parts` chunks of text[0, n), each starting at a
// line start (offset 0 or just after a '\n'); the last entry is n.
inline std::vector<size_t> line_chunks(const char* text, size_t n, size_t parts) {
    std::vector<size_t> cut = {0};
    for (size_t k = 1; k < parts; ++k) {
        size_t pos = n * k / parts;
        if (pos <= cut.back()) continue;
        const char* nl = (const char*)memchr(text + pos - 1, '\n', n - (pos - 1));
        pos = nl ? (size_t)(nl - text) + 1 : n;
        if (pos > cut.back() && pos < n) cut.push_back(pos);
    }
    cut.push_back(n);
    return cut;
}

// strtol(q, &e, 10) on the text up to `end` (the values of candidate lines
// are small): leading white space, an optional sign, decimal digits.  *e = q
// when no digit follows.
inline long read_long(const char* q, const char* end, const char** e) {
    const char* p = q;
    while (p < end && (*p == ' ' || (*p >= '\t' && *p <= '\r'))) ++p;
    bool neg = false;
    if (p < end && (*p == '-' || *p == '+')) {
        neg = *p == '-';
        ++p;
    }
    const char* d0 = p;
    long v = 0;
    while (p < end && *p >= '0' && *p <= '9') {
        v = v * 10 + (*p - '0');
        ++p;
    }
    if (p == d0) {
        *e = q;
        return 0;
    }
    *e = p;
    return neg ? -v : v;
}

// "%d " of a small integer.
inline void put_int_sp(std::string& s, int v) {
    char tmp[12];
    int n = 0;
    unsigned u = v < 0 ? (unsigned)(-(long long)v) : (unsigned)v;
    do {
        tmp[n++] = (char)('0' + u % 10);
        u /= 10;
    } while (u);
    if (v < 0) s.push_back('-');
    while (n) s.push_back(tmp[--n]);
    s.push_back(' ');
}

}  // namespace gp
