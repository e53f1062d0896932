// survivors.h -- the binary survivor file and the text lines it stands for.
//
// Generation writes one line per surviving candidate (src/utils/io.cpp:14-36):
//   "PSD" + the L-1 signature values concatenated + " " + each entry + " " + "\n".
// The binary file holds the same records without the text:
//
//   header (80 bytes, little endian; byte offsets)
//     0 magic "GPSURV01"; 8 version (u32) = 1; then i32 at 12 order,
//     16 compress, 20 paf, 24 L, 28 k (alphabet size), 32 bits per digit,
//     36 role (0 = A file, 1 = B file), 40 sig_bytes (1 or 2), 44 word_bytes;
//     48 count (u64); 56 the alphabet (16 x i8, first k used, ascending);
//     72 eight zero bytes
//   count records, in the order the text file has its lines (FKM order):
//     word_bytes bytes: the packed word, digit 0 in the most significant of
//       its L * bits bits (digit j = index of entry j in the alphabet)
//     (L-1) * sig_bytes bytes: the signature values as written in the line
//
// A record of an order-90 candidate at compression 2 takes 56 bytes; its
// text line about 230.
#pragma once
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "host_math.h"

namespace gp {

constexpr char kSurvMagic[8] = {'G', 'P', 'S', 'U', 'R', 'V', '0', '1'};

struct SurvHeader {
    char magic[8];
    uint32_t version;
    int32_t order, compress, paf, L, k, bits, role, sig_bytes, word_bytes;
    uint64_t count;
    int8_t alpha[16];
    uint8_t reserved1[8];
};
static_assert(sizeof(SurvHeader) == 80, "survivor header layout");

inline bool surv_header_valid(const SurvHeader& h) {
    return std::memcmp(h.magic, kSurvMagic, 8) == 0 && h.version == 1 && h.L >= 2 && h.L <= 128 && h.k >= 1 &&
           h.k <= 16 && h.bits >= 1 && h.bits <= 4 && h.bits * h.L <= 128 && (h.sig_bytes == 1 || h.sig_bytes == 2) &&
           h.word_bytes == (h.bits * h.L + 7) / 8 && (h.role == 0 || h.role == 1);
}

inline size_t surv_record_bytes(const SurvHeader& h) {
    return (size_t)h.word_bytes + (size_t)(h.L - 1) * (size_t)h.sig_bytes;
}

inline void put_uint(std::string& s, unsigned v) {
    char tmp[12];
    int n = 0;
    do {
        tmp[n++] = (char)('0' + v % 10);
        v /= 10;
    } while (v);
    while (n) s.push_back(tmp[--n]);
}

inline void put_int(std::string& s, int v) {
    if (v < 0) {
        s.push_back('-');
        put_uint(s, (unsigned)(-(long long)v));
    } else {
        put_uint(s, (unsigned)v);
    }
}

// One text line (src/utils/io.cpp:14-36): sig holds the L-1 values.
inline void format_survivor_line(std::string& out, int L, int b, const int* alpha, u128 word, const uint16_t* sig) {
    out += "PSD";
    for (int k = 0; k < L - 1; ++k) put_uint(out, sig[k]);
    out.push_back(' ');
    for (int j = 0; j < L; ++j) {
        put_int(out, alpha[word_digit_h(word, b, L, j)]);
        out.push_back(' ');
    }
    out.push_back('\n');
}

inline void surv_put_record(uint8_t* dst, const SurvHeader& h, u128 word, const uint16_t* sig) {
    for (int i = 0; i < h.word_bytes; ++i) dst[i] = (uint8_t)(word >> (8 * i));
    uint8_t* s = dst + h.word_bytes;
    for (int k = 0; k < h.L - 1; ++k) {
        if (h.sig_bytes == 1) {
            s[k] = (uint8_t)sig[k];
        } else {
            s[2 * k] = (uint8_t)sig[k];
            s[2 * k + 1] = (uint8_t)(sig[k] >> 8);
        }
    }
}

inline u128 surv_get_record(const uint8_t* src, const SurvHeader& h, uint16_t* sig) {
    u128 w = 0;
    for (int i = 0; i < h.word_bytes; ++i) w |= (u128)src[i] << (8 * i);
    const uint8_t* s = src + h.word_bytes;
    for (int k = 0; k < h.L - 1; ++k) sig[k] = h.sig_bytes == 1 ? s[k] : (uint16_t)(s[2 * k] | (s[2 * k + 1] << 8));
    return w;
}

// Formats records [lo, hi) of a binary body as text lines.  A digit past
// the alphabet makes the record malformed: returns false.
inline bool surv_format_range(const SurvHeader& h, const uint8_t* body, uint64_t lo, uint64_t hi, std::string& out) {
    const size_t rb = surv_record_bytes(h);
    int alpha[16];
    for (int i = 0; i < 16; ++i) alpha[i] = h.alpha[i];
    std::vector<uint16_t> sig((size_t)h.L);
    out.reserve(out.size() + (size_t)(hi - lo) * (size_t)(4 * h.L + 8));
    for (uint64_t r = lo; r < hi; ++r) {
        const u128 w = surv_get_record(body + r * rb, h, sig.data());
        for (int j = 0; j < h.L; ++j)
            if (word_digit_h(w, h.bits, h.L, j) >= h.k) return false;
        if (h.bits * h.L < 128 && (w >> (h.bits * h.L)) != 0) return false;
        format_survivor_line(out, h.L, h.bits, alpha, w, sig.data());
    }
    return true;
}

// All records as text, formatted by up to 16 host threads.  Returns false
// on a malformed record.
inline bool surv_to_text(const SurvHeader& h, const uint8_t* body, std::string& out) {
    const uint64_t n = h.count;
    const uint64_t per = 1 << 14;
    const uint64_t nblocks = (n + per - 1) / per;
    unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    if (nblocks < nt) nt = (unsigned)std::max<uint64_t>(1, nblocks);
    std::vector<std::string> parts(nblocks);
    std::vector<char> ok(nblocks, 1);
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; ++t)
        th.emplace_back([&, t] {
            for (uint64_t b = t; b < nblocks; b += nt)
                ok[b] = surv_format_range(h, body, b * per, std::min(n, (b + 1) * per), parts[b]);
        });
    for (auto& x : th) x.join();
    for (uint64_t b = 0; b < nblocks; ++b) {
        if (!ok[b]) return false;
        out += parts[b];
    }
    return true;
}

// Splits file bytes into header and body when they start with the magic.
// 0: not a survivor file; 1: survivor file; -1: survivor magic but a bad
// header or a truncated body.
inline int surv_parse(const std::string& bytes, SurvHeader& h, const uint8_t** body) {
    if (bytes.size() < 8 || std::memcmp(bytes.data(), kSurvMagic, 8) != 0) return 0;
    if (bytes.size() < sizeof(SurvHeader)) return -1;
    std::memcpy(&h, bytes.data(), sizeof h);
    if (!surv_header_valid(h)) return -1;
    const size_t rb = surv_record_bytes(h);
    if (h.count > (bytes.size() - sizeof h) / rb || sizeof h + h.count * rb != bytes.size()) return -1;
    *body = reinterpret_cast<const uint8_t*>(bytes.data()) + sizeof h;
    return 1;
}

}  // namespace gp
