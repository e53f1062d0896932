// ref_window_driver.cpp -- runs the reference's own candidate generation
// over a window of word ranks.  Test infrastructure: build_ref.sh links it
// against the reference's unchanged objects into oracle/_ref/golay_ref_window;
// it produces golden files for windowed searches and is never shipped.
//
// The reference enumerates necklaces with generate_necklaces_prefix
// (src/utils/lyndon.cpp:47-85), which resumes the FKM recursion from a
// prefix and its period.  A window [begin, end) of word ranks (base-k
// numbers over the sorted alphabet, first entry most significant) is cut
// into aligned blocks  prefix x alphabet^(L - |prefix|);  the reference's
// generator runs once per block whose prefix is a prenecklace, so necklaces
// come out in lexicographic order, as in the reference's own run.  Each
// necklace goes through the per-necklace body of generate_hybrid
// (src/core/generate/generate_hybrid.cpp:136-156): the row-sum gate per
// decomposition, Fourier::calculate_psd, Fourier::psd_filter, isCanonical
// with generators (0, L) for A and (1, L) for B, and write_seq_psd /
// write_seq_psd_invert.
//
// usage: golay_ref_window ORDER COMPRESS PAF BEGIN END OUT_A OUT_B
//        (BEGIN, END decimal; END is clipped to k^L)
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <functional>
#include <optional>
#include <set>
#include <string>
#include <vector>

#include "decomps.h"
#include "fourier.h"
#include "golay.h"
#include "io.h"
#include "orderly_equivalence.h"

// defined in src/utils/lyndon.cpp and src/core/generate/generate_hybrid.cpp
void generate_necklaces_prefix(const int LEN, const std::vector<int>& alphabet,
                               const std::function<void(const std::vector<int>&, const int)>& callback,
                               std::optional<std::reference_wrapper<std::vector<int>>> partial_seq, const int i,
                               const int p);
int rowsum(const std::vector<int>& seq);
int sum_constant(int order, int paf);

using u128 = unsigned __int128;

static u128 parse_u128(const char* s) {
    u128 v = 0;
    for (; *s; ++s) {
        if (*s < '0' || *s > '9') {
            fprintf(stderr, "bad number\n");
            exit(2);
        }
        v = v * 10 + (u128)(*s - '0');
    }
    return v;
}

// Period of the prefix as a prenecklace, or 0 when it is not one.
static int prenecklace_period(const std::vector<int>& d) {
    int p = 1;
    for (size_t j = 1; j < d.size(); ++j) {
        if (d[j] > d[j - p])
            p = (int)j + 1;
        else if (d[j] < d[j - p])
            return 0;
    }
    return p;
}

int main(int argc, char** argv) {
    if (argc != 8) {
        fprintf(stderr, "usage: %s ORDER COMPRESS PAF BEGIN END OUT_A OUT_B\n", argv[0]);
        return 2;
    }
    const int ORDER = atoi(argv[1]), COMPRESS = atoi(argv[2]), PAF = atoi(argv[3]);
    const int LEN = ORDER / COMPRESS;
    const std::set<int> aset = getalphabet(COMPRESS);
    const std::vector<int> alpha(aset.begin(), aset.end());
    const int k = (int)alpha.size();
    u128 space = 1;
    for (int i = 0; i < LEN; ++i) space *= (u128)k;
    const u128 lo = parse_u128(argv[4]);
    u128 hi = parse_u128(argv[5]);
    if (hi > space) hi = space;
    std::ofstream out_a(argv[6]), out_b(argv[7]);
    const auto decomps = getdecomps(sum_constant(ORDER, PAF));
    if (decomps.empty()) return 1;
    const auto genA = constructGenerators(0, LEN);
    const auto genB = constructGenerators(1, LEN);
    Fourier fourier(LEN);
    long long necklaces = 0;
    auto body = [&](const std::vector<int>& seq) {
        ++necklaces;
        for (const auto& dc : decomps) {
            if (rowsum(seq) == dc.first) {
                const std::vector<double>& psd = fourier.calculate_psd(seq);
                if (fourier.psd_filter(psd, ORDER, PAF) && isCanonical(seq, genA)) write_seq_psd(seq, psd, out_a);
            }
            if (rowsum(seq) == dc.second) {
                const std::vector<double>& psd = fourier.calculate_psd(seq);
                if (fourier.psd_filter(psd, ORDER, PAF) && isCanonical(seq, genB))
                    write_seq_psd_invert(seq, psd, out_b, ORDER * 2 - PAF);
            }
        }
    };
    auto on_word = [&](const std::vector<int>& seq, const int period) {
        if (LEN % period == 0) body(seq);
    };
    // aligned blocks of [lo, hi), in increasing order
    std::vector<int> digits;
    std::function<void(u128, u128)> cover = [&](u128 base, u128 size) {
        if (base >= hi || base + size <= lo) return;
        if (lo <= base && base + size <= hi) {
            const int i = (int)digits.size();
            if (i == 0) {
                generate_necklaces_prefix(LEN, alpha, on_word, std::nullopt, 0, 0);
                return;
            }
            const int p = prenecklace_period(digits);
            if (!p) return;
            std::vector<int> seq(i);
            for (int j = 0; j < i; ++j) seq[j] = alpha[digits[j]];
            if (i == LEN) {
                on_word(seq, p);
                return;
            }
            generate_necklaces_prefix(LEN, alpha, on_word, std::ref(seq), i, p);
            return;
        }
        const u128 sub = size / (u128)k;
        for (int d = 0; d < k; ++d) {
            digits.push_back(d);
            cover(base + sub * (u128)d, sub);
            digits.pop_back();
        }
    };
    cover(0, space);
    printf("necklaces %lld\n", necklaces);
    return 0;
}
