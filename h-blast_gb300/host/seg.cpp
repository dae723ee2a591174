// seg.cpp -- low-complexity masking of protein queries (SEG).
//
// BLASTX masks the translated frames of its query before the word finder
// runs (NCBI's -seg option, default "12 2.2 2.5"; H-BLAST inherits it from
// NCBI's query set-up, NF/blastx_args.cpp:133-134, NF/blast_engine.c:367-433).
// NCBI's implementation is not part of the reference tree; this restates the
// published method of Wootton and Federhen (Comput. Chem. 17:149-163, 1993;
// Methods Enzymol. 266:554-571, 1996):
//
//  1. Every window of `window` letters gets its compositional complexity
//     K2 = -sum_i (n_i / W) log2 (n_i / W) over the 20 standard amino acids.
//     Windows holding any other letter (B, Z, X, U, *, O, J, sentinel) are
//     never low complexity.
//  2. A window with K2 <= locut triggers a segment; it is extended to the
//     left and right over contiguous windows with K2 <= hicut.  The raw
//     segment is the union of those windows' letters.
//  3. Inside the raw segment, the subsequence whose complexity state is
//     least probable is kept: P0 = (N! / prod_k r_k!) (L! / prod_i n_i!) / N^L
//     with N = 20, L its length, n_i its letter counts and r_k the number of
//     letters that occur exactly k times.  Ties go to the leftmost, then the
//     shortest subsequence.  The search trims at most kMaxTrim letters from
//     each end of the raw segment (a bound of this implementation: the search
//     is exhaustive for raw segments of up to 2 x kMaxTrim letters and linear
//     in the length beyond, so a long low-complexity query stays cheap).
//  4. The parts of the raw segment left and right of it are searched again
//     with steps 1-3 as sequences of their own; then the scan resumes after
//     the raw segment.
//
// Masked letters become X (NCBIstdaa 21), NCBI's hard masking.  Logarithms
// are summed in a fixed order (letters, then count classes, ascending) so the
// result does not depend on evaluation order.
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "../../include/hblast_gpu.h"
#include "batch_builder.h"

namespace hbg {

namespace {

constexpr int kN = 20;
constexpr uint8_t kMaskLetter = 21;   // X
constexpr int32_t kMaxTrim = 100;     // letters the optimum may drop from each end of a raw segment

// NCBIstdaa letter -> index among the 20 standard amino acids, -1 otherwise
int std_index(uint8_t c) {
    static const int8_t tab[HBG_ALPHABET] = {-1, 0,  -1, 1,  2,  3,  4,  5,  6,  7,  8,  9,  10, 11,
                                             12, 13, 14, 15, 16, 17, 18, -1, 19, -1, -1, -1, -1, -1};
    return c < HBG_ALPHABET ? tab[c] : -1;
}

struct Seg {
    const uint8_t *s;
    int32_t window;
    double locut, hicut;
    std::vector<double> lf;   // lf[k] = ln k!
    std::vector<uint8_t> *mask;

    // K2 of window [w, w + window), +inf if it holds a non-standard letter
    double k2(int32_t w) const {
        int cnt[kN] = {0};
        for (int32_t i = 0; i < window; ++i) {
            const int x = std_index(s[w + i]);
            if (x < 0)
                return INFINITY;
            cnt[x]++;
        }
        double h = 0.0;
        for (int a = 0; a < kN; ++a)
            if (cnt[a]) {
                const double p = (double)cnt[a] / (double)window;
                h -= p * log2(p);
            }
        return h;
    }

    // ln P0 of the complexity state with these counts
    double log_p0(const int *cnt, int32_t L) const {
        double v = lf[kN] + lf[L] - (double)L * log((double)kN);
        for (int a = 0; a < kN; ++a)
            v -= lf[cnt[a]];
        int r[64] = {0};              // counts of count values; values > 63 go through a map below
        std::vector<int> big;
        for (int a = 0; a < kN; ++a) {
            if (cnt[a] < 64)
                r[cnt[a]]++;
            else
                big.push_back(cnt[a]);
        }
        for (int k = 0; k < 64; ++k)
            v -= lf[r[k]];
        // count values >= 64: group equal values (at most 20 of them)
        for (size_t i = 0; i < big.size(); ++i) {
            bool first = true;
            for (size_t j = 0; j < i; ++j)
                if (big[j] == big[i])
                    first = false;
            if (!first)
                continue;
            int m = 0;
            for (size_t j = 0; j < big.size(); ++j)
                m += big[j] == big[i];
            v -= lf[m];
        }
        return v;
    }

    // Least probable subsequence [*bi, *bj) of [a, b) (standard letters
    // only) that starts within kMaxTrim letters of a and ends within kMaxTrim
    // letters of b.
    void optimise(int32_t a, int32_t b, int32_t *bi, int32_t *bj) const {
        double best = INFINITY;
        *bi = a;
        *bj = b;
        const int32_t i_end = std::min(b, a + kMaxTrim + 1);
        for (int32_t i = a; i < i_end; ++i) {
            const int32_t j_lo = std::max(i, b - kMaxTrim - 1);   // first end index j (inclusive) tried
            int cnt[kN] = {0};
            for (int32_t j = i; j < j_lo; ++j)
                cnt[std_index(s[j])]++;
            for (int32_t j = j_lo; j < b; ++j) {
                cnt[std_index(s[j])]++;
                const double v = log_p0(cnt, j - i + 1);
                if (v < best) {
                    best = v;
                    *bi = i;
                    *bj = j + 1;
                }
            }
        }
    }

    // Steps 1-4 on letters [a, b).
    void run(int32_t a, int32_t b) {
        if (b - a < window)
            return;
        const int32_t nw = b - a - window + 1;
        std::vector<double> k(nw);
        for (int32_t w = 0; w < nw; ++w)
            k[w] = k2(a + w);
        int32_t w = 0;
        while (w < nw) {
            if (!(k[w] <= locut)) {
                ++w;
                continue;
            }
            int32_t lo = w, hi = w;
            while (lo > 0 && k[lo - 1] <= hicut)
                --lo;
            while (hi + 1 < nw && k[hi + 1] <= hicut)
                ++hi;
            const int32_t ra = a + lo, rb = a + hi + window;
            int32_t i = ra, j = rb;
            optimise(ra, rb, &i, &j);
            for (int32_t p = i; p < j; ++p)
                (*mask)[p] = 1;
            run(ra, i);
            run(j, rb);
            w = hi + 1;
        }
    }
};

}  // namespace

int64_t seg_mask(uint8_t *seq, int32_t len, int32_t window, double locut, double hicut) {
    if (!seq || len <= 0 || window < 1)
        return 0;
    std::vector<uint8_t> mask((size_t)len, 0);
    Seg g;
    g.s = seq;
    g.window = window;
    g.locut = locut;
    g.hicut = hicut;
    g.lf.assign((size_t)len + kN + 2, 0.0);
    for (size_t k = 2; k < g.lf.size(); ++k)
        g.lf[k] = g.lf[k - 1] + log((double)k);
    g.mask = &mask;
    g.run(0, len);
    int64_t n = 0;
    for (int32_t p = 0; p < len; ++p)
        if (mask[p]) {
            seq[p] = kMaskLetter;
            ++n;
        }
    return n;
}

}  // namespace hbg
