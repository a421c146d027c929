// Host build of the device primitives (blg_device.cuh) for the CPU tests.
//
// The same step/score/saturation functions the kernels call are compiled
// here with g++ and driven two ways:
//  * blg_host_distance: pattern = shorter trimmed string, words processed
//    top to bottom in one column (the order k_search_seq uses);
//  * blg_host_wavefront: the anti-diagonal lane schedule of the
//    lane-spread kernels, emulated step by step: "lane" w handles column
//    s - w at step s and reads the carry lane w-1 produced one step earlier
//    (what __shfl_up_sync delivers on the GPU), with the max_dist exit
//    decided by the last word's lane.
// Both must equal the oracle for every input.
#include <cstdint>
#include <cstring>
#include <vector>

#include "blg_device.cuh"

using namespace blg;

namespace {

struct Pattern {
    int m = 0, words = 0;
    std::vector<uint64_t> peq;   // 256 x words
    Pattern(const uint8_t *p, int m_) : m(m_), words(m_ > 0 ? (m_ + 63) / 64 : 1), peq(256 * (size_t)words, 0) {
        for (int i = 0; i < m; i++) peq[(size_t)p[i] * words + i / 64] |= 1ull << (i % 64);
    }
    uint64_t eq(uint8_t c, int w) const { return peq[(size_t)c * words + w]; }
};

void normalise(const uint8_t *&a, int &la, const uint8_t *&b, int &lb, int trim) {
    if (trim) trim_affixes(a, la, b, lb);
    if (la > lb) {
        const uint8_t *t = a; a = b; b = t;
        int x = la; la = lb; lb = x;
    }
}

}  // namespace

extern "C" int blg_host_distance(const uint8_t *a, int la, const uint8_t *b, int lb, int trim, int k) {
    normalise(a, la, b, lb, trim);
    if (k >= 0 && lb - la > k) return k + 1;
    if (la == 0) return lb;
    Pattern P(a, la);
    const int W = P.words, lastbit = (la - 1) % 64;
    std::vector<uint64_t> pv(W, ~0ull), mv(W, 0);
    int score = la;
    for (int j = 0; j < lb; j++) {
        uint64_t ph, mh;
        step_top<uint64_t>(pv[0], mv[0], P.eq(b[j], 0), ph, mh);
        int h = hdelta<uint64_t>(ph, mh, W == 1 ? lastbit : 63);
        for (int w = 1; w < W; w++) {
            step_mid<uint64_t>(pv[w], mv[w], P.eq(b[j], w), h, ph, mh);
            h = hdelta<uint64_t>(ph, mh, w == W - 1 ? lastbit : 63);
        }
        score += h;
        if (hopeless(score, j, lb, k)) return k + 1;
    }
    return cap_k(score, k);
}

extern "C" int blg_host_wavefront(const uint8_t *a, int la, const uint8_t *b, int lb, int trim, int k) {
    normalise(a, la, b, lb, trim);
    if (k >= 0 && lb - la > k) return k + 1;
    if (la == 0) return lb;
    Pattern P(a, la);
    const int W = P.words, lastw = W - 1, lastbit = (la - 1) % 64;
    std::vector<uint64_t> pv(W, ~0ull), mv(W, 0);
    std::vector<int> carry(W, 0), next(W, 0);   // carry[w]: what lane w received last step
    int score = la;
    bool done = false;
    for (int s = 0; s < lb + W - 1 && !done; s++) {
        for (int w = 0; w < W; w++) {
            const int j = s - w;
            next[w] = 0;
            if (j < 0 || j >= lb) continue;
            uint64_t ph, mh;
            step_mid<uint64_t>(pv[w], mv[w], P.eq(b[j], w), w == 0 ? 1 : carry[w], ph, mh);
            const int hout = hdelta<uint64_t>(ph, mh, w == lastw ? lastbit : 63);
            next[w] = hout;
            if (w == lastw) {
                score += hout;
                if (hopeless(score, j, lb, k)) done = true;
            }
        }
        for (int w = W - 1; w >= 1; w--) carry[w] = next[w - 1];   // shfl_up by one lane
    }
    if (done) return k + 1;
    return cap_k(score, k);
}

// The pipe-balanced form the search kernels use: 32-bit halves, IMAD-style
// add/shift/score (plain arithmetic on the host), score kept as +1/-1 counts
// of the last word's output bit, words chained top to bottom in a column.
extern "C" int blg_host_distance_halves(const uint8_t *a, int la, const uint8_t *b, int lb, int trim, int k) {
    normalise(a, la, b, lb, trim);
    if (k >= 0 && lb - la > k) return k + 1;
    if (la == 0) return lb;
    Pattern P(a, la);
    const int W = P.words, lastbit = (la - 1) % 64;
    const Units u{1u, 2u};
    const uint32_t mult = u.one << (31 - (lastbit & 31));
    std::vector<Word2> st(W);
    for (auto &x : st) { x.pl = x.ph = ~0u; x.ml = x.mh = 0; }
    uint32_t accP = 0, accM = 0;
    for (int j = 0; j < lb; j++) {
        uint32_t Phl = 0, Phh = 0, Mhl = 0, Mhh = 0, cp = u.one, cm = 0;
        for (int w = 0; w < W; w++) {
            const uint64_t e = P.eq(b[j], w);
            step_h(st[w], (uint32_t)e, (uint32_t)(e >> 32), cp, cm, u, Phl, Phh, Mhl, Mhh);
            cp = top_bit(Phh, u);
            cm = top_bit(Mhh, u);
        }
        if (lastbit >= 32) {
            accP = imad_hi(imad_lo(Phh, mult, 0), u.two, accP);
            accM = imad_hi(imad_lo(Mhh, mult, 0), u.two, accM);
        } else {
            accP = imad_hi(imad_lo(Phl, mult, 0), u.two, accP);
            accM = imad_hi(imad_lo(Mhl, mult, 0), u.two, accM);
        }
        if (hopeless(la + (int)accP - (int)accM, j, lb, k)) return k + 1;
    }
    return cap_k(la + (int)accP - (int)accM, k);
}

// The banded loop (k <= 31) with the window bits read from a full Peq table.
extern "C" int blg_host_band(const uint8_t *a, int la, const uint8_t *b, int lb, int trim, int k) {
    normalise(a, la, b, lb, trim);
    if (k < 0 || k > 31) return -1;
    if (lb - la > k) return k + 1;
    if (la == 0) return lb;
    Pattern P(a, la);
    const Units u{1u, 2u};
    auto text = [&](int j) -> uint32_t { return b[j]; };
    auto eqw = [&](uint32_t c, int p0) -> uint32_t {
        uint32_t v = 0;
        for (int q = 0; q < 32; q++) {
            const int p = p0 + q;
            if (p >= 0 && p < la && ((P.eq((uint8_t)c, p / 64) >> (p % 64)) & 1u)) v |= 1u << q;
        }
        return v;
    };
    return band_core(la, lb, k, text, eqw, u, nullptr);
}

// The banded loop as the pairs path runs it (trimmed, shorter string as
// the pattern), also reporting the text columns it processed before its exit
// fired (0 for pairs settled by the length gap or an empty pattern).
extern "C" int blg_host_band_cols(const uint8_t *a, int la, const uint8_t *b, int lb, int k, int *cols) {
    normalise(a, la, b, lb, 1);
    *cols = 0;
    if (k < 0 || k > 31) return -1;
    if (lb - la > k) return k + 1;
    if (la == 0) return lb;
    Pattern P(a, la);
    const Units u{1u, 2u};
    auto text = [&](int j) -> uint32_t { return b[j]; };
    auto eqw = [&](uint32_t c, int p0) -> uint32_t {
        uint32_t v = 0;
        for (int q = 0; q < 32; q++) {
            const int p = p0 + q;
            if (p >= 0 && p < la && ((P.eq((uint8_t)c, p / 64) >> (p % 64)) & 1u)) v |= 1u << q;
        }
        return v;
    };
    return band_core(la, lb, k, text, eqw, u, cols);
}

// The banded loop with the pairs solver's block tables: nibble rows over a
// 64-position block of the pattern (bit i <-> position 32b - dhi + i), each
// column's window taken with one funnel shift, rows shifted by 32 positions
// and the next 32 bytes entered every 32 columns (k_solve_band's scheme).
extern "C" int blg_host_band_blocks(const uint8_t *a, int la, const uint8_t *b, int lb, int k) {
    normalise(a, la, b, lb, 1);
    if (k < 0 || k > 31) return -1;
    if (lb - la > k) return k + 1;
    if (la == 0) return lb;
    const int m = la, n = lb;
    const BandGeom bg = band_geom(m, n, k);
    const int dhi = bg.dhi;
    uint32_t lo[32] = {0}, hi[32] = {0};
    auto set = [&](uint32_t c, int bitpos) {
        uint32_t *h = bitpos >= 32 ? hi : lo;
        h[c >> 4] |= 1u << (bitpos & 31);
        h[16 + (c & 15)] |= 1u << (bitpos & 31);
    };
    const int first_end = m < 64 - dhi ? m : 64 - dhi;
    for (int p = 0; p < first_end; p++) set(a[p], p + dhi);
    int next_pos = first_end;
    const Units u{1u, 2u};
    auto text = [&](int j) -> uint32_t { return b[j]; };
    auto eqw = [&](uint32_t c, int p0) -> uint32_t {
        const int j = p0 + dhi;
        if ((j & 31) == 0 && j > 0) {
            for (int r = 0; r < 32; r++) { lo[r] = hi[r]; hi[r] = 0; }
            int cnt = m - next_pos;
            if (cnt > 32) cnt = 32;
            for (int i = 0; i < cnt; i++) set(a[next_pos + i], 32 + i);
            if (cnt > 0) next_pos += cnt;
        }
        const uint32_t xl = lo[c >> 4] & lo[16 + (c & 15)], xh = hi[c >> 4] & hi[16 + (c & 15)];
        const int s = j & 31;
        return s == 0 ? xl : (xl >> s) | (xh << (32 - s));
    };
    return band_core(m, n, k, text, eqw, u, nullptr);
}

// Same, with the pattern as the LONGER string (the search kernels' case:
// the query is the pattern whatever the choice's length), no trimming.
extern "C" int blg_host_band_query(const uint8_t *q, int m, const uint8_t *t, int n, int k) {
    if (k < 0 || k > 31) return -1;
    if (m == 0) return cap_k(n, k);
    if ((n > m ? n - m : m - n) > k) return k + 1;
    Pattern P(q, m);
    const Units u{1u, 2u};
    auto text = [&](int j) -> uint32_t { return t[j]; };
    auto eqw = [&](uint32_t c, int p0) -> uint32_t {
        uint32_t v = 0;
        for (int qq = 0; qq < 32; qq++) {
            const int p = p0 + qq;
            if (p >= 0 && p < m && ((P.eq((uint8_t)c, p / 64) >> (p % 64)) & 1u)) v |= 1u << qq;
        }
        return v;
    };
    return band_core(m, n, k, text, eqw, u, nullptr);
}

// The search's banded run stopped after `stop` columns (a multiple of 4) and
// resumed from its saved state with fresh text and window readers, the
// window bits taken from the unpadded Peq words as the resume pass reads
// them (32-bit halves p0 >> 5 and the next, zero outside the pattern).
extern "C" int blg_host_band_resume(const uint8_t *q, int m, const uint8_t *t, int n, int k, int stop) {
    if (k < 0 || k > 31 || stop < 0 || (stop & 3)) return -1;
    if (m == 0) return cap_k(n, k);
    if ((n > m ? n - m : m - n) > k) return k + 1;
    Pattern P(q, m);
    const int nw = (m + 63) / 64;
    auto half = [&](uint32_t c, int r) -> uint32_t {
        if (r < 0 || r >= 2 * nw) return 0u;
        const uint64_t w = P.eq((uint8_t)c, r >> 1);
        return (r & 1) ? (uint32_t)(w >> 32) : (uint32_t)w;
    };
    auto eqw = [&](uint32_t c, int p0) -> uint32_t {
        const int r = p0 >> 5, s = p0 & 31;
        const uint32_t lo = half(c, r), hi = half(c, r + 1);
        return s == 0 ? lo : (lo >> s) | (hi << (32 - s));
    };
    const BandGeom bg = band_geom(m, n, k);
    BandState s = band_start(bg);
    auto text1 = [&](int j) -> uint32_t { return t[j]; };
    if (band_steps(k, bg, s, stop < n ? stop : n, text1, eqw)) return k + 1;
    const BandState saved = s;                          // what the queue item carries
    BandState r = saved;
    const uint8_t *rest = t + saved.j;
    auto text2 = [&](int j) -> uint32_t { return rest[j - saved.j]; };
    if (band_steps(k, bg, r, n, text2, eqw)) return k + 1;
    return band_finish(k, bg, r);
}

extern "C" int blg_host_store(int d, int dtype) {
    if (dtype == DT_UINT8) return (int)saturate_u8(d);
    if (dtype == DT_UINT16) return (int)saturate_u16(d);
    return d;
}
