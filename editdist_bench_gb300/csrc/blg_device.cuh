// Device primitives of the GB300 Levenshtein engine.
//
// Everything in this header compiles as CUDA device code and as plain C++,
// so blg_hostcheck.cpp builds the same functions for the CPU and the tests
// check them against the oracle without a GPU (the reference does the same
// for its own device header: csrc/gpu_hostcheck.cpp).
//
// Algorithm: unit-cost Levenshtein distance by the bit-parallel method of
// Myers (1999) in Hyyro's block formulation: the pattern runs down the bit
// vectors (bit i <-> pattern position i), the text is scanned one column at
// a time, Pv/Mv hold the +1/-1 vertical deltas, and a word passes the
// horizontal delta at its bottom row to the word below (reference:
// csrc/gpu_myers.cuh:45-59, csrc/myers.c:22-36).
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define BLG_HD __host__ __device__ __forceinline__
#else
#define BLG_HD static inline
#endif

namespace blg {

// Output dtype codes shared with the C-ABI (include/bitlev_gb300.h).
enum { DT_INT32 = 0, DT_UINT16 = 1, DT_UINT8 = 2 };

// Saturating store rule: values are already min(d, k+1) when k >= 0; the
// narrow types clamp at their maximum (bitlev/_common.py:25-29,
// csrc/gpu_myers.cuh:149-152).
BLG_HD uint32_t saturate_u8(int d) { return d > 255 ? 255u : (uint32_t)d; }
BLG_HD uint32_t saturate_u16(int d) { return d > 65535 ? 65535u : (uint32_t)d; }

// max_dist rule on a finished distance: min(d, k+1) (k < 0: exact).
BLG_HD int cap_k(int d, int k) { return (k >= 0 && d > k) ? k + 1 : d; }

// One column step on the TOP word of the pattern (the DP's top row grows by
// +1 per column, so the carry-in is always +1). Updates pv/mv and returns the
// +1/-1/0 horizontal delta leaving row `outbit` via ph_out/mh_out bits.
template <typename W>
BLG_HD void step_top(W &pv, W &mv, W eq, W &ph, W &mh) {
    const W xv = eq | mv;
    const W xh = (((eq & pv) + pv) ^ pv) | eq;
    ph = mv | ~(xh | pv);
    mh = pv & xh;
    const W phs = (ph << 1) | (W)1;
    const W mhs = mh << 1;
    pv = mhs | ~(xv | phs);
    mv = phs & xv;
}

// One column step on a word below the top: carry-in hin in {-1,0,+1}
// (a -1 carry is folded in as a match at bit 0, the +1/-1 shifted in).
template <typename W>
BLG_HD void step_mid(W &pv, W &mv, W eq, int hin, W &ph, W &mh) {
    const W neg = (W)(hin < 0), pos = (W)(hin > 0);
    const W xv = eq | mv;
    eq |= neg;
    const W xh = (((eq & pv) + pv) ^ pv) | eq;
    ph = mv | ~(xh | pv);
    mh = pv & xh;
    const W phs = (ph << 1) | pos;
    const W mhs = (mh << 1) | neg;
    pv = mhs | ~(xv | phs);
    mv = phs & xv;
}

// Horizontal delta at bit b of (ph, mh): +1, -1 or 0.
template <typename W>
BLG_HD int hdelta(W ph, W mh, int b) {
    return (int)((ph >> b) & (W)1) - (int)((mh >> b) & (W)1);
}

// Exact early exit of a thresholded run (csrc/myers.c:101-106): after
// column j of n the bottom-row score can fall by at most 1 per remaining
// column, so score - (n - 1 - j) > k already proves d > k.
BLG_HD bool hopeless(int score, int j, int n, int k) { return k >= 0 && score - (n - 1 - j) > k; }

// ---- pipe-balanced step on 32-bit halves --------------------------------
// A 64-bit Myers step is ~25 32-bit instructions; written plainly they all
// land on the ALU pipe, which then limits throughput while the FMA pipe
// (IMAD) idles. The forms below move the low-half shifts, the character
// offsets and the score bits onto IMAD; the 64-bit add stays a carry-chained
// ALU pair, which measured faster than IMAD.WIDE. Multipliers come from
// run-time values (`Units`, loaded from a kernel parameter) so the compiler
// cannot turn the multiply-adds back into shifts. On the host the same
// functions are plain integer arithmetic.
struct Units {
    uint32_t one, two;
};

BLG_HD uint32_t imad_lo(uint32_t a, uint32_t b, uint32_t c) {
#if defined(__CUDA_ARCH__)
    uint32_t r;
    asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
    return r;
#else
    return a * b + c;
#endif
}

// high 32 bits of a*b, plus c
BLG_HD uint32_t imad_hi(uint32_t a, uint32_t b, uint32_t c) {
#if defined(__CUDA_ARCH__)
    uint32_t r;
    asm("mad.hi.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
    return r;
#else
    return (uint32_t)(((uint64_t)a * b) >> 32) + c;
#endif
}

// (hi:lo) << 1, high half
BLG_HD uint32_t shl1_hi(uint32_t lo, uint32_t hi) {
#if defined(__CUDA_ARCH__)
    return __funnelshift_l(lo, hi, 1);
#else
    return (hi << 1) | (lo >> 31);
#endif
}

// (ah:al) + (bh:bl) with the carry passed between the halves.
BLG_HD void add64(uint32_t al, uint32_t ah, uint32_t bl, uint32_t bh, uint32_t &sl, uint32_t &sh) {
#if defined(__CUDA_ARCH__)
    asm("add.cc.u32 %0, %2, %3;\n\taddc.u32 %1, %4, %5;" : "=r"(sl), "=r"(sh) : "r"(al), "r"(bl), "r"(ah), "r"(bh));
#else
    const uint64_t r = (((uint64_t)ah << 32) | al) + (((uint64_t)bh << 32) | bl);
    sl = (uint32_t)r;
    sh = (uint32_t)(r >> 32);
#endif
}

// A pattern word as halves plus its vertical-delta state.
struct Word2 {
    uint32_t pl, ph, ml, mh;   // Pv, Mv
};

// One column on one word. cin_p / cin_m are the +1 / -1 carry-in bits
// (top word: cin_p = 1, cin_m = 0). Returns the pre-shift Ph/Mh halves so
// the caller reads the horizontal delta at its output bit.
BLG_HD void step_h(Word2 &s, uint32_t el, uint32_t eh, uint32_t cin_p, uint32_t cin_m, Units u,
                   uint32_t &Phl, uint32_t &Phh, uint32_t &Mhl, uint32_t &Mhh) {
    const uint32_t vl = el | s.ml, vh = eh | s.mh;            // Xv = Eq | Mv
    const uint32_t el2 = el | cin_m;                           // a -1 carry acts as a match
    // sum = (Eq & Pv) + Pv as a carry-chained pair of 32-bit adds (ALU). An
    // IMAD.WIDE form measured 13% slower in the exact search on GB300.
    uint32_t sl, sh;
    add64(el2 & s.pl, eh & s.ph, s.pl, s.ph, sl, sh);
    const uint32_t xl = (sl ^ s.pl) | el2, xh = (sh ^ s.ph) | eh;   // Xh
    Phl = s.ml | ~(xl | s.pl);
    Phh = s.mh | ~(xh | s.ph);
    Mhl = s.pl & xl;
    Mhh = s.ph & xh;
    const uint32_t psl = imad_lo(Phl, u.two, cin_p), psh = shl1_hi(Phl, Phh);   // Ph << 1 | cin_p
    const uint32_t msl = imad_lo(Mhl, u.two, cin_m), msh = shl1_hi(Mhl, Mhh);   // Mh << 1 | cin_m
    s.pl = msl | ~(vl | psl);
    s.ph = msh | ~(vh | psh);
    s.ml = psl & vl;
    s.mh = psh & vh;
}

// Bit 31 of x as 0/1, on the FMA pipe: hi32(x * 2).
BLG_HD uint32_t top_bit(uint32_t x, Units u) { return imad_hi(x, u.two, 0); }

// ---- banded column loop (max_dist k <= 31) --------------------------------
// Every alignment path of cost <= k keeps its diagonal delta = j - i within
// |delta| + |g - delta| <= k (g = n - m): at most k+1 diagonals [dlo, dhi].
// A 32-row window sliding down one row per text column (rows j - dhi ..
// j - dhi + 31) holds them all, so one 32-bit Myers step per column suffices
// whatever the pattern length. Boundaries: rows <= 0 are virtual rows with
// D[i][j] = j - i (exact under the recurrence since they never match); the
// row leaving the window top is taken to grow by +1 per column and the row
// entering at the bottom gets vertical delta +1. Both are upper bounds of
// the true values and the recurrence is monotone, while the cells of an
// optimal in-band path are computed exactly; so min(D'[m][n], k+1) =
// min(d, k+1). The exit fires once a lower bound of every band cell of the
// current column exceeds k (a path of cost <= k crosses every column inside
// the band, through exactly computed cells).
struct BandGeom {
    int dhi, g, s;          // top diagonal, n - m, window bit of row m at column n
    uint32_t band;          // window bits 1 .. B-1 (B = band width <= k + 1)
};

BLG_HD BandGeom band_geom(int m, int n, int k) {
    BandGeom bg;
    bg.g = n - m;
    const int ag = bg.g < 0 ? -bg.g : bg.g;
    const int half = (k - ag) >> 1;
    bg.dhi = (bg.g > 0 ? bg.g : 0) + half;
    const int dlo = (bg.g < 0 ? bg.g : 0) - half;
    const int B = bg.dhi - dlo + 1;
    bg.band = (B >= 32 ? 0xffffffffu : ((1u << B) - 1u)) & ~1u;
    bg.s = bg.dhi - bg.g;
    return bg;
}

BLG_HD int popc32(uint32_t x) {
#if defined(__CUDA_ARCH__)
    return __popc(x);
#else
    return __builtin_popcount(x);
#endif
}

// The banded loop's state before text column j: the window's vertical
// deltas and D' of its top row. A run may stop at any column and resume
// from the state later with the same results (band_steps).
struct BandState {
    uint32_t pv, mv;
    int A, j;
};

BLG_HD BandState band_start(const BandGeom &bg) {
    const int nv = bg.dhi + 1;                               // virtual rows -dhi .. 0 at column 0
    BandState s;
    s.mv = nv >= 32 ? 0xffffffffu : ((1u << nv) - 1u);
    s.pv = ~s.mv;
    s.A = bg.dhi;                                            // D'[top window row][current column]
    s.j = 0;
    return s;
}

// Text columns s.j .. j_end - 1; s.j is 0 or a multiple of 4. text(j)
// returns text byte j (called once per j in order); eqw(c, p0) returns the
// window's match bits for byte c, where p0 is the 0-based pattern index of
// window bit 0 (positions < 0 or >= m give no bits). Returns true when the
// exit fired (s.j = that column); otherwise s holds the state before column
// j_end. The exit test runs before every 4th column; the main loop takes 4
// columns per iteration, so the readers' per-column alignment tests fold.
template <typename TextFn, typename EqW>
BLG_HD bool band_steps(int k, const BandGeom &bg, BandState &s, int j_end, TextFn text, EqW eqw) {
    uint32_t pv = s.pv, mv = s.mv;
    int A = s.A;
    auto column = [&](int j) {
        const uint32_t c = text(j);
        // column j's deltas re-indexed one row down; the new bottom row enters with +1
        // (plain shifts and add: the IMAD forms of the 32-bit step measured
        // 2-4% slower here, where the column chain is latency-bound)
        pv = (pv >> 1) | 0x80000000u;
        mv >>= 1;
        const uint32_t eq = eqw(c, j - bg.dhi);
        const uint32_t xv = eq | mv;
        const uint32_t sum = (eq & pv) + pv;
        const uint32_t xh = (sum ^ pv) | eq;
        const uint32_t ph = mv | ~(xh | pv);
        const uint32_t mh = pv & xh;
        const uint32_t phs = (ph << 1) | 1u, mhs = mh << 1;
        pv = mhs | ~(xv | phs);
        mv = phs & xv;
        A += 1 + (int)(pv & 1u) - (int)(mv & 1u);
    };
    auto stop = [&](int j) {
        s.pv = pv;
        s.mv = mv;
        s.A = A;
        s.j = j;
    };
    int j = s.j;
    for (; j + 4 <= j_end; j += 4) {
#if defined(__CUDA_ARCH__)
        __builtin_assume((j & 3) == 0);
#endif
        if (j > 0 && A - popc32(mv & bg.band) > k) {          // every band cell > k
            stop(j);
            return true;
        }
        column(j);
        column(j + 1);
        column(j + 2);
        column(j + 3);
    }
    for (; j < j_end; j++) {
        if ((j & 3) == 0 && j > 0 && A - popc32(mv & bg.band) > k) {
            stop(j);
            return true;
        }
        column(j);
    }
    stop(j_end);
    return false;
}

// min(d, k+1) from the state after the last text column.
BLG_HD int band_finish(int k, const BandGeom &bg, const BandState &s) {
    const uint32_t ms = (bg.s >= 31 ? 0xffffffffu : ((2u << bg.s) - 1u)) & ~1u;   // bits 1..s
    return cap_k(s.A + popc32(s.pv & ms) - popc32(s.mv & ms), k);
}

// The whole banded run. Caller guarantees 1 <= m, |n - m| <= k <= 31.
// Returns min(d, k+1); *cols_out = text columns processed.
template <typename TextFn, typename EqW>
BLG_HD int band_core(int m, int n, int k, TextFn text, EqW eqw, Units u, int *cols_out) {
    (void)u;                                                 // plain shifts here (see the column step)
    const BandGeom bg = band_geom(m, n, k);
    BandState s = band_start(bg);
    const bool exited = band_steps(k, bg, s, n, text, eqw);
    if (cols_out) *cols_out = s.j;
    return exited ? k + 1 : band_finish(k, bg, s);
}

// ---- host-side reference of the per-pair device logic ------------------
// pair_distance_plain: trimming + pattern = shorter string + gap exit +
// single/multi-word run with per-character Eq from a 256-row table.  The
// GPU kernels compute exactly this value; the host build checks it.
BLG_HD void trim_affixes(const uint8_t *&a, int &la, const uint8_t *&b, int &lb) {
    const int lim = la < lb ? la : lb;
    int p = 0;
    while (p < lim && a[p] == b[p]) p++;
    int s = 0;
    while (s < lim - p && a[la - 1 - s] == b[lb - 1 - s]) s++;
    a += p; b += p; la -= p + s; lb -= p + s;
}

}  // namespace blg
