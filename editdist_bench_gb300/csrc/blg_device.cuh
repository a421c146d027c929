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
