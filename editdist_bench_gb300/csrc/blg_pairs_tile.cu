// Short-pair tile kernel (pairwise, trimmed patterns of at most 32 bytes).
//
// The reference runs one thread per pair in natural order over global
// memory (csrc/gpu_kernels.cu:6-32, csrc/gpu_myers.cuh:73-119). For short
// pairs that schedule wastes most of every warp: after exact trimming about
// half of the pairs have no work left and the rest keep a handful of
// columns, so a warp runs as long as its slowest lane. Here a persistent CTA
// walks tiles of up to 512 consecutive pairs:
//
//  1. staging: the tile's a and b byte spans are contiguous in the packed
//     layout (csrc/edpy.c:200-224), so one bulk copy (TMA, cp.async.bulk)
//     per side brings them into shared memory, double-buffered: the copy of
//     the CTA's next tile is in flight while this one is computed. Each
//     thread's string offsets for the next tile are prefetched into
//     registers the same way;
//  2. trim + classify from shared memory: common prefix/suffix removed
//     (exact, csrc/myers.c:80-87), trivial pairs (length gap beyond k,
//     empty pattern) finished at once, patterns longer than 32 queued for the
//     lane-spread consumer, the rest listed with their trimmed column count;
//  3. a counting sort of the listed pairs by column count inside the CTA, so
//     each warp takes 32 pairs of nearly equal work;
//  4. solve: one 32-bit Myers/Hyyro word per pair, Eq from per-thread rows
//     (one per byte when the pair set uses at most 15 distinct bytes, else
//     nibble rows), the final score read from the last column's vertical
//     deltas (D[m][n] = n + popc(Pv) - popc(Mv) over the pattern rows);
//  5. the tile's results leave as coalesced vector stores.
#include <algorithm>

#include "blg_kernels.cuh"
#include "blg_tma.cuh"

namespace blg {

constexpr int kTileThreads = 256;
constexpr int kTileMaxPairs = 512;

// Stage of a tile of up to PM pairs: rounded span bytes per side (PM pairs
// of at most 33 bytes), plus 16 bytes of slack before and 32 after.
template <int PM>
struct TileDims {
    static constexpr int Cap = PM * 33;
    static constexpr int Side = Cap + 48;
};
constexpr int kTileKeys = 64;                    // counting-sort keys: min(columns, 63)
constexpr int32_t kNoStore = INT32_MIN;          // result slot filled by the long-pair consumer

// NBUF = 2: the next tile's copy flies while this one computes; NBUF = 1:
// one stage, the copy is issued when the tile is done and the other CTAs of
// the SM compute meanwhile. Up to PM pairs per tile (512 or 256). CTAs per
// SM: 3 (one stage, 512 pairs, nibble rows), 4 (the same with one row per
// byte, or two stages of 256 pairs), 2 (two stages of 512).
template <int NBUF, bool SYM, int PM>
struct __align__(16) TileShared {
    uint8_t stage[NBUF][2][TileDims<PM>::Side];   // [buffer][a|b]
    uint32_t tab[(SYM ? 16 : 32) * kTileThreads]; // pattern rows, row r of thread t at [r*256 + t]
    uint8_t map[SYM ? 256 : 4];                   // byte -> row (SYM)
    uint2 ent[PM];                                // sorted work list
    int32_t res[PM];
    int32_t hist[kTileKeys];
    int32_t start[kTileKeys];
    int64_t span_lo[2][2], span_hi[2][2];         // staged span [lo, hi) per buffer/side, lo < 0: none
    uint64_t bar[2];
    int32_t total, next;
};

// One 32-bit Myers/Hyyro column step on the top word (carry-in +1), with
// the add and the shifts on the FMA pipe (IMAD) and the bitwise work on the ALU.
__device__ __forceinline__ void step32(uint32_t &pv, uint32_t &mv, uint32_t eq, Units u) {
    const uint32_t xv = eq | mv;
    const uint32_t sum = imad_lo(eq & pv, u.one, pv);
    const uint32_t xh = (sum ^ pv) | eq;
    const uint32_t ph = mv | ~(xh | pv);
    const uint32_t mh = pv & xh;
    const uint32_t phs = imad_lo(ph, u.two, u.one);
    const uint32_t mhs = imad_lo(mh, u.two, 0);
    pv = mhs | ~(xv | phs);
    mv = phs & xv;
}

// Per-thread rows of a pattern of m <= 32 bytes (bit i <-> position i), in a
// [row][thread] table. SYM = false: nibble rows, row h (0..15) holds the
// positions whose high nibble is h, row 16 + l those whose low nibble is l,
// Eq(c) = row[c >> 4] & row[16 + (c & 15)]. SYM = true: the pair set uses at
// most 15 distinct bytes and row map[c] holds the positions of byte c (the
// bytes outside the set map to row 15, which stays empty): one row update
// per pattern byte, one row load per text column, half the table.
template <bool SYM>
struct Rows32 {
    static constexpr int R = SYM ? 16 : 32;
    uint32_t *tc;                                  // this thread's row 0
    const uint8_t *map;
    // position bit of byte c (one shared-memory atomic OR per row update
    // instead of a load-or-store chain)
    __device__ __forceinline__ void set(uint32_t c, uint32_t bit) const {
        if (SYM) {
            atomicOr(tc + map[c] * kTileThreads, bit);
        } else {
            atomicOr(tc + (c >> 4) * kTileThreads, bit);
            atomicOr(tc + (16 + (c & 15)) * kTileThreads, bit);
        }
    }
    __device__ __forceinline__ void clear_byte(uint32_t c) const {
        if (SYM) {
            tc[map[c] * kTileThreads] = 0;
        } else {
            tc[(c >> 4) * kTileThreads] = 0;
            tc[(16 + (c & 15)) * kTileThreads] = 0;
        }
    }
    __device__ __forceinline__ void clear_all() const {
#pragma unroll
        for (int r = 0; r < R; r++) tc[r * kTileThreads] = 0;
    }
    __device__ __forceinline__ uint32_t eq(uint32_t c) const {
        if (SYM) return tc[map[c] * kTileThreads];
        return tc[(c >> 4) * kTileThreads] & tc[(16 + (c & 15)) * kTileThreads];
    }
};

// Rows of a pattern read through loader L: set, or clear the rows it touched.
template <typename L, bool SYM>
__device__ __forceinline__ void rows_pattern(const Rows32<SYM> &rw, const uint8_t *p, int m, bool set) {
    TextScanT<L> ps;
    ps.init(p);
    for (int i = 0; i < m; i += 4) {
        const uint32_t w4 = ps.next4();
#pragma unroll
        for (int b = 0; b < 4; b++) {
            if (i + b < m) {
                const uint32_t c = (w4 >> (8 * b)) & 0xffu;
                if (set) rw.set(c, 1u << (i + b));
                else rw.clear_byte(c);
            }
        }
    }
}

// ---- strings in the stage, addressed by byte offset from its 16-byte-aligned
// base: the alignment comes from the offset, so the pointers never pass
// through an integer and stay shared-memory addresses (32-bit loads).
struct StageScan {
    const uint32_t *w;
    uint32_t lo, hi, sh;
    __device__ __forceinline__ void init(const uint8_t *base, uint32_t off) {
        w = reinterpret_cast<const uint32_t *>(base + (off & ~3u));
        sh = (off & 3u) * 8u;
        lo = w[0];
        hi = w[1];
        w += 2;
    }
    __device__ __forceinline__ uint32_t next4() {
        const uint32_t r = __funnelshift_r(lo, hi, sh);
        lo = hi;
        hi = *w++;
        return r;
    }
};

// Exact prefix/suffix trimming of staged strings a (offset oa, length la) and
// b (ob, lb), 4-byte windows (csrc/myers.c:80-87). Each side is read by a
// running pair of aligned words, so a window costs one shared-memory load per
// string plus a funnel shift; the prefix walks forward, the suffix backward
// (a window's alignment remainder does not change as it moves by 4).
__device__ __forceinline__ void stage_trim(const uint8_t *base, uint32_t &oa, int &la, uint32_t &ob, int &lb) {
    const int lim = la < lb ? la : lb;
    int p = 0;
    if (lim > 0) {
        const uint32_t *wa = reinterpret_cast<const uint32_t *>(base + (oa & ~3u));
        const uint32_t *wb = reinterpret_cast<const uint32_t *>(base + (ob & ~3u));
        const uint32_t sa = (oa & 3u) * 8u, sb = (ob & 3u) * 8u;
        uint32_t a0 = wa[0], b0 = wb[0];
        while (p < lim) {
            const uint32_t a1 = *++wa, b1 = *++wb;
            const uint32_t x = __funnelshift_r(a0, a1, sa) ^ __funnelshift_r(b0, b1, sb);
            int q = x ? (__ffs(x) - 1) >> 3 : 4;
            if (q > lim - p) q = lim - p;
            p += q;
            if (q < 4) break;
            a0 = a1;
            b0 = b1;
        }
    }
    const int lim2 = lim - p;
    int s = 0;
    if (lim2 > 0) {
        const uint32_t ea = oa + (uint32_t)la - 4u, eb = ob + (uint32_t)lb - 4u;   // first suffix window
        const uint32_t *wa = reinterpret_cast<const uint32_t *>(base + (ea & ~3u));
        const uint32_t *wb = reinterpret_cast<const uint32_t *>(base + (eb & ~3u));
        const uint32_t sa = (ea & 3u) * 8u, sb = (eb & 3u) * 8u;
        uint32_t a1 = wa[1], b1 = wb[1];
        while (s < lim2) {
            const uint32_t a0 = *wa--, b0 = *wb--;
            const uint32_t x = __funnelshift_r(a0, a1, sa) ^ __funnelshift_r(b0, b1, sb);
            int q = x ? __clz(x) >> 3 : 4;
            if (q > lim2 - s) q = lim2 - s;
            s += q;
            if (q < 4) break;
            a1 = a0;
            b1 = b0;
        }
    }
    oa += p;
    ob += p;
    la -= p + s;
    lb -= p + s;
}

// Rows of a staged pattern: set them, or clear them: all rows with plain
// stores once the pattern touches more rows than that, else just the rows it
// touched.
template <bool SYM>
__device__ __forceinline__ void stage_rows(const Rows32<SYM> &rw, const uint8_t *base, uint32_t op, int m, bool set) {
    if (!set && m > Rows32<SYM>::R / 8) {
        rw.clear_all();
        return;
    }
    StageScan ps;
    ps.init(base, op);
    for (int i = 0; i < m; i += 4) {
        const uint32_t w4 = ps.next4();
#pragma unroll
        for (int b = 0; b < 4; b++) {
            if (i + b < m) {
                const uint32_t c = (w4 >> (8 * b)) & 0xffu;
                if (set) rw.set(c, 1u << (i + b));
                else rw.clear_byte(c);
            }
        }
    }
}

// solve32 for a staged pair (pattern at op, text at ot).
template <bool HASK, bool SYM>
__device__ __forceinline__ int stage_solve32(const Rows32<SYM> &rw, const uint8_t *base, uint32_t op, int m, uint32_t ot,
                                             int n, int k, Units u) {
    stage_rows(rw, base, op, m, true);
    const uint32_t M = m >= 32 ? 0xffffffffu : ((1u << m) - 1u);
    uint32_t pv = 0xffffffffu, mv = 0;
    StageScan ts;
    ts.init(base, ot);
    bool dead = false;
    int j = 0;
    for (; j + 4 <= n; j += 4) {
        const uint32_t w4 = ts.next4();
        step32(pv, mv, rw.eq(w4 & 0xffu), u);
        step32(pv, mv, rw.eq((w4 >> 8) & 0xffu), u);
        step32(pv, mv, rw.eq((w4 >> 16) & 0xffu), u);
        step32(pv, mv, rw.eq(w4 >> 24), u);
        if (HASK && hopeless(j + 4 + popc32(pv & M) - popc32(mv & M), j + 3, n, k)) {
            dead = true;
            break;
        }
    }
    if (!dead && j < n) {
        uint32_t w4 = ts.next4();
        for (; j < n; j++, w4 >>= 8) step32(pv, mv, rw.eq(w4 & 0xffu), u);
    }
    stage_rows(rw, base, op, m, false);
    if (dead) return k + 1;
    const int d = n + popc32(pv & M) - popc32(mv & M);
    return HASK ? cap_k(d, k) : d;
}

// d(p, t) for 1 <= m <= 32, m <= n; min(d, k+1) when HASK.
template <bool HASK, typename L, bool SYM>
__device__ __forceinline__ int solve32(const Rows32<SYM> &rw, const uint8_t *p, int m, const uint8_t *t, int n, int k,
                                       Units u) {
    rows_pattern<L>(rw, p, m, true);
    const uint32_t M = m >= 32 ? 0xffffffffu : ((1u << m) - 1u);
    uint32_t pv = 0xffffffffu, mv = 0;
    TextScanT<L> ts;
    ts.init(t);
    bool dead = false;
    int j = 0;
    for (; j + 4 <= n; j += 4) {
        const uint32_t w4 = ts.next4();
        step32(pv, mv, rw.eq(w4 & 0xffu), u);
        step32(pv, mv, rw.eq((w4 >> 8) & 0xffu), u);
        step32(pv, mv, rw.eq((w4 >> 16) & 0xffu), u);
        step32(pv, mv, rw.eq(w4 >> 24), u);
        // D[m][j+4] from the vertical deltas; the exit test is monotone in j,
        // so testing every 4th column is exact (csrc/myers.c:101-106)
        if (HASK && hopeless(j + 4 + popc32(pv & M) - popc32(mv & M), j + 3, n, k)) {
            dead = true;
            break;
        }
    }
    if (!dead && j < n) {
        uint32_t w4 = ts.next4();
        for (; j < n; j++, w4 >>= 8) step32(pv, mv, rw.eq(w4 & 0xffu), u);
    }
    rows_pattern<L>(rw, p, m, false);
    if (dead) return k + 1;
    const int d = n + popc32(pv & M) - popc32(mv & M);
    return HASK ? cap_k(d, k) : d;
}

// Thread 0: the rounded spans of a tile's strings, one bulk copy per side
// into `buf`, completing on bar[buf]. (a0, a1) and (b0, b1) are the string
// offsets bounding the tile, off[t0] and off[t0 + cnt], of each side.
template <int CAP, typename TS>
__device__ __forceinline__ void tile_issue(TS &S, int buf, const DevStrings &A, const DevStrings &B,
                                           int64_t a0, int64_t a1, int64_t b0, int64_t b1) {
    auto span = [&](const DevStrings &D, int64_t o0, int64_t o1, int side) -> uint32_t {
        const int64_t lo = o0 - D.base, hi = o1 - D.base;
        int64_t lo16 = -1, hi16 = -1;
        if (lo >= 0 && hi >= lo && hi <= D.bytes) {
            lo16 = lo & ~int64_t(15);
            hi16 = (hi + 15) & ~int64_t(15);     // inside the buffer's 16-byte tail slack
            if (hi16 - lo16 > CAP || (reinterpret_cast<uintptr_t>(D.buf + lo16) & 15)) lo16 = hi16 = -1;
        }
        S.span_lo[buf][side] = lo16;
        S.span_hi[buf][side] = hi16;
        return lo16 >= 0 ? (uint32_t)(hi16 - lo16) : 0u;
    };
    const uint32_t la = span(A, a0, a1, 0), lb = span(B, b0, b1, 1);
    mbar_arrive_expect(&S.bar[buf], la + lb);
    if (la) bulk_g2s(S.stage[buf][0] + 16, A.buf + S.span_lo[buf][0], la, &S.bar[buf]);
    if (lb) bulk_g2s(S.stage[buf][1] + 16, B.buf + S.span_lo[buf][1], lb, &S.bar[buf]);
}

// Validated view of string i from prefetched offsets (o0, o1). TRUST: the
// host's pass over the offsets found every pair in order (and the set's
// first and last offsets bound the uploaded buffer), so the checks are left
// out.
template <bool TRUST>
__device__ __forceinline__ const uint8_t *string_from(const DevStrings &S, int64_t o0, int64_t o1, int &len,
                                                      uint32_t *status) {
    if (!TRUST && (o0 < S.base || o1 < o0 || o1 - S.base > S.bytes || o1 - o0 > 0x7fffffff)) {
        atomicOr(status, ST_BAD_OFFSETS);
        len = 0;
        return S.buf;
    }
    len = (int)(o1 - o0);
    return S.buf + (o0 - S.base);
}

struct PairOffs {
    int64_t a0, a1, b0, b1;
};

__device__ __forceinline__ void load_offs(PairOffs &o, const DevStrings &A, const DevStrings &B, int64_t i,
                                          int64_t n) {
    if (i < n) {
        o.a0 = __ldg(A.off + i);
        o.a1 = __ldg(A.off + i + 1);
        o.b0 = __ldg(B.off + i);
        o.b1 = __ldg(B.off + i + 1);
    }
}

// alpha: the pair set's bytes (8 words; SYM builds its byte -> row map from
// them), or null when the host chose the variant. Given to both variants,
// the one that does not apply returns at once.
template <bool HASK, int NBUF, bool TRUST, bool SYM, int PM>
__global__ void __launch_bounds__(kTileThreads, (NBUF == 1 && SYM) || PM == 256 ? 4 : (NBUF == 2 ? 2 : 3))
    k_pairs_tile(DevStrings A, DevStrings B, int P, int k, int dtype, void *out, LongQueue q, uint32_t *status,
                 uint32_t unit, uint32_t wait_polls, const uint32_t *alpha) {
    extern __shared__ __align__(128) uint8_t s_raw[];
    TileShared<NBUF, SYM, PM> &S = *reinterpret_cast<TileShared<NBUF, SYM, PM> *>(s_raw);
    constexpr int kSide = TileDims<PM>::Side, kCap = TileDims<PM>::Cap;
    const Units u{unit, unit + unit};
    const int tid = threadIdx.x;
    if (alpha && (alpha_size(alpha) <= kBandSymbols) != SYM) return;   // uniform: the other variant runs the set
    if (SYM) alpha_map(alpha, S.map);
    const int64_t n = A.n;
    const int64_t ntiles = (n + P - 1) / P;
    const int64_t G = gridDim.x;
    const Rows32<SYM> rw{S.tab + tid, S.map};
    rw.clear_all();
    if (tid < kTileKeys) S.hist[tid] = 0;
    if (tid == 0) {
        mbar_init(&S.bar[0], 1);
        mbar_init(&S.bar[1], 1);
    }
    __syncthreads();

    // thread 0's pipeline of tile bounds: nb = bounds of the CTA's next tile
    PairOffs nb = {0, 0, 0, 0};                     // (a0, a1, b0, b1) bounds of the tile
    auto tile_bounds = [&](int64_t t, PairOffs &bd) {
        const int64_t t0 = t * P, t1 = t0 + P < n ? t0 + P : n;
        bd.a0 = __ldg(A.off + t0);
        bd.a1 = __ldg(A.off + t1);
        bd.b0 = __ldg(B.off + t0);
        bd.b1 = __ldg(B.off + t1);
    };
    const int64_t first = blockIdx.x;
    if (tid == 0 && first < ntiles) {
        PairOffs bd;
        tile_bounds(first, bd);
        tile_issue<kCap>(S, 0, A, B, bd.a0, bd.a1, bd.b0, bd.b1);
        if (first + G < ntiles) tile_bounds(first + G, nb);
    }
    // every thread's offsets for its (up to two) pairs of the current tile
    PairOffs po0 = {0, 0, 0, 0}, po1 = {0, 0, 0, 0};
    if (first < ntiles) {
        load_offs(po0, A, B, first * P + tid, n);
        if (tid + kTileThreads < P) load_offs(po1, A, B, first * P + tid + kTileThreads, n);
    }

    int it = 0;
    for (int64_t t = first; t < ntiles; t += G, it++) {
        const int buf = NBUF == 2 ? (it & 1) : 0;
        const uint32_t parity = NBUF == 2 ? ((uint32_t)(it >> 1) & 1u) : ((uint32_t)it & 1u);
        const int64_t t0 = t * P;
        const int cnt = (int)(n - t0 < P ? n - t0 : P);
        if (NBUF == 2 && tid == 0 && t + G < ntiles) {    // prefetch the next tile's strings
            tile_issue<kCap>(S, buf ^ 1, A, B, nb.a0, nb.a1, nb.b0, nb.b1);
            if (t + 2 * G < ntiles) tile_bounds(t + 2 * G, nb);
        }
        const bool ok = mbar_wait(&S.bar[buf], parity, wait_polls);
        if (__syncthreads_or(!ok)) {
            // a copy did not complete in time: report, wait (bounded, at the
            // normal bound whatever `wait_polls` was) for the copies still in
            // flight, and stop
            if (tid == 0) {
                atomicOr(status, ST_QUEUE_TIMEOUT);
                mbar_wait(&S.bar[buf], parity);
                if (NBUF == 2 && t + G < ntiles) mbar_wait(&S.bar[buf ^ 1], (uint32_t)((it + 1) >> 1) & 1u);
            }
            return;
        }
        const int64_t alo = S.span_lo[buf][0], ahi = S.span_hi[buf][0];
        const int64_t blo = S.span_lo[buf][1], bhi = S.span_hi[buf][1];
        const uint8_t *stage = S.stage[buf][0];

        // ---- phase 1: trim, finish trivial pairs, queue long ones, list the rest
        int key0 = -1, key1 = -1, rank0 = 0, rank1 = 0;
        uint2 ent0 = make_uint2(0, 0), ent1 = make_uint2(0, 0);
        auto classify = [&](const PairOffs &o, int j, int &key, int &rank, uint2 &ent) {
            const int64_t i = t0 + j;
            int la, lb;
            const uint8_t *ga = string_from<TRUST>(A, o.a0, o.a1, la, status);
            const uint8_t *gb = string_from<TRUST>(B, o.b0, o.b1, lb, status);
            const int64_t ra = ga - A.buf, rb = gb - B.buf;
            const bool sa = alo >= 0 && ra >= alo && ra + la <= ahi;
            const bool sb = blo >= 0 && rb >= blo && rb + lb <= bhi;
            const uint8_t *a, *b;
            int64_t pre;
            uint32_t oa = 0, ob = 0;
            if (sa && sb) {                                 // both staged: 32-bit shared offsets
                oa = 16 + (uint32_t)(ra - alo);
                ob = kSide + 16 + (uint32_t)(rb - blo);
                const uint32_t oa0 = oa;
                stage_trim(stage, oa, la, ob, lb);
                pre = oa - oa0;
                a = stage + oa;
                b = stage + ob;
            } else {
                a = sa ? stage + 16 + (ra - alo) : ga;
                b = sb ? stage + kSide + 16 + (rb - blo) : gb;
                const uint8_t *a_start = a;
                trim_windows<GenericLoad>(a, la, b, lb);
                pre = a - a_start;
            }
            const uint8_t *gpa = ga + pre, *gpb = gb + pre;
            if (la > lb) {                                  // the shorter string is the pattern
                const uint8_t *x = a; a = b; b = x;
                x = gpa; gpa = gpb; gpb = x;
                const uint32_t z = oa; oa = ob; ob = z;
                const int y = la; la = lb; lb = y;
            }
            int d = kNoStore;
            if (HASK && lb - la > k) d = k + 1;             // length gap alone exceeds k
            else if (la == 0) d = lb;
            else if (la > 32) {
                const int cls = long_class(la);
                d = -1;
                if (cls < 0) atomicOr(status, ST_TOO_LONG);
                else {
                    const int pos = atomicAdd(&q.counts[cls], 1);
                    if (pos < q.cap[cls]) {
                        LongItem itm;
                        itm.pat = gpa; itm.txt = gpb; itm.m = la; itm.n = lb; itm.idx = i;
                        q.items[cls][pos] = itm;
                        d = kNoStore;
                    } else {
                        atomicOr(status, ST_QUEUE_OVERFLOW);
                    }
                }
            } else if (sa && sb) {
                key = lb < kTileKeys - 1 ? lb : kTileKeys - 1;
                rank = atomicAdd(&S.hist[key], 1);
                ent = make_uint2(oa | (ob << 16), (uint32_t)lb | ((uint32_t)la << 16) | ((uint32_t)j << 22));
            } else {
                d = solve32<HASK, GenericLoad>(rw, a, la, b, lb, k, u);   // not staged: read in place
            }
            S.res[j] = d;
        };
        if (tid < cnt) classify(po0, tid, key0, rank0, ent0);
        if (tid + kTileThreads < cnt) classify(po1, tid + kTileThreads, key1, rank1, ent1);
        // the next tile's offsets, in flight during the rest of this one
        if (t + G < ntiles) {
            load_offs(po0, A, B, (t + G) * P + tid, n);
            if (tid + kTileThreads < P) load_offs(po1, A, B, (t + G) * P + tid + kTileThreads, n);
        }
        __syncthreads();
        // ---- phase 2: bucket starts (largest column count first)
        if (tid < 32) {
            const int h0 = S.hist[kTileKeys - 1 - 2 * tid], h1 = S.hist[kTileKeys - 2 - 2 * tid];
            int incl = h0 + h1;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(kFull, incl, o);
                if (tid >= o) incl += v;
            }
            const int excl = incl - h0 - h1;
            S.start[kTileKeys - 1 - 2 * tid] = excl;
            S.start[kTileKeys - 2 - 2 * tid] = excl + h0;
            if (tid == 31) {
                S.total = incl;
                S.next = 0;
            }
        }
        __syncthreads();
        if (key0 >= 0) S.ent[S.start[key0] + rank0] = ent0;
        if (key1 >= 0) S.ent[S.start[key1] + rank1] = ent1;
        __syncthreads();
        // ---- phase 3: solve in sorted order, longest first: warps pull 32-pair
        //      chunks of the list from a shared counter
        const int total = S.total;
        while (true) {
            int c = 0;
            if ((tid & 31) == 0) c = atomicAdd(&S.next, 1);
            c = __shfl_sync(kFull, c, 0);
            if (c * 32 >= total) break;
            const int e = c * 32 + (tid & 31);
            if (e < total) {
                const uint2 E = S.ent[e];
                const int m = (int)((E.y >> 16) & 63u), nn = (int)(E.y & 0xffffu), j = (int)(E.y >> 22);
                S.res[j] = stage_solve32<HASK>(rw, stage, E.x & 0xffffu, m, E.x >> 16, nn, k, u);
            }
        }
        __syncthreads();
        // ---- phase 4: coalesced stores of the tile's results
        for (int j4 = tid * 4; j4 < cnt; j4 += 4 * kTileThreads) {
            const int c4 = cnt - j4 < 4 ? cnt - j4 : 4;
            const int d0 = S.res[j4], d1 = c4 > 1 ? S.res[j4 + 1] : 0, d2 = c4 > 2 ? S.res[j4 + 2] : 0,
                      d3 = c4 > 3 ? S.res[j4 + 3] : 0;
            if (c4 == 4 && d0 != kNoStore && d1 != kNoStore && d2 != kNoStore && d3 != kNoStore) {
                store4(out, dtype, t0 + j4, 4, d0, d1, d2, d3);
            } else {
                if (d0 != kNoStore) store1(out, dtype, t0 + j4, d0);
                if (c4 > 1 && d1 != kNoStore) store1(out, dtype, t0 + j4 + 1, d1);
                if (c4 > 2 && d2 != kNoStore) store1(out, dtype, t0 + j4 + 2, d2);
                if (c4 > 3 && d3 != kNoStore) store1(out, dtype, t0 + j4 + 3, d3);
            }
        }
        if (tid < kTileKeys) S.hist[tid] = 0;
        __syncthreads();                                    // the stage buffer and lists are reused
        if (NBUF == 1 && tid == 0 && t + G < ntiles) {    // the single stage is free: next tile's copy
            tile_issue<kCap>(S, 0, A, B, nb.a0, nb.a1, nb.b0, nb.b1);
            if (t + 2 * G < ntiles) tile_bounds(t + 2 * G, nb);
        }
    }
}

// ------------------------------------------------------------- launcher --
template <bool HASK, int NBUF, bool TRUST, bool SYM, int PM>
static cudaError_t launch_tile(cudaStream_t st, int sms, const DevStrings &A, const DevStrings &B, int P, int k,
                               int dtype, void *out, const LongQueue &q, uint32_t *status, uint32_t polls,
                               const uint32_t *alpha) {
    P = std::max(32, (P * PM / kTileMaxPairs) & ~3);       // the caller sized P for a 512-pair stage
    const int64_t ntiles = (A.n + P - 1) / P;
    const int per_sm = (NBUF == 1 && SYM) || PM == 256 ? 4 : (NBUF == 2 ? 2 : 3);
    const int grid = (int)std::min<int64_t>(ntiles, (int64_t)sms * per_sm);
    const size_t smem = sizeof(TileShared<NBUF, SYM, PM>);
    cudaFuncSetAttribute(k_pairs_tile<HASK, NBUF, TRUST, SYM, PM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    k_pairs_tile<HASK, NBUF, TRUST, SYM, PM><<<grid, kTileThreads, smem, st>>>(A, B, P, k, dtype, out, q, status, 1u,
                                                                              polls, alpha);
    return cudaGetLastError();
}

// variant: 1 = one row per byte (alpha: the set's bytes), 0 = nibble rows,
// -1 = both launch and alpha, computed on the stream before, picks.
template <bool HASK, int NBUF, bool TRUST, int PM>
static cudaError_t launch_tile_v(int variant, const uint32_t *alpha, cudaStream_t st, int sms, const DevStrings &A,
                                 const DevStrings &B, int P, int k, int dtype, void *out, const LongQueue &q,
                                 uint32_t *status, uint32_t polls) {
    cudaError_t e = cudaSuccess;
    if (variant != 0)
        e = launch_tile<HASK, NBUF, TRUST, true, PM>(st, sms, A, B, P, k, dtype, out, q, status, polls, alpha);
    if (e == cudaSuccess && variant != 1)
        e = launch_tile<HASK, NBUF, TRUST, false, PM>(st, sms, A, B, P, k, dtype, out, q, status, polls,
                                                      variant < 0 ? alpha : nullptr);
    return e;
}

template <bool HASK, int NBUF, int PM>
static cudaError_t launch_tile_t(bool trusted, int variant, const uint32_t *alpha, cudaStream_t st, int sms,
                                 const DevStrings &A, const DevStrings &B, int P, int k, int dtype, void *out,
                                 const LongQueue &q, uint32_t *status, uint32_t polls) {
    return trusted
               ? launch_tile_v<HASK, NBUF, true, PM>(variant, alpha, st, sms, A, B, P, k, dtype, out, q, status, polls)
               : launch_tile_v<HASK, NBUF, false, PM>(variant, alpha, st, sms, A, B, P, k, dtype, out, q, status, polls);
}

template <bool HASK>
static cudaError_t launch_tile_shape(int shape, bool trusted, int variant, const uint32_t *alpha, cudaStream_t st,
                                     int sms, const DevStrings &A, const DevStrings &B, int P, int k, int dtype,
                                     void *out, const LongQueue &q, uint32_t *status, uint32_t polls) {
    if (shape == 1)
        return launch_tile_t<HASK, 1, 512>(trusted, variant, alpha, st, sms, A, B, P, k, dtype, out, q, status, polls);
    if (shape == 3)
        return launch_tile_t<HASK, 2, 256>(trusted, variant, alpha, st, sms, A, B, P, k, dtype, out, q, status, polls);
    return launch_tile_t<HASK, 2, 512>(trusted, variant, alpha, st, sms, A, B, P, k, dtype, out, q, status, polls);
}

// shape: 1 = one stage of up to 512 pairs, 2 = two stages of 512, 3 = two
// stages of 256 (the autotuner picks). trusted: the offsets were checked on
// the host (every pair in order). variant / alpha: the row layout, as for
// launch_tile_v.
cudaError_t launch_pairs_tile(cudaStream_t st, int sms, int shape, bool hask, const DevStrings &A,
                              const DevStrings &B, int tile_pairs, int k, int dtype, void *out, const LongQueue &q,
                              uint32_t *status, int32_t wait_polls, bool trusted, int variant, const uint32_t *alpha) {
    if (A.n <= 0) return cudaSuccess;
    const uint32_t polls = wait_polls < 0 ? kMbarPolls : (uint32_t)wait_polls;
    int P = tile_pairs;
    if (P > kTileMaxPairs) P = kTileMaxPairs;
    if (P < 32) P = 32;
    P &= ~3;                                                // 4-aligned tiles keep the vector stores aligned
    return hask ? launch_tile_shape<true>(shape, trusted, variant, alpha, st, sms, A, B, P, k, dtype, out, q, status,
                                          polls)
                : launch_tile_shape<false>(shape, trusted, variant, alpha, st, sms, A, B, P, k, dtype, out, q, status,
                                           polls);
}

}  // namespace blg
