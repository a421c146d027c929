// GB300 (sm_103a) kernels of the bit-parallel Levenshtein engine.
//
// The reference computes the same distances with two CUDA kernel families
// (csrc/gpu_kernels.cu:6-69): one thread per pair with the pattern packed in
// registers and Eq built by SWAR byte compares, and one block per query with
// a Peq table in shared memory.  The kernels here are designed for GB300:
//
//  * k_search_seq<NW>   cdist for queries of NW <= 8 words: a CTA owns a tile
//                       of 1024 candidates (4 consecutive per thread, so the
//                       narrow results leave as one vector store) and loops
//                       over a chunk of queries, staging each query's
//                       prebuilt Peq table (k_build_peq) into shared memory.
//  * k_search_lanes     cdist for queries longer than 512: a query's words
//                       are spread over L lanes, the add-carry travels lane to
//                       lane with __shfl_up_sync on an anti-diagonal wavefront.
//  * k_pairs_main       pairwise: one thread per pair, exact prefix/suffix
//                       trimming on 4-byte windows, single-word solve with
//                       per-lane nibble Peq tables in shared memory; pairs
//                       whose trimmed pattern exceeds 64 go to a device queue.
//  * k_pairs_long       persistent consumer of that queue, lane-spread.
//
// All arithmetic is integer bit logic on the ALU/FMA pipes; no tensor cores.
#include "blg_device.cuh"
#include "blg_internal.h"

namespace blg {

constexpr unsigned kFull = 0xffffffffu;

// ---------------------------------------------------------------- loads --
// Four bytes starting at an arbitrary address: two aligned 32-bit loads and
// a funnel shift. Callers keep 16 bytes of slack around every string buffer
// so the aligned words never leave the allocation.
__device__ __forceinline__ uint32_t load4(const uint8_t *p) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(p);
    const uint32_t *w = reinterpret_cast<const uint32_t *>(a & ~uintptr_t(3));
    return __funnelshift_r(__ldg(w), __ldg(w + 1), (uint32_t)(a & 3) * 8u);
}

// Sequential reader: 4 characters per call, one aligned load per call.
struct TextScan {
    const uint32_t *w;
    uint32_t lo, sh;
    __device__ __forceinline__ void init(const uint8_t *p) {
        const uintptr_t a = reinterpret_cast<uintptr_t>(p);
        w = reinterpret_cast<const uint32_t *>(a & ~uintptr_t(3));
        sh = (uint32_t)(a & 3) * 8u;
        lo = __ldg(w);
    }
    __device__ __forceinline__ uint32_t next4() {
        const uint32_t hi = __ldg(++w);
        const uint32_t r = __funnelshift_r(lo, hi, sh);
        lo = hi;
        return r;
    }
};

// Validated string view; a corrupt offset pair raises ST_BAD_OFFSETS and
// yields an empty string instead of an out-of-range read.
__device__ __forceinline__ const uint8_t *string_at(const DevStrings &S, int64_t i, int &len,
                                                    uint32_t *status) {
    const int64_t o0 = S.off[i], o1 = S.off[i + 1];
    if (o0 < S.base || o1 < o0 || o1 - S.base > S.bytes || o1 - o0 > 0x7fffffff) {
        atomicOr(status, ST_BAD_OFFSETS);
        len = 0;
        return S.buf;
    }
    len = (int)(o1 - o0);
    return S.buf + (o0 - S.base);
}

// --------------------------------------------------------------- stores --
__device__ __forceinline__ void store1(void *out, int dtype, int64_t i, int d) {
    if (dtype == DT_UINT8) reinterpret_cast<uint8_t *>(out)[i] = (uint8_t)saturate_u8(d);
    else if (dtype == DT_UINT16) reinterpret_cast<uint16_t *>(out)[i] = (uint16_t)saturate_u16(d);
    else reinterpret_cast<int32_t *>(out)[i] = d;
}

// cnt (1..4) consecutive results from element i; one vector store when the
// four land on an aligned group (uint8: 4 B, uint16: 8 B, int32: 16 B).
__device__ __forceinline__ void store4(void *out, int dtype, int64_t i, int cnt, int d0, int d1,
                                       int d2, int d3) {
    if (cnt == 4 && (i & 3) == 0 && (reinterpret_cast<uintptr_t>(out) & 15) == 0) {
        if (dtype == DT_UINT8) {
            const uint32_t v = saturate_u8(d0) | (saturate_u8(d1) << 8) | (saturate_u8(d2) << 16) |
                               (saturate_u8(d3) << 24);
            reinterpret_cast<uint32_t *>(out)[i >> 2] = v;
        } else if (dtype == DT_UINT16) {
            uint2 v;
            v.x = saturate_u16(d0) | (saturate_u16(d1) << 16);
            v.y = saturate_u16(d2) | (saturate_u16(d3) << 16);
            reinterpret_cast<uint2 *>(out)[i >> 2] = v;
        } else {
            reinterpret_cast<int4 *>(out)[i >> 2] = make_int4(d0, d1, d2, d3);
        }
        return;
    }
    store1(out, dtype, i, d0);
    if (cnt > 1) store1(out, dtype, i + 1, d1);
    if (cnt > 2) store1(out, dtype, i + 2, d2);
    if (cnt > 3) store1(out, dtype, i + 3, d3);
}

// ------------------------------------------------------------- Peq build --
// One CTA per query: zero a 256 x nwc table in shared memory, set one bit
// per query position (shared-memory atomics), copy it out coalesced.
__global__ void __launch_bounds__(256) k_build_peq(DevStrings Q, const int32_t *qidx, int nwc,
                                                   uint64_t *peq_out, uint32_t *status) {
    extern __shared__ uint64_t tab[];
    const int qi = blockIdx.x;
    int m;
    const uint8_t *p = string_at(Q, qidx[qi], m, status);
    const int words = 256 * nwc;
    for (int x = threadIdx.x; x < words; x += blockDim.x) tab[x] = 0;
    __syncthreads();
    if (m > 64 * nwc) m = 64 * nwc;   // class construction guarantees this; keep the write in range
    for (int i = threadIdx.x; i < m; i += blockDim.x)
        atomicOr(reinterpret_cast<unsigned long long *>(&tab[(int)p[i] * nwc + (i >> 6)]),
                 1ull << (i & 63));
    __syncthreads();
    uint64_t *dst = peq_out + (size_t)qi * words;
    for (int x = threadIdx.x; x < words; x += blockDim.x) dst[x] = tab[x];
}

// --------------------------------------------------- search, NW <= 8 words --
// One text column through NW pattern words (word 0 takes the +1 top-row carry).
template <int NW, bool TOP63>
__device__ __forceinline__ void column_seq(uint64_t (&pv)[NW], uint64_t (&mv)[NW],
                                           const uint64_t *row, int lastbit, int &score) {
    uint64_t ph, mh;
    step_top<uint64_t>(pv[0], mv[0], row[0], ph, mh);
    if (NW == 1) {
        score += TOP63 ? hdelta<uint64_t>(ph, mh, 63) : hdelta<uint64_t>(ph, mh, lastbit);
        return;
    }
    int h = hdelta<uint64_t>(ph, mh, 63);
#pragma unroll
    for (int w = 1; w < NW - 1; w++) {
        step_mid<uint64_t>(pv[w], mv[w], row[w], h, ph, mh);
        h = hdelta<uint64_t>(ph, mh, 63);
    }
    step_mid<uint64_t>(pv[NW - 1], mv[NW - 1], row[NW - 1], h, ph, mh);
    score += TOP63 ? hdelta<uint64_t>(ph, mh, 63) : hdelta<uint64_t>(ph, mh, lastbit);
}

// d(query, t) with the query's Peq table in shared memory (NW = ceil(m/64)).
template <int NW, bool HASK, bool TOP63>
__device__ __forceinline__ int dist_seq(const uint64_t *peq, int m, const uint8_t *t, int n, int k) {
    if (m == 0) return cap_k(n, k);                    // csrc/gpu_kernels.cu:53
    if (HASK && (n > m ? n - m : m - n) > k) return k + 1;
    uint64_t pv[NW], mv[NW];
#pragma unroll
    for (int w = 0; w < NW; w++) { pv[w] = ~0ull; mv[w] = 0; }
    const int lastbit = (m - 1) & 63;
    int score = m;
    TextScan ts;
    ts.init(t);
    int j = 0;
    for (; j + 4 <= n; j += 4) {
        const uint32_t w4 = ts.next4();
#pragma unroll
        for (int b = 0; b < 4; b++)
            column_seq<NW, TOP63>(pv, mv, peq + ((w4 >> (8 * b)) & 0xffu) * NW, lastbit, score);
        // the exit test is monotone in j, so testing every 4th column is exact
        if (HASK && hopeless(score, j + 3, n, k)) return k + 1;
    }
    if (j < n) {
        uint32_t w4 = ts.next4();
        for (; j < n; j++, w4 >>= 8) column_seq<NW, TOP63>(pv, mv, peq + (w4 & 0xffu) * NW, lastbit, score);
    }
    return HASK ? cap_k(score, k) : score;
}

template <int NW, bool HASK>
__device__ __forceinline__ int dist_seq_any(const uint64_t *peq, int m, const uint8_t *t, int n, int k) {
    // the last pattern bit is bit 63 for full words: cheaper score extraction
    if (((m - 1) & 63) == 63) return dist_seq<NW, HASK, true>(peq, m, t, n, k);
    return dist_seq<NW, HASK, false>(peq, m, t, n, k);
}

// grid: x = candidate tiles of 4*blockDim.x, y = query chunks of `qpb`.
template <int NW, bool HASK>
__global__ void __launch_bounds__(256) k_search_seq(DevStrings C, SearchClass cls, int qpb, int k,
                                                    int dtype, void *out, uint32_t *status) {
    extern __shared__ uint64_t s_peq[];
    const int64_t nc = C.n;
    const int64_t c0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * 4;
    const uint8_t *tp0 = C.buf, *tp1 = C.buf, *tp2 = C.buf, *tp3 = C.buf;
    int tn0 = 0, tn1 = 0, tn2 = 0, tn3 = 0;
    const int cnt = (int)(c0 >= nc ? 0 : (nc - c0 < 4 ? nc - c0 : 4));
    if (cnt > 0) tp0 = string_at(C, c0, tn0, status);
    if (cnt > 1) tp1 = string_at(C, c0 + 1, tn1, status);
    if (cnt > 2) tp2 = string_at(C, c0 + 2, tn2, status);
    if (cnt > 3) tp3 = string_at(C, c0 + 3, tn3, status);
    const int q_begin = blockIdx.y * qpb;
    const int q_end = min(q_begin + qpb, cls.nq);
    constexpr int kWords = 256 * NW;
    for (int qi = q_begin; qi < q_end; qi++) {
        __syncthreads();
        const uint64_t *src = cls.peq + (size_t)qi * kWords;
        for (int x = threadIdx.x; x < kWords; x += blockDim.x) s_peq[x] = __ldg(src + x);
        __syncthreads();
        if (cnt == 0) continue;
        const int m = cls.qlen[qi];
        const int64_t row = cls.qidx[qi];
        const int d0 = dist_seq_any<NW, HASK>(s_peq, m, tp0, tn0, k);
        const int d1 = cnt > 1 ? dist_seq_any<NW, HASK>(s_peq, m, tp1, tn1, k) : 0;
        const int d2 = cnt > 2 ? dist_seq_any<NW, HASK>(s_peq, m, tp2, tn2, k) : 0;
        const int d3 = cnt > 3 ? dist_seq_any<NW, HASK>(s_peq, m, tp3, tn3, k) : 0;
        store4(out, dtype, row * nc + c0, cnt, d0, d1, d2, d3);
    }
}

// ------------------------------------------------ lane-spread core (L lanes) --
// One pair per group of L lanes; lane w owns pattern word w and processes
// text column j = s - w at wavefront step s. The horizontal delta leaving a
// word's bottom row is the only coupling between words (csrc/myers.c:24-27):
// it reaches lane w+1 one step later through __shfl_up_sync. The lane of
// the last word keeps the score and decides the max_dist exit, which the
// group learns through __ballot_sync.
template <bool HASK, typename EqFn>
__device__ __forceinline__ int lane_wavefront(bool valid, int m, const uint8_t *txt, int n, int L,
                                              int w, int g, int k, EqFn eqfn, bool &is_last) {
    const int W = valid ? (m + 63) >> 6 : 0;
    const bool own = valid && w < W;
    const int lastw = W - 1;
    is_last = valid && w == lastw;
    const int ob = is_last ? ((m - 1) & 63) : 63;
    uint64_t pv = ~0ull, mv = 0;
    int score = m;
    const int steps = valid ? n + W - 1 : 0;
    const int maxsteps = __reduce_max_sync(kFull, steps);
    int hrecv = 0;
    bool done = false;
    TextScan ts;
    uint32_t win = 0;
    if (own) ts.init(txt);
    for (int s = 0; s < maxsteps; s++) {
        const int j = s - w;
        const bool act = own && !done && j >= 0 && j < n;
        int hout = 0;
        if (act) {
            if ((j & 3) == 0) win = ts.next4();
            const uint32_t c = (win >> (8 * (j & 3))) & 0xffu;
            uint64_t ph, mh;
            step_mid<uint64_t>(pv, mv, eqfn(c), w == 0 ? 1 : hrecv, ph, mh);
            hout = hdelta<uint64_t>(ph, mh, ob);
            if (is_last) score += hout;
        }
        hrecv = __shfl_up_sync(kFull, hout, 1, L);
        if (HASK) {
            const bool ex = act && is_last && hopeless(score, j, n, k);
            const unsigned bal = __ballot_sync(kFull, ex);
            if (valid && ((bal >> (g * L + lastw)) & 1u)) done = true;
        }
    }
    if (done) return k + 1;
    return HASK ? cap_k(score, k) : score;
}

// ----------------------------------------------- search, long queries (lanes) --
// grid: x = candidate tiles of (warps * 32/L), y = queries of the class.
template <bool HASK>
__global__ void __launch_bounds__(256) k_search_lanes(DevStrings C, SearchClass cls, int nwc, int L,
                                                      int k, int dtype, void *out, uint32_t *status) {
    extern __shared__ uint64_t s_peq[];
    const int words = 256 * nwc;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int G = 32 / L, g = lane / L, w = lane & (L - 1);
    const int64_t c = ((int64_t)blockIdx.x * (blockDim.x >> 5) + warp) * G + g;
    const bool valid = c < C.n;
    int n = 0;
    const uint8_t *t = valid ? string_at(C, c, n, status) : C.buf;
    for (int qi = blockIdx.y; qi < cls.nq; qi += gridDim.y) {
        __syncthreads();
        const uint64_t *src = cls.peq + (size_t)qi * words;
        for (int x = threadIdx.x; x < words; x += blockDim.x) s_peq[x] = __ldg(src + x);
        __syncthreads();
        const int m = cls.qlen[qi];
        const int64_t row = cls.qidx[qi];
        // a length gap beyond k needs no wavefront
        const bool quick = valid && HASK && (n > m ? n - m : m - n) > k;
        bool is_last = false;
        const int d = lane_wavefront<HASK>(valid && !quick, m, t, n, L, w, g, k,
                                           [&](uint32_t ch) { return s_peq[ch * nwc + w]; }, is_last);
        if (quick && w == 0) store1(out, dtype, row * C.n + c, k + 1);
        else if (is_last) store1(out, dtype, row * C.n + c, d);
    }
}

// ------------------------------------------------------------ pairs: main --
// Trim the common prefix and suffix with 4-byte window compares (exact:
// d(xPy, xQy) = d(P, Q), csrc/myers.c:80-87).
__device__ __forceinline__ void trim_windows(const uint8_t *&a, int &la, const uint8_t *&b, int &lb) {
    const int lim = la < lb ? la : lb;
    int p = 0;
    while (p < lim) {
        const uint32_t x = load4(a + p) ^ load4(b + p);
        int q = x ? (__ffs(x) - 1) >> 3 : 4;               // equal leading bytes
        if (q > lim - p) q = lim - p;
        p += q;
        if (q < 4) break;
    }
    const int lim2 = lim - p;
    int s = 0;
    while (s < lim2) {
        const uint32_t x = load4(a + la - s - 4) ^ load4(b + lb - s - 4);
        int q = x ? __clz(x) >> 3 : 4;                     // equal trailing bytes
        if (q > lim2 - s) q = lim2 - s;
        s += q;
        if (q < 4) break;
    }
    a += p; b += p;
    la -= p + s; lb -= p + s;
}

// Per-lane nibble Peq tables: rows 0..15 hold the positions whose high
// nibble is r, rows 16..31 those whose low nibble is r; Eq(c) is the AND of
// the two rows. Layout [row][lane] (stride 32 words) keeps every access
// bank-conflict free. `tc` points at this lane's column.
__device__ __forceinline__ uint64_t nib_eq(const uint64_t *tc, uint32_t c) {
    return tc[(c >> 4) * 32] & tc[(16 + (c & 15)) * 32];
}

__device__ __forceinline__ void nib_build(uint64_t *tc, const uint8_t *p, int m) {
    TextScan ps;
    ps.init(p);
    for (int i = 0; i < m; i += 4) {
        const uint32_t w4 = ps.next4();
#pragma unroll
        for (int b = 0; b < 4; b++) {
            if (i + b < m) {
                const uint32_t c = (w4 >> (8 * b)) & 0xffu;
                const uint64_t bit = 1ull << (i + b);
                tc[(c >> 4) * 32] |= bit;
                tc[(16 + (c & 15)) * 32] |= bit;
            }
        }
    }
}

__device__ __forceinline__ void nib_clear(uint64_t *tc, const uint8_t *p, int m) {
    TextScan ps;
    ps.init(p);
    for (int i = 0; i < m; i += 4) {
        const uint32_t w4 = ps.next4();
#pragma unroll
        for (int b = 0; b < 4; b++) {
            if (i + b < m) {
                const uint32_t c = (w4 >> (8 * b)) & 0xffu;
                tc[(c >> 4) * 32] = 0;
                tc[(16 + (c & 15)) * 32] = 0;
            }
        }
    }
}

// Single-word pair (1 <= m <= 64, m <= n): pattern p, text t.
template <bool HASK>
__device__ __forceinline__ int solve_word(uint64_t *tc, const uint8_t *p, int m, const uint8_t *t,
                                          int n, int k) {
    nib_build(tc, p, m);
    uint64_t pv = ~0ull, mv = 0;
    const int lastbit = m - 1;
    int score = m;
    bool dead = false;
    TextScan ts;
    ts.init(t);
    int j = 0;
    for (; j + 4 <= n; j += 4) {
        const uint32_t w4 = ts.next4();
#pragma unroll
        for (int b = 0; b < 4; b++) {
            uint64_t ph, mh;
            step_top<uint64_t>(pv, mv, nib_eq(tc, (w4 >> (8 * b)) & 0xffu), ph, mh);
            score += hdelta<uint64_t>(ph, mh, lastbit);
        }
        if (HASK && hopeless(score, j + 3, n, k)) { dead = true; break; }
    }
    if (!dead && j < n) {
        uint32_t w4 = ts.next4();
        for (; j < n; j++, w4 >>= 8) {
            uint64_t ph, mh;
            step_top<uint64_t>(pv, mv, nib_eq(tc, w4 & 0xffu), ph, mh);
            score += hdelta<uint64_t>(ph, mh, lastbit);
        }
    }
    nib_clear(tc, p, m);
    if (dead) return k + 1;
    return HASK ? cap_k(score, k) : score;
}

__device__ __forceinline__ int long_class(int m) {
    const int W = (m + 63) >> 6;
    return W <= 2 ? 0 : W <= 4 ? 1 : W <= 8 ? 2 : W <= 16 ? 3 : W <= 32 ? 4 : -1;
}

// One thread per pair (grid-stride). Dynamic shared memory: 8 KB per warp.
template <bool HASK>
__global__ void __launch_bounds__(256) k_pairs_main(DevStrings A, DevStrings B, int k, int dtype,
                                                    void *out, LongQueue q, uint32_t *status) {
    extern __shared__ uint64_t s_tab[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t *tc = s_tab + warp * 1024 + lane;
#pragma unroll
    for (int r = 0; r < 32; r++) tc[r * 32] = 0;
    const int64_t n = A.n;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        int la, lb;
        const uint8_t *a = string_at(A, i, la, status);
        const uint8_t *b = string_at(B, i, lb, status);
        trim_windows(a, la, b, lb);
        if (la > lb) {                                  // the shorter string is the pattern
            const uint8_t *t = a; a = b; b = t;
            const int x = la; la = lb; lb = x;
        }
        int d;
        if (HASK && lb - la > k) d = k + 1;             // length gap alone exceeds k
        else if (la == 0) d = lb;
        else if (la <= 64) d = solve_word<HASK>(tc, a, la, b, lb, k);
        else {
            const int cls = long_class(la);
            if (cls < 0) { atomicOr(status, ST_TOO_LONG); d = -1; }
            else {
                const int pos = atomicAdd(&q.counts[cls], 1);
                if (pos < q.cap[cls]) {
                    LongItem it;
                    it.pat = a; it.txt = b; it.m = la; it.n = lb; it.idx = i;
                    q.items[cls][pos] = it;
                    continue;
                }
                atomicOr(status, ST_QUEUE_OVERFLOW);
                d = -1;
            }
        }
        store1(out, dtype, i, d);
    }
}

// Persistent consumer of the long-pair queues: each warp takes 32/L pairs
// of one class at a time until every class queue is drained.
template <bool HASK>
__global__ void __launch_bounds__(256) k_pairs_long(LongQueue q, int k, int dtype, void *out) {
    extern __shared__ uint64_t s_tab[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t *tc = s_tab + warp * 1024 + lane;
#pragma unroll
    for (int r = 0; r < 32; r++) tc[r * 32] = 0;
    for (int cls = 0; cls < kLongClasses; cls++) {
        const int L = 2 << cls, G = 32 / L, g = lane / L, w = lane & (L - 1);
        const int count = (int)min((int64_t)q.counts[cls], q.cap[cls]);
        if (count == 0) continue;
        while (true) {
            int base = 0;
            if (lane == 0) base = atomicAdd(&q.heads[cls], G);
            base = __shfl_sync(kFull, base, 0);
            if (base >= count) break;
            const int it_i = base + g;
            const bool valid = it_i < count;
            LongItem it;
            if (valid) it = q.items[cls][it_i];
            else { it.pat = nullptr; it.txt = nullptr; it.m = 0; it.n = 0; it.idx = 0; }
            const bool own = valid && w < ((it.m + 63) >> 6);
            const uint8_t *pw = own ? it.pat + 64 * w : nullptr;
            const int plen = own ? min(64, it.m - 64 * w) : 0;
            if (own) nib_build(tc, pw, plen);
            bool is_last = false;
            const int d = lane_wavefront<HASK>(valid, it.m, it.txt, it.n, L, w, g, k,
                                               [&](uint32_t ch) { return nib_eq(tc, ch); }, is_last);
            if (own) nib_clear(tc, pw, plen);
            if (is_last) store1(out, dtype, it.idx, d);
        }
    }
}

// ------------------------------------------------------------- launchers --
template <int NW>
static cudaError_t launch_seq(bool hask, dim3 grid, size_t smem, cudaStream_t st, const DevStrings &C,
                              const SearchClass &cls, int qpb, int k, int dtype, void *out,
                              uint32_t *status) {
    if (hask) {
        cudaFuncSetAttribute(k_search_seq<NW, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_search_seq<NW, true><<<grid, 256, smem, st>>>(C, cls, qpb, k, dtype, out, status);
    } else {
        cudaFuncSetAttribute(k_search_seq<NW, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_search_seq<NW, false><<<grid, 256, smem, st>>>(C, cls, qpb, k, dtype, out, status);
    }
    return cudaGetLastError();
}

cudaError_t launch_build_peq(cudaStream_t st, const DevStrings &Q, const int32_t *qidx, int nq, int nwc,
                             uint64_t *peq, uint32_t *status) {
    if (nq <= 0) return cudaSuccess;
    const size_t smem = (size_t)256 * nwc * sizeof(uint64_t);
    cudaFuncSetAttribute(k_build_peq, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_build_peq<<<nq, 256, smem, st>>>(Q, qidx, nwc, peq, status);
    return cudaGetLastError();
}

cudaError_t launch_search_seq(cudaStream_t st, int nw, bool hask, const DevStrings &C,
                              const SearchClass &cls, int qpb, int k, int dtype, void *out,
                              uint32_t *status) {
    if (cls.nq <= 0 || C.n <= 0) return cudaSuccess;
    const int64_t tiles = (C.n + 1023) / 1024;
    dim3 grid((unsigned)tiles, (unsigned)((cls.nq + qpb - 1) / qpb));
    const size_t smem = (size_t)256 * nw * sizeof(uint64_t);
    switch (nw) {
    case 1: return launch_seq<1>(hask, grid, smem, st, C, cls, qpb, k, dtype, out, status);
    case 2: return launch_seq<2>(hask, grid, smem, st, C, cls, qpb, k, dtype, out, status);
    case 3: return launch_seq<3>(hask, grid, smem, st, C, cls, qpb, k, dtype, out, status);
    case 4: return launch_seq<4>(hask, grid, smem, st, C, cls, qpb, k, dtype, out, status);
    case 5: return launch_seq<5>(hask, grid, smem, st, C, cls, qpb, k, dtype, out, status);
    case 6: return launch_seq<6>(hask, grid, smem, st, C, cls, qpb, k, dtype, out, status);
    case 7: return launch_seq<7>(hask, grid, smem, st, C, cls, qpb, k, dtype, out, status);
    case 8: return launch_seq<8>(hask, grid, smem, st, C, cls, qpb, k, dtype, out, status);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_search_lanes(cudaStream_t st, bool hask, const DevStrings &C, const SearchClass &cls,
                                int nwc, int k, int dtype, void *out, uint32_t *status) {
    if (cls.nq <= 0 || C.n <= 0) return cudaSuccess;
    int L = 1;
    while (L < nwc) L <<= 1;
    if (L > 32) return cudaErrorInvalidValue;
    const int per_cta = 8 * (32 / L);
    dim3 grid((unsigned)((C.n + per_cta - 1) / per_cta), (unsigned)min(cls.nq, 65535));
    const size_t smem = (size_t)256 * nwc * sizeof(uint64_t);
    if (hask) {
        cudaFuncSetAttribute(k_search_lanes<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_search_lanes<true><<<grid, 256, smem, st>>>(C, cls, nwc, L, k, dtype, out, status);
    } else {
        cudaFuncSetAttribute(k_search_lanes<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_search_lanes<false><<<grid, 256, smem, st>>>(C, cls, nwc, L, k, dtype, out, status);
    }
    return cudaGetLastError();
}

cudaError_t launch_pairs_main(cudaStream_t st, int grid, bool hask, const DevStrings &A,
                              const DevStrings &B, int k, int dtype, void *out, const LongQueue &q,
                              uint32_t *status) {
    const size_t smem = 8 * 1024 * sizeof(uint64_t);
    if (hask) {
        cudaFuncSetAttribute(k_pairs_main<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_pairs_main<true><<<grid, 256, smem, st>>>(A, B, k, dtype, out, q, status);
    } else {
        cudaFuncSetAttribute(k_pairs_main<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_pairs_main<false><<<grid, 256, smem, st>>>(A, B, k, dtype, out, q, status);
    }
    return cudaGetLastError();
}

cudaError_t launch_pairs_long(cudaStream_t st, int grid, bool hask, const LongQueue &q, int k,
                              int dtype, void *out) {
    const size_t smem = 8 * 1024 * sizeof(uint64_t);
    if (hask) {
        cudaFuncSetAttribute(k_pairs_long<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_pairs_long<true><<<grid, 256, smem, st>>>(q, k, dtype, out);
    } else {
        cudaFuncSetAttribute(k_pairs_long<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_pairs_long<false><<<grid, 256, smem, st>>>(q, k, dtype, out);
    }
    return cudaGetLastError();
}

}  // namespace blg
