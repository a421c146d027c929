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
//  * k_pairs_staged     pairwise in natural order: one thread per pair, warp
//                       spans staged in shared memory, exact prefix/suffix
//                       trimming on 4-byte windows, single-word solve with
//                       per-lane nibble Peq tables; pairs whose trimmed
//                       pattern exceeds 64 go to a device queue.
//  * k_pairs_long       persistent consumer of that queue, lane-spread.
//  * k_search_surv      thresholded cdist with max_dist > 31 (full-word loop);
//                       max_dist <= 31 runs in blg_search_lpt.cu.
//
// All arithmetic is integer bit logic on the ALU/FMA pipes; no tensor cores.
#include <algorithm>

#include "blg_kernels.cuh"

namespace blg {

// ------------------------------------------------------------- Peq build --
// One CTA per query: zero a 256 x nwc table in shared memory, set one bit
// per query position (shared-memory atomics), copy it out coalesced.
__global__ void __launch_bounds__(256) k_build_peq(DevStrings Q, const int32_t *qidx, int nwc,
                                                   uint64_t *peq_out, uint32_t *status) {
    extern __shared__ uint64_t tab[];
    const int qi = blockIdx.x;
    int m;
    const uint8_t *p = string_at(Q, qidx[qi], m, status);
    build_peq_block(p, m, nwc, tab, peq_out + (size_t)qi * 256 * nwc);
}

// grid: x = candidate tiles of 4*blockDim.x, y = query chunks of `qpb`.
template <int NW, bool HASK>
__global__ void __launch_bounds__(256) k_search_seq(DevStrings C, SearchClass cls, int qpb, int k,
                                                    int dtype, void *out, uint32_t *status, uint32_t unit) {
    extern __shared__ uint64_t s_peq[];
    const Units u{unit, unit + unit};
    RowAddr<NW> ra;
    ra.init(u);
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
        const int d0 = dist_seq_any<NW, HASK>(s_peq, m, tp0, tn0, k, u, ra);
        const int d1 = cnt > 1 ? dist_seq_any<NW, HASK>(s_peq, m, tp1, tn1, k, u, ra) : 0;
        const int d2 = cnt > 2 ? dist_seq_any<NW, HASK>(s_peq, m, tp2, tn2, k, u, ra) : 0;
        const int d3 = cnt > 3 ? dist_seq_any<NW, HASK>(s_peq, m, tp3, tn3, k, u, ra) : 0;
        store4(out, dtype, row * nc + c0, cnt, d0, d1, d2, d3);
    }
}

// Exact-capable search over tile-transposed choices: grid x = choice tiles
// of kTileCands, y = query chunks of `qpb`. Thread t owns choices t, t+256,
// t+512, t+768 of the tile, so a warp's text loads and its result stores are
// each one contiguous line.
template <int NW, bool HASK>
__global__ void __launch_bounds__(256) k_search_tt(TransposedChoices T, SearchClass cls, int qpb, int k,
                                                   int dtype, void *out, uint32_t unit) {
    extern __shared__ uint64_t s_peq[];
    const Units u{unit, unit + unit};
    RowAddr<NW> ra;
    ra.init(u);
    const int64_t nc = T.n;
    const int64_t tile = blockIdx.x;
    const int64_t c0 = tile * kTileCands + threadIdx.x;
    const uint32_t *tw = T.words + T.base[tile] + threadIdx.x;
    const int q_begin = blockIdx.y * qpb;
    const int q_end = min(q_begin + qpb, cls.nq);
    constexpr int kWords = 256 * NW;
    for (int qi = q_begin; qi < q_end; qi++) {
        __syncthreads();
        const uint64_t *src = cls.peq + (size_t)qi * kWords;
        for (int x = threadIdx.x; x < kWords; x += blockDim.x) s_peq[x] = __ldg(src + x);
        __syncthreads();
        const int m = cls.qlen[qi];
        const int64_t row = cls.qidx[qi] * nc;
#pragma unroll 1
        for (int t = 0; t < 4; t++) {
            const int64_t c = c0 + 256 * t;
            if (c >= nc) break;
            const int d = dist_tt<NW, HASK>(s_peq, m, tw + 256 * t, __ldg(T.len + c), k, u, ra);
            store1(out, dtype, row + c, d);
        }
    }
}

// Exact search of short queries, QI queries per thread: the CTA stages the
// Peq tables of QI consecutive queries of its chunk and every thread runs its
// 4 choices against all QI at once (dist_tt_q). Partial groups at the end of
// a chunk run with zero tables and store nothing for the missing queries.
template <int NW, int QI>
__global__ void __launch_bounds__(256) k_search_ttq(TransposedChoices T, SearchClass cls, int qpb, int dtype,
                                                    void *out, uint32_t unit) {
    extern __shared__ uint64_t s_peq[];
    const Units u{unit, unit + unit};
    RowAddr<NW> ra;
    ra.init(u);
    const int64_t nc = T.n;
    const int64_t tile = blockIdx.x;
    const int64_t c0 = tile * kTileCands + threadIdx.x;
    const uint32_t *tw = T.words + T.base[tile] + threadIdx.x;
    const int q_begin = blockIdx.y * qpb;
    const int q_end = min(q_begin + qpb, cls.nq);
    constexpr int kWords = 256 * NW;
    for (int qg = q_begin; qg < q_end; qg += QI) {
        const int nqg = min(QI, q_end - qg);
        __syncthreads();
        const uint64_t *src = cls.peq + (size_t)qg * kWords;
        for (int x = threadIdx.x; x < QI * kWords; x += blockDim.x) s_peq[x] = x < nqg * kWords ? __ldg(src + x) : 0;
        __syncthreads();
#pragma unroll 1
        for (int t = 0; t < 4; t++) {
            const int64_t c = c0 + 256 * t;
            if (c >= nc) break;
            int d[QI];
            dist_tt_q<NW, QI>(s_peq, cls.qlen + qg, nqg, tw + 256 * t, __ldg(T.len + c), u, ra, d);
#pragma unroll
            for (int i = 0; i < QI; i++)
                if (i < nqg) store1(out, dtype, cls.qidx[qg + i] * nc + c, d[i]);
        }
    }
}

// ------------------------------------------- exact search with prefix reuse --
// Choices sorted lexicographically share prefixes with their neighbours: the
// column state of a query after the first c text columns depends on those c
// characters only, so a choice that shares c characters with the previous
// one can start at column c from the state the previous run passed there.
// Here a warp's 32 lanes hold QI queries each (QI*32 per warp, the same block
// of queries for the whole CTA) and share one choice at a time: the text, the
// choice length and the restart column are warp-uniform, so a skipped column
// is skipped by the whole warp. Each warp walks a chain of `chain`
// consecutive sorted choices (a divisor of kPfxChain), saving its lanes'
// column states at the launch's checkpoint columns in shared memory; the
// chain's first choice starts from column 0 and every other one restarts
// from the checkpoint P.restart names (computed on the host for chains of
// kPfxChain, whose starts are chain starts here too). Shorter chains give a
// launch over few queries enough work items to fill the GPU. The block's Peq rows
// are staged per alphabet symbol as [symbol][query][lane] (conflict-free
// 64-bit loads) and the text carries each character's row offset, so a
// column's row address is one half-word extract for QI queries. A persistent
// grid pulls (query block, chain group) items from a device counter, query
// block outermost, so a CTA restages its Peq rows only when the block changes.
// Results leave through the sort's permutation (P.orig).
template <int NW, int QI>
__global__ void __launch_bounds__(256) k_search_pfx(PrefixChoices P, SearchClass cls, unsigned long long *work,
                                                    int64_t items, int chain, int dtype, void *out, uint32_t unit) {
    static_assert(QI * NW * 32 * 8 == kPfxRowBytes, "one symbol's entries fill a row");
    static_assert(kPfxCheckpoints == 2, "two checkpoint columns");
    static_assert(kPfxWarps * 32 == 256, "256 threads");
    extern __shared__ uint64_t s_peq[];                        // [nsym][QI][32][NW], then the checkpoints
    constexpr int kState = QI * NW * 4;                        // u32 of one lane's column states
    uint32_t *s_ck = reinterpret_cast<uint32_t *>(s_peq + (size_t)P.nsym * (kPfxRowBytes / 8));
    __shared__ int64_t s_item;
    const Units u{unit, unit + unit};
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t nc = P.n;
    const int64_t seg_len = (int64_t)kPfxWarps * chain, segs = (nc + seg_len - 1) / seg_len;
    const int ck0 = P.ck[0], ck1 = P.ck[1];                    // (no dynamic index into the parameter block)
    const uint32_t hi16 = u.one << 16;
    const char *pl = reinterpret_cast<const char *>(s_peq) + lane * NW * 8;
    Word2 st[QI][NW];
    auto col = [&](uint32_t off) {
#pragma unroll
        for (int i = 0; i < QI; i++)
            column_v<NW>(st[i], reinterpret_cast<const uint64_t *>(pl + off + i * (32 * NW * 8)), u);
    };
    auto col2 = [&](uint32_t w) {                              // the two characters of a text word
        col(w & 0xffffu);
        col(imad_hi(w, hi16, 0));
    };
    int cur = -1;
    while (true) {
        __syncthreads();                                       // the previous item is done with s_item
        if (tid == 0) s_item = (int64_t)atomicAdd(work, 1ull);
        __syncthreads();
        const int64_t item = s_item;
        if (item >= items) break;
        const int qb = (int)(item / segs);
        const int64_t seg = item - (int64_t)qb * segs;
        const int q0 = qb * (QI * 32);
        if (qb != cur) {                                       // uniform: every thread read the same item
            const int entries = P.nsym * (QI * 32 * NW);
            for (int x = tid; x < entries; x += 256) {
                const int w = x % NW, ql = (x / NW) % (QI * 32), a = x / (NW * QI * 32);
                const int q = q0 + ql;                         // ql = i * 32 + lane
                s_peq[x] = q < cls.nq ? __ldg(cls.peq + ((size_t)q * 256 + P.sym[a]) * NW + w) : 0;
            }
            __syncthreads();
            cur = qb;
        }
        const int64_t p0 = seg * seg_len + (int64_t)warp * chain;
#pragma unroll 1
        for (int r = 0; r < chain; r++) {
            const int64_t p = p0 + r;
            if (p >= nc) break;                                // warp-uniform
            const int n = __ldg(P.len + p);
            const int b = r == 0 ? 0 : __ldg(P.restart + p);
            const uint32_t *tx = P.text + __ldg(P.woff + p);
            if (b == 0) {
#pragma unroll
                for (int i = 0; i < QI; i++)
#pragma unroll
                    for (int w = 0; w < NW; w++) { st[i][w].pl = st[i][w].ph = ~0u; st[i][w].ml = st[i][w].mh = 0; }
            } else {
                const uint32_t *ck = s_ck + (b == ck1 ? kState * 256 : 0) + tid;
#pragma unroll
                for (int i = 0; i < QI; i++)
#pragma unroll
                    for (int w = 0; w < NW; w++) {
                        const int x = (i * NW + w) * 4;
                        st[i][w].pl = ck[(x + 0) * 256];
                        st[i][w].ph = ck[(x + 1) * 256];
                        st[i][w].ml = ck[(x + 2) * 256];
                        st[i][w].mh = ck[(x + 3) * 256];
                    }
            }
            // columns [b, n): up to the checkpoints it passes (saving there), then to the end
            int j = b;
#pragma unroll 1
            for (int sg = 0; sg <= kPfxCheckpoints; sg++) {
                int end = n;
                if (sg < kPfxCheckpoints) {
                    end = sg == 0 ? ck0 : ck1;
                    if (!(j < end && end <= n)) continue;
                }
                if ((j & 1) && j < end) {                      // the second character of a started word
                    col(imad_hi(__ldg(tx + (j >> 1)), hi16, 0));
                    j++;
                }
                if (j + 8 <= end) {                            // 8 columns per step, the next 4 words in flight
                    const uint32_t *q = tx + (j >> 1);
                    uint32_t a0 = __ldg(q), a1 = __ldg(q + 1), a2 = __ldg(q + 2), a3 = __ldg(q + 3);
                    for (; j + 8 <= end; j += 8) {
                        const uint32_t c0 = a0, c1 = a1, c2 = a2, c3 = a3;
                        q += 4;
                        a0 = __ldg(q);                         // may read up to 4 words past the choice
                        a1 = __ldg(q + 1);
                        a2 = __ldg(q + 2);
                        a3 = __ldg(q + 3);
                        col2(c0);
                        col2(c1);
                        col2(c2);
                        col2(c3);
                    }
                }
                for (; j + 2 <= end; j += 2) col2(__ldg(tx + (j >> 1)));
                if (j < end) {
                    col(__ldg(tx + (j >> 1)) & 0xffffu);
                    j++;
                }
                if (sg < kPfxCheckpoints) {                    // the state after `end` columns
                    uint32_t *ck = s_ck + sg * kState * 256 + tid;
#pragma unroll
                    for (int i = 0; i < QI; i++)
#pragma unroll
                        for (int w = 0; w < NW; w++) {
                            const int x = (i * NW + w) * 4;
                            ck[(x + 0) * 256] = st[i][w].pl;
                            ck[(x + 1) * 256] = st[i][w].ph;
                            ck[(x + 2) * 256] = st[i][w].ml;
                            ck[(x + 3) * 256] = st[i][w].mh;
                        }
                }
            }
            const int64_t c = __ldg(P.orig + p);
#pragma unroll
            for (int i = 0; i < QI; i++) {
                const int q = q0 + i * 32 + lane;
                if (q >= cls.nq) continue;
                const int m = __ldg(cls.qlen + q);
                const int lb = m - 64 * (NW - 1);
                const uint32_t ml = m <= 0 ? 0u : (lb >= 32 ? ~0u : ((1u << lb) - 1u));
                const uint32_t mh = m <= 0 ? 0u : (lb >= 64 ? ~0u : (lb <= 32 ? 0u : ((1u << (lb - 32)) - 1u)));
                store1(out, dtype, (int64_t)__ldg(cls.qidx + q) * nc + c, n + vsum<NW>(st[i], ml, mh));
            }
        }
    }
}

// The prefix layout's text (PrefixChoices): one thread per sorted choice p
// reads its original string (order[p]) and writes each character's Peq row
// offset (rowoff[byte]), two per word, from word woff[p]; and its length.
__global__ void __launch_bounds__(256) k_prefix_text(DevStrings C, const int32_t *order, const int64_t *woff,
                                                     const uint16_t *rowoff, uint32_t *text, int32_t *len,
                                                     uint32_t *status) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < C.n; p += (int64_t)gridDim.x * blockDim.x) {
        int n;
        const uint8_t *s = string_at(C, order[p], n, status);
        len[p] = n;
        uint32_t *t = text + woff[p];
        for (int j = 0; j < n; j += 2) {
            const uint32_t lo = rowoff[s[j]], hi = j + 1 < n ? rowoff[s[j + 1]] : 0u;
            t[j >> 1] = lo | (hi << 16);
        }
    }
}

// Transpose choices into tiles (see TransposedChoices); one thread per
// (choice, word), bytes past a choice's end are zero.
__global__ void __launch_bounds__(256) k_transpose_choices(DevStrings C, const int64_t *base, uint32_t *words,
                                                           int32_t *len, uint32_t *status) {
    const int64_t nc = C.n;
    const int64_t tiles = (nc + kTileCands - 1) / kTileCands;
    for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const int64_t b0 = base[tile];
        const int nwords = (int)((base[tile + 1] - b0) / kTileCands);
        for (int cl = threadIdx.x; cl < kTileCands; cl += blockDim.x) {
            const int64_t c = tile * kTileCands + cl;
            int n = 0;
            const uint8_t *p = c < nc ? string_at(C, c, n, status) : C.buf;
            if (c < nc) len[c] = n;
            for (int w = 0; w < nwords; w++) {
                uint32_t v = 0;
                const int rem = n - 4 * w;
                if (rem > 0) {
                    v = load4(p + 4 * w);
                    if (rem < 4) v &= (1u << (8 * rem)) - 1u;
                }
                words[b0 + (int64_t)w * kTileCands + cl] = v;
            }
        }
    }
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

// Pairs in natural order (the reference's schedule, one thread per pair):
// each warp takes 32 consecutive pairs,
// copies the byte spans of their a and b strings into shared memory with
// coalesced 16-byte loads (one round trip instead of a chain of dependent
// global reads per pair), then trims and solves from shared memory. Groups
// whose span does not fit read global memory directly; long patterns are
// queued with their global addresses. 128 threads: per warp 8 KB of nibble
// tables and two staging buffers.
constexpr int kStageSpan = 1536;
constexpr int kStageBuf = kStageSpan + 48;      // 16 bytes before, 32 after the span

__device__ __forceinline__ int64_t warp_min64(int64_t v) {
    for (int o = 16; o; o >>= 1) { const int64_t w = __shfl_xor_sync(kFull, v, o); v = w < v ? w : v; }
    return v;
}
__device__ __forceinline__ int64_t warp_max64(int64_t v) {
    for (int o = 16; o; o >>= 1) { const int64_t w = __shfl_xor_sync(kFull, v, o); v = w > v ? w : v; }
    return v;
}

// Copy bytes [lo, hi) of a 16-byte-aligned buffer into stage + 16 (lo, hi
// rounded out to 16 bytes; the buffer's 16-byte slack covers the rounding).
__device__ __forceinline__ void stage_span(uint8_t *stage, const uint8_t *buf, int64_t lo16, int64_t hi16, int lane) {
    for (int64_t x = (int64_t)lane * 16; x < hi16 - lo16; x += 32 * 16)
        *reinterpret_cast<uint4 *>(stage + 16 + x) = __ldg(reinterpret_cast<const uint4 *>(buf + lo16 + x));
}

template <bool HASK>
__global__ void __launch_bounds__(128) k_pairs_staged(DevStrings A, DevStrings B, int k, int dtype, void *out,
                                                      LongQueue q, uint32_t *status) {
    extern __shared__ uint64_t s_mem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t *tc = s_mem + warp * 1024 + lane;
    uint8_t *sa = reinterpret_cast<uint8_t *>(s_mem + 4 * 1024) + warp * 2 * kStageBuf;
    uint8_t *sb = sa + kStageBuf;
#pragma unroll
    for (int r = 0; r < 32; r++) tc[r * 32] = 0;
    const int64_t n = A.n;
    const int64_t nwarps = (int64_t)gridDim.x * 4;
    for (int64_t grp = (int64_t)blockIdx.x * 4 + warp; grp * 32 < n; grp += nwarps) {
        const int64_t i = grp * 32 + lane;
        const bool valid = i < n;
        int la = 0, lb = 0;
        const uint8_t *ga = valid ? string_at(A, i, la, status) : A.buf;
        const uint8_t *gb = valid ? string_at(B, i, lb, status) : B.buf;
        const int64_t a0 = ga - A.buf, b0 = gb - B.buf;
        const int64_t alo = warp_min64(valid ? a0 : INT64_MAX) & ~int64_t(15);
        const int64_t ahi = (warp_max64(valid ? a0 + la : 0) + 15) & ~int64_t(15);
        const int64_t blo = warp_min64(valid ? b0 : INT64_MAX) & ~int64_t(15);
        const int64_t bhi = (warp_max64(valid ? b0 + lb : 0) + 15) & ~int64_t(15);
        const bool staged = ahi - alo <= kStageSpan && bhi - blo <= kStageSpan;
        if (staged) {
            stage_span(sa, A.buf, alo, ahi, lane);
            stage_span(sb, B.buf, blo, bhi, lane);
        }
        __syncwarp();
        if (valid) {
            const uint8_t *a = staged ? sa + 16 + (a0 - alo) : ga;
            const uint8_t *b = staged ? sb + 16 + (b0 - blo) : gb;
            const uint8_t *a_start = a;
            trim_windows<GenericLoad>(a, la, b, lb);
            const int64_t pre = a - a_start;                 // common prefix removed
            const uint8_t *gta = ga + pre, *gtb = gb + pre;  // the same trimmed strings in global memory
            if (la > lb) {
                const uint8_t *t = a; a = b; b = t;
                t = gta; gta = gtb; gtb = t;
                const int x = la; la = lb; lb = x;
            }
            int d;
            bool queued = false;
            if (HASK && lb - la > k) d = k + 1;
            else if (la == 0) d = lb;
            else if (la <= 64) d = solve_word<HASK, GenericLoad>(tc, a, la, b, lb, k);
            else {
                const int cls = long_class(la);
                d = -1;
                if (cls < 0) atomicOr(status, ST_TOO_LONG);
                else {
                    const int pos = atomicAdd(&q.counts[cls], 1);
                    if (pos < q.cap[cls]) {
                        LongItem it;
                        it.pat = gta; it.txt = gtb; it.m = la; it.n = lb; it.idx = i;
                        q.items[cls][pos] = it;
                        queued = true;
                    } else {
                        atomicOr(status, ST_QUEUE_OVERFLOW);
                    }
                }
            }
            if (!queued) store1(out, dtype, i, d);
        }
        __syncwarp();                                        // staging reused by the next group
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

// ------------------------------------------- thresholded search: survivors --
// With max_dist = k, a (query, choice) pair whose lengths differ by more than
// k is decided by the lengths alone (csrc/myers.c:101-106): its result is
// k+1. Choices are kept in a length-sorted copy, so the pairs that need the
// column loop ("survivors") of a query of length m are one contiguous range
// of that copy: lengths m-k .. m+k. The output is first filled with k+1;
// survivors are computed in tiles of 1024 and only results <= k are written.

// out[0..n) = v (dtype-sized), 16-byte stores for the aligned middle.
__global__ void __launch_bounds__(256) k_fill(void *out, int64_t n, int dtype, uint32_t v) {
    fill_share(out, n, dtype, v, (int64_t)blockIdx.x * blockDim.x + threadIdx.x, (int64_t)gridDim.x * blockDim.x);
}

// dst string i = src string perm[i]; one warp per string, byte-wise copy.
__global__ void __launch_bounds__(256) k_gather_strings(DevStrings src, const int32_t *perm,
                                                        const int64_t *dst_off, uint8_t *dst, int64_t n,
                                                        uint32_t *status) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = warp; i < n; i += nwarps) {
        int len;
        const uint8_t *p = string_at(src, perm[i], len, status);
        uint8_t *q = dst + dst_off[i];
        const int64_t cap = dst_off[i + 1] - dst_off[i];
        if (len > cap) len = (int)cap;
        for (int x = lane; x < len; x += 32) q[x] = p[x];
    }
}

// Per class (one block each): survivor range [lo, hi) of every query
// (queries sorted by length), tile counts, and their exclusive prefix
// tile_start[0..nq]; the class's work counter cleared. The scan walks the
// queries 1024 at a time.
__global__ void __launch_bounds__(1024) k_surv_plan(SurvClasses C, const int64_t *lstart, int64_t min_len,
                                                    int64_t n_len, int k, int tile) {
    __shared__ __align__(16) unsigned char s_raw[sizeof(SurvClasses)];   // (no constructor runs on shared memory)
    SurvClasses &s_c = *reinterpret_cast<SurvClasses *>(s_raw);
    __shared__ int64_t s_sum[1024];
    __shared__ int64_t s_carry;
    if (threadIdx.x == 0) {
        s_c = C;
        s_carry = 0;
    }
    __syncthreads();
    const SearchClass &cls = s_c.cls[blockIdx.x];
    int32_t *lo = s_c.lo[blockIdx.x], *hi = s_c.hi[blockIdx.x];
    int64_t *tile_start = s_c.tile_start[blockIdx.x];
    if (threadIdx.x == 0) *s_c.work[blockIdx.x] = 0;
    for (int base = 0; base < cls.nq; base += 1024) {
        const int qi = base + threadIdx.x;
        int64_t tiles = 0;
        if (qi < cls.nq) {
            const int64_t m = cls.qlen[qi];
            int64_t a = m - k - min_len, b = m + k - min_len + 1;   // length window, index space
            a = a < 0 ? 0 : (a > n_len ? n_len : a);
            b = b < 0 ? 0 : (b > n_len ? n_len : b);
            const int64_t l = lstart[a], h = b > a ? lstart[b] : l;
            lo[qi] = (int32_t)l;
            hi[qi] = (int32_t)h;
            tiles = (h - l + tile - 1) / tile;
        }
        s_sum[threadIdx.x] = tiles;
        __syncthreads();
        for (int off = 1; off < 1024; off <<= 1) {                     // inclusive scan
            const int64_t v = threadIdx.x >= off ? s_sum[threadIdx.x - off] : 0;
            __syncthreads();
            s_sum[threadIdx.x] += v;
            __syncthreads();
        }
        if (qi < cls.nq) tile_start[qi] = s_carry + s_sum[threadIdx.x] - tiles;
        __syncthreads();
        if (threadIdx.x == 0) s_carry += s_sum[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0) tile_start[cls.nq] = s_carry;
}

// Persistent: every CTA pulls tiles from the device work counter until the
// plan is exhausted (the counter only grows, so the loop always ends).
template <int NW>
__global__ void __launch_bounds__(256) k_search_surv(DevStrings CS, const int32_t *perm, SearchClass cls,
                                                     const int32_t *lo, const int32_t *hi,
                                                     const int64_t *tile_start, int32_t *work, int k,
                                                     int dtype, void *out, int64_t nc, uint32_t *status,
                                                     uint32_t unit) {
    extern __shared__ uint64_t s_peq[];
    __shared__ int s_tile;
    const Units u{unit, unit + unit};
    RowAddr<NW> ra;
    ra.init(u);
    const int64_t total = tile_start[cls.nq];
    int cur = -1;
    while (true) {
        if (threadIdx.x == 0) s_tile = atomicAdd(work, 1);
        __syncthreads();
        const int64_t tile = s_tile;
        if (tile >= total) break;
        int a = 0, b = cls.nq;                        // tile_start[a] <= tile < tile_start[b]
        while (b - a > 1) {
            const int mid = (a + b) >> 1;
            if (tile_start[mid] <= tile) a = mid; else b = mid;
        }
        const int qi = a;
        const bool banded = k <= 31;                  // uniform: one band word holds every path <= k
        if (qi != cur) {
            const uint64_t *src = cls.peq + (size_t)qi * 256 * NW;
            if (banded) stage_band_rows(src, NW, reinterpret_cast<uint32_t *>(s_peq));
            else for (int x = threadIdx.x; x < 256 * NW; x += blockDim.x) s_peq[x] = __ldg(src + x);
            cur = qi;
        }
        __syncthreads();
        const int m = cls.qlen[qi];
        const int64_t row = cls.qidx[qi];
        const int64_t s_end = hi[qi];
        const int64_t s0 = lo[qi] + (tile - tile_start[qi]) * 1024 + threadIdx.x * 4;
        const uint32_t *rows32 = reinterpret_cast<const uint32_t *>(s_peq);
        constexpr int kStride = 2 * NW + 6;
#pragma unroll 1
        for (int t = 0; t < 4; t++) {
            const int64_t sidx = s0 + t;
            if (sidx >= s_end) break;
            int n;
            const uint8_t *tp = string_at(CS, sidx, n, status);
            int d;
            if (!banded) d = dist_seq_any<NW, true>(s_peq, m, tp, n, k, u, ra);
            else if (m == 0) d = cap_k(n, k);
            else if ((n > m ? n - m : m - n) > k) d = k + 1;
            else d = band_distance(m, tp, n, k,
                                   [&](uint32_t c, int p0) { return band_row_bits(rows32 + c * kStride, p0); }, u);
            if (d <= k) store1(out, dtype, row * nc + perm[sidx], d);
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------- launchers --
template <int NW>
static cudaError_t launch_seq(bool hask, dim3 grid, size_t smem, cudaStream_t st, const DevStrings &C,
                              const SearchClass &cls, int qpb, int k, int dtype, void *out,
                              uint32_t *status) {
    if (hask) {
        cudaFuncSetAttribute(k_search_seq<NW, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_search_seq<NW, true><<<grid, 256, smem, st>>>(C, cls, qpb, k, dtype, out, status, 1u);
    } else {
        cudaFuncSetAttribute(k_search_seq<NW, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_search_seq<NW, false><<<grid, 256, smem, st>>>(C, cls, qpb, k, dtype, out, status, 1u);
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

template <int NW, int QI>
static cudaError_t launch_ttq(dim3 grid, cudaStream_t st, const TransposedChoices &T, const SearchClass &cls,
                              int qpb, int dtype, void *out) {
    const size_t smem = (size_t)QI * 256 * NW * sizeof(uint64_t);
    cudaFuncSetAttribute(k_search_ttq<NW, QI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_search_ttq<NW, QI><<<grid, 256, smem, st>>>(T, cls, qpb, dtype, out, 1u);
    return cudaGetLastError();
}

template <int NW>
static cudaError_t launch_tt(bool hask, dim3 grid, size_t smem, cudaStream_t st, const TransposedChoices &T,
                             const SearchClass &cls, int qpb, int k, int dtype, void *out) {
    // exact short queries: several queries per thread (one text pass serves them all)
    // (measured on 1024 x 65536 L64: 1 query per thread 4.48 ms, 2: 4.19 ms, 4: 4.09 ms, 8: 5.0 ms)
    if (!hask && NW == 1) return launch_ttq<1, 4>(grid, st, T, cls, qpb, dtype, out);
    if (!hask && NW == 2) return launch_ttq<2, 2>(grid, st, T, cls, qpb, dtype, out);
    if (hask) {
        cudaFuncSetAttribute(k_search_tt<NW, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_search_tt<NW, true><<<grid, 256, smem, st>>>(T, cls, qpb, k, dtype, out, 1u);
    } else {
        cudaFuncSetAttribute(k_search_tt<NW, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_search_tt<NW, false><<<grid, 256, smem, st>>>(T, cls, qpb, k, dtype, out, 1u);
    }
    return cudaGetLastError();
}

cudaError_t launch_search_tt(cudaStream_t st, int nw, bool hask, const TransposedChoices &T,
                             const SearchClass &cls, int qpb, int k, int dtype, void *out) {
    if (cls.nq <= 0 || T.n <= 0) return cudaSuccess;
    const int64_t tiles = (T.n + kTileCands - 1) / kTileCands;
    dim3 grid((unsigned)tiles, (unsigned)((cls.nq + qpb - 1) / qpb));
    const size_t smem = (size_t)256 * nw * sizeof(uint64_t);
    switch (nw) {
    case 1: return launch_tt<1>(hask, grid, smem, st, T, cls, qpb, k, dtype, out);
    case 2: return launch_tt<2>(hask, grid, smem, st, T, cls, qpb, k, dtype, out);
    case 3: return launch_tt<3>(hask, grid, smem, st, T, cls, qpb, k, dtype, out);
    case 4: return launch_tt<4>(hask, grid, smem, st, T, cls, qpb, k, dtype, out);
    case 5: return launch_tt<5>(hask, grid, smem, st, T, cls, qpb, k, dtype, out);
    case 6: return launch_tt<6>(hask, grid, smem, st, T, cls, qpb, k, dtype, out);
    case 7: return launch_tt<7>(hask, grid, smem, st, T, cls, qpb, k, dtype, out);
    case 8: return launch_tt<8>(hask, grid, smem, st, T, cls, qpb, k, dtype, out);
    default: return cudaErrorInvalidValue;
    }
}

// Chain length: the longest (most prefix reuse) that still gives the grid
// at least 6 waves of (query block, chain group) items; 4 at the least.
template <int NW, int QI>
static cudaError_t launch_pfx_nw(cudaStream_t st, int grid, const PrefixChoices &P, const SearchClass &cls,
                                 unsigned long long *work, int dtype, void *out) {
    const size_t smem = (size_t)P.nsym * kPfxRowBytes + (size_t)kPfxCheckpoints * QI * NW * 4 * 256 * 4;
    const int64_t qblocks = (cls.nq + QI * 32 - 1) / (QI * 32);
    int chain = kPfxChain;
    auto items_of = [&](int ch) { return qblocks * ((P.n + (int64_t)kPfxWarps * ch - 1) / ((int64_t)kPfxWarps * ch)); };
    while (chain > 4 && items_of(chain) < 6 * (int64_t)grid) chain >>= 1;
    cudaFuncSetAttribute(k_search_pfx<NW, QI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_search_pfx<NW, QI><<<grid, 256, smem, st>>>(P, cls, work, items_of(chain), chain, dtype, out, 1u);
    return cudaGetLastError();
}

bool search_pfx_supported(int nw) { return nw == 1 || nw == 2; }

// `work` must be zero when the launch starts (the caller clears it on the stream).
cudaError_t launch_search_pfx(cudaStream_t st, int sms, int ctas_per_sm, int nw, const PrefixChoices &P,
                              const SearchClass &cls, unsigned long long *work, int dtype, void *out) {
    if (cls.nq <= 0 || P.n <= 0) return cudaSuccess;
    if (P.nsym < 1 || P.nsym > kPfxMaxSymbols) return cudaErrorInvalidValue;
    const int grid = sms * std::max(1, std::min(ctas_per_sm, 8));
    if (nw == 1) return launch_pfx_nw<1, 4>(st, grid, P, cls, work, dtype, out);
    if (nw == 2) return launch_pfx_nw<2, 2>(st, grid, P, cls, work, dtype, out);
    return cudaErrorInvalidValue;
}

cudaError_t launch_prefix_text(cudaStream_t st, int sms, const DevStrings &C, const int32_t *order,
                               const int64_t *woff, const uint16_t *rowoff, uint32_t *text, int32_t *len,
                               uint32_t *status) {
    if (C.n <= 0) return cudaSuccess;
    const int grid = (int)std::min<int64_t>((C.n + 255) / 256, (int64_t)sms * 8);
    k_prefix_text<<<grid, 256, 0, st>>>(C, order, woff, rowoff, text, len, status);
    return cudaGetLastError();
}

cudaError_t launch_transpose_choices(cudaStream_t st, int sms, const DevStrings &C, const int64_t *base,
                                     uint32_t *words, int32_t *len, uint32_t *status) {
    if (C.n <= 0) return cudaSuccess;
    const int64_t tiles = (C.n + kTileCands - 1) / kTileCands;
    const int grid = (int)std::min<int64_t>(tiles, (int64_t)sms * 8);
    k_transpose_choices<<<grid, 256, 0, st>>>(C, base, words, len, status);
    return cudaGetLastError();
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

cudaError_t launch_pairs_staged(cudaStream_t st, int sms, bool hask, const DevStrings &A, const DevStrings &B,
                                int k, int dtype, void *out, const LongQueue &q, uint32_t *status) {
    const size_t smem = 4 * 1024 * sizeof(uint64_t) + 4 * 2 * kStageBuf;
    const int64_t want = (A.n + 127) / 128;
    const int grid = (int)std::min<int64_t>(want, (int64_t)sms * 5 * 8);
    if (hask) {
        cudaFuncSetAttribute(k_pairs_staged<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_pairs_staged<true><<<grid, 128, smem, st>>>(A, B, k, dtype, out, q, status);
    } else {
        cudaFuncSetAttribute(k_pairs_staged<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_pairs_staged<false><<<grid, 128, smem, st>>>(A, B, k, dtype, out, q, status);
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

cudaError_t launch_fill(cudaStream_t st, int sms, void *out, int64_t n, int dtype, uint32_t v) {
    if (n <= 0) return cudaSuccess;
    const int64_t es = dtype == DT_UINT8 ? 1 : dtype == DT_UINT16 ? 2 : 4;
    int64_t blocks = (n * es / 16 + 255) / 256;
    blocks = blocks < 1 ? 1 : (blocks > (int64_t)sms * 16 ? (int64_t)sms * 16 : blocks);
    k_fill<<<(unsigned)blocks, 256, 0, st>>>(out, n, dtype, v);
    return cudaGetLastError();
}

// Offsets of the length-sorted copy: every string of length bucket b
// (positions lstart[b] .. lstart[b+1]-1) is min_len + b bytes long, so
// soff[j] = bstart[b] + (j - lstart[b]) * (min_len + b); soff[n] = the total.
__global__ void __launch_bounds__(256) k_sorted_offsets(const int64_t *lstart, int64_t n_len, int64_t min_len,
                                                        const int64_t *bstart, int64_t n, int64_t *soff) {
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j <= n; j += (int64_t)gridDim.x * blockDim.x) {
        const int b = j < n ? upper_index(lstart, (int)n_len, j) : (int)n_len - 1;
        soff[j] = bstart[b] + (j - lstart[b]) * (min_len + b);
    }
}

cudaError_t launch_sorted_offsets(cudaStream_t st, int sms, const int64_t *lstart, int64_t n_len, int64_t min_len,
                                  const int64_t *bstart, int64_t n, int64_t *soff) {
    if (n < 0 || n_len <= 0) return cudaSuccess;
    const int64_t blocks = std::min<int64_t>((n + 256) / 256, (int64_t)sms * 8);
    k_sorted_offsets<<<(unsigned)blocks, 256, 0, st>>>(lstart, n_len, min_len, bstart, n, soff);
    return cudaGetLastError();
}

cudaError_t launch_gather_strings(cudaStream_t st, int sms, const DevStrings &src, const int32_t *perm,
                                  const int64_t *dst_off, uint8_t *dst, int64_t n, uint32_t *status) {
    if (n <= 0) return cudaSuccess;
    int64_t blocks = (n + 7) / 8;
    blocks = blocks > (int64_t)sms * 32 ? (int64_t)sms * 32 : blocks;
    k_gather_strings<<<(unsigned)blocks, 256, 0, st>>>(src, perm, dst_off, dst, n, status);
    return cudaGetLastError();
}

cudaError_t launch_surv_plan(cudaStream_t st, const SurvClasses &C, const int64_t *lstart, int64_t min_len,
                             int64_t n_len, int k, int tile) {
    if (C.n <= 0) return cudaSuccess;
    if (C.n > kSurvClasses) return cudaErrorInvalidValue;
    k_surv_plan<<<C.n, 1024, 0, st>>>(C, lstart, min_len, n_len, k, tile);
    return cudaGetLastError();
}

template <int NW>
static cudaError_t launch_surv_nw(cudaStream_t st, int grid, const DevStrings &CS, const int32_t *perm,
                                  const SearchClass &cls, const int32_t *lo, const int32_t *hi,
                                  const int64_t *tile_start, int32_t *work, int k, int dtype, void *out,
                                  int64_t nc, uint32_t *status) {
    const size_t smem = std::max((size_t)256 * NW * sizeof(uint64_t), (size_t)256 * (2 * NW + 6) * sizeof(uint32_t));
    cudaFuncSetAttribute(k_search_surv<NW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_search_surv<NW><<<grid, 256, smem, st>>>(CS, perm, cls, lo, hi, tile_start, work, k, dtype, out, nc,
                                                status, 1u);
    return cudaGetLastError();
}

cudaError_t launch_search_surv(cudaStream_t st, int sms, int nw, const DevStrings &CS, const int32_t *perm,
                               const SearchClass &cls, const int32_t *lo, const int32_t *hi,
                               const int64_t *tile_start, int32_t *work, int k, int dtype, void *out,
                               int64_t nc, uint32_t *status) {
    if (cls.nq <= 0) return cudaSuccess;
    const int grid = sms * 4;
    switch (nw) {
    case 1: return launch_surv_nw<1>(st, grid, CS, perm, cls, lo, hi, tile_start, work, k, dtype, out, nc, status);
    case 2: return launch_surv_nw<2>(st, grid, CS, perm, cls, lo, hi, tile_start, work, k, dtype, out, nc, status);
    case 3: return launch_surv_nw<3>(st, grid, CS, perm, cls, lo, hi, tile_start, work, k, dtype, out, nc, status);
    case 4: return launch_surv_nw<4>(st, grid, CS, perm, cls, lo, hi, tile_start, work, k, dtype, out, nc, status);
    case 5: return launch_surv_nw<5>(st, grid, CS, perm, cls, lo, hi, tile_start, work, k, dtype, out, nc, status);
    case 6: return launch_surv_nw<6>(st, grid, CS, perm, cls, lo, hi, tile_start, work, k, dtype, out, nc, status);
    case 7: return launch_surv_nw<7>(st, grid, CS, perm, cls, lo, hi, tile_start, work, k, dtype, out, nc, status);
    case 8: return launch_surv_nw<8>(st, grid, CS, perm, cls, lo, hi, tile_start, work, k, dtype, out, nc, status);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace blg
