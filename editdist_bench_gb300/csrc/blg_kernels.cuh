// Device-side building blocks shared by the kernel translation units:
// string access, stores, the per-query Peq column loop (search), the
// lane-spread wavefront and the pair-solving helpers (trimming, per-lane
// nibble Peq tables). Device code only; the host-testable primitives live in
// blg_device.cuh.
#pragma once
#include "blg_device.cuh"
#include "blg_internal.h"

namespace blg {

constexpr unsigned kFull = 0xffffffffu;

// ---------------------------------------------------------------- loads --
// Load policies: strings in global memory go through the read-only cache;
// strings staged in shared memory are read with generic loads.
struct LdgLoad {
    static __device__ __forceinline__ uint32_t ld(const uint32_t *p) { return __ldg(p); }
};
struct GenericLoad {
    static __device__ __forceinline__ uint32_t ld(const uint32_t *p) { return *p; }
};

// Four bytes starting at an arbitrary address: two aligned 32-bit loads and
// a funnel shift. Callers keep 16 bytes of slack around every string buffer
// so the aligned words never leave the allocation.
template <typename L = LdgLoad>
__device__ __forceinline__ uint32_t load4(const uint8_t *p) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(p);
    const uint32_t *w = reinterpret_cast<const uint32_t *>(a & ~uintptr_t(3));
    return __funnelshift_r(L::ld(w), L::ld(w + 1), (uint32_t)(a & 3) * 8u);
}

// Sequential reader: 4 characters per call, one aligned load per call,
// issued one call ahead so its latency overlaps the caller's columns. Reads
// at most 12 bytes past the last character returned (the 16-byte slack).
template <typename L = LdgLoad>
struct TextScanT {
    const uint32_t *w;
    uint32_t lo, hi, sh;
    __device__ __forceinline__ void init(const uint8_t *p) {
        const uintptr_t a = reinterpret_cast<uintptr_t>(p);
        w = reinterpret_cast<const uint32_t *>(a & ~uintptr_t(3));
        sh = (uint32_t)(a & 3) * 8u;
        lo = L::ld(w);
        hi = L::ld(++w);
    }
    __device__ __forceinline__ uint32_t next4() {
        const uint32_t r = __funnelshift_r(lo, hi, sh);
        lo = hi;
        hi = L::ld(++w);
        return r;
    }
};
using TextScan = TextScanT<LdgLoad>;

// Non-prefetching variant for register-bound loops (the full-word search
// loop), where the extra live word costs more than the load latency saves.
struct TextScanLean {
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

// ------------------------------------------------------- byte alphabets --
// A set's bytes as an 8-word presence bitmap (k_byte_presence): its size,
// and the byte -> row map of the one-row-per-byte pattern tables (bytes in
// increasing order get rows 0, 1, ...; the rest row kBandSymbols). The map
// is built by the whole block into shared memory.
__device__ __forceinline__ int alpha_size(const uint32_t *alpha) {
    int total = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) total += __popc(__ldg(alpha + i));
    return total;
}

__device__ __forceinline__ void alpha_map(const uint32_t *alpha, uint8_t *map) {
    for (int b = threadIdx.x; b < 256; b += blockDim.x) {
        const uint32_t w = __ldg(alpha + (b >> 5));
        int rank = __popc(w & ((1u << (b & 31)) - 1u));
        for (int i = 0; i < (b >> 5); i++) rank += __popc(__ldg(alpha + i));
        map[b] = (uint8_t)(((w >> (b & 31)) & 1u) ? rank : kBandSymbols);
    }
    __syncthreads();
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

// --------------------------------------------------- search, NW <= 8 words --
// Address arithmetic for the Peq row of text byte b (0..3) of a 4-byte
// window: byte offset = c * 8 * NW. For power-of-two NW the byte is shifted
// straight into place by one IMAD (hi or lo) and masked; otherwise it is
// extracted and scaled by IMAD. Multipliers are run-time values.
template <int NW>
struct RowAddr {
    static constexpr bool kPow2 = (NW & (NW - 1)) == 0;
    static constexpr int kSh = 3 + (NW >= 8 ? 3 : NW >= 4 ? 2 : NW >= 2 ? 1 : 0);
    uint32_t mul[4], mask, stride, ext[4];
    __device__ __forceinline__ void init(Units u) {
        if (kPow2) {
            mul[0] = u.one << kSh;
            mul[1] = u.one << (24 + kSh);
            mul[2] = u.one << (16 + kSh);
            mul[3] = u.one << (8 + kSh);
            mask = 0xffu << kSh;
        }
        ext[1] = u.one << 24;
        ext[2] = u.one << 16;
        ext[3] = u.one << 8;
        stride = imad_lo(u.one, 8u * NW, 0);
    }
    template <int B>
    __device__ __forceinline__ uint32_t off(uint32_t w4) const {
        // the top byte needs no mask: hi32(w4 * 2^8) is that byte alone
        if (kPow2 && B == 3) return imad_lo(imad_hi(w4, ext[3], 0), stride, 0);
        if (kPow2) return (B == 0 ? imad_lo(w4, mul[0], 0) : imad_hi(w4, mul[B], 0)) & mask;
        const uint32_t c = B == 0 ? (w4 & 0xffu) : B == 3 ? imad_hi(w4, ext[3], 0)
                                                          : (imad_hi(w4, ext[B], 0) & 0xffu);
        return imad_lo(c, stride, 0);
    }
};

// One text column through the NW words of the query (word 0 takes the +1
// top-row carry); the last word's horizontal delta is accumulated as +1/-1
// counts. LAST: 0 = score bit is bit 63, 1 = bit (lastbit-32) of the high
// half, 2 = bit lastbit of the low half (`mult` = 2^(31 - that bit)).
template <int NW, int LAST>
__device__ __forceinline__ void column_h(Word2 (&st)[NW], const uint64_t *row, Units u, uint32_t mult,
                                         uint32_t &accP, uint32_t &accM) {
    uint32_t Phl, Phh, Mhl, Mhh;
    uint32_t cp = u.one, cm = 0;
#pragma unroll
    for (int w = 0; w < NW; w++) {
        const uint64_t e = row[w];
        step_h(st[w], (uint32_t)e, (uint32_t)(e >> 32), cp, cm, u, Phl, Phh, Mhl, Mhh);
        if (w < NW - 1) {
            cp = top_bit(Phh, u);
            cm = top_bit(Mhh, u);
        }
    }
    if (LAST == 0) {
        accP = imad_hi(Phh, u.two, accP);
        accM = imad_hi(Mhh, u.two, accM);
    } else if (LAST == 1) {
        accP = imad_hi(imad_lo(Phh, mult, 0), u.two, accP);
        accM = imad_hi(imad_lo(Mhh, mult, 0), u.two, accM);
    } else {
        accP = imad_hi(imad_lo(Phl, mult, 0), u.two, accP);
        accM = imad_hi(imad_lo(Mhl, mult, 0), u.two, accM);
    }
}

// d(query, t) with the query's Peq table in shared memory (NW = ceil(m/64)).
template <int NW, bool HASK, int LAST>
__device__ __forceinline__ int dist_seq(const uint64_t *peq, int m, const uint8_t *t, int n, int k,
                                        Units u, const RowAddr<NW> &ra) {
    if (m == 0) return cap_k(n, k);                    // csrc/gpu_kernels.cu:53
    if (HASK && (n > m ? n - m : m - n) > k) return k + 1;
    Word2 st[NW];
#pragma unroll
    for (int w = 0; w < NW; w++) { st[w].pl = st[w].ph = ~0u; st[w].ml = st[w].mh = 0; }
    const int lastbit = (m - 1) & 63;
    const uint32_t mult = u.one << (31 - (lastbit & 31));
    uint32_t accP = 0, accM = 0;                        // score = m + accP - accM
    const char *base = reinterpret_cast<const char *>(peq);
    TextScanLean ts;
    ts.init(t);
    int j = 0;
    for (; j + 4 <= n; j += 4) {
        const uint32_t w4 = ts.next4();
        column_h<NW, LAST>(st, reinterpret_cast<const uint64_t *>(base + ra.template off<0>(w4)), u, mult, accP, accM);
        column_h<NW, LAST>(st, reinterpret_cast<const uint64_t *>(base + ra.template off<1>(w4)), u, mult, accP, accM);
        column_h<NW, LAST>(st, reinterpret_cast<const uint64_t *>(base + ra.template off<2>(w4)), u, mult, accP, accM);
        column_h<NW, LAST>(st, reinterpret_cast<const uint64_t *>(base + ra.template off<3>(w4)), u, mult, accP, accM);
        // the exit test is monotone in j, so testing every 4th column is exact
        if (HASK && hopeless(m + (int)accP - (int)accM, j + 3, n, k)) return k + 1;
    }
    if (j < n) {
        uint32_t w4 = ts.next4();
        for (; j < n; j++, w4 >>= 8)
            column_h<NW, LAST>(st, reinterpret_cast<const uint64_t *>(base + ra.template off<0>(w4)), u, mult,
                               accP, accM);
    }
    const int score = m + (int)accP - (int)accM;
    return HASK ? cap_k(score, k) : score;
}

// One text column through the NW words of the query without the score
// (the score is read from the vertical deltas when needed).
template <int NW>
__device__ __forceinline__ void column_v(Word2 (&st)[NW], const uint64_t *row, Units u) {
    uint32_t Phl, Phh, Mhl, Mhh;
    uint32_t cp = u.one, cm = 0;
#pragma unroll
    for (int w = 0; w < NW; w++) {
        const uint64_t e = row[w];
        step_h(st[w], (uint32_t)e, (uint32_t)(e >> 32), cp, cm, u, Phl, Phh, Mhl, Mhh);
        if (w < NW - 1) {
            cp = top_bit(Phh, u);
            cm = top_bit(Mhh, u);
        }
    }
}

// Sum of the vertical deltas of the pattern rows (the last word masked to
// its `lastbits` = m - 64 (NW - 1) rows): D[m][j] = j + this, after j columns.
template <int NW>
__device__ __forceinline__ int vsum(const Word2 (&st)[NW], uint32_t ml, uint32_t mh) {
    int s = 0;
#pragma unroll
    for (int w = 0; w < NW - 1; w++)
        s += popc32(st[w].pl) + popc32(st[w].ph) - popc32(st[w].ml) - popc32(st[w].mh);
    s += popc32(st[NW - 1].pl & ml) + popc32(st[NW - 1].ph & mh) - popc32(st[NW - 1].ml & ml) -
         popc32(st[NW - 1].mh & mh);
    return s;
}

// d(query, choice) with the choice in tile-transposed form: word w of the
// text at txt[w * kTileCands] (one coalesced line per warp). The loop runs 16
// columns (4 words) per iteration with the next 4 words already in flight, so
// the loop's own bookkeeping is spread over 16 columns; the prefetch may read
// up to 4 words past the text (the transposed buffer has kTtSlackRows spare
// rows after its last tile).
template <int NW, bool HASK>
__device__ __forceinline__ int dist_tt(const uint64_t *peq, int m, const uint32_t *txt, int n, int k, Units u,
                                       const RowAddr<NW> &ra) {
    if (m == 0) return cap_k(n, k);                    // csrc/gpu_kernels.cu:53
    if (HASK && (n > m ? n - m : m - n) > k) return k + 1;
    Word2 st[NW];
#pragma unroll
    for (int w = 0; w < NW; w++) { st[w].pl = st[w].ph = ~0u; st[w].ml = st[w].mh = 0; }
    const int lb = m - 64 * (NW - 1);                  // rows of the last word, 1..64
    const uint32_t ml = lb >= 32 ? ~0u : ((1u << lb) - 1u);
    const uint32_t mh = lb >= 64 ? ~0u : (lb <= 32 ? 0u : ((1u << (lb - 32)) - 1u));
    const char *base = reinterpret_cast<const char *>(peq);
    auto col4 = [&](uint32_t w4) {
        column_v<NW>(st, reinterpret_cast<const uint64_t *>(base + ra.template off<0>(w4)), u);
        column_v<NW>(st, reinterpret_cast<const uint64_t *>(base + ra.template off<1>(w4)), u);
        column_v<NW>(st, reinterpret_cast<const uint64_t *>(base + ra.template off<2>(w4)), u);
        column_v<NW>(st, reinterpret_cast<const uint64_t *>(base + ra.template off<3>(w4)), u);
    };
    const uint32_t *p = txt;
    uint32_t w0 = __ldg(p), w1 = __ldg(p + kTileCands), w2 = __ldg(p + 2 * kTileCands),
             w3 = __ldg(p + 3 * kTileCands);
    int j = 0;
    for (; j + 16 <= n; j += 16) {
        const uint32_t a0 = w0, a1 = w1, a2 = w2, a3 = w3;
        p += 4 * kTileCands;
        w0 = __ldg(p);
        w1 = __ldg(p + kTileCands);
        w2 = __ldg(p + 2 * kTileCands);
        w3 = __ldg(p + 3 * kTileCands);
        // the exit test is monotone in j, so testing every 4th column is exact
        col4(a0);
        if (HASK && hopeless(j + 4 + vsum<NW>(st, ml, mh), j + 3, n, k)) return k + 1;
        col4(a1);
        if (HASK && hopeless(j + 8 + vsum<NW>(st, ml, mh), j + 7, n, k)) return k + 1;
        col4(a2);
        if (HASK && hopeless(j + 12 + vsum<NW>(st, ml, mh), j + 11, n, k)) return k + 1;
        col4(a3);
        if (HASK && hopeless(j + 16 + vsum<NW>(st, ml, mh), j + 15, n, k)) return k + 1;
    }
    // up to 15 columns left, in w0..w3
    const uint32_t rest[4] = {w0, w1, w2, w3};
#pragma unroll
    for (int q = 0; q < 4; q++) {
        if (j + 4 <= n) {
            col4(rest[q]);
            if (HASK && hopeless(j + 4 + vsum<NW>(st, ml, mh), j + 3, n, k)) return k + 1;
            j += 4;
        } else {
            for (uint32_t w4 = rest[q]; j < n; j++, w4 >>= 8)
                column_v<NW>(st, reinterpret_cast<const uint64_t *>(base + ra.template off<0>(w4)), u);
            break;
        }
    }
    const int d = n + vsum<NW>(st, ml, mh);
    return HASK ? cap_k(d, k) : d;
}

// Exact distances of QI queries (Peq tables consecutive in shared memory,
// 256 * NW words apart) against one tile-transposed choice: each text word
// is loaded and each character's row offset computed once for the QI
// queries, whose column chains are independent (instruction-level
// parallelism). Queries past `nq` (a partial group) and queries of length 0
// have all-zero tables and masks, so their result is n, as the exact rule
// wants for an empty query.
template <int NW, int QI>
__device__ __forceinline__ void dist_tt_q(const uint64_t *peq, const int32_t *qlen, int nq, const uint32_t *txt,
                                          int n, Units u, const RowAddr<NW> &ra, int (&d)[QI]) {
    Word2 st[QI][NW];
#pragma unroll
    for (int i = 0; i < QI; i++)
#pragma unroll
        for (int w = 0; w < NW; w++) { st[i][w].pl = st[i][w].ph = ~0u; st[i][w].ml = st[i][w].mh = 0; }
    const char *base = reinterpret_cast<const char *>(peq);
    auto col = [&](uint32_t off) {
#pragma unroll
        for (int i = 0; i < QI; i++)
            column_v<NW>(st[i], reinterpret_cast<const uint64_t *>(base + i * (256 * NW * 8) + off), u);
    };
    auto col4 = [&](uint32_t w4) {
        col(ra.template off<0>(w4));
        col(ra.template off<1>(w4));
        col(ra.template off<2>(w4));
        col(ra.template off<3>(w4));
    };
    const uint32_t *p = txt;
    uint32_t w0 = __ldg(p), w1 = __ldg(p + kTileCands), w2 = __ldg(p + 2 * kTileCands),
             w3 = __ldg(p + 3 * kTileCands);
    int j = 0;
    for (; j + 16 <= n; j += 16) {
        const uint32_t a0 = w0, a1 = w1, a2 = w2, a3 = w3;
        p += 4 * kTileCands;
        w0 = __ldg(p);
        w1 = __ldg(p + kTileCands);
        w2 = __ldg(p + 2 * kTileCands);
        w3 = __ldg(p + 3 * kTileCands);
        col4(a0);
        col4(a1);
        col4(a2);
        col4(a3);
    }
    const uint32_t rest[4] = {w0, w1, w2, w3};
#pragma unroll
    for (int q = 0; q < 4; q++) {
        if (j + 4 <= n) {
            col4(rest[q]);
            j += 4;
        } else {
            for (uint32_t w4 = rest[q]; j < n; j++, w4 >>= 8) col(ra.template off<0>(w4));
            break;
        }
    }
#pragma unroll
    for (int i = 0; i < QI; i++) {
        const int m = i < nq ? __ldg(qlen + i) : 0;    // lengths read here, not held through the loop
        const int lb = m - 64 * (NW - 1);
        const uint32_t ml = m <= 0 ? 0u : (lb >= 32 ? ~0u : ((1u << lb) - 1u));
        const uint32_t mh = m <= 0 ? 0u : (lb >= 64 ? ~0u : (lb <= 32 ? 0u : ((1u << (lb - 32)) - 1u)));
        d[i] = n + vsum<NW>(st[i], ml, mh);
    }
}

template <int NW, bool HASK>
__device__ __forceinline__ int dist_seq_any(const uint64_t *peq, int m, const uint8_t *t, int n, int k,
                                            Units u, const RowAddr<NW> &ra) {
    const int lastbit = (m - 1) & 63;
    if (m > 0 && lastbit == 63) return dist_seq<NW, HASK, 0>(peq, m, t, n, k, u, ra);
    if (lastbit >= 32) return dist_seq<NW, HASK, 1>(peq, m, t, n, k, u, ra);
    return dist_seq<NW, HASK, 2>(peq, m, t, n, k, u, ra);
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
                                              int w, int g, int k, EqFn eqfn, bool &is_last,
                                              int *cols_out = nullptr) {
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
            if (valid && ((bal >> (g * L + lastw)) & 1u)) {
                if (!done && cols_out) *cols_out = s - lastw + 1;   // columns the last word processed
                done = true;
            }
        }
    }
    if (done) return k + 1;
    if (cols_out) *cols_out = n;
    return HASK ? cap_k(score, k) : score;
}

// ------------------------------------------------------------ pairs: main --
// Trim the common prefix and suffix with 4-byte window compares (exact:
// d(xPy, xQy) = d(P, Q), csrc/myers.c:80-87). Each side is read by a running
// pair of aligned words with the next word already requested, so a window
// costs one load per string and its latency overlaps the previous compare.
// The reads stay within 11 bytes of the strings' ends (the buffers' slack is
// 16 bytes before and at least 32 after).
template <typename L = LdgLoad>
__device__ __forceinline__ void trim_windows(const uint8_t *&a, int &la, const uint8_t *&b, int &lb) {
    const int lim = la < lb ? la : lb;
    int p = 0;
    if (lim > 0) {
        const uintptr_t ua = reinterpret_cast<uintptr_t>(a), ub = reinterpret_cast<uintptr_t>(b);
        const uint32_t *wa = reinterpret_cast<const uint32_t *>(ua & ~uintptr_t(3));
        const uint32_t *wb = reinterpret_cast<const uint32_t *>(ub & ~uintptr_t(3));
        const uint32_t sa = (uint32_t)(ua & 3) * 8u, sb = (uint32_t)(ub & 3) * 8u;
        uint32_t a0 = L::ld(wa), a1 = L::ld(wa + 1), b0 = L::ld(wb), b1 = L::ld(wb + 1);
        while (p < lim) {
            const uint32_t a2 = L::ld(wa + 2), b2 = L::ld(wb + 2);     // the next window's new words
            const uint32_t x = __funnelshift_r(a0, a1, sa) ^ __funnelshift_r(b0, b1, sb);
            int q = x ? (__ffs(x) - 1) >> 3 : 4;               // equal leading bytes
            if (q > lim - p) q = lim - p;
            p += q;
            if (q < 4) break;
            a0 = a1; a1 = a2; b0 = b1; b1 = b2;
            wa++; wb++;
        }
    }
    const int lim2 = lim - p;
    int s = 0;
    if (lim2 > 0) {
        const uintptr_t ua = reinterpret_cast<uintptr_t>(a + la - 4), ub = reinterpret_cast<uintptr_t>(b + lb - 4);
        const uint32_t *wa = reinterpret_cast<const uint32_t *>(ua & ~uintptr_t(3));
        const uint32_t *wb = reinterpret_cast<const uint32_t *>(ub & ~uintptr_t(3));
        const uint32_t sa = (uint32_t)(ua & 3) * 8u, sb = (uint32_t)(ub & 3) * 8u;
        uint32_t a0 = L::ld(wa), a1 = L::ld(wa + 1), b0 = L::ld(wb), b1 = L::ld(wb + 1);
        while (s < lim2) {
            const uint32_t am = L::ld(wa - 1), bm = L::ld(wb - 1);     // the next window's new words
            const uint32_t x = __funnelshift_r(a0, a1, sa) ^ __funnelshift_r(b0, b1, sb);
            int q = x ? __clz(x) >> 3 : 4;                     // equal trailing bytes
            if (q > lim2 - s) q = lim2 - s;
            s += q;
            if (q < 4) break;
            a1 = a0; a0 = am; b1 = b0; b0 = bm;
            wa--; wb--;
        }
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

template <typename L = LdgLoad>
__device__ __forceinline__ void nib_build(uint64_t *tc, const uint8_t *p, int m) {
    TextScanT<L> ps;
    ps.init(p);
    for (int i = 0; i < m; i += 4) {
        const uint32_t w4 = ps.next4();
#pragma unroll
        for (int b = 0; b < 4; b++) {
            if (i + b < m) {
                const uint32_t c = (w4 >> (8 * b)) & 0xffu;
                const unsigned long long bit = 1ull << (i + b);
                // one shared-memory atomic per row update instead of a load-or-store chain
                atomicOr(reinterpret_cast<unsigned long long *>(tc + (c >> 4) * 32), bit);
                atomicOr(reinterpret_cast<unsigned long long *>(tc + (16 + (c & 15)) * 32), bit);
            }
        }
    }
}

// Clear a pattern's rows: all 32 with plain stores once it has more than 4
// bytes (fewer instructions than revisiting its bytes), else the rows it set.
template <typename L = LdgLoad>
__device__ __forceinline__ void nib_clear(uint64_t *tc, const uint8_t *p, int m) {
    if (m > 4) {
#pragma unroll
        for (int r = 0; r < 32; r++) tc[r * 32] = 0;
        return;
    }
    TextScanT<L> ps;
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
template <bool HASK, typename L = LdgLoad>
__device__ __forceinline__ int solve_word(uint64_t *tc, const uint8_t *p, int m, const uint8_t *t,
                                          int n, int k, int *cols_out = nullptr) {
    nib_build<L>(tc, p, m);
    uint64_t pv = ~0ull, mv = 0;
    const int lastbit = m - 1;
    int score = m;
    bool dead = false;
    TextScanT<L> ts;
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
        if (HASK && hopeless(score, j + 3, n, k)) {
            dead = true;
            if (cols_out) *cols_out = j + 4;
            break;
        }
    }
    if (!dead && j < n) {
        uint32_t w4 = ts.next4();
        for (; j < n; j++, w4 >>= 8) {
            uint64_t ph, mh;
            step_top<uint64_t>(pv, mv, nib_eq(tc, w4 & 0xffu), ph, mh);
            score += hdelta<uint64_t>(ph, mh, lastbit);
        }
    }
    nib_clear<L>(tc, p, m);
    if (dead) return k + 1;
    if (cols_out) *cols_out = n;
    return HASK ? cap_k(score, k) : score;
}

__device__ __forceinline__ int long_class(int m) {
    const int W = (m + 63) >> 6;
    return W <= 2 ? 0 : W <= 4 ? 1 : W <= 8 ? 2 : W <= 16 ? 3 : W <= 32 ? 4 : -1;
}

// Banded column loop (blg_device.cuh: band_core) reading the text with 4-byte loads.
template <typename EqW>
__device__ __forceinline__ int band_distance(int m, const uint8_t *t, int n, int k, EqW eqw, Units u,
                                             int *cols_out = nullptr) {
    TextScan ts;
    ts.init(t);
    uint32_t w4 = 0;
    auto text = [&](int j) -> uint32_t {
        if ((j & 3) == 0) w4 = ts.next4();
        const uint32_t c = w4 & 0xffu;
        w4 >>= 8;
        return c;
    };
    return band_core(m, n, k, text, eqw, u, cols_out);
}

// The banded loop of one pair with per-thread block rows (the pairs
// kernels): rows over a 64-position block of the pattern, bit i <->
// position 32b - dhi + i in block b, in a [row][thread] table of stride T
// starting at this thread's row 0 (tc). Columns 32b .. 32b+31 read their
// 32-bit windows out of the block with one funnel shift; every 32 columns
// the rows shift down by 32 positions and the next 32 pattern bytes enter.
// SYM: one row per byte (map: byte -> row, kBandSymbols + 1 rows); else
// nibble rows, Eq(c) = row[c >> 4] & row[16 + (c & 15)] (32 rows).
// pat_at(pos) / txt_at(pos) return readers (next4()) positioned at pattern
// / text byte pos. Caller guarantees 1 <= m, |n - m| <= k <= 31.
template <bool SYM, int T, typename PatAt, typename TxtAt>
__device__ __forceinline__ int band_rows_distance(uint2 *tc, const uint8_t *map, PatAt pat_at, TxtAt txt_at, int m,
                                                  int n, int k, int *cols_out) {
    constexpr int R = SYM ? kBandSymbols + 1 : 32;
    auto enter = [&](uint32_t c, int bitpos) {                  // pattern byte c at block bit bitpos (0..63)
        const uint32_t bit = 1u << (bitpos & 31);
        if (SYM) {
            atomicOr(reinterpret_cast<uint32_t *>(tc + map[c] * T) + (bitpos >> 5), bit);
        } else {
            atomicOr(reinterpret_cast<uint32_t *>(tc + (c >> 4) * T) + (bitpos >> 5), bit);
            atomicOr(reinterpret_cast<uint32_t *>(tc + (16 + (c & 15)) * T) + (bitpos >> 5), bit);
        }
    };
    auto rowbits = [&](uint32_t c) -> uint2 {
        if (SYM) return tc[map[c] * T];
        const uint2 h = tc[(c >> 4) * T], l = tc[(16 + (c & 15)) * T];
        return make_uint2(h.x & l.x, h.y & l.y);
    };
    const BandGeom bg = band_geom(m, n, k);
    const int dhi = bg.dhi;
#pragma unroll
    for (int r = 0; r < R; r++) tc[r * T] = make_uint2(0, 0);
    // block 0: positions 0 .. min(m, 64 - dhi) - 1 at bits pos + dhi
    const int first_end = min(m, 64 - dhi);
    {
        auto fs = pat_at(0);
        for (int p = 0; p < first_end; p += 4) {
            const uint32_t w4 = fs.next4();
#pragma unroll
            for (int b = 0; b < 4; b++)
                if (p + b < first_end) enter((w4 >> (8 * b)) & 0xffu, p + b + dhi);
        }
    }
    // later blocks enter the positions from 64 - dhi on, 32 at a time
    auto ps = pat_at(first_end);
    int next_pos = first_end;
    auto eqw = [&](uint32_t c, int p0) -> uint32_t {
        const int j = p0 + dhi;
        if ((j & 31) == 0 && j > 0) {
#pragma unroll
            for (int r = 0; r < R; r++) {
                const uint32_t hi = tc[r * T].y;
                tc[r * T] = make_uint2(hi, 0);
            }
            const int cnt = min(32, m - next_pos);
            for (int i = 0; i < cnt; i += 4) {
                const uint32_t w4 = ps.next4();
#pragma unroll
                for (int b = 0; b < 4; b++)
                    if (i + b < cnt) enter((w4 >> (8 * b)) & 0xffu, 32 + i + b);
            }
            next_pos += cnt > 0 ? cnt : 0;
        }
        const uint2 x = rowbits(c);
        return __funnelshift_r(x.x, x.y, (uint32_t)(j & 31));
    };
    auto ts = txt_at(0);
    uint32_t w4 = 0;
    auto text = [&](int j) -> uint32_t {
        if ((j & 3) == 0) w4 = ts.next4();
        const uint32_t c = w4 & 0xffu;
        w4 >>= 8;
        return c;
    };
    return band_core(m, n, k, text, eqw, Units{1u, 2u}, cols_out);
}

// Query Peq rows as 32-bit halves with zero padding (2 halves before, 4
// after): row stride 2*NW + 6 halves. Window bits at pattern index p0:
// halves around p0 + 64, one funnel shift.
__device__ __forceinline__ uint32_t band_row_bits(const uint32_t *row, int p0) {
    const int P = p0 + 64;
    return __funnelshift_r(row[P >> 5], row[(P >> 5) + 1], (uint32_t)(P & 31));
}

// The same window bits from an unpadded [256][nw] u64 Peq row in global
// memory (row = table + byte * nw): halves p0 >> 5 and the next one, zero
// outside the row (p0 >= -32 may be negative).
__device__ __forceinline__ uint32_t peq_window(const uint64_t *row, int nw, int p0) {
    const uint32_t *h = reinterpret_cast<const uint32_t *>(row);
    const int r = p0 >> 5;
    const uint32_t lo = (unsigned)r < (unsigned)(2 * nw) ? __ldg(h + r) : 0u;
    const uint32_t hi = (unsigned)(r + 1) < (unsigned)(2 * nw) ? __ldg(h + r + 1) : 0u;
    return __funnelshift_r(lo, hi, (uint32_t)(p0 & 31));
}

// Stage a [256][nw] u64 Peq table as padded halves (stride 2*nw + 6).
__device__ __forceinline__ void stage_band_rows(const uint64_t *src, int nw, uint32_t *dst) {
    const int stride = 2 * nw + 6;
    for (int x = threadIdx.x; x < 256 * stride; x += blockDim.x) {
        const int r = x / stride, h = x - r * stride - 2;
        uint32_t v = 0;
        if (h >= 0 && h < 2 * nw) {
            const uint64_t wd = src[r * nw + (h >> 1)];
            v = (h & 1) ? (uint32_t)(wd >> 32) : (uint32_t)wd;
        }
        dst[x] = v;
    }
}

// Build the Peq table of one query into shared memory `tab` (256 x nwc
// words) and copy it to `dst`: one block, shared-memory atomics.
__device__ __forceinline__ void build_peq_block(const uint8_t *p, int m, int nwc, uint64_t *tab,
                                                uint64_t *dst) {
    const int words = 256 * nwc;
    for (int x = threadIdx.x; x < words; x += blockDim.x) tab[x] = 0;
    __syncthreads();
    if (m > 64 * nwc) m = 64 * nwc;   // callers guarantee m <= 64*nwc; keep the write in range
    for (int i = threadIdx.x; i < m; i += blockDim.x)
        atomicOr(reinterpret_cast<unsigned long long *>(&tab[(int)p[i] * nwc + (i >> 6)]),
                 1ull << (i & 63));
    __syncthreads();
    for (int x = threadIdx.x; x < words; x += blockDim.x) dst[x] = tab[x];
}

// 4-gram sketch of a string: its first kSketchWindow bytes set one bit of a
// 64-bit mask per 4-gram (hashed into 64 bins). popc(sketch(x) ^ sketch(y))
// counts the bins present in one string and not the other: each edit changes
// at most 4 grams of each string, so near-identical strings score low and
// unrelated ones high. A few register operations per byte, no shared memory.
constexpr int kSketchWindow = 64;

__device__ __forceinline__ uint64_t gram_sketch(const uint8_t *p, int m) {
    if (m > kSketchWindow) m = kSketchWindow;
    uint64_t sk = 0;
    uint32_t g = 0;
    TextScan ts;
    ts.init(p);
    for (int i = 0; i < m; i += 4) {
        const uint32_t w4 = ts.next4();
#pragma unroll
        for (int b = 0; b < 4; b++) {
            if (i + b < m) {
                g = __funnelshift_l(w4 << (24 - 8 * b), g, 8);     // g = (g << 8) | byte b
                if (i + b >= 3) sk |= 1ull << ((g * 0x9E3779B1u) >> 26);
            }
        }
    }
    return sk;
}

// 4-gram counts of a string, binned: its 4-grams hashed into 16 bins (the
// top 4 bits of gram_sketch's hash), one saturating byte counter per bin. An
// edit removes at most 4 grams of a string and adds at most 4, so it changes
// the sum over bins of |count(x) - count(y)| by at most 8: for any x, y,
// gram_bound(x, y) = that sum / 8 <= d(x, y) (q-gram lemma, q = 4; merging
// grams into bins and saturating counters only lower the sum). It is the
// scheduler network's similarity feature, and an exact filter: a pair whose
// bound exceeds max_dist has distance > max_dist.
__device__ __forceinline__ uint4 gram_counts(const uint8_t *p, int m) {
    // plain byte adds into l0..l3 (a byte cannot pass 255 within 252 grams),
    // folded into the saturating totals c0..c3 every 252 bytes and at the end
    uint32_t c0 = 0, c1 = 0, c2 = 0, c3 = 0, l0 = 0, l1 = 0, l2 = 0, l3 = 0;
    uint32_t g = 0;
    TextScan ts;
    ts.init(p);
    for (int i = 0; i < m; i += 4) {
        const uint32_t w4 = ts.next4();
#pragma unroll
        for (int b = 0; b < 4; b++) {
            if (i + b < m) {
                g = __funnelshift_l(w4 << (24 - 8 * b), g, 8);     // g = (g << 8) | byte b
                if (i + b >= 3) {
                    const uint32_t h = (g * 0x9E3779B1u) >> 28;    // bin 0..15
                    const uint32_t add = 1u << (8 * (h & 3u)), word = h >> 2;
                    l0 += word == 0 ? add : 0u;
                    l1 += word == 1 ? add : 0u;
                    l2 += word == 2 ? add : 0u;
                    l3 += word == 3 ? add : 0u;
                }
            }
        }
        if (i % 252 == 248) {
            c0 = __vaddus4(c0, l0); c1 = __vaddus4(c1, l1); c2 = __vaddus4(c2, l2); c3 = __vaddus4(c3, l3);
            l0 = l1 = l2 = l3 = 0;
        }
    }
    return make_uint4(__vaddus4(c0, l0), __vaddus4(c1, l1), __vaddus4(c2, l2), __vaddus4(c3, l3));
}

// Sum over the 16 bins of |count(x) - count(y)| (8 x gram_bound).
__device__ __forceinline__ uint32_t gram_dist(uint4 a, uint4 b) {
    return __vsadu4(a.x, b.x) + __vsadu4(a.y, b.y) + __vsadu4(a.z, b.z) + __vsadu4(a.w, b.w);
}

// -------------------------------- thresholded search: filter and band solve --
// The survivors of a query (choices within max_dist k <= 31 of its length, a
// contiguous range of the length-sorted choices) go through the 4-gram count
// bound, and the ones it does not rule out through the banded loop, one lane
// per survivor. Their costs differ by two orders of magnitude: most leave
// the band within 2k + 2 columns, near-copies of the query run the whole
// text. So warps run without CTA barriers and their lanes advance in rounds
// of R columns (a tuned launch shape: 8, 16 or 32); between rounds the warp
// hands the passers it has
// found to the lanes whose survivor finished, scanning further survivors
// (128 per step, four independent count loads per lane) while lanes are
// free. The window bits come from the query's Peq table in global memory
// (L1-resident while a warp works on the query). Results <= k are stored
// (the output holds k+1 already).
constexpr int kSurvPend = 128;         // passers one scan step can buffer

// One query's survivor range, read by all lanes of a warp (kept in shared
// memory: warp-uniform values that would otherwise take registers).
struct SurvJob {
    DevStrings CS;                     // the problem's length-sorted choices
    const int32_t *perm;               // sorted -> original choice index
    const uint4 *ccnt;                 // binned 4-gram counts of the sorted choices
    const uint64_t *peq;               // the query's Peq table [256][nw]
    void *out;
    int64_t row, nc;                   // the query's output row, row length
    int64_t s, s1;                     // next and end survivor (sorted choice index)
    uint4 qc;                          // the query's binned 4-gram counts
    int m, nw, k, dtype;
};

// largest j in [0, n) with pre[j] <= x (pre non-decreasing, pre[0] <= x)
__device__ __forceinline__ int upper_index(const int64_t *pre, int n, int64_t x) {
    int a = 0, b = n;
    while (b - a > 1) {
        const int mid = (a + b) >> 1;
        if (pre[mid] <= x) a = mid; else b = mid;
    }
    return a;
}

// ---- deferred results and the output fill as work items
// A survivor kernel that also fills its output with k+1 (fill items taken
// between survivor jobs, so the HBM-bound fill overlaps the latency-bound
// search) cannot store results in place: a fill item may reach an element
// after its result. Its results <= k go to a list instead, one 64-bit entry
// each (element address << 8 | dtype << 6 | value; value <= 63), and a
// scatter kernel stores them after the kernel (ResultList). A list that ran
// full (count > cap) is seen on the device: the search then runs again in
// place. Fill work is FillItems: arrays cut into kFillChunk-byte items.
__device__ __forceinline__ void list_emit(const ResultList &L, void *out, int dtype, int64_t idx, int d) {
    const int es = dtype == DT_UINT8 ? 1 : dtype == DT_UINT16 ? 2 : 4;
    const unsigned long long a = (unsigned long long)reinterpret_cast<uintptr_t>(out) + (unsigned long long)(idx * es);
    const unsigned long long at = atomicAdd(L.count, 1ull);
    if (at < L.cap) L.item[at] = (a << 8) | ((unsigned long long)dtype << 6) | (unsigned long long)d;
}

// out[0..n) = v (dtype-sized) by this thread's share (tid of stride): 16-byte
// stores for the aligned middle, element stores for the ends (out is
// element-aligned, so the unaligned head is whole elements).
__device__ __forceinline__ void fill_share(void *out, int64_t n, int dtype, uint32_t v, int64_t tid,
                                           int64_t stride) {
    const int es = dtype == DT_UINT8 ? 1 : dtype == DT_UINT16 ? 2 : 4;
    uint32_t word = v;
    if (es == 1) word = v * 0x01010101u;
    else if (es == 2) word = v | (v << 16);
    const int64_t bytes = n * es;
    uint8_t *b = reinterpret_cast<uint8_t *>(out);
    const int64_t head = (16 - (reinterpret_cast<uintptr_t>(b) & 15)) & 15;
    const int64_t nvec = bytes > head ? (bytes - head) / 16 : 0;
    uint4 *vp = reinterpret_cast<uint4 *>(b + head);
    const uint4 vv = make_uint4(word, word, word, word);
    for (int64_t i = tid; i < nvec; i += stride) __stcs(vp + i, vv);   // streaming: no L2 residency wanted
    const int64_t tail0 = head + nvec * 16;
    for (int64_t r = tid * es; r < head + (bytes - tail0); r += stride * es) {
        const int64_t x = r < head ? r : tail0 + (r - head);
        if (x >= bytes) break;
        if (es == 1) b[x] = (uint8_t)v;
        else if (es == 2) *reinterpret_cast<uint16_t *>(b + x) = (uint16_t)v;
        else *reinterpret_cast<uint32_t *>(b + x) = v;
    }
}

// The warp claims one fill item and fills it (every lane calls it); false
// when every item was claimed.
__device__ __forceinline__ bool fill_one(const FillItems &F) {
    unsigned long long i = 0;
    if ((threadIdx.x & 31) == 0) i = atomicAdd(F.ctr, 1ull);
    i = __shfl_sync(kFull, i, 0);
    if ((int64_t)i >= F.total) return false;
    BatchFill f = F.one;
    int64_t li = (int64_t)i;
    if (F.fills) {
        const int a = upper_index(F.start, F.nfill, li);
        f = F.fills[a];
        li -= F.start[a];
    }
    const int es = f.dtype == DT_UINT8 ? 1 : f.dtype == DT_UINT16 ? 2 : 4;
    const int64_t per = kFillChunk / es, e0 = li * per, e1 = min(f.n, e0 + per);
    fill_share(reinterpret_cast<uint8_t *>(f.out) + e0 * es, e1 - e0, f.dtype, f.value, threadIdx.x & 31, 32);
    return true;
}

// Called by every lane of a warp. next_job(J) fills the warp's job (every
// lane calls it; lane 0 writes J) and returns false when none is left.
// s_pend: the warp's kSurvPend passer slots (sorted choice index), s_pgd
// their 4-gram count distances. log(sidx, m, n, cols, gd) sees every
// survivor the banded loop finished; emit(out, dtype, index, d) takes every
// result <= k (a store in place, or list_emit).
template <int R, typename NextJob, typename LogFn, typename Emit>
__device__ __forceinline__ void survivor_warp(SurvJob &J, NextJob next_job, int32_t *s_pend, uint16_t *s_pgd,
                                              uint32_t *status, LogFn log, Emit emit) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    bool have_job = false, jobs_done = false;
    int pend = 0;                                          // warp-uniform
    // this lane's survivor
    bool busy = false;
    TextScan ts{};
    uint32_t w4 = 0;
    const uint64_t *peq = nullptr;
    void *out = nullptr;
    int64_t oidx = 0;
    int n = 0, m = 0, nw = 1, k = 0, dtype = 0, sidx = 0;
    uint32_t gd = 0;
    BandGeom bg{};
    BandState bs{};
    while (true) {
        unsigned freem = __ballot_sync(kFull, !busy);
        while (freem) {
            if (pend == 0) {
                if (!have_job || J.s >= J.s1) {
                    if (jobs_done) break;
                    have_job = next_job(J);
                    __syncwarp();
                    if (!have_job) {
                        jobs_done = true;
                        break;
                    }
                    if (J.m == 0) {                        // empty query: d = n for every survivor
                        for (int64_t x = J.s + lane; x < J.s1; x += 32) {
                            int nn;
                            string_at(J.CS, x, nn, status);
                            emit(J.out, J.dtype, J.row * J.nc + J.perm[x], cap_k(nn, J.k));
                        }
                        __syncwarp();
                        if (lane == 0) J.s = J.s1;
                        __syncwarp();
                        continue;
                    }
                }
                // scan 128 survivors: four independent count loads per lane
                const int64_t base = J.s, s1 = J.s1;
                const uint4 qc = J.qc;
                const uint32_t gmax = 8u * (uint32_t)J.k;
                uint4 c[4];
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const int64_t x = base + i * 32 + lane;
                    c[i] = x < s1 ? __ldg(J.ccnt + x) : make_uint4(0, 0, 0, 0);
                }
                uint32_t g[4];
#pragma unroll
                for (int i = 0; i < 4; i++) g[i] = base + i * 32 + lane < s1 ? gram_dist(qc, c[i]) : 0xffffffffu;
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const bool pass = g[i] <= gmax;        // else the bound alone proves d > k
                    const unsigned pm = __ballot_sync(kFull, pass);
                    if (pass) {
                        const int at = pend + __popc(pm & lt);
                        s_pend[at] = (int32_t)(base + i * 32 + lane);
                        s_pgd[at] = (uint16_t)g[i];
                    }
                    pend += __popc(pm);
                }
                __syncwarp();
                if (lane == 0) J.s = base + 4 * 32;
                __syncwarp();
                continue;
            }
            // hand buffered passers to free lanes, from the end of the buffer
            const int take = min(pend, __popc(freem));
            const int r = __popc(freem & lt);
            if (!busy && r < take) {
                const int e = pend - take + r;
                sidx = s_pend[e];
                gd = s_pgd[e];
                const uint8_t *t = string_at(J.CS, sidx, n, status);
                m = J.m;
                k = J.k;
                dtype = J.dtype;
                out = J.out;
                peq = J.peq;
                nw = J.nw;
                oidx = J.row * J.nc + J.perm[sidx];
                if ((n > m ? n - m : m - n) > k) {
                    // outside the length window: the output keeps its k+1
                } else {
                    bg = band_geom(m, n, k);
                    bs = band_start(bg);
                    ts.init(t);
                    w4 = 0;
                    busy = true;
                }
            }
            pend -= take;
            __syncwarp();
            freem = __ballot_sync(kFull, !busy);
        }
        if (!__any_sync(kFull, busy)) {
            if (jobs_done && pend == 0) break;
            continue;
        }
        if (busy) {
            auto text = [&](int j) -> uint32_t {
                if ((j & 3) == 0) w4 = ts.next4();
                const uint32_t c = w4 & 0xffu;
                w4 >>= 8;
                return c;
            };
            const uint64_t *pq = peq;
            const int nwl = nw;
            auto eqw = [&](uint32_t c, int p0) { return peq_window(pq + c * nwl, nwl, p0); };
            const bool exited = band_steps(k, bg, bs, min(n, bs.j + R), text, eqw);
            if (exited || bs.j == n) {
                const int d = exited ? k + 1 : band_finish(k, bg, bs);
                if (d <= k) emit(out, dtype, oidx, d);
                log((int64_t)sidx, m, n, bs.j, gd);
                busy = false;
            }
        }
    }
}

}  // namespace blg
