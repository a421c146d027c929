// Scheduled pairwise path: prep -> order -> solve.
//
// One thread per pair in natural order (the reference's schedule,
// csrc/gpu_kernels.cu:6-32) leaves most lanes of a warp idle: after exact
// trimming the remaining work of neighbouring pairs differs by an order of
// magnitude (trimmed lengths, max_dist exits). Here
//   1. k_pairs_prep trims every pair, finishes the trivial ones (length gap
//      beyond k, empty pattern) and writes the rest as 32-byte work records
//      into per-class regions (class 0: pattern <= 64, one thread; classes
//      1..5: 2..32 lanes), each with a cost key and, for the learned
//      schedule, a feature row;
//   2. k_order_segments counting-sorts every 1024-record segment of a class
//      by cost key, largest cost first: warps get pairs of similar cost
//      while their strings stay in one neighbourhood of memory (a sort over
//      the whole class scatters them, and the solvers' per-lane string
//      reads lose more to cache misses than the order saves);
//   3. k_solve_word / k_solve_lanes consume the sorted records from device
//      work counters, so a warp takes pairs of similar cost.
// Which pairs are computed and their values never change: only the order.
#include <algorithm>

#include "blg_kernels.cuh"
#include "blg_sched.h"

namespace blg {

// Cost bucket of an estimated work amount (columns x words), log-spaced so
// 256 buckets cover 1 .. 2^32.
__device__ __forceinline__ int cost_bucket(float work) {
    if (work < 1.f) return 0;
    const int b = (int)(__log2f(work) * 8.f) + 1;
    return b > kCostBuckets - 1 ? kCostBuckets - 1 : b;
}

// Features of one trimmed pair (pattern p of m, text t of n; la0, lb0
// untrimmed): lengths, trimmed lengths, length gap, k, and a 4-gram count
// lower bound from the first kSketchWindow (64) trimmed bytes of each string:
// with A, B those prefixes, d(A, B) <= 2 d(a, b) (an optimal alignment of a
// and b aligns A with some prefix B' of b at cost <= d, and |B'| differs from
// |B| by at most d), and gram_dist(A, B) / 8 <= d(A, B), so gram_dist / 16 <=
// d(a, b). The window keeps the count pass short (whole strings cost the
// learned pipeline more than its order gains).

template <bool HASK, bool FEAT>
__global__ void __launch_bounds__(256) k_pairs_prep(DevStrings A, DevStrings B, int k, int dtype, void *out,
                                                    PairsPlan plan, int band, int lengap_key, uint32_t *status) {
    const int lane = threadIdx.x & 31;
    const int64_t n = A.n;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    // whole warps iterate together so the slot claim below can be warp-aggregated
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < n; base += stride) {
        const int64_t i = base + lane;
        int cls = -1, la = 0, lb = 0, la0 = 0, lb0 = 0;
        const uint8_t *a = nullptr, *b = nullptr;
        if (i < n) {
            a = string_at(A, i, la, status);
            b = string_at(B, i, lb, status);
            la0 = la;
            lb0 = lb;
            trim_windows(a, la, b, lb);
            if (la > lb) {
                const uint8_t *t = a; a = b; b = t;
                const int x = la; la = lb; lb = x;
            }
            const int W = (la + 63) >> 6;
            if (HASK && lb - la > k) store1(out, dtype, i, k + 1);          // length gap alone exceeds k
            else if (la == 0) store1(out, dtype, i, lb);
            else if (W > 32) { atomicOr(status, ST_TOO_LONG); store1(out, dtype, i, -1); }
            else cls = W <= 1 ? 0 : W <= 2 ? 1 : W <= 4 ? 2 : W <= 8 ? 3 : W <= 16 ? 4 : 5;
        }
        // claim record slots: one atomic per class present in the warp
        const unsigned peers = __match_any_sync(kFull, cls);
        const int leader = __ffs(peers) - 1;
        int pos = 0;
        if (cls >= 0 && lane == leader) pos = atomicAdd(&plan.count[cls], __popc(peers));
        pos = __shfl_sync(kFull, pos, leader) + __popc(peers & ((1u << lane) - 1));
        if (cls < 0) continue;
        if (pos >= plan.cap[cls]) { atomicOr(status, ST_QUEUE_OVERFLOW); store1(out, dtype, i, -1); continue; }
        LongItem it;
        it.pat = a; it.txt = b; it.m = la; it.n = lb; it.idx = i;
        plan.raw[cls][pos] = it;
        // the banded loop costs columns plus a window fill, the word solvers
        // columns x words; the length-difference order (an ablation) puts
        // equal lengths first
        int key = lengap_key ? 255 - min(255, 8 * (lb - la))
                             : cost_bucket(band ? (float)lb + 16.f : (float)lb * (float)((la + 63) >> 6));
        if (FEAT) {
            const float gd = (float)gram_dist(gram_counts(a, min(la, kSketchWindow)), gram_counts(b, min(lb, kSketchWindow)));
            half *f = plan.feat[cls] + (size_t)pos * kFeatures;
            f[0] = __float2half((float)la * (1.f / 256.f));
            f[1] = __float2half((float)lb * (1.f / 256.f));
            f[2] = __float2half((float)la0 * (1.f / 256.f));
            f[3] = __float2half((float)lb0 * (1.f / 256.f));
            f[4] = __float2half((float)(lb - la) * (1.f / 16.f));
            f[5] = __float2half(gd * (1.f / 256.f));   // the windowed lower bound gd / 16, over 16
            f[6] = __float2half(HASK ? (float)k * (1.f / 16.f) : 16.f);
            key = 0;                       // the network's prediction sets the key later
        }
        plan.key[cls][pos] = (uint8_t)key;
    }
}

// Segmented counting sort: every segment of kSegRecords consecutive records
// of a class is sorted by key, largest first, into the same index range of
// plan.sorted. A persistent grid walks (class, segment) pairs; one CTA owns
// a segment (shared-memory histogram, scan, scatter; order inside a key is
// free).
constexpr int kSegRecords = 1024;

__global__ void __launch_bounds__(kSegRecords) k_order_segments(PairsPlan plan) {
    __shared__ int s_cnt[kCostBuckets];
    __shared__ int s_start[kCostBuckets];
    const int t = threadIdx.x;
    for (int cls = 0; cls < kPairClasses; cls++) {
        const int cnt = min(plan.count[cls], (int)plan.cap[cls]);
        const int nseg = (cnt + kSegRecords - 1) / kSegRecords;
        for (int seg = blockIdx.x; seg < nseg; seg += gridDim.x) {
            const int base = seg * kSegRecords, i = base + t;
            if (t < kCostBuckets) s_cnt[t] = 0;
            __syncthreads();
            const int key = i < cnt ? plan.key[cls][i] : -1;
            const int rank = key >= 0 ? atomicAdd(&s_cnt[key], 1) : 0;
            __syncthreads();
            // exclusive scan over keys in descending order (one warp of 8 keys per lane)
            if (t < 32) {
                int v[8], sum = 0;
#pragma unroll
                for (int q = 0; q < 8; q++) { v[q] = s_cnt[kCostBuckets - 1 - (t * 8 + q)]; sum += v[q]; }
                int incl = sum;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int x = __shfl_up_sync(kFull, incl, o);
                    if (t >= o) incl += x;
                }
                int run = incl - sum;
#pragma unroll
                for (int q = 0; q < 8; q++) { s_start[kCostBuckets - 1 - (t * 8 + q)] = run; run += v[q]; }
            }
            __syncthreads();
            if (key >= 0) plan.sorted[cls][base + s_start[key] + rank] = plan.raw[cls][i];
            __syncthreads();
        }
    }
}

// Class 0: one thread per record (pattern <= 64), records in sorted order.
template <bool HASK>
__global__ void __launch_bounds__(256) k_solve_word(PairsPlan plan, int k, int dtype, void *out,
                                                    int32_t *exit_log) {
    extern __shared__ uint64_t s_tab[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t *tc = s_tab + warp * 1024 + lane;
#pragma unroll
    for (int r = 0; r < 32; r++) tc[r * 32] = 0;
    const int cnt = min(plan.count[0], (int)plan.cap[0]);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
        const LongItem it = plan.sorted[0][i];
        int cols = 0;
        const int d = solve_word<HASK>(tc, it.pat, it.m, it.txt, it.n, k, exit_log ? &cols : nullptr);
        store1(out, dtype, it.idx, d);
        if (exit_log) exit_log[it.idx] = cols;
    }
}

// Classes 1..5: lane-spread, pulling 32/L records at a time from the class's counter.
template <bool HASK>
__global__ void __launch_bounds__(256) k_solve_lanes(PairsPlan plan, int k, int dtype, void *out,
                                                     int32_t *exit_log) {
    extern __shared__ uint64_t s_tab[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t *tc = s_tab + warp * 1024 + lane;
#pragma unroll
    for (int r = 0; r < 32; r++) tc[r * 32] = 0;
    for (int cls = 1; cls < kPairClasses; cls++) {
        const int L = 1 << cls, G = 32 / L, g = lane / L, w = lane & (L - 1);
        const int count = min(plan.count[cls], (int)plan.cap[cls]);
        if (count == 0) continue;
        while (true) {
            int base = 0;
            if (lane == 0) base = atomicAdd(&plan.head[cls], G);
            base = __shfl_sync(kFull, base, 0);
            if (base >= count) break;
            const int it_i = base + g;
            const bool valid = it_i < count;
            LongItem it;
            if (valid) it = plan.sorted[cls][it_i];
            else { it.pat = nullptr; it.txt = nullptr; it.m = 0; it.n = 0; it.idx = 0; }
            const bool own = valid && w < ((it.m + 63) >> 6);
            const uint8_t *pw = own ? it.pat + 64 * w : nullptr;
            const int plen = own ? min(64, it.m - 64 * w) : 0;
            if (own) nib_build(tc, pw, plen);
            bool is_last = false;
            int cols = 0;
            const int d = lane_wavefront<HASK>(valid, it.m, it.txt, it.n, L, w, g, k,
                                               [&](uint32_t ch) { return nib_eq(tc, ch); }, is_last,
                                               exit_log ? &cols : nullptr);
            if (own) nib_clear(tc, pw, plen);
            if (is_last) {
                store1(out, dtype, it.idx, d);
                if (exit_log) exit_log[it.idx] = cols;
            }
        }
    }
}

// max_dist <= 31: every record (any pattern length) solved by the banded
// loop, one thread per record. The window's match bits come from per-thread
// rows over a 64-position block of the pattern (bit i <-> position
// 32b - dhi + i in block b), in a [row][thread] table (every access
// bank-conflict free). Columns 32b .. 32b+31 read their 32-bit windows out
// of the same block with one funnel shift, so within a block the table is
// read-only and the match loads stay off the column chain; every 32 columns
// the rows shift down by 32 positions and the next 32 pattern bytes are
// entered. Two row layouts:
//   SYM = false: nibble rows, 0..15 / 16..31 for each high / low nibble
//     value; Eq(c) = row[c >> 4] & row[16 + (c & 15)], any byte alphabet,
//     two row updates per pattern byte, 64 KB per CTA (3 CTAs per SM);
//   SYM = true: when the pair set uses at most 15 distinct bytes, one row
//     per byte (rank of the byte among the set's bytes; the bytes outside
//     the set share row 15, which stays empty): one update per pattern
//     byte, one row load per column, and 32 KB per CTA, so twice the warps
//     per SM hide the latency of the lanes' string loads (the kernel's
//     stall: each lane walks its own strings).
// alpha: the set's bytes (8 words), or null when the host has chosen the
// variant; given, each variant checks it and the one that does not apply
// returns at once (one launch of each, no host round trip).
constexpr int kBandThreads = 256;
constexpr int kSymRows = kBandSymbols + 1;           // the last row stays empty

template <bool LOG, bool SYM>
__global__ void __launch_bounds__(kBandThreads) k_solve_band(PairsPlan plan, int k, int dtype, void *out,
                                                             int32_t *exit_log, const uint32_t *alpha) {
    extern __shared__ uint2 s_rows2[];                      // [rows][kBandThreads] 64-bit rows
    __shared__ uint8_t s_map[256];                          // byte -> row (SYM)
    if (alpha && (alpha_size(alpha) <= kBandSymbols) != SYM) return;   // uniform: the other variant runs the set
    if (SYM) alpha_map(alpha, s_map);
    uint2 *tc = s_rows2 + threadIdx.x;                      // row r at tc[r * kBandThreads]
    const int lane = threadIdx.x & 31;
    for (int cls = kPairClasses - 1; cls >= 0; cls--) {
        const int count = min(plan.count[cls], (int)plan.cap[cls]);
        while (true) {
            int base = 0;
            if (lane == 0) base = atomicAdd(&plan.head[cls], 32);
            base = __shfl_sync(kFull, base, 0);
            if (base >= count) break;
            const int ri = base + lane;
            if (ri >= count) continue;
            const LongItem it = plan.sorted[cls][ri];
            const int m = it.m, n = it.n;
            int d, cols = 0;
            if (n - m > k || m - n > k) {
                d = k + 1;
            } else {
                auto at = [](const uint8_t *base) {
                    return [base](int pos) {
                        TextScan s;
                        s.init(base + pos);
                        return s;
                    };
                };
                d = band_rows_distance<SYM, kBandThreads>(tc, s_map, at(it.pat), at(it.txt), m, n, k,
                                                          LOG ? &cols : nullptr);
            }
            store1(out, dtype, it.idx, d);
            if (LOG) exit_log[it.idx] = cols;
        }
    }
}

// Bytes present in the strings of A and B (each over its own offset range):
// 16-byte aligned loads, a block-wide bitmap in shared memory set at a
// byte's first sighting in the block, OR-ed into `mask` (8 words, zero
// before the launch).
__device__ __forceinline__ void presence_scan(const DevStrings &S, uint32_t *s_m) {
    if (S.n <= 0) return;
    int64_t lo = S.off[0] - S.base, hi = S.off[S.n] - S.base;
    lo = lo < 0 ? 0 : (lo > S.bytes ? S.bytes : lo);
    hi = hi < lo ? lo : (hi > S.bytes ? S.bytes : hi);
    const int64_t a0 = lo & ~int64_t(15);
    const uint4 *v = reinterpret_cast<const uint4 *>(S.buf + a0);   // buf is 16-byte aligned, 16 bytes of slack
    const int64_t nv = (hi - a0 + 15) >> 4;
    for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < nv; x += (int64_t)gridDim.x * blockDim.x) {
        const uint4 q = __ldg(v + x);
        const uint32_t w[4] = {q.x, q.y, q.z, q.w};
        const int64_t p0 = a0 + 16 * x;
#pragma unroll
        for (int i = 0; i < 16; i++) {
            const int64_t p = p0 + i;
            if (p < lo || p >= hi) continue;
            const uint32_t c = (w[i >> 2] >> (8 * (i & 3))) & 0xffu, bit = 1u << (c & 31);
            if (!(s_m[c >> 5] & bit)) atomicOr(&s_m[c >> 5], bit);
        }
    }
}

__global__ void __launch_bounds__(256) k_byte_presence(DevStrings A, DevStrings B, uint32_t *mask) {
    __shared__ uint32_t s_m[8];
    if (threadIdx.x < 8) s_m[threadIdx.x] = 0;
    __syncthreads();
    presence_scan(A, s_m);
    presence_scan(B, s_m);
    __syncthreads();
    if (threadIdx.x < 8 && s_m[threadIdx.x]) atomicOr(mask + threadIdx.x, s_m[threadIdx.x]);
}

// ------------------------------------------------------------- launchers --
cudaError_t launch_pairs_prep(cudaStream_t st, int grid, bool hask, bool feat, bool band, const DevStrings &A,
                              const DevStrings &B, int k, int dtype, void *out, const PairsPlan &plan,
                              bool lengap_key, uint32_t *status) {
    const int bd = band ? 1 : 0, lg = lengap_key ? 1 : 0;
    if (hask) {
        if (feat) k_pairs_prep<true, true><<<grid, 256, 0, st>>>(A, B, k, dtype, out, plan, bd, lg, status);
        else k_pairs_prep<true, false><<<grid, 256, 0, st>>>(A, B, k, dtype, out, plan, bd, lg, status);
    } else {
        if (feat) k_pairs_prep<false, true><<<grid, 256, 0, st>>>(A, B, k, dtype, out, plan, bd, lg, status);
        else k_pairs_prep<false, false><<<grid, 256, 0, st>>>(A, B, k, dtype, out, plan, bd, lg, status);
    }
    return cudaGetLastError();
}

cudaError_t launch_order(cudaStream_t st, int sms, const PairsPlan &plan) {
    k_order_segments<<<sms * 2, kSegRecords, 0, st>>>(plan);
    return cudaGetLastError();
}

template <bool LOG, bool SYM>
static cudaError_t launch_band_v(cudaStream_t st, int sms, int ctas_per_sm, const PairsPlan &plan, int k, int dtype,
                                 void *out, int32_t *exit_log, const uint32_t *alpha) {
    const size_t smem = sizeof(uint2) * (SYM ? kSymRows : 32) * kBandThreads;
    cudaFuncSetAttribute(k_solve_band<LOG, SYM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = ctas_per_sm;
    if (SYM) {                                           // as many CTAs as fit: the point of the small rows
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_solve_band<LOG, SYM>, kBandThreads, smem) !=
                cudaSuccess || per_sm < 1)
            per_sm = 1;
    } else {                                             // 64 KB of nibble rows per CTA: at most three per SM
        per_sm = per_sm < 1 ? 1 : (per_sm > 3 ? 3 : per_sm);
    }
    k_solve_band<LOG, SYM><<<sms * per_sm, kBandThreads, smem, st>>>(plan, k, dtype, out, exit_log, alpha);
    return cudaGetLastError();
}

// variant: 1 = one row per byte (the set's alphabet fits; `alpha` its bytes),
// 0 = nibble rows, -1 = unknown: both launch and the alphabet in `alpha`
// (computed on the stream before) picks the one that runs.
cudaError_t launch_solve_band(cudaStream_t st, int sms, int ctas_per_sm, const PairsPlan &plan, int k, int dtype,
                              void *out, int32_t *exit_log, int variant, const uint32_t *alpha) {
    cudaError_t e = cudaSuccess;
    if (variant != 0) {
        e = exit_log ? launch_band_v<true, true>(st, sms, ctas_per_sm, plan, k, dtype, out, exit_log, alpha)
                     : launch_band_v<false, true>(st, sms, ctas_per_sm, plan, k, dtype, out, exit_log, alpha);
        if (e != cudaSuccess) return e;
    }
    if (variant != 1) {
        const uint32_t *a = variant < 0 ? alpha : nullptr;
        e = exit_log ? launch_band_v<true, false>(st, sms, ctas_per_sm, plan, k, dtype, out, exit_log, a)
                     : launch_band_v<false, false>(st, sms, ctas_per_sm, plan, k, dtype, out, exit_log, a);
    }
    return e;
}

cudaError_t launch_byte_presence(cudaStream_t st, int sms, const DevStrings &A, const DevStrings &B, uint32_t *mask) {
    const int64_t bytes = std::max<int64_t>(A.n > 0 ? 1 : 0, (A.bytes + B.bytes) / 16);
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((bytes + 255) / 256, (int64_t)sms * 8));
    k_byte_presence<<<grid, 256, 0, st>>>(A, B, mask);
    return cudaGetLastError();
}

cudaError_t launch_solve(cudaStream_t st, int sms, bool hask, const PairsPlan &plan, int k, int dtype,
                         void *out, int32_t *exit_log, bool any_long) {
    const size_t smem = 8 * 1024 * sizeof(uint64_t);
    if (hask) {
        cudaFuncSetAttribute(k_solve_word<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_solve_word<true><<<sms * 3 * 4, 256, smem, st>>>(plan, k, dtype, out, exit_log);
        if (any_long) {
            cudaFuncSetAttribute(k_solve_lanes<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            k_solve_lanes<true><<<sms * 3, 256, smem, st>>>(plan, k, dtype, out, exit_log);
        }
    } else {
        cudaFuncSetAttribute(k_solve_word<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_solve_word<false><<<sms * 3 * 4, 256, smem, st>>>(plan, k, dtype, out, exit_log);
        if (any_long) {
            cudaFuncSetAttribute(k_solve_lanes<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            k_solve_lanes<false><<<sms * 3, 256, smem, st>>>(plan, k, dtype, out, exit_log);
        }
    }
    return cudaGetLastError();
}

}  // namespace blg
