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
// untrimmed): lengths, trimmed lengths, length gap, k, and the 4-gram sketch
// distance of their first 64 trimmed bytes (gram_sketch, blg_kernels.cuh).

template <bool HASK, bool FEAT>
__global__ void __launch_bounds__(256) k_pairs_prep(DevStrings A, DevStrings B, int k, int dtype, void *out,
                                                    PairsPlan plan, int band, uint32_t *status) {
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
        // the banded loop costs columns plus a window fill, the word solvers columns x words
        int key = cost_bucket(band ? (float)lb + 16.f : (float)lb * (float)((la + 63) >> 6));
        if (FEAT) {
            const float qb = (float)__popcll(gram_sketch(a, la) ^ gram_sketch(b, lb));
            half *f = plan.feat[cls] + (size_t)pos * kFeatures;
            f[0] = __float2half((float)la * (1.f / 256.f));
            f[1] = __float2half((float)lb * (1.f / 256.f));
            f[2] = __float2half((float)la0 * (1.f / 256.f));
            f[3] = __float2half((float)lb0 * (1.f / 256.f));
            f[4] = __float2half((float)(lb - la) * (1.f / 16.f));
            f[5] = __float2half(qb * (1.f / 16.f));
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
// loop, one thread per record. The window's match bits come from a 32-slot
// ring per thread: rows 0..15 / 16..31 of a [row][thread] u32 table hold,
// for each high / low nibble value, the ring slots whose pattern byte has
// it; slot (p & 31) holds pattern position p. Each column the position
// leaving the window top and the one entering at its bottom share a slot:
// the leaving byte (kept in a per-thread byte ring) is cleared, the entering
// one set, and the slot order is rotated into window order. Both tables are
// laid out [row or slot][thread], so every access is bank-conflict free.
template <bool LOG>
__global__ void __launch_bounds__(256) k_solve_band(PairsPlan plan, int k, int dtype, void *out,
                                                    int32_t *exit_log, uint32_t unit) {
    __shared__ uint32_t s_tab[32 * 256];
    __shared__ uint8_t s_ring[256 * 32];
    const Units u{unit, unit + unit};
    uint32_t *tc = s_tab + threadIdx.x;                     // row r at tc[r * 256]
    uint8_t *ring = s_ring + threadIdx.x;                  // slot q at ring[q * 256] (conflict-free)
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
            const uint8_t *pat = it.pat;
            int d, cols = 0;
            if (n - m > k || m - n > k) d = k + 1;
            else {
                const BandGeom bg = band_geom(m, n, k);
#pragma unroll
                for (int r = 0; r < 32; r++) tc[r * 256] = 0;
                // window of column 1 holds positions -dhi .. 30 - dhi; real ones first
                {
                    const int fill = min(31 - bg.dhi, m);
                    TextScan fs;
                    fs.init(pat);
                    uint32_t f4 = 0;
                    for (int p = 0; p < fill; p++) {
                        if ((p & 3) == 0) f4 = fs.next4();
                        const uint32_t c = f4 & 0xffu, bit = 1u << p;
                        f4 >>= 8;
                        tc[(c >> 4) * 256] |= bit;
                        tc[(16 + (c & 15)) * 256] |= bit;
                        ring[p * 256] = (uint8_t)c;
                    }
                }
                // entering positions p0 + 31 = 31 - dhi + j advance one per column:
                // a 4-byte cursor keeps the pattern loads off the column chain
                const int pin0 = 31 - bg.dhi;
                TextScan ps;
                if (pin0 < m) ps.init(pat + pin0);
                uint32_t pw = 0;
                auto eqw = [&](uint32_t c, int p0) -> uint32_t {
                    const int pin = p0 + 31, pout = p0 - 1;   // same ring slot
                    const uint32_t slot = (uint32_t)pin & 31u, bit = 1u << slot;
                    // match bits from the table before this column's update; window
                    // bit 31 (the entering position) from a register compare instead
                    const uint32_t x = tc[(c >> 4) * 256] & tc[(16 + (c & 15)) * 256];
                    uint32_t eq = __funnelshift_r(x, x, (uint32_t)(p0 & 31)) & 0x7fffffffu;
                    if (pin < m) {
                        if (((pin - pin0) & 3) == 0) pw = ps.next4();
                        const uint32_t cn = pw & 0xffu;
                        pw >>= 8;
                        if (cn == c) eq |= 0x80000000u;
                        if (pout >= 0) {
                            const uint32_t co = ring[slot * 256];
                            tc[(co >> 4) * 256] &= ~bit;
                            tc[(16 + (co & 15)) * 256] &= ~bit;
                        }
                        tc[(cn >> 4) * 256] |= bit;
                        tc[(16 + (cn & 15)) * 256] |= bit;
                        ring[slot * 256] = (uint8_t)cn;
                    } else if (pout >= 0 && pout < m) {
                        const uint32_t co = ring[slot * 256];
                        tc[(co >> 4) * 256] &= ~bit;
                        tc[(16 + (co & 15)) * 256] &= ~bit;
                    }
                    return eq;
                };
                d = band_distance(m, it.txt, n, k, eqw, u, LOG ? &cols : nullptr);
            }
            store1(out, dtype, it.idx, d);
            if (LOG) exit_log[it.idx] = cols;
        }
    }
}

// ------------------------------------------------------------- launchers --
cudaError_t launch_pairs_prep(cudaStream_t st, int grid, bool hask, bool feat, bool band, const DevStrings &A,
                              const DevStrings &B, int k, int dtype, void *out, const PairsPlan &plan,
                              uint32_t *status) {
    const int bd = band ? 1 : 0;
    if (hask) {
        if (feat) k_pairs_prep<true, true><<<grid, 256, 0, st>>>(A, B, k, dtype, out, plan, bd, status);
        else k_pairs_prep<true, false><<<grid, 256, 0, st>>>(A, B, k, dtype, out, plan, bd, status);
    } else {
        if (feat) k_pairs_prep<false, true><<<grid, 256, 0, st>>>(A, B, k, dtype, out, plan, bd, status);
        else k_pairs_prep<false, false><<<grid, 256, 0, st>>>(A, B, k, dtype, out, plan, bd, status);
    }
    return cudaGetLastError();
}

cudaError_t launch_order(cudaStream_t st, int sms, const PairsPlan &plan) {
    k_order_segments<<<sms * 2, kSegRecords, 0, st>>>(plan);
    return cudaGetLastError();
}

cudaError_t launch_solve_band(cudaStream_t st, int sms, int ctas_per_sm, const PairsPlan &plan, int k, int dtype,
                              void *out, int32_t *exit_log) {
    // 40 KB of ring tables per CTA: at most five CTAs per SM
    const int grid = sms * (ctas_per_sm < 1 ? 1 : (ctas_per_sm > 5 ? 5 : ctas_per_sm));
    if (exit_log) k_solve_band<true><<<grid, 256, 0, st>>>(plan, k, dtype, out, exit_log, 1u);
    else k_solve_band<false><<<grid, 256, 0, st>>>(plan, k, dtype, out, nullptr, 1u);
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
