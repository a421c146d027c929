// Thresholded search: the survivor kernel for max_dist <= 31.
//
// With max_dist = k only (query, choice) pairs whose lengths differ by at
// most k need the column loop (csrc/myers.c:101-106); they are a contiguous
// range of the length-sorted choices per query (the "survivors"). A
// persistent grid of barrier-free warps pulls jobs of survivors of one query
// from one device counter over every query class of the run, filters them by
// the 4-gram count bound and solves the rest with the banded loop, lanes
// refilled between rounds of columns (survivor_warp). Unrelated pairs leave
// the band after a few columns and near-copies run the whole text; a lane
// whose survivor finished takes the next passer instead of waiting for its
// warp's longest one.
// Only results <= k are written. DEFER = false: the output was filled with
// k+1 before and results are stored in place; a launch given a list that
// ran full (L.count) re-runs the search only then, else returns at once.
// DEFER = true: the kernel fills the output itself, one fill item per job
// claimed (the rest once the jobs are gone), so the HBM-bound fill spreads
// over the latency-bound search, and its results go to the list for
// k_list_scatter (config 4: 0.37 ms per step against 0.41 with the fill
// kernel first; warp 0 of each CTA filling alone: 0.43).
#include <cuda_fp16.h>

#include <algorithm>

#include "blg_kernels.cuh"
#include "blg_sched.h"

namespace blg {

// sketch[i] = gram_sketch(string i), counts[i] = gram_counts(string i),
// one warp per string: lane l takes the 4-grams starting at l, l + 32, ...
// (one unaligned 4-byte read each, consecutive across the warp) and counts
// them in its own 16 byte counters (4 registers); every 255 steps, before a
// lane counter can wrap, and at the end the counters are folded into
// saturating totals, then summed over the warp: with plain adds when the
// string has fewer than 256 grams, else with saturating byte adds.
// The sketch bits are an OR over the warp. The values equal the per-thread
// functions' (the same grams, hash and saturation at 255).
__global__ void __launch_bounds__(256) k_sketch_strings(DevStrings S, uint64_t *sketch, uint4 *counts,
                                                        uint32_t *status) {
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < S.n; i += nwarps) {
        int n;
        const uint8_t *p = string_at(S, i, n, status);
        uint32_t sk_lo = 0, sk_hi = 0;
        uint32_t t[4] = {0, 0, 0, 0};                          // saturating totals, bins 4w .. 4w+3
        for (int c0 = 0; c0 + 3 < n; c0 += 32 * 255) {
            uint32_t c[4] = {0, 0, 0, 0};                      // this lane's counts of the chunk
            const int c1 = min(n - 3, c0 + 32 * 255);          // grams starting before c1
            for (int s = c0 + lane; s < c1; s += 32) {
                const uint32_t g = __byte_perm(load4(p + s), 0u, 0x0123);   // b[s] << 24 | .. | b[s+3]
                const uint32_t h = g * 0x9E3779B1u;
                const uint32_t bin = h >> 28, inc = 1u << (8 * (bin & 3));
#pragma unroll
                for (int w = 0; w < 4; w++) c[w] += (bin >> 2) == (uint32_t)w ? inc : 0u;
                if (s + 3 < kSketchWindow) {
                    const uint32_t bit = h >> 26;
                    if (bit < 32) sk_lo |= 1u << bit;
                    else sk_hi |= 1u << (bit - 32);
                }
            }
#pragma unroll
            for (int w = 0; w < 4; w++) t[w] = __vaddus4(t[w], c[w]);
        }
        if (n <= 256) {                // fewer than 256 grams: plain adds never carry into the next byte
#pragma unroll
            for (int w = 0; w < 4; w++) t[w] = __reduce_add_sync(kFull, t[w]);
        } else {
#pragma unroll
            for (int off = 16; off > 0; off >>= 1)
#pragma unroll
                for (int w = 0; w < 4; w++) t[w] = __vaddus4(t[w], __shfl_xor_sync(kFull, t[w], off));
        }
        sk_lo = __reduce_or_sync(kFull, sk_lo);
        sk_hi = __reduce_or_sync(kFull, sk_hi);
        if (lane == 0) {
            sketch[i] = ((uint64_t)sk_hi << 32) | sk_lo;
            counts[i] = make_uint4(t[0], t[1], t[2], t[3]);
        }
    }
}

// At most 64 registers (4 CTAs of 256 threads per SM, the largest tuned
// shape): left free, the fill and deferred-result paths took the kernel to
// 76, which fits only 3 CTAs per SM, so a 4-per-SM grid ran a quarter of
// its CTAs as a second wave (the cap costs at most 40 bytes of spills).
template <int R, bool LOG, bool DEFER>
__global__ void __launch_bounds__(256, 4) k_search_band(DevStrings CS, const int32_t *perm, const uint4 *ccnt,
                                                     const uint4 *qcnt, SurvClasses C, int jobsz,
                                                     int k, int dtype, void *out, int64_t nc, SurvRows rows,
                                                     ResultList L, FillItems F, uint32_t *status) {
    if (!DEFER && L.count && *L.count <= L.cap) return;   // the repair launch: the list held every result
    // raw shared bytes: no constructor runs on shared memory
    constexpr size_t kJobs = (sizeof(SurvClasses) + 15) & ~size_t(15);
    __shared__ __align__(16) unsigned char s_raw[kJobs + 8 * sizeof(SurvJob)];
    SurvClasses &s_cls = *reinterpret_cast<SurvClasses *>(s_raw);
    SurvJob *s_job = reinterpret_cast<SurvJob *>(s_raw + kJobs);
    __shared__ int32_t s_pend[8][kSurvPend];
    __shared__ uint16_t s_pgd[8][kSurvPend];
    if (threadIdx.x == 0) s_cls = C;
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int32_t *work = s_cls.work[0];                 // one counter for the launch
    bool fill_on = DEFER;                          // warp-uniform
    auto next_job = [&](SurvJob &J) -> bool {
        if (DEFER && fill_on) fill_on = fill_one(F);
        int job = 0;
        if (lane == 0) job = atomicAdd(work, 1);
        job = __shfl_sync(kFull, job, 0);
        int c = 0;
        int64_t first = 0;
        for (; c < s_cls.n; c++) {
            const int64_t t = s_cls.tile_start[c][s_cls.cls[c].nq];
            if (job < first + t) break;
            first += t;
        }
        if (c >= s_cls.n) {
            if (DEFER)
                while (fill_on) fill_on = fill_one(F);
            return false;
        }
        if (lane == 0) {
            const SearchClass &cl = s_cls.cls[c];
            const int64_t lj = job - first;
            const int qi = upper_index(s_cls.tile_start[c], cl.nq, lj);
            const int64_t row = cl.qidx[qi];
            J.CS = CS;
            J.perm = perm;
            J.ccnt = ccnt;
            J.peq = cl.peq + (size_t)qi * 256 * cl.nw;
            J.out = out;
            J.row = row;
            J.nc = nc;
            J.s = s_cls.lo[c][qi] + (lj - s_cls.tile_start[c][qi]) * jobsz;
            J.s1 = min(J.s + jobsz, (int64_t)s_cls.hi[c][qi]);
            J.qc = qcnt[row];
            J.m = cl.qlen[qi];
            J.nw = cl.nw;
            J.k = k;
            J.dtype = dtype;
        }
        return true;
    };
    survivor_warp<R>(s_job[w], next_job, s_pend[w], s_pgd[w], status,
                  [&](int64_t sidx, int m, int n, int cols, uint32_t gd) {
                      if (!LOG || m == 0 || n == 0 || (sidx % rows.stride) != 0) return;
                      const int64_t at = atomicAdd((unsigned long long *)rows.count, 1ull);
                      if (at >= rows.cap) return;
                      half *f = rows.x + at * 7;
                      f[0] = __float2half((float)m * (1.f / 256.f));
                      f[1] = __float2half((float)n * (1.f / 256.f));
                      f[2] = f[0];
                      f[3] = f[1];
                      f[4] = __float2half((float)(n - m) * (1.f / 16.f));
                      f[5] = __float2half((float)gd * (1.f / 128.f));
                      f[6] = __float2half((float)k * (1.f / 16.f));
                      rows.y[at] = (float)cols / (float)n;
                  },
                  [&](void *o, int dt, int64_t idx, int d) {
                      if (DEFER) list_emit(L, o, dt, idx, d);
                      else store1(o, dt, idx, d);
                  });
}

// The list's entries into their outputs (after the search kernel). A list
// that ran full re-arms the job counter for the repair launch that follows.
__global__ void __launch_bounds__(256) k_list_scatter(ResultList L, int32_t *work) {
    const unsigned long long cnt = *L.count, n = cnt < L.cap ? cnt : L.cap;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const unsigned long long e = L.item[i];
        uint8_t *a = reinterpret_cast<uint8_t *>((uintptr_t)(e >> 8));
        const int dt = (int)((e >> 6) & 3u), d = (int)(e & 63u);
        store1(a, dt, 0, d);
    }
    if (cnt > L.cap && blockIdx.x == 0 && threadIdx.x == 0) *work = 0;
}

// ------------------------------------------------------------- launchers --
cudaError_t launch_sketch_strings(cudaStream_t st, int sms, const DevStrings &S, uint64_t *sketch, uint4 *counts,
                                  uint32_t *status) {
    if (S.n <= 0) return cudaSuccess;
    const int grid = (int)std::min<int64_t>((S.n + 7) / 8, (int64_t)sms * 8);     // a warp per string
    k_sketch_strings<<<grid, 256, 0, st>>>(S, sketch, counts, status);
    return cudaGetLastError();
}

template <int R>
static void launch_band_r(cudaStream_t st, int grid, int jobsz, const SurvClasses &C, const DevStrings &CS,
                          const int32_t *perm, const uint4 *ccnt, const uint4 *qcnt, int k, int dtype, void *out,
                          int64_t nc, const SurvRows *rows, const ResultList *list, const FillItems *fill,
                          uint32_t *status) {
    const SurvRows none{nullptr, nullptr, 0, nullptr, 1};
    const ResultList L = list ? *list : ResultList{nullptr, nullptr, 0};
    const FillItems F = fill ? *fill : FillItems{};
    if (rows)
        k_search_band<R, true, false><<<grid, 256, 0, st>>>(CS, perm, ccnt, qcnt, C, jobsz, k, dtype, out, nc, *rows,
                                                             L, F, status);
    else if (fill)
        k_search_band<R, false, true><<<grid, 256, 0, st>>>(CS, perm, ccnt, qcnt, C, jobsz, k, dtype, out, nc, none,
                                                             L, F, status);
    else
        k_search_band<R, false, false><<<grid, 256, 0, st>>>(CS, perm, ccnt, qcnt, C, jobsz, k, dtype, out, nc, none,
                                                              L, F, status);
}

// The job counter is C.work[0], zero when the launch starts (the plan
// clears it on the stream). round: columns per round, 8, 16 or 32.
// fill != null: the kernel fills the output and defers its results to
// `list`; fill == null, list != null: the repair launch (runs only if the
// list ran full); both null: results stored in place.
cudaError_t launch_search_band(cudaStream_t st, int sms, int ctas_per_sm, int round, int jobsz, const SurvClasses &C,
                               const DevStrings &CS, const int32_t *perm, const uint4 *ccnt, const uint4 *qcnt, int k,
                               int dtype, void *out, int64_t nc, const SurvRows *rows, const ResultList *list,
                               const FillItems *fill, uint32_t *status) {
    if (C.n <= 0) return cudaSuccess;
    if (C.n > kSurvClasses || k < 0 || k > 31 || jobsz < 128 || (fill && (!list || rows))) return cudaErrorInvalidValue;
    const int grid = sms * std::max(1, std::min(ctas_per_sm, 8));
    if (round == 8) launch_band_r<8>(st, grid, jobsz, C, CS, perm, ccnt, qcnt, k, dtype, out, nc, rows, list, fill, status);
    else if (round == 16)
        launch_band_r<16>(st, grid, jobsz, C, CS, perm, ccnt, qcnt, k, dtype, out, nc, rows, list, fill, status);
    else if (round == 32)
        launch_band_r<32>(st, grid, jobsz, C, CS, perm, ccnt, qcnt, k, dtype, out, nc, rows, list, fill, status);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}

cudaError_t launch_list_scatter(cudaStream_t st, int sms, const ResultList &L, int32_t *work) {
    k_list_scatter<<<sms * 2, 256, 0, st>>>(L, work);
    return cudaGetLastError();
}

}  // namespace blg
