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
// Only results <= k are written; the output was filled with k+1 before.
#include <cuda_fp16.h>

#include <algorithm>

#include "blg_kernels.cuh"
#include "blg_sched.h"

namespace blg {

// sketch[i] = gram_sketch(string i), counts[i] = gram_counts(string i),
// one warp per string: lane l takes the 4-grams starting at l, l + 32, ...
// (one unaligned 4-byte read each, consecutive across the warp), the 16 bin
// counts are summed by one ballot per bin, the sketch bits by an OR over the
// warp. The values equal the per-thread functions' (the same grams, hash and
// saturation at 255).
__global__ void __launch_bounds__(256) k_sketch_strings(DevStrings S, uint64_t *sketch, uint4 *counts,
                                                        uint32_t *status) {
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < S.n; i += nwarps) {
        int n;
        const uint8_t *p = string_at(S, i, n, status);
        uint32_t sk_lo = 0, sk_hi = 0, cnt = 0;              // lane b < 16 counts bin b
        for (int s0 = 0; s0 + 3 < n; s0 += 32) {
            const int s = s0 + lane;                          // the gram of bytes s .. s+3
            const bool act = s + 3 < n;
            const uint32_t g = act ? __byte_perm(load4(p + s), 0u, 0x0123) : 0u;   // b[s] << 24 | .. | b[s+3]
            const uint32_t h = g * 0x9E3779B1u;
            const uint32_t bin = act ? (h >> 28) : 16u;
            if (act && s + 3 < kSketchWindow) {
                const uint32_t bit = h >> 26;
                if (bit < 32) sk_lo |= 1u << bit;
                else sk_hi |= 1u << (bit - 32);
            }
#pragma unroll
            for (uint32_t b = 0; b < 16; b++) {
                const unsigned m = __ballot_sync(kFull, bin == b);
                if ((uint32_t)lane == b) cnt += __popc(m);
            }
        }
        sk_lo = __reduce_or_sync(kFull, sk_lo);
        sk_hi = __reduce_or_sync(kFull, sk_hi);
        uint32_t v = (lane < 16 ? min(cnt, 255u) : 0u) << (8 * (lane & 3));   // byte lane & 3 of word lane >> 2
        v |= __shfl_xor_sync(kFull, v, 1);
        v |= __shfl_xor_sync(kFull, v, 2);
        const uint32_t w0 = __shfl_sync(kFull, v, 0), w1 = __shfl_sync(kFull, v, 4), w2 = __shfl_sync(kFull, v, 8),
                       w3 = __shfl_sync(kFull, v, 12);
        if (lane == 0) {
            sketch[i] = ((uint64_t)sk_hi << 32) | sk_lo;
            counts[i] = make_uint4(w0, w1, w2, w3);
        }
    }
}

// Every non-lane-spread query class of one thresholded run in one launch.
struct SurvClasses {
    int n;                                     // classes
    SearchClass cls[kSurvClasses];
    const int32_t *lo[kSurvClasses];           // survivor range per query
    const int32_t *hi[kSurvClasses];
    const int64_t *tile_start[kSurvClasses];   // job prefix per query (nq + 1)
};

template <bool LOG>
__global__ void __launch_bounds__(256) k_search_band(DevStrings CS, const int32_t *perm, const uint4 *ccnt,
                                                     const uint4 *qcnt, SurvClasses C, int32_t *work, int jobsz,
                                                     int k, int dtype, void *out, int64_t nc, SurvRows rows,
                                                     uint32_t *status) {
    __shared__ SurvClasses s_cls;
    __shared__ SurvJob s_job[8];
    __shared__ int32_t s_pend[8][kSurvPend];
    __shared__ uint16_t s_pgd[8][kSurvPend];
    if (threadIdx.x == 0) s_cls = C;
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    auto next_job = [&](SurvJob &J) -> bool {
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
        if (c >= s_cls.n) return false;
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
    survivor_warp(s_job[w], next_job, s_pend[w], s_pgd[w], status,
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
                  });
}

// ------------------------------------------------------------- launchers --
cudaError_t launch_sketch_strings(cudaStream_t st, int sms, const DevStrings &S, uint64_t *sketch, uint4 *counts,
                                  uint32_t *status) {
    if (S.n <= 0) return cudaSuccess;
    const int grid = (int)std::min<int64_t>((S.n + 7) / 8, (int64_t)sms * 8);     // a warp per string
    k_sketch_strings<<<grid, 256, 0, st>>>(S, sketch, counts, status);
    return cudaGetLastError();
}

// `work` must be zero when the launch starts (the first class's survivor
// plan clears it on the stream).
cudaError_t launch_search_band(cudaStream_t st, int sms, int ctas_per_sm, int jobsz, int ncls,
                               const SearchClass *cls, const int32_t *const *lo, const int32_t *const *hi,
                               const int64_t *const *tile_start, int32_t *work, const DevStrings &CS,
                               const int32_t *perm, const uint4 *ccnt, const uint4 *qcnt, int k, int dtype, void *out,
                               int64_t nc, const SurvRows *rows, uint32_t *status) {
    if (ncls <= 0) return cudaSuccess;
    if (ncls > kSurvClasses || k < 0 || k > 31 || jobsz < 128) return cudaErrorInvalidValue;
    SurvClasses C{};
    C.n = ncls;
    for (int c = 0; c < ncls; c++) {
        C.cls[c] = cls[c];
        C.lo[c] = lo[c];
        C.hi[c] = hi[c];
        C.tile_start[c] = tile_start[c];
    }
    const int grid = sms * std::max(1, std::min(ctas_per_sm, 8));
    if (rows) {
        k_search_band<true><<<grid, 256, 0, st>>>(CS, perm, ccnt, qcnt, C, work, jobsz, k, dtype, out, nc, *rows,
                                                   status);
    } else {
        const SurvRows none{nullptr, nullptr, 0, nullptr, 1};
        k_search_band<false><<<grid, 256, 0, st>>>(CS, perm, ccnt, qcnt, C, work, jobsz, k, dtype, out, nc, none,
                                                    status);
    }
    return cudaGetLastError();
}

}  // namespace blg
