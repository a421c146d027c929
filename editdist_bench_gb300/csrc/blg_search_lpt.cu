// Thresholded search, longest-predicted-first: the survivor kernel for
// max_dist <= 31.
//
// With max_dist = k only (query, choice) pairs whose lengths differ by at
// most k need the column loop (csrc/myers.c:101-106); they are a contiguous
// range of the length-sorted choices per query. Their cost is very uneven:
// unrelated pairs leave the banded loop after a few columns, near-copies run
// the whole text. A CTA that gives each thread a fixed share waits at its
// barrier for the slowest thread. Here a persistent CTA takes a job of up to
// 4096 survivors of one query and
//   1. gives every survivor a predicted-cost key: the 4-gram sketch distance
//      of query and choice (near-copies score low and run long), or, under
//      the learned schedule, the scheduler network's prediction for
//      (query length, length gap, sketch distance) read from a per-query table;
//   2. counting-sorts the job by key in shared memory, most expensive first;
//   3. lets its warps pull 32-survivor chunks from a shared counter in that
//      order (longest processing time first), so the expensive pairs start
//      early and cheap ones fill the gaps;
//   4. runs each survivor for at most 4 (k + 4) columns: unrelated pairs
//      leave the band by then, and the rest (near-copies, which run the whole
//      text, a few per job) are queued with their column state. One resume
//      launch after all jobs finishes them 32 to a warp; left in their jobs
//      they would run on a few lanes of one warp while the CTA's other
//      warps wait for them at the job's last barrier.
// Only results <= k are written; the output was filled with k+1 before.
// The job body (lpt_job) is shared with the multi-problem batch kernel.
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

template <int NW, bool LOG>
__global__ void __launch_bounds__(256) k_search_lpt(DevStrings CS, const int32_t *perm, const uint64_t *csk,
                                                    const uint64_t *qsk, const uint4 *ccnt, const uint4 *qcnt,
                                                    SearchClass cls, const int32_t *lo,
                                                    const int32_t *hi, const int64_t *tile_start, int32_t *work,
                                                    const uint8_t *keytab, int64_t keystride, int k, int dtype,
                                                    void *out, int64_t nc, int jobsz, SurvRows rows, DeferQueue dq,
                                                    uint32_t *status, uint32_t unit) {
    extern __shared__ uint32_t s_rows[];              // the query's padded Peq halves (banded layout)
    __shared__ LptShared S;
    const Units u{unit, unit + unit};
    const int tid = threadIdx.x;
    const int64_t total = tile_start[cls.nq];
    int cur = -1;
    while (true) {
        if (tid == 0) S.job = atomicAdd(work, 1);
        __syncthreads();
        const int64_t job = S.job;
        if (job >= total) break;
        const int qi = upper_index(tile_start, cls.nq, job);
        if (qi != cur) {
            stage_band_rows(cls.peq + (size_t)qi * 256 * NW, NW, s_rows);
            cur = qi;
        }
        const int m = cls.qlen[qi];
        const int64_t row = cls.qidx[qi];
        const uint64_t qs = qsk[row];
        const int64_t s0 = lo[qi] + (job - tile_start[qi]) * jobsz;
        const int cnt = (int)min((int64_t)jobsz, (int64_t)hi[qi] - s0);
        lpt_job(S, CS, perm, csk, ccnt, qs, qcnt[row], s_rows, 2 * NW + 6, m, row, s0, cnt, k,
                keytab ? keytab + qi * keystride : nullptr, dtype, out, nc, dq, cls.peq + (size_t)qi * 256 * NW, NW,
                status, u,
                [&](int64_t sidx, int n, int cols, uint32_t gd) {
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
}

// The resume pass of the deferred survivors (all query classes of a run, or
// every banded problem of a batch): a thread per item.
__global__ void __launch_bounds__(256) k_band_resume(DeferQueue dq) {
    const unsigned long long claimed = *dq.count;
    const uint32_t total = claimed < (unsigned long long)dq.cap ? (uint32_t)claimed : (uint32_t)dq.cap;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x)
        band_resume_item(dq.items[i]);
}

// ------------------------------------------------------------- launchers --
cudaError_t launch_band_resume(cudaStream_t st, int sms, const DeferQueue &dq) {
    if (!dq.items) return cudaSuccess;
    k_band_resume<<<sms * 4, 256, 0, st>>>(dq);
    return cudaGetLastError();
}

cudaError_t launch_sketch_strings(cudaStream_t st, int sms, const DevStrings &S, uint64_t *sketch, uint4 *counts,
                                  uint32_t *status) {
    if (S.n <= 0) return cudaSuccess;
    const int grid = (int)std::min<int64_t>((S.n + 7) / 8, (int64_t)sms * 8);     // a warp per string
    k_sketch_strings<<<grid, 256, 0, st>>>(S, sketch, counts, status);
    return cudaGetLastError();
}

template <int NW>
static cudaError_t launch_lpt_nw(cudaStream_t st, int grid, const DevStrings &CS, const int32_t *perm,
                                 const uint64_t *csk, const uint64_t *qsk, const uint4 *ccnt, const uint4 *qcnt,
                                 const SearchClass &cls, const int32_t *lo, const int32_t *hi, const int64_t *tile_start, int32_t *work, const uint8_t *keytab,
                                 int64_t keystride, int k, int dtype, void *out, int64_t nc, int jobsz,
                                 const SurvRows *rows, const DeferQueue &dq, uint32_t *status) {
    const size_t smem = (size_t)256 * (2 * NW + 6) * sizeof(uint32_t);
    if (rows) {
        cudaFuncSetAttribute(k_search_lpt<NW, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_search_lpt<NW, true><<<grid, 256, smem, st>>>(CS, perm, csk, qsk, ccnt, qcnt, cls, lo, hi, tile_start, work, keytab,
                                                        keystride, k, dtype, out, nc, jobsz, *rows, DeferQueue{},
                                                        status, 1u);
    } else {
        const SurvRows none{nullptr, nullptr, 0, nullptr, 1};
        cudaFuncSetAttribute(k_search_lpt<NW, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_search_lpt<NW, false><<<grid, 256, smem, st>>>(CS, perm, csk, qsk, ccnt, qcnt, cls, lo, hi, tile_start, work, keytab,
                                                         keystride, k, dtype, out, nc, jobsz, none, dq, status, 1u);
    }
    return cudaGetLastError();
}

cudaError_t launch_search_lpt(cudaStream_t st, int sms, int ctas_per_sm, int jobsz, int nw, const DevStrings &CS,
                              const int32_t *perm, const uint64_t *csk, const uint64_t *qsk, const uint4 *ccnt,
                              const uint4 *qcnt, const SearchClass &cls, const int32_t *lo, const int32_t *hi,
                              const int64_t *tile_start, int32_t *work,
                              const uint8_t *keytab, int64_t keystride, int k, int dtype, void *out, int64_t nc,
                              const SurvRows *rows, const DeferQueue &dq, uint32_t *status) {
    if (cls.nq <= 0) return cudaSuccess;
    if (k < 0 || k > 31 || jobsz < 256 || jobsz > kSurvJob) return cudaErrorInvalidValue;
    const int grid = sms * std::max(1, std::min(ctas_per_sm, 8));
    switch (nw) {
#define BLG_LPT(W) \
    case W: return launch_lpt_nw<W>(st, grid, CS, perm, csk, qsk, ccnt, qcnt, cls, lo, hi, tile_start, work, keytab, keystride, k, dtype, out, nc, jobsz, rows, dq, status);
    BLG_LPT(1) BLG_LPT(2) BLG_LPT(3) BLG_LPT(4) BLG_LPT(5) BLG_LPT(6) BLG_LPT(7) BLG_LPT(8)
#undef BLG_LPT
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace blg
