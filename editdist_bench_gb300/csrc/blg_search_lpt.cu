// Thresholded search, longest-predicted-first: the survivor kernel for
// max_dist <= 31 (configs 2b, 4).
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
//      early and cheap ones fill the gaps.
// Only results <= k are written; the output was filled with k+1 before.
#include <cuda_fp16.h>

#include <algorithm>

#include "blg_kernels.cuh"
#include "blg_sched.h"

namespace blg {

constexpr int kSurvJob = 4096;                      // survivors per job
constexpr int kSketchBins = kSketchWindow + 1;      // sketch distances 0..64

// sketch[i] = gram_sketch(string i)
__global__ void __launch_bounds__(256) k_sketch_strings(DevStrings S, uint64_t *sketch, uint32_t *status) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < S.n; i += (int64_t)gridDim.x * blockDim.x) {
        int n;
        const uint8_t *p = string_at(S, i, n, status);
        sketch[i] = gram_sketch(p, n);
    }
}

template <int NW, bool LOG>
__global__ void __launch_bounds__(256) k_search_lpt(DevStrings CS, const int32_t *perm, const uint64_t *csk,
                                                    const uint64_t *qsk, SearchClass cls, const int32_t *lo,
                                                    const int32_t *hi, const int64_t *tile_start, int32_t *work,
                                                    const uint8_t *keytab, int k, int dtype, void *out, int64_t nc,
                                                    SurvRows rows, uint32_t *status, uint32_t unit) {
    extern __shared__ uint32_t s_rows[];              // the query's padded Peq halves (banded layout)
    __shared__ uint16_t s_list[kSurvJob];
    __shared__ int s_cnt[256], s_start[256];
    __shared__ int64_t s_job;
    __shared__ int s_next;
    const Units u{unit, unit + unit};
    const int tid = threadIdx.x, lane = tid & 31;
    constexpr int kStride = 2 * NW + 6;
    constexpr int kPer = kSurvJob / 256;
    const int64_t total = tile_start[cls.nq];
    const int E = (2 * k + 1) * kSketchBins;
    int cur = -1;
    uint64_t qs = 0;
    while (true) {
        if (tid == 0) {
            s_job = atomicAdd(work, 1);
            s_next = 0;
        }
        s_cnt[tid] = 0;
        __syncthreads();
        const int64_t job = s_job;
        if (job >= total) break;
        int a = 0, b = cls.nq;                        // tile_start[a] <= job < tile_start[b]
        while (b - a > 1) {
            const int mid = (a + b) >> 1;
            if (tile_start[mid] <= job) a = mid; else b = mid;
        }
        const int qi = a;
        if (qi != cur) {
            stage_band_rows(cls.peq + (size_t)qi * 256 * NW, NW, s_rows);
            cur = qi;
        }
        const int m = cls.qlen[qi];
        const int64_t row = cls.qidx[qi];
        qs = qsk[row];
        const int64_t s0 = lo[qi] + (job - tile_start[qi]) * kSurvJob;
        const int cnt = (int)min((int64_t)kSurvJob, (int64_t)hi[qi] - s0);
        // 1. keys (a larger key = more predicted work)
        int key[kPer], rank[kPer];
#pragma unroll
        for (int r = 0; r < kPer; r++) {
            const int l = tid + 256 * r;
            key[r] = -1;
            if (l < cnt) {
                const int64_t sidx = s0 + l;
                const int n = (int)(CS.off[sidx + 1] - CS.off[sidx]);
                const int sd = __popcll(qs ^ csk[sidx]);
                int g = n - m + k;
                g = g < 0 ? 0 : (g > 2 * k ? 2 * k : g);
                key[r] = keytab ? keytab[(size_t)qi * E + g * kSketchBins + sd] : kSketchWindow - sd;
                rank[r] = atomicAdd(&s_cnt[key[r]], 1);
            }
        }
        __syncthreads();
        // 2. bucket starts, largest key first (one warp, 8 keys per lane)
        if (tid < 32) {
            int v[8], sum = 0;
#pragma unroll
            for (int q = 0; q < 8; q++) { v[q] = s_cnt[255 - (tid * 8 + q)]; sum += v[q]; }
            int incl = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int x = __shfl_up_sync(kFull, incl, o);
                if (tid >= o) incl += x;
            }
            int run = incl - sum;
#pragma unroll
            for (int q = 0; q < 8; q++) { s_start[255 - (tid * 8 + q)] = run; run += v[q]; }
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < kPer; r++)
            if (key[r] >= 0) s_list[s_start[key[r]] + rank[r]] = (uint16_t)(tid + 256 * r);
        __syncthreads();
        // 3. warps pull 32-survivor chunks in that order
        while (true) {
            int c = 0;
            if (lane == 0) c = atomicAdd(&s_next, 1);
            c = __shfl_sync(kFull, c, 0);
            if (c * 32 >= cnt) break;
            const int e = c * 32 + lane;
            if (e < cnt) {
                const int l = s_list[e];
                const int64_t sidx = s0 + l;
                int n;
                const uint8_t *tp = string_at(CS, sidx, n, status);
                int d, cols = 0;
                if (m == 0) d = cap_k(n, k);
                else if ((n > m ? n - m : m - n) > k) d = k + 1;
                else d = band_distance(m, tp, n, k,
                                       [&](uint32_t ch, int p0) { return band_row_bits(s_rows + ch * kStride, p0); }, u,
                                       LOG ? &cols : nullptr);
                if (d <= k) store1(out, dtype, row * nc + perm[sidx], d);
                if (LOG && m > 0 && n > 0 && ((s0 + l) % rows.stride) == 0) {
                    const int64_t at = atomicAdd((unsigned long long *)rows.count, 1ull);
                    if (at < rows.cap) {
                        half *f = rows.x + at * 7;
                        f[0] = __float2half((float)m * (1.f / 256.f));
                        f[1] = __float2half((float)n * (1.f / 256.f));
                        f[2] = f[0];
                        f[3] = f[1];
                        f[4] = __float2half((float)(n - m) * (1.f / 16.f));
                        f[5] = __float2half((float)__popcll(qs ^ csk[sidx]) * (1.f / 16.f));
                        f[6] = __float2half((float)k * (1.f / 16.f));
                        rows.y[at] = (float)cols / (float)n;
                    }
                }
            }
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------- launchers --
cudaError_t launch_sketch_strings(cudaStream_t st, int sms, const DevStrings &S, uint64_t *sketch, uint32_t *status) {
    if (S.n <= 0) return cudaSuccess;
    const int grid = (int)std::min<int64_t>((S.n + 255) / 256, (int64_t)sms * 8);
    k_sketch_strings<<<grid, 256, 0, st>>>(S, sketch, status);
    return cudaGetLastError();
}

template <int NW>
static cudaError_t launch_lpt_nw(cudaStream_t st, int grid, const DevStrings &CS, const int32_t *perm,
                                 const uint64_t *csk, const uint64_t *qsk, const SearchClass &cls, const int32_t *lo,
                                 const int32_t *hi, const int64_t *tile_start, int32_t *work, const uint8_t *keytab,
                                 int k, int dtype, void *out, int64_t nc, const SurvRows *rows, uint32_t *status) {
    const size_t smem = (size_t)256 * (2 * NW + 6) * sizeof(uint32_t);
    if (rows) {
        cudaFuncSetAttribute(k_search_lpt<NW, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_search_lpt<NW, true><<<grid, 256, smem, st>>>(CS, perm, csk, qsk, cls, lo, hi, tile_start, work, keytab, k,
                                                        dtype, out, nc, *rows, status, 1u);
    } else {
        const SurvRows none{nullptr, nullptr, 0, nullptr, 1};
        cudaFuncSetAttribute(k_search_lpt<NW, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_search_lpt<NW, false><<<grid, 256, smem, st>>>(CS, perm, csk, qsk, cls, lo, hi, tile_start, work, keytab, k,
                                                         dtype, out, nc, none, status, 1u);
    }
    return cudaGetLastError();
}

cudaError_t launch_search_lpt(cudaStream_t st, int sms, int nw, const DevStrings &CS, const int32_t *perm,
                              const uint64_t *csk, const uint64_t *qsk, const SearchClass &cls, const int32_t *lo,
                              const int32_t *hi, const int64_t *tile_start, int32_t *work, const uint8_t *keytab,
                              int k, int dtype, void *out, int64_t nc, const SurvRows *rows, uint32_t *status) {
    if (cls.nq <= 0) return cudaSuccess;
    if (k < 0 || k > 31) return cudaErrorInvalidValue;
    const int grid = sms * 4;
    switch (nw) {
#define BLG_LPT(W) \
    case W: return launch_lpt_nw<W>(st, grid, CS, perm, csk, qsk, cls, lo, hi, tile_start, work, keytab, k, dtype, out, nc, rows, status);
    BLG_LPT(1) BLG_LPT(2) BLG_LPT(3) BLG_LPT(4) BLG_LPT(5) BLG_LPT(6) BLG_LPT(7) BLG_LPT(8)
#undef BLG_LPT
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace blg
