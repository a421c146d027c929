// Many independent cdist problems in one persistent launch.
//
// A batch is a set of problems, each with its own queries, choices, max_dist,
// output dtype and device output. Every problem keeps the layout of a
// resident search (length-sorted choices, per-query Peq tables); a "job" is
// one (problem, query word-class). These kernels run the whole batch:
//   k_batch_fill    max_dist+1 into every thresholded problem's output
//   k_batch_plan    one block per job: survivor ranges and tile prefix
//   k_batch_scan    job tile prefix (the global tile space)
//   k_batch_band    persistent warps: banded jobs (max_dist <= 31), units of
//                   survivors of one query filtered by the 4-gram bound and
//                   solved with lanes refilled between rounds (survivor_warp)
//   k_batch_search  persistent: every CTA pulls (job, query, 1024-survivor)
//                   tiles from one device counter until the space is done
// The host captures them once into a CUDA graph and replays it per run.
#include "blg_batch.h"
#include "blg_kernels.cuh"

namespace blg {

// Peq staging of the exact / wide-threshold kernel: [256][NW] u64 for NW =
// kBatchMaxWords.
constexpr int kBatchSearchSmem = 256 * kBatchMaxWords * 8;

// out[0..n) = v (dtype-sized) by this thread's share (tid of stride).
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
    for (int64_t i = tid; i < nvec; i += stride) vp[i] = vv;
    const int64_t tail0 = head + nvec * 16;
    for (int64_t r = tid * es; r < head + (bytes - tail0); r += stride * es) {
        const int64_t x = r < head ? r : tail0 + (r - head);
        if (x >= bytes) break;
        if (es == 1) b[x] = (uint8_t)v;
        else if (es == 2) *reinterpret_cast<uint16_t *>(b + x) = (uint16_t)v;
        else *reinterpret_cast<uint32_t *>(b + x) = v;
    }
}

__global__ void __launch_bounds__(256) k_batch_fill(const BatchFill *fills) {
    const BatchFill f = fills[blockIdx.y];
    fill_share(f.out, f.n, f.dtype, f.value, (int64_t)blockIdx.x * blockDim.x + threadIdx.x,
               (int64_t)gridDim.x * blockDim.x);
}

// One block per job: survivor range of every query (all choices for exact
// problems), tile counts and their prefix, the job's tile total.
__global__ void __launch_bounds__(1024) k_batch_plan(BatchPlan plan) {
    __shared__ int64_t s_sum[1024];
    __shared__ int64_t s_carry;
    const BatchJob &job = plan.jobs[blockIdx.x];
    const SearchClass &cls = job.cls;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    for (int base = 0; base < cls.nq; base += 1024) {
        const int qi = base + threadIdx.x;
        int64_t tiles = 0;
        if (qi < cls.nq) {
            int64_t a = 0, b = job.n_len;
            if (job.k >= 0) {
                const int64_t m = cls.qlen[qi];
                a = m - job.k - job.min_len;
                b = m + job.k - job.min_len + 1;
                a = a < 0 ? 0 : (a > job.n_len ? job.n_len : a);
                b = b < 0 ? 0 : (b > job.n_len ? job.n_len : b);
            }
            const int64_t l = job.lstart[a], h = b > a ? job.lstart[b] : l;
            job.lo[qi] = (int32_t)l;
            job.hi[qi] = (int32_t)h;
            tiles = (h - l + job.tile - 1) / job.tile;
        }
        s_sum[threadIdx.x] = tiles;
        __syncthreads();
        for (int off = 1; off < 1024; off <<= 1) {
            const int64_t v = threadIdx.x >= off ? s_sum[threadIdx.x - off] : 0;
            __syncthreads();
            s_sum[threadIdx.x] += v;
            __syncthreads();
        }
        if (qi < cls.nq) job.tile_start[qi] = s_carry + s_sum[threadIdx.x] - tiles;
        __syncthreads();
        if (threadIdx.x == 0) s_carry += s_sum[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        job.tile_start[cls.nq] = s_carry;
        plan.job_tiles[blockIdx.x] = s_carry;
    }
}

__global__ void __launch_bounds__(1024) k_batch_scan(BatchPlan plan) {
    __shared__ int64_t s_sum[1024];
    __shared__ int64_t s_carry;
    if (threadIdx.x == 0) {
        s_carry = 0;
        plan.work[0] = 0;
        plan.work[1] = 0;
    }
    __syncthreads();
    for (int base = 0; base < plan.njobs; base += 1024) {
        const int j = base + threadIdx.x;
        const int64_t t = j < plan.njobs ? plan.job_tiles[j] : 0;
        s_sum[threadIdx.x] = t;
        __syncthreads();
        for (int off = 1; off < 1024; off <<= 1) {
            const int64_t v = threadIdx.x >= off ? s_sum[threadIdx.x - off] : 0;
            __syncthreads();
            s_sum[threadIdx.x] += v;
            __syncthreads();
        }
        if (j < plan.njobs) plan.tile_base[j] = s_carry + s_sum[threadIdx.x] - t;
        __syncthreads();
        if (threadIdx.x == 0) s_carry += s_sum[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0) plan.tile_base[plan.njobs] = s_carry;
}

template <int NW>
__device__ __forceinline__ void batch_tile(const BatchJob &job, const uint64_t *s_peq, int qi, int64_t s0, Units u,
                                           uint32_t *status) {
    RowAddr<NW> ra;
    ra.init(u);
    const int m = job.cls.qlen[qi];
    const int64_t row = job.cls.qidx[qi];
    const int64_t s_end = job.hi[qi];
    const int k = job.k >= 0 ? job.k : 0x3fffffff;    // exact problems: no exit can fire
#pragma unroll 1
    for (int t = 0; t < 4; t++) {
        const int64_t sidx = s0 + t;
        if (sidx >= s_end) break;
        int n;
        const uint8_t *tp = string_at(job.CS, sidx, n, status);
        const int d = dist_seq_any<NW, true>(s_peq, m, tp, n, k, u, ra);
        if (d <= k) store1(job.out, job.dtype, row * job.nc + job.perm[sidx], d);
    }
}

// Banded jobs (0 <= k <= 31): persistent warps pull (job, query, survivor
// unit) tiles of the banded part of the tile space.
template <int R>
__global__ void __launch_bounds__(256) k_batch_band(BatchPlan plan, uint32_t *status) {
    __shared__ __align__(16) unsigned char s_raw[8 * sizeof(SurvJob)];   // (no constructor runs on shared memory)
    SurvJob *s_job = reinterpret_cast<SurvJob *>(s_raw);
    __shared__ int32_t s_pend[8][kSurvPend];
    __shared__ uint16_t s_pgd[8][kSurvPend];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t total = plan.tile_base[plan.nbanded];
    auto next_job = [&](SurvJob &J) -> bool {
        int64_t tile = 0;
        if (lane == 0) tile = atomicAdd(&plan.work[0], 1);
        tile = __shfl_sync(kFull, tile, 0);
        if (tile >= total) return false;
        if (lane == 0) {
            const int j = upper_index(plan.tile_base, plan.nbanded, tile);
            const BatchJob &job = plan.jobs[j];
            const int64_t lt = tile - plan.tile_base[j];
            const int qi = upper_index(job.tile_start, job.cls.nq, lt);
            const int64_t row = job.cls.qidx[qi];
            J.CS = job.CS;
            J.perm = job.perm;
            J.ccnt = job.ccnt;
            J.peq = job.cls.peq + (size_t)qi * 256 * job.nw;
            J.out = job.out;
            J.row = row;
            J.nc = job.nc;
            J.s = job.lo[qi] + (lt - job.tile_start[qi]) * job.tile;
            J.s1 = min(J.s + job.tile, (int64_t)job.hi[qi]);
            J.qc = job.qcnt[row];
            J.m = job.cls.qlen[qi];
            J.nw = job.nw;
            J.k = job.k;
            J.dtype = job.dtype;
        }
        return true;
    };
    survivor_warp<R>(s_job[w], next_job, s_pend[w], s_pgd[w], status, [](int64_t, int, int, int, uint32_t) {});
}

// The other jobs (exact, or max_dist > 31): 1024-choice tiles, 4 per thread.
__global__ void __launch_bounds__(256) k_batch_search(BatchPlan plan, uint32_t *status, uint32_t unit) {
    extern __shared__ uint64_t s_peq[];
    __shared__ int64_t s_tile;
    const Units u{unit, unit + unit};
    const int64_t first = plan.tile_base[plan.nbanded], total = plan.tile_base[plan.njobs];
    int cur_j = -1, cur_q = -1;
    while (true) {
        if (threadIdx.x == 0) s_tile = first + atomicAdd(&plan.work[1], 1);
        __syncthreads();
        const int64_t tile = s_tile;
        if (tile >= total) break;
        const int j = upper_index(plan.tile_base, plan.njobs, tile);
        const BatchJob &job = plan.jobs[j];
        const int64_t lt = tile - plan.tile_base[j];
        const int qi = upper_index(job.tile_start, job.cls.nq, lt);
        const int nw = job.nw;
        if (j != cur_j || qi != cur_q) {
            const uint64_t *src = job.cls.peq + (size_t)qi * 256 * nw;
            for (int x = threadIdx.x; x < 256 * nw; x += blockDim.x) s_peq[x] = __ldg(src + x);
            cur_j = j;
            cur_q = qi;
        }
        __syncthreads();
        const int64_t s0 = job.lo[qi] + (lt - job.tile_start[qi]) * 1024 + threadIdx.x * 4;
        switch (nw) {
        case 1: batch_tile<1>(job, s_peq, qi, s0, u, status); break;
        case 2: batch_tile<2>(job, s_peq, qi, s0, u, status); break;
        case 3: batch_tile<3>(job, s_peq, qi, s0, u, status); break;
        default: batch_tile<4>(job, s_peq, qi, s0, u, status); break;
        }
        __syncthreads();
    }
}

cudaError_t batch_set_attributes() {
    return cudaFuncSetAttribute(k_batch_search, cudaFuncAttributeMaxDynamicSharedMemorySize, kBatchSearchSmem);
}

// The launches of one batch run, on `st` (capturable: no allocation, no
// attribute change, no synchronisation). The queries' Peq tables were built
// at upload.
cudaError_t launch_batch(cudaStream_t st, int sms, const BatchPlan &plan, const BatchFill *fills, int nfill,
                         int64_t max_fill, uint32_t *status) {
    if (nfill > 0) {
        int64_t bx = (max_fill / 16 + 255) / 256;
        bx = bx < 1 ? 1 : (bx > 1024 ? 1024 : bx);
        k_batch_fill<<<dim3((unsigned)bx, (unsigned)nfill), 256, 0, st>>>(fills);
    }
    if (plan.njobs > 0) {
        k_batch_plan<<<plan.njobs, 1024, 0, st>>>(plan);
        k_batch_scan<<<1, 1024, 0, st>>>(plan);
        // 32 columns per round: the batch's short strings mostly end within
        // one (config 5: 1.38 ms per step, 1.70 with 16 columns, 1.72 with 8)
        if (plan.nbanded > 0) k_batch_band<32><<<sms * 4, 256, 0, st>>>(plan, status);
        if (plan.nbanded < plan.njobs) k_batch_search<<<sms * 3, 256, kBatchSearchSmem, st>>>(plan, status, 1u);
    }
    return cudaGetLastError();
}

}  // namespace blg
