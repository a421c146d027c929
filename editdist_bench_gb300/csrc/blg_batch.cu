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
#include <algorithm>

#include "blg_batch.h"
#include "blg_kernels.cuh"

namespace blg {

// Peq staging of the exact / wide-threshold kernel: [256][NW] u64 for NW =
// kBatchMaxWords.
constexpr int kBatchSearchSmem = 256 * kBatchMaxWords * 8;

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
// DEFER: fills every thresholded output (one fill item per unit claimed, the
// rest once the units are gone; config 5: 0.75 ms per step against 0.92 with
// the fill kernel first) and defers its results to plan.list; else
// stores in place, and a launch given the list runs only if it ran full.
// At most 64 registers, so its 4-CTA-per-SM grid is resident at once (78
// registers left free; config 5: 0.730 vs 0.747 ms per step).
template <int R, bool DEFER>
__global__ void __launch_bounds__(256, 4) k_batch_band(BatchPlan plan, bool repair, uint32_t *status) {
    if (!DEFER && repair && *plan.list.count <= plan.list.cap) return;
    __shared__ __align__(16) unsigned char s_raw[8 * sizeof(SurvJob)];   // (no constructor runs on shared memory)
    SurvJob *s_job = reinterpret_cast<SurvJob *>(s_raw);
    __shared__ int32_t s_pend[8][kSurvPend];
    __shared__ uint16_t s_pgd[8][kSurvPend];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t total = plan.tile_base[plan.nbanded];
    bool fill_on = DEFER;                          // warp-uniform
    auto next_job = [&](SurvJob &J) -> bool {
        if (DEFER && fill_on) fill_on = fill_one(plan.fill);
        int64_t tile = 0;
        if (lane == 0) tile = atomicAdd(&plan.work[0], 1);
        tile = __shfl_sync(kFull, tile, 0);
        if (tile >= total) {
            if (DEFER)
                while (fill_on) fill_on = fill_one(plan.fill);
            return false;
        }
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
    survivor_warp<R>(s_job[w], next_job, s_pend[w], s_pgd[w], status, [](int64_t, int, int, int, uint32_t) {},
                     [&](void *o, int dt, int64_t idx, int d) {
                         if (DEFER) list_emit(plan.list, o, dt, idx, d);
                         else store1(o, dt, idx, d);
                     });
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

// ------------------------------------------------------- batch upload --
// Length sort of every set's choices: count, bucket starts, slots.
__global__ void __launch_bounds__(256) k_len_count(const LenSortSet *sets, const int64_t *start, int nsets,
                                                   int64_t first, int64_t total) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x, end = first + total;
    for (int64_t J = first + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; J < end; J += stride) {
        const int s = upper_index(start, nsets, J);
        const LenSortSet &L = sets[s];
        const int64_t i = J - start[s];
        const int64_t b = L.off[i + 1] - L.off[i] - L.min_len;
        if (b >= 0 && b < L.n_len) atomicAdd(L.hist + b, 1ull);   // the host's length range bounds b
    }
}

// One block per set: exclusive scan of the counts into the bucket starts
// (index and byte), 1024 buckets per pass; hist becomes the cursors.
__global__ void __launch_bounds__(1024) k_len_scan(const LenSortSet *sets) {
    __shared__ int64_t s_i[1024], s_b[1024];
    __shared__ int64_t s_ci, s_cb;
    const LenSortSet &L = sets[blockIdx.x];
    const int t = threadIdx.x;
    if (t == 0) {
        s_ci = 0;
        s_cb = 0;
    }
    __syncthreads();
    for (int64_t b0 = 0; b0 < L.n_len; b0 += 1024) {
        const int64_t b = b0 + t;
        const int64_t cnt = b < L.n_len ? (int64_t)L.hist[b] : 0;
        s_i[t] = cnt;
        s_b[t] = cnt * (L.min_len + b);
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {            // inclusive scans (Hillis-Steele)
            const int64_t vi = t >= o ? s_i[t - o] : 0, vb = t >= o ? s_b[t - o] : 0;
            __syncthreads();
            s_i[t] += vi;
            s_b[t] += vb;
            __syncthreads();
        }
        const int64_t ci = s_ci, cb = s_cb;
        if (b < L.n_len) {
            const int64_t li = ci + s_i[t] - cnt;
            L.lstart[b] = li;
            L.bstart[b] = cb + s_b[t] - cnt * (L.min_len + b);
            L.hist[b] = (unsigned long long)li;
        }
        __syncthreads();
        if (t == 1023) {
            s_ci = ci + s_i[1023];
            s_cb = cb + s_b[1023];
        }
        __syncthreads();
    }
    if (t == 0) L.lstart[L.n_len] = s_ci;
}

__global__ void __launch_bounds__(256) k_len_scatter(const LenSortSet *sets, const int64_t *start, int nsets,
                                                     int64_t first, int64_t total) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x, end = first + total;
    for (int64_t J = first + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; J < end; J += stride) {
        const int s = upper_index(start, nsets, J);
        const LenSortSet &L = sets[s];
        const int64_t i = J - start[s];
        const int64_t b = L.off[i + 1] - L.off[i] - L.min_len;
        if (b >= 0 && b < L.n_len) L.perm[atomicAdd(L.hist + b, 1ull)] = (int32_t)i;
    }
}

cudaError_t launch_length_sort(cudaStream_t st, int sms, const LenSortSet *sets, const int64_t *start, int nsets,
                               int64_t first, int64_t total) {
    if (nsets <= 0 || total <= 0) return cudaSuccess;
    const int64_t blocks = std::min<int64_t>((total + 255) / 256, (int64_t)sms * 8);
    k_len_count<<<(unsigned)blocks, 256, 0, st>>>(sets, start, nsets, first, total);
    k_len_scan<<<nsets, 1024, 0, st>>>(sets);
    k_len_scatter<<<(unsigned)blocks, 256, 0, st>>>(sets, start, nsets, first, total);
    return cudaGetLastError();
}

// Per problem (item 0 also zeroes the problem's slack bytes): the sorted
// copy's offsets from its length buckets -- every string of bucket b has
// length min_len + b, so offset j is the bucket's first byte plus whole
// strings after it.
__global__ void __launch_bounds__(256) k_upload_prep(const UploadPrep *sets, const int64_t *start, int nsets,
                                                     int64_t first, int64_t total) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x, end = first + total;
    for (int64_t J = first + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; J < end; J += stride) {
        const int s = upper_index(start, nsets, J);
        const UploadPrep &P = sets[s];
        const int64_t j = J - start[s];
        if (j == 0)
            for (int b = 0; b < 3; b++) {
                if (!P.buf[b]) continue;
                for (int x = 1; x <= kSlackBefore; x++) P.buf[b][-x] = 0;
                for (int x = 0; x < kSlackAfter; x++) P.buf[b][P.bytes[b] + x] = 0;
            }
        if (P.n_sorted > 0) {
            const int b = j < P.n_sorted ? upper_index(P.lstart, (int)P.n_len, j) : (int)P.n_len - 1;
            P.soff[j] = P.bstart[b] + (j - P.lstart[b]) * (P.min_len + b);
        }
    }
}

// Every set's strings: the byte copy into sorted order (when the set has a
// permutation), the 4-gram sketch and the binned 4-gram counts, a warp per
// string. A warp takes 32 consecutive items; each lane first resolves one
// item (set, source string, destination) so the 32 lookups overlap, then
// the warp walks the 32 strings, lane l taking the grams that start at
// l, l + 32, .... A string of at most 256 bytes is read from shared memory,
// where its window was copied asynchronously while the warp worked on the
// previous string; longer ones are read in place. Strings of at most 256
// bytes have fewer than 256 grams, so the warp sums its byte counters with
// plain adds; longer ones fold per-lane counters into saturating totals
// every 255 grams and sum them with saturating byte adds. The sketch bits
// are an OR over the warp.
// Values equal gram_sketch / gram_counts of each string.
__device__ __forceinline__ void gram_add(uint32_t g, int s, int n, uint32_t (&c)[4], uint32_t &sk_lo,
                                         uint32_t &sk_hi) {
    if (s + 3 >= n) return;
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

// Asynchronous 16-byte copies global -> shared (cp.async, no registers held
// while they fly), grouped per string.
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    const uint32_t sa = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_prev() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

constexpr int kSketchWarps = 8;
constexpr int kSketchStage = 320;     // a string's 16-byte-aligned window (<= 256 + 30 bytes) and word slack

__global__ void __launch_bounds__(256) k_sketch_sets(const SketchSet *sets, const int64_t *start, int nsets,
                                                     int64_t first, int64_t total, uint32_t *status) {
    __shared__ __align__(16) uint8_t s_stage[kSketchWarps][2][kSketchStage];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t g0 = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; g0 < total; g0 += nwarps * 32) {
        // this lane's item (items first .. first + total - 1)
        const int64_t J = first + g0 + lane;
        const uint8_t *my_p = nullptr;
        uint8_t *my_q = nullptr;
        int my_n = 0, my_s = 0;
        int64_t my_i = 0;
        if (g0 + lane < total) {
            my_s = upper_index(start, nsets, J);
            const SketchSet &S = sets[my_s];
            my_i = J - start[my_s];
            my_p = string_at(S.src, S.perm ? (int64_t)S.perm[my_i] : my_i, my_n, status);
            if (S.perm) {
                const int64_t o0 = S.dst_off[my_i], cap = S.dst_off[my_i + 1] - o0;
                if (my_n > cap) my_n = (int)cap;
                my_q = S.dst + o0;
            }
        }
        const int cnt = total - g0 < 32 ? (int)(total - g0) : 32;
        // string t's window into stage buffer t & 1 (strings of at most 256
        // bytes; one commit group per string either way). The window lies
        // in the buffer's slack: 16 bytes before every string set, 48 after.
        auto stage = [&](int t) {
            const uintptr_t p = (uintptr_t)__shfl_sync(kFull, (unsigned long long)reinterpret_cast<uintptr_t>(my_p), t);
            const int n = __shfl_sync(kFull, my_n, t);
            if (n > 0 && n <= 256) {
                const uintptr_t base = p & ~uintptr_t(15);
                const int chunks = (int)((((p + (uintptr_t)n + 15) & ~uintptr_t(15)) - base) >> 4);   // <= 17
                if (lane < chunks)
                    cp_async16(s_stage[wib][t & 1] + 16 * lane, reinterpret_cast<const void *>(base + 16 * (uintptr_t)lane));
            }
            cp_async_commit();
        };
        uint64_t my_sk = 0;
        uint4 my_cnt = make_uint4(0, 0, 0, 0);
        stage(0);
        for (int t = 0; t < cnt; t++) {
            if (t + 1 < cnt) stage(t + 1);
            else cp_async_commit();
            cp_async_wait_prev();                              // string t's window has landed
            __syncwarp();
            const uint8_t *p = reinterpret_cast<const uint8_t *>(
                __shfl_sync(kFull, (unsigned long long)reinterpret_cast<uintptr_t>(my_p), t));
            uint8_t *q = reinterpret_cast<uint8_t *>(
                __shfl_sync(kFull, (unsigned long long)reinterpret_cast<uintptr_t>(my_q), t));
            const int n = __shfl_sync(kFull, my_n, t);
            uint32_t sk_lo = 0, sk_hi = 0;
            uint32_t tot[4] = {0, 0, 0, 0};                    // totals, bins 4w .. 4w+3
            if (n <= 256) {
                // lane l takes positions 128c + 4l .. +3 of chunks c = 0, 1:
                // three aligned words of the window give its 7 bytes, and one
                // byte permute gives each big-endian gram. At most 8 grams per
                // lane: its bin counts fit in nibbles (bin b at bits 4b..4b+3
                // of lo:hi), spread into byte counters once per string.
                const uint32_t *sw = reinterpret_cast<const uint32_t *>(s_stage[wib][t & 1]);
                const uint32_t off = (uint32_t)(reinterpret_cast<uintptr_t>(p) & 15);
                uint32_t lo = 0, hi = 0;
#pragma unroll
                for (int c = 0; c < 2; c++) {
                    const int s0 = 128 * c + 4 * lane;
                    if (128 * c >= n) break;
                    if (s0 < n) {
                        const uint32_t o = off + (uint32_t)s0, wi = o >> 2, sh = (o & 3u) * 8u;
                        const uint32_t w0 = sw[wi], w1 = sw[wi + 1], w2 = sw[wi + 2];
                        const uint32_t a0 = __funnelshift_r(w0, w1, sh), a1 = __funnelshift_r(w1, w2, sh);
#pragma unroll
                        for (int k = 0; k < 4; k++) {
                            const int sp = s0 + k;
                            if (sp + 3 < n) {
                                // bytes sp .. sp+3 as b[sp] << 24 | .. | b[sp+3]
                                const uint32_t g = __byte_perm(a0, a1, (uint32_t)((k + 3) | (k + 2) << 4 | (k + 1) << 8 | k << 12));
                                const uint32_t h = g * 0x9E3779B1u;
                                const uint32_t amt = (h >> 26) & 0x3cu;          // 4 x bin
                                const uint32_t one = 1u << (amt & 31u);
                                if (amt & 32u) hi += one;
                                else lo += one;
                                if (c == 0 && sp + 3 < kSketchWindow) {
                                    const uint32_t bit = h >> 26;
                                    if (bit < 32) sk_lo |= 1u << bit;
                                    else sk_hi |= 1u << (bit - 32);
                                }
                            }
                            if (q && sp < n) q[sp] = (uint8_t)(a0 >> (8 * k));
                        }
                    }
                }
                // nibbles -> bytes: bins 4x .. 4x+3 into word x
                auto spread = [](uint32_t v) {
                    v &= 0xffffu;
                    v = (v | (v << 8)) & 0x00ff00ffu;
                    return (v | (v << 4)) & 0x0f0f0f0fu;
                };
                tot[0] = spread(lo);
                tot[1] = spread(lo >> 16);
                tot[2] = spread(hi);
                tot[3] = spread(hi >> 16);
                // at most n - 3 <= 253 grams in all: no bin of the warp's sum
                // reaches 256, so plain adds never carry into the next byte
#pragma unroll
                for (int x = 0; x < 4; x++) tot[x] = __reduce_add_sync(kFull, tot[x]);
            } else {
                for (int c0 = 0; c0 < n; c0 += 32 * 255) {
                    uint32_t c[4] = {0, 0, 0, 0};              // this lane's counts of the chunk
                    const int c1 = min(n, c0 + 32 * 255);
                    for (int s = c0 + lane; s < c1; s += 32) {
                        const uint32_t w4 = load4(p + s);
                        gram_add(__byte_perm(w4, 0u, 0x0123), s, n, c, sk_lo, sk_hi);
                        if (q) q[s] = (uint8_t)w4;
                    }
#pragma unroll
                    for (int x = 0; x < 4; x++) tot[x] = __vaddus4(tot[x], c[x]);
                }
#pragma unroll
                for (int off = 16; off > 0; off >>= 1)
#pragma unroll
                    for (int x = 0; x < 4; x++) tot[x] = __vaddus4(tot[x], __shfl_xor_sync(kFull, tot[x], off));
            }
            sk_lo = __reduce_or_sync(kFull, sk_lo);
            sk_hi = __reduce_or_sync(kFull, sk_hi);
            if (lane == t) {
                my_sk = ((uint64_t)sk_hi << 32) | sk_lo;
                my_cnt = make_uint4(tot[0], tot[1], tot[2], tot[3]);
            }
            __syncwarp();                                      // buffer t & 1 is restaged for string t + 2
        }
        if (g0 + lane < total) {
            const SketchSet &S = sets[my_s];
            S.sketch[my_i] = my_sk;
            S.counts[my_i] = my_cnt;
        }
    }
}

// One CTA per query of every class: its Peq table (build_peq_block).
__global__ void __launch_bounds__(256) k_peq_sets(const PeqSet *sets, const int64_t *start, int nsets,
                                                  int64_t first, uint32_t *status) {
    extern __shared__ uint64_t tab[];
    const int64_t J = first + blockIdx.x;
    const int s = upper_index(start, nsets, J);
    const PeqSet &P = sets[s];
    const int64_t qi = J - start[s];
    int m;
    const uint8_t *p = string_at(P.Q, P.qidx[qi], m, status);
    build_peq_block(p, m, P.nwc, tab, P.peq + qi * 256 * P.nwc);
}

cudaError_t launch_upload_prep(cudaStream_t st, int sms, const UploadPrep *sets, const int64_t *start, int nsets,
                               int64_t first, int64_t total) {
    if (nsets <= 0 || total <= 0) return cudaSuccess;
    const int64_t blocks = std::min<int64_t>((total + 255) / 256, (int64_t)sms * 8);
    k_upload_prep<<<(unsigned)blocks, 256, 0, st>>>(sets, start, nsets, first, total);
    return cudaGetLastError();
}

cudaError_t launch_sketch_sets(cudaStream_t st, int sms, const SketchSet *sets, const int64_t *start, int nsets,
                               int64_t first, int64_t total, uint32_t *status) {
    if (nsets <= 0 || total <= 0) return cudaSuccess;
    const int64_t blocks = std::min<int64_t>((total + 255) / 256, (int64_t)sms * 4);   // 32 items per warp; 64 regs
    k_sketch_sets<<<(unsigned)blocks, 256, 0, st>>>(sets, start, nsets, first, total, status);
    return cudaGetLastError();
}

cudaError_t launch_peq_sets(cudaStream_t st, const PeqSet *sets, const int64_t *start, int nsets, int64_t first,
                            int64_t total, int max_nwc, uint32_t *status) {
    if (nsets <= 0 || total <= 0) return cudaSuccess;
    if (total > INT32_MAX || max_nwc < 1 || max_nwc > 32) return cudaErrorInvalidValue;
    const size_t smem = (size_t)256 * max_nwc * sizeof(uint64_t);
    cudaError_t e = cudaFuncSetAttribute(k_peq_sets, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_peq_sets<<<(unsigned)total, 256, smem, st>>>(sets, start, nsets, first, status);
    return cudaGetLastError();
}

cudaError_t batch_set_attributes() {
    return cudaFuncSetAttribute(k_batch_search, cudaFuncAttributeMaxDynamicSharedMemorySize, kBatchSearchSmem);
}

// The launches of one batch run, on `st` (capturable: no allocation, no
// attribute change, no synchronisation). The queries' Peq tables were built
// at upload. With the deferred list the banded kernel fills the outputs
// (the fill overlaps the survivor search) and the scatter follows, then
// the in-place repair launch that runs only if the list ran full; else the
// fill kernel runs first. *kernels: the kernels launched.
cudaError_t launch_batch(cudaStream_t st, int sms, const BatchPlan &plan, const BatchFill *fills, int nfill,
                         int64_t max_fill, uint32_t *status, int *kernels) {
    int nk = 0;
    const bool defer = plan.list.item && plan.nbanded > 0;
    if (defer) {
        cudaError_t e = cudaMemsetAsync(plan.hdr, 0, 2 * sizeof(unsigned long long), st);
        if (e != cudaSuccess) return e;
    } else if (nfill > 0) {
        int64_t bx = (max_fill / 16 + 255) / 256;
        bx = bx < 1 ? 1 : (bx > 1024 ? 1024 : bx);
        k_batch_fill<<<dim3((unsigned)bx, (unsigned)nfill), 256, 0, st>>>(fills);
        nk++;
    }
    if (plan.njobs > 0) {
        k_batch_plan<<<plan.njobs, 1024, 0, st>>>(plan);
        k_batch_scan<<<1, 1024, 0, st>>>(plan);
        nk += 2;
        // 32 columns per round: the batch's short strings mostly end within
        // one (config 5: 1.38 ms per step, 1.70 with 16 columns, 1.72 with 8)
        if (defer) {
            k_batch_band<32, true><<<sms * 4, 256, 0, st>>>(plan, false, status);
            launch_list_scatter(st, sms, plan.list, plan.work);
            k_batch_band<32, false><<<sms * 4, 256, 0, st>>>(plan, true, status);
            nk += 3;
        } else if (plan.nbanded > 0) {
            k_batch_band<32, false><<<sms * 4, 256, 0, st>>>(plan, false, status);
            nk++;
        }
        if (plan.nbanded < plan.njobs) {
            k_batch_search<<<sms * 3, 256, kBatchSearchSmem, st>>>(plan, status, 1u);
            nk++;
        }
    }
    if (kernels) *kernels = nk;
    return cudaGetLastError();
}

}  // namespace blg
