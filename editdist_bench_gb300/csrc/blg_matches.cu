// Matches-only output of a thresholded search: every (query, choice) whose
// distance is <= max_dist, as (query, choice, distance) records in row-major
// order, instead of the dense query x choice matrix. The reference names
// this as the output fuzzy search usually wants and leaves it undone
// (README.md:319-321); it cuts the result stream from nq*nc elements to the
// matches.
//
// The search fills a dense scratch matrix (uint8 while k+1 fits, else
// uint16 or int32) on the device; a stream compaction then keeps the
// matches:
//   1. k_match_count: every CTA counts the elements <= k of its block of
//      kMatchBlock elements (16-byte loads, SWAR compares for bytes);
//   2. k_match_scan: one CTA turns the block counts into exclusive offsets
//      and the total;
//   3. k_match_emit: every CTA re-reads its block, ranks its matches (per
//      thread a contiguous run of elements, then a CTA scan) and writes each
//      match's record at its block offset + rank, so the records come out in
//      element order, i.e. sorted by (query, choice).
// Records past `capacity` are not written; the total is reported anyway.
#include "../../include/bitlev_gb300.h"
#include "blg_kernels.cuh"

#include <algorithm>

namespace blg {

constexpr int kMatchThreads = 256;
constexpr int kMatchPerThread = 64;                          // elements per thread per block
constexpr int64_t kMatchBlock = (int64_t)kMatchThreads * kMatchPerThread;

// Elements <= k among the 16 bytes / 8 halves / 4 words of one 16-byte chunk,
// as a bit mask in element order (bit i = element i matches).
__device__ __forceinline__ uint32_t match_mask(const uint4 v, uint32_t k, uint8_t) {
    const uint32_t kk = k * 0x01010101u;
    uint32_t m = 0;
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const uint32_t le = __vcmpleu4(w[i], kk);            // 0xff per byte <= k
        // gather the four byte flags into 4 bits
        m |= ((le & 0x01u) | ((le >> 7) & 0x02u) | ((le >> 14) & 0x04u) | ((le >> 21) & 0x08u)) << (4 * i);
    }
    return m;
}
__device__ __forceinline__ uint32_t match_mask(const uint4 v, uint32_t k, uint16_t) {
    const uint32_t kk = k * 0x00010001u;
    uint32_t m = 0;
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const uint32_t le = __vcmpleu2(w[i], kk);            // 0xffff per half <= k
        m |= ((le & 0x1u) | ((le >> 15) & 0x2u)) << (2 * i);
    }
    return m;
}
__device__ __forceinline__ uint32_t match_mask(const uint4 v, uint32_t k, int32_t) {
    return ((uint32_t)v.x <= k ? 1u : 0u) | ((uint32_t)v.y <= k ? 2u : 0u) | ((uint32_t)v.z <= k ? 4u : 0u) |
           ((uint32_t)v.w <= k ? 8u : 0u);
}

// Mask of the matches among this thread's elements [e0, e0 + 64) of the
// matrix (elements >= n never match), one bit per element, 64 bits.
template <typename T>
__device__ __forceinline__ uint64_t thread_matches(const T *dense, int64_t n, int64_t e0, uint32_t k) {
    constexpr int kPerChunk = 16 / sizeof(T);
    uint64_t bits = 0;
    if (e0 + kMatchPerThread <= n) {
        const uint4 *p = reinterpret_cast<const uint4 *>(dense + e0);
#pragma unroll
        for (int c = 0; c < kMatchPerThread / kPerChunk; c++)
            bits |= (uint64_t)match_mask(__ldg(p + c), k, T()) << (c * kPerChunk);
    } else {
        for (int i = 0; i < kMatchPerThread && e0 + i < n; i++)
            if ((uint32_t)dense[e0 + i] <= k) bits |= 1ull << i;
    }
    return bits;
}

template <typename T>
__global__ void __launch_bounds__(kMatchThreads) k_match_count(const T *dense, int64_t n, uint32_t k,
                                                               int64_t *counts) {
    __shared__ int warp_sum[kMatchThreads / 32];
    const int64_t nblocks = (n + kMatchBlock - 1) / kMatchBlock;
    for (int64_t b = blockIdx.x; b < nblocks; b += gridDim.x) {
        const int64_t e0 = b * kMatchBlock + (int64_t)threadIdx.x * kMatchPerThread;
        int cnt = e0 < n ? __popcll(thread_matches(dense, n, e0, k)) : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(kFull, cnt, o);
        if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = cnt;
        __syncthreads();
        if (threadIdx.x == 0) {
            int64_t s = 0;
            for (int w = 0; w < kMatchThreads / 32; w++) s += warp_sum[w];
            counts[b] = s;
        }
        __syncthreads();
    }
}

// One CTA: counts[0..nb) -> exclusive offsets in place; *total = the sum.
__global__ void __launch_bounds__(1024) k_match_scan(int64_t *counts, int64_t nb, int64_t *total) {
    __shared__ int64_t part[1024];
    const int t = threadIdx.x;
    const int64_t per = (nb + 1023) / 1024;
    const int64_t i0 = min(nb, t * per), i1 = min(nb, i0 + per);
    int64_t s = 0;
    for (int64_t i = i0; i < i1; i++) s += counts[i];
    part[t] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {                     // inclusive Hillis-Steele scan of the parts
        const int64_t v = t >= o ? part[t - o] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    int64_t run = part[t] - s;
    for (int64_t i = i0; i < i1; i++) {
        const int64_t c = counts[i];
        counts[i] = run;
        run += c;
    }
    if (t == 1023) *total = part[1023];
}

template <typename T>
__global__ void __launch_bounds__(kMatchThreads) k_match_emit(const T *dense, int64_t n, uint32_t k,
                                                              const int64_t *offsets, int64_t nc, int64_t row0,
                                                              blg_match *out, int64_t capacity) {
    __shared__ int warp_sum[kMatchThreads / 32];
    const int64_t nblocks = (n + kMatchBlock - 1) / kMatchBlock;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int64_t b = blockIdx.x; b < nblocks; b += gridDim.x) {
        const int64_t e0 = b * kMatchBlock + (int64_t)threadIdx.x * kMatchPerThread;
        uint64_t bits = e0 < n ? thread_matches(dense, n, e0, k) : 0;
        const int cnt = __popcll(bits);
        int incl = cnt;                                      // rank among the CTA's threads
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += v;
        }
        if (lane == 31) warp_sum[warp] = incl;
        __syncthreads();
        int before = 0;
        for (int w = 0; w < warp; w++) before += warp_sum[w];
        int64_t at = offsets[b] + before + incl - cnt;
        while (bits) {
            const int i = __ffsll((long long)bits) - 1;
            bits &= bits - 1;
            if (at < capacity) {
                const int64_t e = e0 + i;
                blg_match r;
                r.query = row0 + e / nc;
                r.choice = e % nc;
                r.dist = (int32_t)dense[e];
                r.reserved = 0;
                out[at] = r;
            }
            at++;
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------- launchers --
template <typename T>
static cudaError_t match_compact_t(cudaStream_t st, int sms, const void *dense, int64_t n, int k,
                                   int64_t *counts, int64_t *total, int64_t nc, int64_t row0, blg_match *out,
                                   int64_t capacity, bool emit) {
    const int64_t nb = (n + kMatchBlock - 1) / kMatchBlock;
    const int grid = (int)std::min<int64_t>(nb, (int64_t)sms * 8);
    if (!emit) {
        k_match_count<T><<<grid, kMatchThreads, 0, st>>>(static_cast<const T *>(dense), n, (uint32_t)k, counts);
        k_match_scan<<<1, 1024, 0, st>>>(counts, nb, total);
    } else {
        k_match_emit<T><<<grid, kMatchThreads, 0, st>>>(static_cast<const T *>(dense), n, (uint32_t)k, counts, nc,
                                                        row0, out, capacity);
    }
    return cudaGetLastError();
}

int64_t match_blocks(int64_t n) { return (n + kMatchBlock - 1) / kMatchBlock; }

// Pass 1+2 (emit = false): block offsets into `counts` (match_blocks(n)
// entries) and the total into *total (device). Pass 3 (emit = true): the
// records. `dense` is 16-byte aligned, n elements of dtype.
cudaError_t launch_match_compact(cudaStream_t st, int sms, int dtype, const void *dense, int64_t n, int k,
                                 int64_t *counts, int64_t *total, int64_t nc, int64_t row0, blg_match *out,
                                 int64_t capacity, bool emit) {
    if (n <= 0) return cudaSuccess;
    if (dtype == DT_UINT8)
        return match_compact_t<uint8_t>(st, sms, dense, n, k, counts, total, nc, row0, out, capacity, emit);
    if (dtype == DT_UINT16)
        return match_compact_t<uint16_t>(st, sms, dense, n, k, counts, total, nc, row0, out, capacity, emit);
    return match_compact_t<int32_t>(st, sms, dense, n, k, counts, total, nc, row0, out, capacity, emit);
}

// ---------------------------------------------------- 4-bit packed results --
// Results e0 .. e1-1 of a uint8 result array, each saturated at 15, two per
// byte: element e goes to byte e / 2, the low nibble for even e. e0 is even,
// so every output byte comes from two elements of this range (the last one
// has a zero high nibble when e1 is odd). One thread per 16 output bytes:
// two 16-byte loads, one 16-byte store where the addresses line up, else
// byte by byte.
__device__ __forceinline__ uint32_t nibble_pack4(uint32_t x) {    // 4 bytes -> 2 bytes (low 16 bits)
    x = __vminu4(x, 0x0f0f0f0fu);
    const uint32_t y = (x & 0x000f000fu) | ((x >> 4) & 0x00f000f0u);
    return __byte_perm(y, 0u, 0x4420);                             // bytes 0 and 2
}

__global__ void __launch_bounds__(256) k_pack_nibbles(const uint8_t *src, int64_t e0, int64_t e1, uint8_t *dst) {
    const int64_t b0 = e0 >> 1, b1 = (e1 + 1) >> 1;              // output bytes [b0, b1)
    const int64_t nb = b1 - b0;
    const bool vec = ((reinterpret_cast<uintptr_t>(src + e0) | reinterpret_cast<uintptr_t>(dst + b0)) & 15) == 0;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t * 16 < nb; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t o = b0 + t * 16;                             // first output byte of this thread
        if (vec && o + 16 <= b1 && 2 * (o + 16) <= e1) {
            const uint4 a = *reinterpret_cast<const uint4 *>(src + 2 * o);
            const uint4 b = *reinterpret_cast<const uint4 *>(src + 2 * o + 16);
            uint4 r;
            r.x = nibble_pack4(a.x) | (nibble_pack4(a.y) << 16);
            r.y = nibble_pack4(a.z) | (nibble_pack4(a.w) << 16);
            r.z = nibble_pack4(b.x) | (nibble_pack4(b.y) << 16);
            r.w = nibble_pack4(b.z) | (nibble_pack4(b.w) << 16);
            *reinterpret_cast<uint4 *>(dst + o) = r;
        } else {
            for (int64_t q = o; q < b1 && q < o + 16; q++) {
                const uint32_t lo = min((uint32_t)src[2 * q], 15u);
                const uint32_t hi = 2 * q + 1 < e1 ? min((uint32_t)src[2 * q + 1], 15u) : 0u;
                dst[q] = (uint8_t)(lo | (hi << 4));
            }
        }
    }
}

cudaError_t launch_pack_nibbles(cudaStream_t st, int sms, const uint8_t *src, int64_t e0, int64_t e1, uint8_t *dst) {
    if (e1 <= e0) return cudaSuccess;
    if (e0 & 1) return cudaErrorInvalidValue;
    const int64_t threads = ((e1 - e0 + 1) / 2 + 15) / 16;
    const int grid = (int)std::min<int64_t>((threads + 255) / 256, (int64_t)sms * 16);
    k_pack_nibbles<<<grid, 256, 0, st>>>(src, e0, e1, dst);
    return cudaGetLastError();
}

}  // namespace blg

