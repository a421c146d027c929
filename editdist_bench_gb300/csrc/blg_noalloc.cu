// cdist without any device allocation: blg_cdist_noalloc.
//
// Who needs it: programs that host this library inside an engine that owns
// the GPU's memory — a database or stream processor whose plugins must run
// inside the memory the engine reserved up front, or a latency-bound service
// that must not call cudaMalloc on its request path (an allocation can block
// on the device, fail under memory pressure, or fragment the engine's own
// pool). Those callers place the strings and the output in device memory
// they already own and need the distance computation itself to allocate
// nothing.
//
// How: the only scratch memory of the search path — the per-query Peq
// tables — lives in the file-scope array below, a fixed 2 MiB per device,
// held for as long as the library is loaded. Queries are processed in
// chunks of kChunkQueries, so any number of queries fits; the limit is the
// query length (kMaxQueryLen bytes, i.e. 4 Peq words per table).
//
// Host code must not pass `g_noalloc_peq` itself to a kernel: on the host
// that name is a stand-in, not a device address. The device address comes
// from cudaGetSymbolAddress, looked up once per device (first call on that
// device, with the device current) and cached. With CUDA's lazy module
// loading that first call is also when this file's kernels and the 2 MiB
// array are loaded onto the device, so it can still fail for lack of memory:
// callers make one small call at start-up, before any stream capture. The
// cached address belongs to the device's primary context; after a device
// reset (cudaDeviceReset) this entry point must not be used again in the
// process.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/bitlev_gb300.h"
#include "blg_context.h"
#include "blg_kernels.cuh"

namespace {

using namespace blg;

constexpr int kNoAllocWords = 4;                       // Peq words per query table
constexpr int kMaxQueryLen = 64 * kNoAllocWords;      // 256 bytes
constexpr int kChunkQueries = 256;                     // tables per chunk
constexpr int kTableWords = 256 * kNoAllocWords;       // u64 per table
constexpr int kMaxDevices = 64;

// 256 tables x 256 rows x 4 words x 8 B = 2 MiB per device.
static __device__ __align__(256) uint64_t g_noalloc_peq[(size_t)kChunkQueries * kTableWords];

std::mutex g_sym_mu;
uint64_t *g_sym_ptr[kMaxDevices] = {nullptr};

// One CTA per query of the chunk: validate the length, build its table.
__global__ void __launch_bounds__(256) k_na_build(DevStrings Q, int64_t q0, uint64_t *scratch,
                                                  uint32_t *status) {
    extern __shared__ uint64_t tab[];
    int m;
    const uint8_t *p = string_at(Q, q0 + blockIdx.x, m, status);
    if (m > kMaxQueryLen) {
        if (threadIdx.x == 0) atomicOr(status, ST_TOO_LONG);
        m = 0;                                     // the search skips this row
    }
    build_peq_block(p, m, kNoAllocWords, tab, scratch + (size_t)blockIdx.x * kTableWords);
}

template <bool HASK>
__device__ __forceinline__ int na_dist(int nw, const uint64_t *peq, int m, const uint8_t *t, int n, int k,
                                       Units u) {
    switch (nw) {
    case 1: { RowAddr<1> ra; ra.init(u); return dist_seq_any<1, HASK>(peq, m, t, n, k, u, ra); }
    case 2: { RowAddr<2> ra; ra.init(u); return dist_seq_any<2, HASK>(peq, m, t, n, k, u, ra); }
    case 3: { RowAddr<3> ra; ra.init(u); return dist_seq_any<3, HASK>(peq, m, t, n, k, u, ra); }
    default: { RowAddr<4> ra; ra.init(u); return dist_seq_any<4, HASK>(peq, m, t, n, k, u, ra); }
    }
}

// grid: x = candidate tiles of 4*blockDim.x, y = groups of `qpb` chunk queries.
template <bool HASK>
__global__ void __launch_bounds__(256) k_na_search(DevStrings C, DevStrings Q, int64_t q0, int cnt,
                                                   int qpb, const uint64_t *scratch, int k, int dtype,
                                                   void *out, uint32_t *status, uint32_t unit) {
    extern __shared__ uint64_t s_peq[];
    const Units u{unit, unit + unit};
    const int64_t nc = C.n;
    const int64_t c0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * 4;
    const int ccnt = (int)(c0 >= nc ? 0 : (nc - c0 < 4 ? nc - c0 : 4));
    const uint8_t *tp0 = C.buf, *tp1 = C.buf, *tp2 = C.buf, *tp3 = C.buf;
    int tn0 = 0, tn1 = 0, tn2 = 0, tn3 = 0;
    if (ccnt > 0) tp0 = string_at(C, c0, tn0, status);
    if (ccnt > 1) tp1 = string_at(C, c0 + 1, tn1, status);
    if (ccnt > 2) tp2 = string_at(C, c0 + 2, tn2, status);
    if (ccnt > 3) tp3 = string_at(C, c0 + 3, tn3, status);
    const int i_begin = blockIdx.y * qpb;
    const int i_end = min(i_begin + qpb, cnt);
    for (int i = i_begin; i < i_end; i++) {
        int m;
        string_at(Q, q0 + i, m, status);
        if (m > kMaxQueryLen) continue;            // uniform per block; flagged by k_na_build
        const int nw = m > 64 ? (m + 63) >> 6 : 1;
        __syncthreads();
        const uint64_t *src = scratch + (size_t)i * kTableWords;
        for (int x = threadIdx.x; x < 256 * nw; x += blockDim.x)
            s_peq[x] = src[(x / nw) * kNoAllocWords + (x % nw)];
        __syncthreads();
        if (ccnt == 0) continue;
        const int d0 = na_dist<HASK>(nw, s_peq, m, tp0, tn0, k, u);
        const int d1 = ccnt > 1 ? na_dist<HASK>(nw, s_peq, m, tp1, tn1, k, u) : 0;
        const int d2 = ccnt > 2 ? na_dist<HASK>(nw, s_peq, m, tp2, tn2, k, u) : 0;
        const int d3 = ccnt > 3 ? na_dist<HASK>(nw, s_peq, m, tp3, tn3, k, u) : 0;
        store4(out, dtype, (q0 + i) * nc + c0, ccnt, d0, d1, d2, d3);
    }
}

// Device address of the scratch array for the current device (looked up once).
int scratch_address(blg_ctx *c, uint64_t **out) {
    if (c->device < 0 || c->device >= kMaxDevices) return fail(c, BLG_ERR_ARG, "device index out of range");
    std::lock_guard<std::mutex> lock(g_sym_mu);
    if (!g_sym_ptr[c->device]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_peq);
        if (e != cudaSuccess) return cuda_fail(c, e, "cudaGetSymbolAddress(no-alloc scratch)");
        g_sym_ptr[c->device] = static_cast<uint64_t *>(p);
    }
    *out = g_sym_ptr[c->device];
    return BLG_OK;
}

bool aligned(const void *p, uintptr_t a) { return (reinterpret_cast<uintptr_t>(p) & (a - 1)) == 0; }

}  // namespace

extern "C" int blg_cdist_noalloc(blg_ctx *c, const uint8_t *d_buf_q, size_t q_bytes,
                                 const int64_t *d_off_q, int64_t nq, const uint8_t *d_buf_c,
                                 size_t c_bytes, const int64_t *d_off_c, int64_t nc, int32_t max_dist,
                                 int32_t dtype, void *d_out) {
    if (!c) return BLG_ERR_ARG;
    std::lock_guard<std::mutex> lock(c->mu);
    c->err.clear();
    if (cudaSetDevice(c->device) != cudaSuccess) return fail(c, BLG_ERR_CUDA, "cudaSetDevice");
    if (dtype != BLG_INT32 && dtype != BLG_UINT16 && dtype != BLG_UINT8)
        return fail(c, BLG_ERR_ARG, "dtype must be int32, uint16 or uint8");
    if (nq < 0 || nc < 0) return fail(c, BLG_ERR_ARG, "negative count");
    if (nq == 0 || nc == 0) return BLG_OK;
    if (!d_buf_q || !d_off_q || !d_buf_c || !d_off_c || !d_out)
        return fail(c, BLG_ERR_ARG, "null device pointer");
    // the string buffers feed aligned 4-byte window loads from their 16-byte
    // aligned start; offsets are read as int64; results are stored as whole
    // elements (vector stores only where 16 bytes line up)
    if (!aligned(d_buf_q, 16) || !aligned(d_buf_c, 16))
        return fail(c, BLG_ERR_ARG, "string buffers must be 16-byte aligned");
    if (!aligned(d_off_q, 8) || !aligned(d_off_c, 8))
        return fail(c, BLG_ERR_ARG, "offset arrays must be 8-byte aligned");
    if (!aligned(d_out, dtype == BLG_INT32 ? 4 : dtype == BLG_UINT16 ? 2 : 1))
        return fail(c, BLG_ERR_ARG, "output must be aligned to its element size");
    if (q_bytes < 16 || c_bytes < 16)
        return fail(c, BLG_ERR_ARG, "string buffers need 16 readable bytes after the last string");
    uint64_t *scratch = nullptr;
    int rc = scratch_address(c, &scratch);
    if (rc) return rc;
    // offsets are relative to the buffer start; the last 16 bytes are read slack
    DevStrings Q, C;
    Q.buf = d_buf_q; Q.off = d_off_q; Q.n = nq; Q.base = 0; Q.bytes = (int64_t)q_bytes - 16;
    C.buf = d_buf_c; C.off = d_off_c; C.n = nc; C.base = 0; C.bytes = (int64_t)c_bytes - 16;
    const bool hask = max_dist >= 0;
    const size_t smem = (size_t)kTableWords * sizeof(uint64_t);
    const int64_t tiles = (nc + 1023) / 1024;
    for (int64_t q0 = 0; q0 < nq; q0 += kChunkQueries) {
        const int cnt = (int)(nq - q0 < kChunkQueries ? nq - q0 : kChunkQueries);
        k_na_build<<<cnt, 256, smem, c->stream>>>(Q, q0, scratch, c->d_status);
        int qpb = (int)((int64_t)cnt * tiles / ((int64_t)c->sms * 8));
        qpb = qpb < 1 ? 1 : (qpb > 16 ? 16 : qpb);
        const dim3 grid((unsigned)tiles, (unsigned)((cnt + qpb - 1) / qpb));
        if (hask)
            k_na_search<true><<<grid, 256, smem, c->stream>>>(C, Q, q0, cnt, qpb, scratch, max_dist,
                                                              dtype, d_out, c->d_status, 1u);
        else
            k_na_search<false><<<grid, 256, smem, c->stream>>>(C, Q, q0, cnt, qpb, scratch, max_dist,
                                                               dtype, d_out, c->d_status, 1u);
        c->launches += 2;
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            // earlier chunks may still be running on the caller's buffers:
            // let them finish and clear any status they raised before
            // reporting the launch error
            const int rc_launch = cuda_fail(c, e, "blg_cdist_noalloc launch");
            const std::string msg = c->err;
            sync_and_status(c);
            c->err = msg;
            return rc_launch;
        }
    }
    rc = sync_and_status(c);
    if (rc == BLG_ERR_ARG && c->err.find("longer than") != std::string::npos)
        c->err = "a query is longer than 256 bytes, the limit of blg_cdist_noalloc's fixed scratch";
    return rc;
}
