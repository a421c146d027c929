// Host runtime of the C-ABI (include/bitlev_gb300.h).
//
// Replaces the CuPy driver of the reference (bitlev/gpu.py:54-138,
// bench/cudamyers.py:83-174): packing stays with the caller, classification
// of work by length happens here in C++ (queries) or on the device (pairs,
// after trimming), kernels run on the context's stream, device memory comes
// from the stream-ordered allocator (cudaMallocAsync) so repeated calls do
// not synchronise on allocation.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <array>
#include <condition_variable>
#include <functional>
#include <thread>
#include <cstdio>
#include <cstdlib>
#include <unistd.h>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/bitlev_gb300.h"
#include "blg_context.h"
#include "blg_device.cuh"
#include "blg_batch.h"
#include "blg_internal.h"
#include "blg_sched.h"

namespace blg {
cudaError_t launch_build_peq(cudaStream_t st, const DevStrings &Q, const int32_t *qidx, int nq, int nwc,
                             uint64_t *peq, uint32_t *status);
cudaError_t launch_search_seq(cudaStream_t st, int nw, bool hask, const DevStrings &C,
                              const SearchClass &cls, int qpb, int k, int dtype, void *out,
                              uint32_t *status);
bool search_pfx_supported(int nw);
cudaError_t launch_search_pfx(cudaStream_t st, int sms, int ctas_per_sm, int nw, const PrefixChoices &P,
                              const SearchClass &cls, unsigned long long *work, int dtype, void *out);
cudaError_t launch_prefix_text(cudaStream_t st, int sms, const DevStrings &C, const int32_t *order,
                               const int64_t *woff, const uint16_t *rowoff, uint32_t *text, int32_t *len,
                               uint32_t *status);
cudaError_t launch_search_tt(cudaStream_t st, int nw, bool hask, const TransposedChoices &T,
                             const SearchClass &cls, int qpb, int k, int dtype, void *out);
cudaError_t launch_transpose_choices(cudaStream_t st, int sms, const DevStrings &C, const int64_t *base,
                                     uint32_t *words, int32_t *len, uint32_t *status);
cudaError_t launch_search_lanes(cudaStream_t st, bool hask, const DevStrings &C, const SearchClass &cls,
                                int nwc, int k, int dtype, void *out, uint32_t *status);
cudaError_t launch_pairs_long(cudaStream_t st, int grid, bool hask, const LongQueue &q, int k,
                              int dtype, void *out);
cudaError_t launch_pairs_staged(cudaStream_t st, int sms, bool hask, const DevStrings &A, const DevStrings &B,
                                int k, int dtype, void *out, const LongQueue &q, uint32_t *status);
cudaError_t launch_fill(cudaStream_t st, int sms, void *out, int64_t n, int dtype, uint32_t v);
cudaError_t launch_match_compact(cudaStream_t st, int sms, int dtype, const void *dense, int64_t n, int k,
                                 int64_t *counts, int64_t *total, int64_t nc, int64_t row0, blg_match *out,
                                 int64_t capacity, bool emit);
int64_t match_blocks(int64_t n);
cudaError_t launch_pack_nibbles(cudaStream_t st, int sms, const uint8_t *src, int64_t e0, int64_t e1, uint8_t *dst);
cudaError_t launch_pairs_tile(cudaStream_t st, int sms, int buffers, bool hask, const DevStrings &A,
                              const DevStrings &B, int tile_pairs, int k, int dtype, void *out, const LongQueue &q,
                              uint32_t *status, int32_t wait_polls, bool trusted, int variant, const uint32_t *alpha);
cudaError_t launch_pairs_prep(cudaStream_t st, int grid, bool hask, bool feat, bool band, const DevStrings &A,
                              const DevStrings &B, int k, int dtype, void *out, const PairsPlan &plan,
                              bool lengap_key, uint32_t *status);
cudaError_t launch_order(cudaStream_t st, int sms, const PairsPlan &plan);
cudaError_t launch_solve(cudaStream_t st, int sms, bool hask, const PairsPlan &plan, int k, int dtype,
                         void *out, int32_t *exit_log, bool any_long);
cudaError_t launch_solve_band(cudaStream_t st, int sms, int ctas_per_sm, const PairsPlan &plan, int k, int dtype, void *out,
                              int32_t *exit_log, int variant, const uint32_t *alpha);
cudaError_t launch_byte_presence(cudaStream_t st, int sms, const DevStrings &A, const DevStrings &B, uint32_t *mask);
}  // namespace blg
int sched_model_ensure(blg_ctx *c, blg_sched_model **out);
cudaError_t launch_mlp_keys(cudaStream_t st, int sms, const blg_sched_model *m, const blg::PairsPlan &plan,
                            bool band);
cudaError_t launch_collect_rows(cudaStream_t st, int sms, const blg::PairsPlan &plan, const int32_t *cols,
                                int64_t stride, int64_t max_rows, half *x, float *y, int64_t *n_rows);
int sched_train_rows(blg_ctx *c, blg_sched_model *m, half *x, float *y, const int64_t *d_rows, int64_t rows,
                     int epochs, float lr, int batch, float *loss_out);
bool sched_model_trained(const blg_sched_model *m);
namespace blg {
cudaError_t launch_sorted_offsets(cudaStream_t st, int sms, const int64_t *lstart, int64_t n_len, int64_t min_len,
                                  const int64_t *bstart, int64_t n, int64_t *soff);
cudaError_t launch_gather_strings(cudaStream_t st, int sms, const DevStrings &src, const int32_t *perm,
                                  const int64_t *dst_off, uint8_t *dst, int64_t n, uint32_t *status);
cudaError_t launch_sketch_strings(cudaStream_t st, int sms, const DevStrings &S, uint64_t *sketch, uint4 *counts,
                                  uint32_t *status);
cudaError_t launch_search_band(cudaStream_t st, int sms, int ctas_per_sm, int round, int jobsz, const SurvClasses &C,
                               const DevStrings &CS, const int32_t *perm, const uint4 *ccnt, const uint4 *qcnt, int k,
                               int dtype, void *out, int64_t nc, const SurvRows *rows, const ResultList *list,
                               const FillItems *fill, uint32_t *status);
cudaError_t launch_surv_plan(cudaStream_t st, const SurvClasses &C, const int64_t *lstart, int64_t min_len,
                             int64_t n_len, int k, int tile);
cudaError_t launch_search_surv(cudaStream_t st, int sms, int nw, const DevStrings &CS, const int32_t *perm,
                               const SearchClass &cls, const int32_t *lo, const int32_t *hi,
                               const int64_t *tile_start, int32_t *work, int k, int dtype, void *out,
                               int64_t nc, uint32_t *status);
}  // namespace blg

using namespace blg;

namespace {

constexpr int kSeqMaxWords = 8;          // queries up to 512: sequential words per thread
constexpr int kLaneMaxWords = 32;        // queries up to 2048: lane-spread

struct OwnedStrings {
    DevStrings d;
    void *mem_buf = nullptr;   // the one allocation: d.buf - 16, with the offsets after the bytes
};

}  // namespace


struct blg_pairs {
    OwnedStrings a, b;
    int64_t n = 0;
    int64_t cap[kLongClasses] = {0, 0, 0, 0, 0};
    int64_t short_pairs = 0;      // pairs whose shorter string is at most 32 bytes
    bool trusted = false;         // the host pass found every offset pair in order (kernels skip their checks)
    int64_t len_max_side = 0;     // total bytes of the larger side (a or b)
    void *q_items = nullptr;      // all class regions, one allocation
    int32_t *q_ctr = nullptr;     // counts[5], heads[5]
    // scheduled path (prep -> order -> solve), allocated on first use
    int64_t pcap[kPairClasses] = {0, 0, 0, 0, 0, 0};
    void *plan_mem = nullptr;     // raw + sorted records, keys
    half *feat_mem = nullptr;     // feature rows (learned schedule)
    int32_t *plan_ctr = nullptr;  // count, head, hist, cursor
    // the bytes the set uses (8 words) and their count on the host (-1: not
    // known; the banded solver's one-row-per-byte variant needs at most 15)
    uint32_t *d_alpha = nullptr;
    int nsym = -1;
    // resident runs as a CUDA graph (pairs_run_graph): the launches of one
    // run, captured once its parameters repeat, replayed while they stay
    struct GraphKey {
        int k = 0, dtype = -1, sched = -1, learned = 0, band_ctas = 0, tile_shape = 0;
        void *out = nullptr;
        bool operator==(const GraphKey &o) const {
            return k == o.k && dtype == o.dtype && sched == o.sched && learned == o.learned &&
                   band_ctas == o.band_ctas && tile_shape == o.tile_shape && out == o.out;
        }
    };
    GraphKey g_last;              // parameters of the previous run
    bool g_have_last = false;
    cudaGraphExec_t gexec = nullptr;
    GraphKey g_key;               // parameters gexec was captured with
    int64_t g_launches = 0;       // kernels in gexec
};

struct blg_search {
    OwnedStrings q, c;
    int64_t nq = 0, nc = 0;
    struct Cls {
        int nw;          // words (seq) or table stride (lanes)
        bool lanes;
        int nq;
        int32_t *qidx, *qlen;      // queries of the class, sorted by length
        uint64_t *peq;
        int32_t *lo, *hi, *work;   // survivor plan (thresholded runs)
        int64_t *tile_start;
        void *mem;                 // the one device block all of the above live in
        std::vector<int32_t> h_qlen;   // host copy of qlen
    };
    std::vector<Cls> cls;
    std::vector<int64_t> h_oq;    // host copy of the query offsets (resident searches: class rebuilds)
    // choices sorted by length (thresholded runs): cs = sorted copy,
    // perm[i] = original index of sorted choice i, lstart[L - min_len] =
    // first sorted index of length L (n_len + 1 entries)
    bool lsorted = false;
    OwnedStrings cs;
    void *sorted_mem = nullptr;   // one device block: perm, lstart, bucket starts, offsets, sketches, bytes
    int32_t *perm = nullptr;
    int64_t *lstart = nullptr;
    int64_t min_len = 0, n_len = 0;
    std::vector<int64_t> h_lstart;   // host copy of lstart
    // 4-gram sketches and binned 4-gram counts: of the length-sorted choices
    // and of the queries
    uint64_t *csk = nullptr, *qsk = nullptr;
    uint4 *ccnt = nullptr, *qcnt = nullptr;
    void *sk_mem = nullptr;           // the queries' sketch block when this search owns it
    // choices in tile-transposed form (exact and unsorted runs), when the
    // padding to each tile's longest choice stays small
    bool tt = false;
    // choices sorted lexicographically for the exact search with prefix
    // reuse (PrefixChoices), when the sorted neighbours share enough
    bool pfx = false;
    void *pfx_mem = nullptr;          // one device block: order, restarts, base, words, len, orig, work
    PrefixChoices pd;
    unsigned long long *pfx_work = nullptr;
    double pfx_saving = 0.0;          // fraction of text columns the restarts skip
    uint32_t *tt_words = nullptr;
    int64_t *tt_base = nullptr;
    int32_t *tt_len = nullptr;
};

// ------------------------------------------------------------ helpers --
int fail(blg_ctx *c, int code, const std::string &msg) {
    if (c) c->err = msg;
    return code;
}

int cuda_fail(blg_ctx *c, cudaError_t e, const char *what) {
    if (e == cudaErrorMemoryAllocation)
        return fail(c, BLG_ERR_ALLOC, std::string(what) + ": " + cudaGetErrorString(e));
    return fail(c, BLG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}


template <typename F>
static cudaError_t launch(blg_ctx *c, const char *name, F &&fn) {
    blg_ctx::ProfRec r{name, nullptr, nullptr};
    if (c->prof) {
        cudaEventCreate(&r.e0);
        cudaEventCreate(&r.e1);
        cudaEventRecord(r.e0, c->stream);
    }
    cudaError_t e = fn();
    c->launches++;
    if (c->prof) {
        cudaEventRecord(r.e1, c->stream);
        c->prof_recs.push_back(r);
    }
    return e;
}

static cudaError_t dev_alloc(blg_ctx *c, void **p, size_t bytes) {
    if (c->fault_alloc_after >= 0 && c->fault_alloc_after-- == 0) {   // injected failure (tests)
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMallocAsync(p, bytes ? bytes : 16, c->stream);
}

static void dev_free(blg_ctx *c, void *p) {
    if (p) cudaFreeAsync(p, c->stream);
}

static int check_offsets_host(blg_ctx *c, const int64_t *off, int64_t n) {
    if (n < 0) return fail(c, BLG_ERR_ARG, "negative count");
    if (n > 0 && !off) return fail(c, BLG_ERR_ARG, "null offsets");
    if (n > 0 && (off[0] < 0 || off[n] < off[0]))
        return fail(c, BLG_ERR_ARG, "offsets must start >= 0 and end >= start");
    return BLG_OK;
}

// Device storage for a packed string set: the bytes with 16 bytes of
// (zeroed) slack on both sides, and the offsets. Nothing is copied yet.
static int alloc_strings(blg_ctx *c, const uint8_t *buf, const int64_t *off, int64_t n, OwnedStrings &o) {
    int rc = check_offsets_host(c, off, n);
    if (rc) return rc;
    const int64_t base = n > 0 ? off[0] : 0;
    const int64_t bytes = n > 0 ? off[n] - off[0] : 0;
    if (bytes > 0 && !buf) return fail(c, BLG_ERR_ARG, "null buffer");
    // one block: 16 bytes of slack | the bytes | 48 bytes of slack | offsets (256-byte aligned)
    const size_t o_off = ((size_t)bytes + kSlackBefore + kSlackAfter + 255) & ~size_t(255);
    CK(dev_alloc(c, &o.mem_buf, o_off + sizeof(int64_t) * (size_t)(n + 1)), "cudaMallocAsync(strings)");
    uint8_t *dbuf = (uint8_t *)o.mem_buf + kSlackBefore;
    // only the slack on either side needs defined contents
    CK(cudaMemsetAsync(o.mem_buf, 0, kSlackBefore, c->stream), "cudaMemsetAsync(slack)");
    CK(cudaMemsetAsync(dbuf + bytes, 0, kSlackAfter, c->stream), "cudaMemsetAsync(slack)");
    o.d.buf = dbuf;
    o.d.off = (const int64_t *)((uint8_t *)o.mem_buf + o_off);
    o.d.n = n;
    o.d.base = base;
    o.d.bytes = bytes;
    return BLG_OK;
}

// Copy strings [i0, i1) of a packed set (and offsets i0..i1) into storage
// made by alloc_strings, on stream `st`.
static int copy_strings(blg_ctx *c, const uint8_t *buf, const int64_t *off, int64_t i0, int64_t i1,
                        OwnedStrings &o, cudaStream_t st) {
    if (i1 <= i0) return BLG_OK;
    const int64_t b0 = off[i0] - o.d.base, b1 = off[i1] - o.d.base;
    if (b1 > b0)
        CK(cudaMemcpyAsync((uint8_t *)o.d.buf + b0, buf + off[i0], (size_t)(b1 - b0), cudaMemcpyHostToDevice, st),
           "H2D strings");
    CK(cudaMemcpyAsync(const_cast<int64_t *>(o.d.off) + i0, off + i0, sizeof(int64_t) * (size_t)(i1 - i0 + 1),
                       cudaMemcpyHostToDevice, st), "H2D offsets");
    return BLG_OK;
}

// Copy a packed string set into HBM with 16 bytes of slack on both sides.
static int upload_strings(blg_ctx *c, const uint8_t *buf, const int64_t *off, int64_t n,
                          OwnedStrings &o) {
    int rc = alloc_strings(c, buf, off, n, o);
    if (!rc) rc = copy_strings(c, buf, off, 0, n, o, c->stream);
    return rc;
}

static void free_strings(blg_ctx *c, OwnedStrings &o) {
    dev_free(c, o.mem_buf);
    o = OwnedStrings();
}

static int status_to_rc(blg_ctx *c, uint32_t st) {
    if (!st) return BLG_OK;
    if (st & ST_QUEUE_TIMEOUT) return fail(c, BLG_ERR_TIMEOUT, "a bounded device wait timed out");
    if (st & ST_BAD_OFFSETS) return fail(c, BLG_ERR_ARG, "corrupt offsets (not monotone or out of range)");
    if (st & ST_TOO_LONG)
        return fail(c, BLG_ERR_ARG, "a pattern is longer than 2048 bytes after trimming (unsupported)");
    if (st & ST_QUEUE_OVERFLOW) return fail(c, BLG_ERR_CUDA, "internal work queue overflow");
    return fail(c, BLG_ERR_CUDA, "device status " + std::to_string(st));
}

int sync_and_status(blg_ctx *c) {
    uint32_t st = 0;
    CK(cudaMemcpyAsync(&st, c->d_status, sizeof(st), cudaMemcpyDeviceToHost, c->stream), "D2H status");
    CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    if (st) {
        CK(cudaMemsetAsync(c->d_status, 0, sizeof(uint32_t), c->stream), "reset status");
        CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    }
    return status_to_rc(c, st);
}

// The tuned shapes of the banded kernels for a run's max_dist k (the max_dist
// axis of the autotuner: small k and the rest up to 31 are tuned apart).
static int surv_ctas(const blg_ctx *c, int k) { return k < kSurvWideK ? c->tune.lpt_ctas : c->tune.lpt_ctas_wide; }
static int surv_round(const blg_ctx *c, int k) {
    return k < kSurvWideK ? c->tune.surv_round : c->tune.surv_round_wide;
}
static int band_ctas(const blg_ctx *c, int k) { return k < kBandWideK ? c->tune.band_ctas : c->tune.band_ctas_wide; }

static size_t dtype_size(int dt) { return dt == BLG_UINT8 ? 1 : dt == BLG_UINT16 ? 2 : 4; }

static bool dtype_ok(int dt) { return dt == BLG_INT32 || dt == BLG_UINT16 || dt == BLG_UINT8; }

// 4-bit results (BLG_UINT4): the kernels write uint8, then k_pack_nibbles
// saturates at 15 and packs two results per byte.
static bool dtype_ok_out(int dt) { return dtype_ok(dt) || dt == BLG_UINT4; }
static size_t out_bytes(int dt, int64_t n) {
    return dt == BLG_UINT4 ? (size_t)(n + 1) / 2 : dtype_size(dt) * (size_t)n;
}
static int pack_u4(blg_ctx *c, const void *d8, int64_t e0, int64_t e1, void *d4) {
    CK(launch(c, "pack_u4", [&] {
           return launch_pack_nibbles(c->stream, c->sms, (const uint8_t *)d8, e0, e1, (uint8_t *)d4);
       }), "pack_u4");
    return BLG_OK;
}

// ------------------------------------------------------------- pairs --
// Host pass over the offsets: how many pairs are short (shorter string <= 32
// bytes) and the long-queue capacity per class. Trimming only shortens a
// pattern, so a pair can land in class j only if its untrimmed shorter
// length reaches it. The tile kernel queues every pattern longer than 32
// (32 < m <= 64 goes to class 0 too); the other pairs kernels queue
// patterns longer than 64.
// Persistent host threads for the passes over offsets. Spawning threads per
// call cost about 0.3 ms on the GPU host (Grace), as much as the pass itself,
// and the one-call pipeline waits for the pass before its first kernel.
// run(nt, fn) runs fn(0) on the caller and fn(1..nt-1) on workers, and
// returns when all are done; calls from several contexts take turns.
class HostPool {
public:
    static HostPool &get() {
        static HostPool pool;
        return pool;
    }
    int size() const { return (int)workers_->size() + 1; }
    void run(int nt, const std::function<void(int)> &fn) {
        nt = std::max(1, std::min(nt, size()));
        if (getpid() != owner_) {                   // a forked child: the workers stayed with the parent
            for (int t = 0; t < nt; t++) fn(t);
            return;
        }
        if (nt == 1) {
            fn(0);
            return;
        }
        std::lock_guard<std::mutex> turn(turn_);
        {
            std::lock_guard<std::mutex> g(m_);
            job_ = &fn;
            njob_ = nt;
            remaining_ = nt - 1;
            gen_++;
        }
        cv_.notify_all();
        fn(0);
        std::unique_lock<std::mutex> g(m_);
        done_.wait(g, [&] { return remaining_ == 0; });
        job_ = nullptr;
    }
    ~HostPool() {
        // a forked child has no running workers: their thread objects are
        // left alone (destroying or detaching them there is not defined)
        if (getpid() != owner_) return;
        {
            std::lock_guard<std::mutex> g(m_);
            stop_ = true;
            gen_++;
        }
        cv_.notify_all();
        for (auto &t : *workers_) t.join();
        delete workers_;
    }

private:
    HostPool() : owner_(getpid()) {
        const int n = (int)std::min<unsigned>(8, std::max(1u, std::thread::hardware_concurrency()));
        for (int i = 1; i < n; i++) workers_->emplace_back([this, i] { loop(i); });
    }
    void loop(int idx) {
        uint64_t seen = 0;
        while (true) {
            const std::function<void(int)> *job;
            int nj;
            {
                std::unique_lock<std::mutex> g(m_);
                cv_.wait(g, [&] { return stop_ || gen_ != seen; });
                if (stop_) return;
                seen = gen_;
                job = job_;
                nj = njob_;
            }
            if (idx < nj) {
                (*job)(idx);
                std::lock_guard<std::mutex> g(m_);
                if (--remaining_ == 0) done_.notify_one();
            }
        }
    }
    pid_t owner_;
    std::vector<std::thread> *workers_ = new std::vector<std::thread>();
    std::mutex m_, turn_;
    std::condition_variable cv_, done_;
    const std::function<void(int)> *job_ = nullptr;
    int njob_ = 0, remaining_ = 0;
    uint64_t gen_ = 0;
    bool stop_ = false;
};

static int pairs_classify(blg_ctx *c, const int64_t *oa, const int64_t *ob, int64_t n, blg_pairs *p) {
    int rc = check_offsets_host(c, oa, n);
    if (!rc) rc = check_offsets_host(c, ob, n);
    if (rc) return rc;
    int64_t hist[kLongClasses + 1] = {0, 0, 0, 0, 0, 0};
    p->n = n;
    p->len_max_side = n > 0 ? std::max(oa[n] - oa[0], ob[n] - ob[0]) : 0;
    // the pass reads 16 bytes of offsets per pair: large sets are split
    // over host threads
    const int nt = n >= (1 << 17) ? HostPool::get().size() : 1;
    // per thread: class counts, short pairs, and whether an offset pair is out of order
    std::vector<std::array<int64_t, kLongClasses + 3>> part(nt);
    auto work = [&](int t) {
        std::array<int64_t, kLongClasses + 3> h{};
        const int64_t i0 = n * t / nt, i1 = n * (t + 1) / nt;
        int64_t shorts = 0, bad = 0;
        for (int64_t i = i0; i < i1; i++) {                  // branch-free, vectorisable
            const int64_t la = oa[i + 1] - oa[i], lb = ob[i + 1] - ob[i];
            shorts += (la <= 32) | (lb <= 32);
            bad |= (la < 0) | (lb < 0) | (la > INT32_MAX) | (lb > INT32_MAX);
        }
        if (shorts < i1 - i0) {
            for (int64_t i = i0; i < i1; i++) {
                const int64_t la = oa[i + 1] - oa[i], lb = ob[i + 1] - ob[i];
                const int64_t m = la < lb ? la : lb;
                if (m <= 32) continue;
                const int64_t W = (m + 63) >> 6;
                h[W <= 2 ? 0 : W <= 4 ? 1 : W <= 8 ? 2 : W <= 16 ? 3 : W <= 32 ? 4 : 5]++;
            }
        }
        h[kLongClasses + 1] = shorts;
        h[kLongClasses + 2] = bad;
        part[t] = h;
    };
    if (nt == 1) work(0);
    else HostPool::get().run(nt, work);
    p->short_pairs = 0;
    bool bad = false;
    for (int t = 0; t < nt; t++) {
        for (int j = 0; j <= kLongClasses; j++) hist[j] += part[t][j];
        p->short_pairs += part[t][kLongClasses + 1];
        bad |= part[t][kLongClasses + 2] != 0;
    }
    // off[0] >= 0 and off[n] >= off[0] were checked above: with every pair in
    // order, every string lies inside the uploaded buffer
    p->trusted = !bad;
    int64_t total = 0, above = hist[kLongClasses];
    for (int j = kLongClasses - 1; j >= 0; j--) {
        above += hist[j];
        p->cap[j] = above;
        total += above;
    }
    // scheduled classes: 0 = one word (any pair), 1..5 = the lane classes
    p->pcap[0] = n;
    for (int j = 0; j < kLongClasses; j++) p->pcap[j + 1] = p->cap[j];
    if (total > 0) {
        CK(dev_alloc(c, &p->q_items, sizeof(LongItem) * (size_t)total), "cudaMallocAsync(queue)");
        CK(dev_alloc(c, (void **)&p->q_ctr, sizeof(int32_t) * 2 * kLongClasses), "cudaMallocAsync(ctr)");
    }
    return BLG_OK;
}

static int pairs_upload(blg_ctx *c, const uint8_t *ba, const int64_t *oa, const uint8_t *bb,
                        const int64_t *ob, int64_t n, blg_pairs *p) {
    int rc = upload_strings(c, ba, oa, n, p->a);
    if (!rc) rc = upload_strings(c, bb, ob, n, p->b);
    if (!rc) rc = pairs_classify(c, oa, ob, n, p);
    return rc;
}

constexpr size_t kPlanCounters = 2 * kPairClasses;   // count, head

static int plan_alloc(blg_ctx *c, blg_pairs *p, bool feat) {
    int64_t slots = 0;
    for (int j = 0; j < kPairClasses; j++) slots += p->pcap[j];
    // each buffer on its own: after a failed allocation a resident plan must
    // not keep one buffer and run with the other missing
    if (!p->plan_mem)
        CK(dev_alloc(c, &p->plan_mem, (size_t)slots * (2 * sizeof(LongItem) + 1) + 64), "cudaMallocAsync(plan)");
    if (!p->plan_ctr)
        CK(dev_alloc(c, (void **)&p->plan_ctr, sizeof(int32_t) * kPlanCounters), "cudaMallocAsync(plan ctr)");
    if (feat && !p->feat_mem)
        CK(dev_alloc(c, (void **)&p->feat_mem, sizeof(half) * kFeatures * (size_t)slots + 16), "cudaMallocAsync(features)");
    return BLG_OK;
}

static PairsPlan plan_view(blg_pairs *p) {
    PairsPlan pl{};
    int64_t slots = 0;
    for (int j = 0; j < kPairClasses; j++) slots += p->pcap[j];
    LongItem *raw = (LongItem *)p->plan_mem, *sorted = raw + slots;
    uint8_t *key = (uint8_t *)(sorted + slots);
    int64_t off = 0;
    for (int j = 0; j < kPairClasses; j++) {
        pl.raw[j] = raw + off;
        pl.sorted[j] = sorted + off;
        pl.key[j] = key + off;
        pl.feat[j] = p->feat_mem ? p->feat_mem + off * kFeatures : nullptr;
        pl.cap[j] = p->pcap[j];
        off += p->pcap[j];
    }
    pl.count = p->plan_ctr;
    pl.head = p->plan_ctr + kPairClasses;
    return pl;
}

// The bytes an uploaded set uses, scanned once (synchronises): p->nsym then
// picks the pairs kernels' row layout for every run of the set.
static int pairs_learn_alphabet(blg_ctx *c, blg_pairs *p) {
    if (p->n <= 0) return BLG_OK;
    uint32_t alpha[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (!p->d_alpha) CK(dev_alloc(c, (void **)&p->d_alpha, sizeof(alpha)), "cudaMallocAsync(alphabet)");
    CK(cudaMemsetAsync(p->d_alpha, 0, sizeof(alpha), c->stream), "reset alphabet");
    CK(launch(c, "byte_presence", [&] { return launch_byte_presence(c->stream, c->sms, p->a.d, p->b.d, p->d_alpha); }),
       "byte_presence");
    CK(cudaMemcpyAsync(alpha, p->d_alpha, sizeof(alpha), cudaMemcpyDeviceToHost, c->stream), "D2H alphabet");
    CK(cudaStreamSynchronize(c->stream), "sync alphabet");
    int nsym = 0;
    for (uint32_t w : alpha) nsym += __builtin_popcount(w);
    p->nsym = nsym;
    return BLG_OK;
}

// The row layout of the pairs kernels for strings A, B of set p: 1 = one
// row per byte, 0 = nibble rows, from the alphabet a resident set's upload
// found; -1 = unknown: the bytes of A and B are scanned into p->d_alpha on
// the stream and both variants launch, the one that does not apply
// returning at once.
static int pairs_alphabet(blg_ctx *c, blg_pairs *p, const DevStrings &A, const DevStrings &B, int *variant) {
    if (!p->d_alpha) CK(dev_alloc(c, (void **)&p->d_alpha, 8 * sizeof(uint32_t)), "cudaMallocAsync(alphabet)");
    if (p->nsym >= 0) {
        *variant = p->nsym <= kBandSymbols ? 1 : 0;
        return BLG_OK;
    }
    *variant = -1;
    CK(cudaMemsetAsync(p->d_alpha, 0, 8 * sizeof(uint32_t), c->stream), "reset alphabet");
    CK(launch(c, "byte_presence", [&] { return launch_byte_presence(c->stream, c->sms, A, B, p->d_alpha); }),
       "byte_presence");
    return BLG_OK;
}

// prep -> order -> solve (every schedule but PLAIN). exit_log (optional,
// device int32[n]) receives the columns each pair's column loop processed.
static int pairs_run_scheduled(blg_ctx *c, blg_pairs *p, const DevStrings &A, const DevStrings &B, int k,
                               int dtype, void *d_out, int32_t *exit_log, bool want_features = false) {
    const bool hask = k >= 0;
    // the learned order needs a trained network; otherwise cost buckets order the work
    const bool learned = want_features || (c->sched == BLG_SCHED_LEARNED && c->model && sched_model_trained(c->model));
    int rc = plan_alloc(c, p, learned);
    if (rc) return rc;
    const PairsPlan plan = plan_view(p);
    CK(cudaMemsetAsync(p->plan_ctr, 0, sizeof(int32_t) * kPlanCounters, c->stream), "reset plan");
    if (exit_log) CK(cudaMemsetAsync(exit_log, 0, sizeof(int32_t) * (size_t)A.n, c->stream), "reset log");
    const int grid = (int)std::min<int64_t>((A.n + 255) / 256, (int64_t)c->sms * 8);
    const bool band = hask && k <= 31;
    CK(launch(c, "pairs_prep", [&] {
           return launch_pairs_prep(c->stream, grid, hask, learned, band, A, B, k, dtype, d_out, plan,
                                    c->sched == BLG_SCHED_LENSORT, c->d_status);
       }), "pairs_prep");
    if (learned && !want_features)
        CK(launch(c, "sched_keys", [&] { return launch_mlp_keys(c->stream, c->sms, c->model, plan, band); }),
           "sched_keys");
    CK(launch(c, "pairs_order", [&] { return launch_order(c->stream, c->sms, plan); }), "pairs_order");
    bool any_long = false;
    for (int j = 1; j < kPairClasses; j++) any_long |= p->pcap[j] > 0;
    if (band) {
        int variant = -1;
        rc = pairs_alphabet(c, p, A, B, &variant);
        if (rc) return rc;
        CK(launch(c, "pairs_band", [&] {
               return launch_solve_band(c->stream, c->sms, band_ctas(c, k), plan, k, dtype, d_out, exit_log, variant,
                                        p->d_alpha);
           }), "pairs_band");
    } else {
        CK(launch(c, "pairs_solve", [&] {
               return launch_solve(c->stream, c->sms, hask, plan, k, dtype, d_out, exit_log, any_long);
           }), "pairs_solve");
    }
    return BLG_OK;
}

// Short pairs (the shorter string <= 32 bytes for at least 3 in 4 pairs)
// run in the tile kernel under the automatic schedule: trimming, the
// in-CTA work sort and the 32-bit solve need no global work plan.
static bool pairs_use_tile(const blg_ctx *c, const blg_pairs *p) {
    return c->sched == BLG_SCHED_AUTO && 4 * p->short_pairs >= 3 * p->n;
}

// One launch of the direct pairs path (tile or staged kernel + the long-pair
// consumer) over strings A, B (a range of the pair set), results at d_out.
static int pairs_run_direct(blg_ctx *c, blg_pairs *p, const DevStrings &A, const DevStrings &B, bool use_tile,
                            int k, int dtype, void *d_out) {
    const bool hask = k >= 0;
    LongQueue q{};
    int64_t total = 0;
    for (int j = 0; j < kLongClasses; j++) {
        q.items[j] = (LongItem *)p->q_items + total;
        q.cap[j] = p->cap[j];
        total += p->cap[j];
    }
    q.counts = p->q_ctr;
    q.heads = p->q_ctr ? p->q_ctr + kLongClasses : nullptr;
    if (total > 0)
        CK(cudaMemsetAsync(p->q_ctr, 0, sizeof(int32_t) * 2 * kLongClasses, c->stream), "reset queue");
    if (use_tile) {
        // 512 pairs per tile while each side averages <= 32 bytes; longer
        // strings get smaller tiles so a tile's span still fits the stage
        const double avg = (double)p->len_max_side / (double)p->n;
        const int tile = avg <= 32.0 ? 512 : std::max(32, (int)(16384.0 / avg) & ~31);
        int variant = -1;
        int rc = pairs_alphabet(c, p, A, B, &variant);
        if (rc) return rc;
        CK(launch(c, "pairs_tile", [&] {
               return launch_pairs_tile(c->stream, c->sms, c->tune.tile_shape, hask, A, B, tile, k, dtype, d_out, q,
                                        c->d_status, c->fault_wait_polls, p->trusted, variant, p->d_alpha);
           }), "pairs_tile");
    } else {
        CK(launch(c, "pairs_staged", [&] {
               return launch_pairs_staged(c->stream, c->sms, hask, A, B, k, dtype, d_out, q, c->d_status);
           }), "pairs_staged");
    }
    if (total > 0)
        CK(launch(c, "pairs_long", [&] {
               return launch_pairs_long(c->stream, c->sms * 3, hask, q, k, dtype, d_out);
           }), "pairs_long");
    return BLG_OK;
}

// Pairs A, B (the whole uploaded set or a range of it) by the context's
// schedule: the tile kernel, the prep -> order -> solve plan, or the
// reference's natural order.
static int pairs_run_range(blg_ctx *c, blg_pairs *p, const DevStrings &A, const DevStrings &B, int k, int dtype,
                           void *d_out, int32_t *exit_log) {
    if (A.n == 0) return BLG_OK;
    const bool use_tile = !exit_log && pairs_use_tile(c, p);
    if (!use_tile && (c->sched != BLG_SCHED_PLAIN || exit_log))
        return pairs_run_scheduled(c, p, A, B, k, dtype, d_out, exit_log);
    return pairs_run_direct(c, p, A, B, use_tile, k, dtype, d_out);
}

static int pairs_run(blg_ctx *c, blg_pairs *p, int k, int dtype, void *d_out, int32_t *exit_log = nullptr) {
    if (!dtype_ok(dtype)) return fail(c, BLG_ERR_ARG, "dtype must be int32, uint16 or uint8");
    if (p->n == 0) return BLG_OK;
    if (!d_out) return fail(c, BLG_ERR_ARG, "null output");
    return pairs_run_range(c, p, p->a.d, p->b.d, k, dtype, d_out, exit_log);
}

// Strings [i0, i1) of an uploaded set, as their own set (offsets are shared).
static DevStrings sub_strings(const DevStrings &S, int64_t i0, int64_t i1) {
    DevStrings r = S;
    r.off = S.off + i0;
    r.n = i1 - i0;
    return r;
}

// Pipeline of the one-call pairwise with host results: the pair set is cut
// into chunks; every chunk's copy to the device is issued first (stream
// `up`), the host's pass over the offsets (path choice, queue capacities)
// runs while they are in flight, then each chunk's kernels (context stream,
// any schedule, ordered within the chunk) start as soon as its bytes have
// landed and its results go back on stream `down` while later chunks
// compute. Pinned buffers overlap fully; pageable ones block the host on
// each copy and overlap less.
static int pairwise_pipelined(blg_ctx *c, const uint8_t *ba, const int64_t *oa, const uint8_t *bb,
                              const int64_t *ob, int64_t n, int k, int dtype, void *out_host, void *d_out,
                              blg_pairs *p) {
    const size_t es = dtype_size(dtype);
    const int nch = (int)std::min<int64_t>(4, std::max<int64_t>(1, n / (1 << 17)));
    std::vector<cudaEvent_t> ev(2 * nch + 2, nullptr);
    int rc = BLG_OK;
    for (auto &e : ev)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) rc = BLG_ERR_CUDA;
    auto fin = [&](int r) {
        cudaStreamSynchronize(c->up);
        cudaStreamSynchronize(c->down);
        cudaStreamSynchronize(c->stream);
        for (auto &e : ev)
            if (e) cudaEventDestroy(e);
        return r;
    };
    if (rc) return fin(fail(c, rc, "cudaEventCreate"));
    // storage was allocated on the context stream: order both copy streams after it
    if (cudaEventRecord(ev[0], c->stream) != cudaSuccess || cudaStreamWaitEvent(c->up, ev[0], 0) != cudaSuccess ||
        cudaStreamWaitEvent(c->down, ev[0], 0) != cudaSuccess)
        return fin(fail(c, BLG_ERR_CUDA, "stream ordering"));
    for (int ch = 0; ch < nch && !rc; ch++) {
        const int64_t i0 = n * ch / nch, i1 = n * (ch + 1) / nch;
        rc = copy_strings(c, ba, oa, i0, i1, p->a, c->up);
        if (!rc) rc = copy_strings(c, bb, ob, i0, i1, p->b, c->up);
        if (!rc && cudaEventRecord(ev[1 + ch], c->up) != cudaSuccess) rc = fail(c, BLG_ERR_CUDA, "event");
    }
    if (!rc) rc = pairs_classify(c, oa, ob, n, p);          // overlaps the copies
    for (int ch = 0; ch <= nch && !rc; ch++) {
        if (ch < nch) {
            const int64_t i0 = n * ch / nch, i1 = n * (ch + 1) / nch;
            if (cudaStreamWaitEvent(c->stream, ev[1 + ch], 0) != cudaSuccess) { rc = fail(c, BLG_ERR_CUDA, "wait"); break; }
            rc = pairs_run_range(c, p, sub_strings(p->a.d, i0, i1), sub_strings(p->b.d, i0, i1), k, dtype,
                                 (uint8_t *)d_out + i0 * es, nullptr);
            if (rc) break;
            if (cudaEventRecord(ev[1 + nch + ch], c->stream) != cudaSuccess) { rc = fail(c, BLG_ERR_CUDA, "event"); break; }
        }
        // the results of the previous chunk go back while this one computes
        if (ch >= 1) {
            const int64_t i0 = n * (ch - 1) / nch, i1 = n * ch / nch;
            if (cudaStreamWaitEvent(c->down, ev[nch + ch], 0) != cudaSuccess) { rc = fail(c, BLG_ERR_CUDA, "wait"); break; }
            cudaError_t e = cudaMemcpyAsync((uint8_t *)out_host + i0 * es, (uint8_t *)d_out + i0 * es,
                                            (i1 - i0) * es, cudaMemcpyDeviceToHost, c->down);
            if (e != cudaSuccess) rc = cuda_fail(c, e, "D2H results");
        }
    }
    // frees on the context stream must follow the last copy back
    if (cudaEventRecord(ev[2 * nch + 1], c->down) == cudaSuccess) cudaStreamWaitEvent(c->stream, ev[2 * nch + 1], 0);
    return fin(rc);
}

static void pairs_graph_drop(blg_pairs *p) {
    if (p->gexec) cudaGraphExecDestroy(p->gexec);
    p->gexec = nullptr;
}

static void pairs_release(blg_ctx *c, blg_pairs *p) {
    pairs_graph_drop(p);
    free_strings(c, p->a);
    free_strings(c, p->b);
    dev_free(c, p->q_items);
    dev_free(c, p->q_ctr);
    dev_free(c, p->plan_mem);
    dev_free(c, p->plan_ctr);
    dev_free(c, p->feat_mem);
    dev_free(c, p->d_alpha);
    p->d_alpha = nullptr;
    p->plan_mem = nullptr;
    p->plan_ctr = nullptr;
    p->feat_mem = nullptr;
}

// ------------------------------------------------------------ search --
static void free_classes(blg_ctx *c, blg_search *s) {
    for (auto &k : s->cls) dev_free(c, k.mem);
    s->cls.clear();
}

// Length buckets of a choice set (the sorted copy of thresholded runs): a
// stable counting sort by length on nt threads of the host pool (nt = 1
// runs on the caller alone, so a pool task may call it). Every string of a
// bucket has the bucket's length, so the sorted offsets follow from the
// bucket starts. perm_at() gives the room for the permutation (pinned) once
// the histogram is done.
struct LengthSort {
    int64_t mn = 0, n_len = 0, bytes = 0;
    std::vector<int64_t> lstart;      // first sorted index per length (n_len + 1)
    std::vector<int64_t> bstart;      // first sorted byte per length (n_len)
};

// 1: sorted; 0: the lengths spread over 2^22 or more values (no buckets);
// -1: perm_at() gave no room.
template <typename PermAt>
static int length_sort(const int64_t *oc, int64_t nc, int nt, LengthSort &L, PermAt &&perm_at) {
    HostPool &pool = HostPool::get();
    auto lo_of = [&](int t, int parts) { return nc * t / parts; };
    std::vector<int64_t> tmn(nt, INT64_MAX), tmx(nt, 0);
    pool.run(nt, [&](int t) {
        int64_t a = INT64_MAX, b = 0;
        for (int64_t i = lo_of(t, nt), e = lo_of(t + 1, nt); i < e; i++) {
            const int64_t l = oc[i + 1] - oc[i];
            a = std::min(a, l);
            b = std::max(b, l);
        }
        tmn[t] = a;
        tmx[t] = b;
    });
    const int64_t mn = *std::min_element(tmn.begin(), tmn.end()), mx = *std::max_element(tmx.begin(), tmx.end());
    if (mx - mn >= (1 << 22)) return 0;
    const int64_t n_len = mx - mn + 1;
    // per-thread histograms [thread][bucket] while they stay small
    const int nh = n_len * nt <= (1 << 22) ? nt : 1;
    std::vector<int64_t> hist((size_t)(n_len * nh), 0);
    pool.run(nh, [&](int t) {
        int64_t *h = hist.data() + (size_t)t * n_len;
        for (int64_t i = lo_of(t, nh), e = lo_of(t + 1, nh); i < e; i++) h[oc[i + 1] - oc[i] - mn]++;
    });
    // bucket starts; each thread's cursor per bucket after the lower threads (stable)
    L.lstart.assign(n_len + 1, 0);
    L.bstart.assign(n_len, 0);
    int64_t run = 0, bytes = 0;
    for (int64_t b = 0; b < n_len; b++) {
        L.lstart[b] = run;
        L.bstart[b] = bytes;
        for (int t = 0; t < nh; t++) {
            const int64_t cnt = hist[(size_t)t * n_len + b];
            hist[(size_t)t * n_len + b] = run;
            run += cnt;
        }
        bytes += (run - L.lstart[b]) * (b + mn);
    }
    L.lstart[n_len] = run;
    int32_t *perm = perm_at();
    if (!perm) return -1;
    pool.run(nh, [&](int t) {
        int64_t *cur = hist.data() + (size_t)t * n_len;
        for (int64_t i = lo_of(t, nh), e = lo_of(t + 1, nh); i < e; i++) perm[cur[oc[i + 1] - oc[i] - mn]++] = (int32_t)i;
    });
    L.mn = mn;
    L.n_len = n_len;
    L.bytes = bytes;
    return 1;
}

// Queries [q0, q1) by word class (bitlev/gpu.py:116-118 uses 1,2,4,8 and the
// CPU above 512; here every length has a GPU class): the sequential classes
// of 1..kSeqMaxWords words, then one lane-spread class (nw = its longest
// query's words), each sorted by length so consecutive survivor tiles share
// choices in L2. false: a query is longer than the lane-spread limit.
struct QueryClass {
    bool lanes = false;
    int nw = 0;
    std::vector<int32_t> idx, len;
};

static bool query_classes(const int64_t *oq, int64_t q0, int64_t q1, std::vector<QueryClass> &out) {
    out.clear();
    std::vector<std::vector<int32_t>> idx(kSeqMaxWords + 1), len(kSeqMaxWords + 1);
    int lanes_nw = 0;
    for (int64_t i = q0; i < q1; i++) {
        const int64_t m = oq[i + 1] - oq[i];
        int64_t W = (m + 63) >> 6;
        if (W < 1) W = 1;
        if (W > kLaneMaxWords) return false;
        const int slot = W <= kSeqMaxWords ? (int)W - 1 : kSeqMaxWords;
        idx[slot].push_back((int32_t)i);
        len[slot].push_back((int32_t)m);
        if (slot == kSeqMaxWords) lanes_nw = std::max(lanes_nw, (int)W);
    }
    for (int slot = 0; slot <= kSeqMaxWords; slot++) {
        if (idx[slot].empty()) continue;
        std::vector<size_t> ord(idx[slot].size());
        for (size_t i = 0; i < ord.size(); i++) ord[i] = i;
        std::stable_sort(ord.begin(), ord.end(), [&](size_t x, size_t y) { return len[slot][x] < len[slot][y]; });
        QueryClass k;
        k.lanes = slot == kSeqMaxWords;
        k.nw = k.lanes ? lanes_nw : slot + 1;
        k.idx.resize(ord.size());
        k.len.resize(ord.size());
        for (size_t i = 0; i < ord.size(); i++) { k.idx[i] = idx[slot][ord[i]]; k.len[i] = len[slot][ord[i]]; }
        out.push_back(std::move(k));
    }
    return true;
}

// Query classes of queries [q0, q1) (query_classes), each in one device
// block with its Peq tables; replaces the previous classes.
static int search_build_classes(blg_ctx *c, const int64_t *oq, int64_t q0, int64_t q1, blg_search *s) {
    free_classes(c, s);
    std::vector<QueryClass> qc;
    if (!query_classes(oq, q0, q1, qc)) return fail(c, BLG_ERR_ARG, "query longer than 2048 bytes is not supported");
    for (auto &q : qc) {
        blg_search::Cls k{};
        k.lanes = q.lanes;
        k.nw = q.nw;
        k.nq = (int)q.idx.size();
        // one device block per class: [qidx | qlen] (filled by one copy), lo,
        // hi, work, tile_start, peq — 256-byte aligned parts. A class joins
        // the search only once its block exists, so a failed allocation never
        // leaves a class without memory behind for a later run.
        auto up = [](size_t x) { return (x + 255) & ~size_t(255); };
        const size_t nq = (size_t)k.nq;
        const size_t o_qidx = 0, o_qlen = nq * 4, o_lo = up(2 * nq * 4), o_hi = o_lo + up(nq * 4),
                     o_work = o_hi + up(nq * 4), o_ts = o_work + 256, o_peq = o_ts + up((nq + 1) * 8),
                     total = o_peq + sizeof(uint64_t) * 256 * (size_t)k.nw * nq;
        CK(dev_alloc(c, &k.mem, total), "cudaMallocAsync(class)");
        s->cls.push_back(k);
        blg_search::Cls &kk = s->cls.back();
        kk.h_qlen = q.len;
        uint8_t *m = (uint8_t *)kk.mem;
        kk.qidx = (int32_t *)(m + o_qidx);
        kk.qlen = (int32_t *)(m + o_qlen);
        kk.lo = (int32_t *)(m + o_lo);
        kk.hi = (int32_t *)(m + o_hi);
        kk.work = (int32_t *)(m + o_work);
        kk.tile_start = (int64_t *)(m + o_ts);
        kk.peq = (uint64_t *)(m + o_peq);
        std::vector<int32_t> both(2 * nq);
        std::copy(q.idx.begin(), q.idx.end(), both.begin());
        std::copy(q.len.begin(), q.len.end(), both.begin() + nq);
        CK(cudaMemcpyAsync(kk.qidx, both.data(), sizeof(int32_t) * 2 * nq, cudaMemcpyHostToDevice, c->stream),
           "H2D class queries");
    }
    // the host vectors above are pageable: the copies completed before return.
    // Peq tables once per class set: every run of these queries reads them.
    for (auto &k_ : s->cls)
        CK(launch(c, "build_peq", [&] {
               return launch_build_peq(c->stream, s->q.d, k_.qidx, k_.nq, k_.nw, k_.peq, c->d_status);
           }), "build_peq");
    return BLG_OK;
}

// Choices: the packed strings, a length-sorted copy (thresholded runs) and
// the tile-transposed form (exact runs).
// Pinned host room for `bytes` of host-built data on its way to the device:
// the context's staging buffer, grown when needed, after the last copy out
// of it has finished.
static void *host_stage(blg_ctx *c, size_t bytes) {
    if (c->stage_done) cudaEventSynchronize(c->stage_done);
    if (bytes > c->stage_bytes) {
        const size_t want = std::max(bytes, c->stage_bytes * 2);
        if (c->stage) cudaFreeHost(c->stage);
        c->stage = nullptr;
        c->stage_bytes = 0;
        if (cudaHostAlloc(&c->stage, want, cudaHostAllocDefault) != cudaSuccess) return nullptr;
        c->stage_bytes = want;
    }
    if (!c->stage_done && cudaEventCreateWithFlags(&c->stage_done, cudaEventDisableTiming) != cudaSuccess)
        return nullptr;
    return c->stage;
}

// What a search needs beside the choices themselves: the length-sorted copy
// with sketches (survivor kernels of max_dist runs) and the tile-transposed
// copy (exact and plain-order runs). A resident search set builds both; a
// one-call search knows its max_dist and schedule and builds one.
enum { NEED_SORTED = 1, NEED_TT = 2, NEED_PFX = 4, NEED_ALL = 7 };

// perm_stage: pinned room for the permutation (nc int32) reserved by the
// caller for this upload alone (a batch reserves one region per problem, so
// no upload waits for an earlier one's copy); null: the context's stage.
// ---- exact search with prefix reuse (k_search_pfx): the choices sorted
// lexicographically on the host's thread pool by their first 16 bytes (ties
// in any order: only the exact common prefixes computed next matter), the
// common prefix of every sorted neighbour pair, and the two checkpoint
// columns that skip the most text columns over the warps' chains of
// kPfxChain consecutive choices. Built when the choices use at most
// kPfxMaxSymbols distinct bytes and at least kPfxMinSaving of the columns
// are skipped; the text is laid out on the device (k_prefix_text).
constexpr int64_t kPfxMinChoices = 4096;
constexpr double kPfxMinSaving = 0.02;

static int search_build_prefix(blg_ctx *c, const uint8_t *bc, const int64_t *oc, int64_t nc, blg_search *s) {
    if (nc < kPfxMinChoices || nc >= INT32_MAX) return BLG_OK;
    const int64_t cols = oc[nc] - oc[0];
    if (cols <= 0) return BLG_OK;
    HostPool &pool = HostPool::get();
    const int nt = pool.size();
    std::vector<int64_t> cut((size_t)nt + 1);
    for (int t = 0; t <= nt; t++) cut[t] = nc * t / nt;
    // the alphabet: the bytes the choices use
    std::vector<std::array<uint8_t, 256>> seen((size_t)nt);
    pool.run(nt, [&](int t) {
        seen[t].fill(0);
        for (int64_t x = oc[cut[t]]; x < oc[cut[t + 1]]; x++) seen[t][bc[x]] = 1;
    });
    std::vector<uint8_t> sym;
    std::vector<uint16_t> rowoff(256, 0);
    for (int v = 0; v < 256; v++) {
        bool any = false;
        for (int t = 0; t < nt; t++) any |= seen[t][v] != 0;
        if (any) {
            rowoff[v] = (uint16_t)(sym.size() * kPfxRowBytes);
            sym.push_back((uint8_t)v);
        }
    }
    if (sym.empty() || (int)sym.size() > kPfxMaxSymbols) return BLG_OK;
    struct Key {
        uint64_t hi, lo;
        int32_t idx;
    };
    std::vector<Key> keys((size_t)nc);
    auto be8 = [](const uint8_t *p, int64_t len, int64_t from) {
        uint64_t v = 0;
        for (int b = 0; b < 8; b++) v = (v << 8) | (from + b < len ? p[from + b] : 0u);
        return v;
    };
    auto less = [](const Key &a, const Key &b) { return a.hi != b.hi ? a.hi < b.hi : a.lo < b.lo; };
    pool.run(nt, [&](int t) {
        for (int64_t i = cut[t]; i < cut[t + 1]; i++) {
            const uint8_t *p = bc + oc[i];
            const int64_t len = oc[i + 1] - oc[i];
            keys[i] = Key{be8(p, len, 0), be8(p, len, 8), (int32_t)i};
        }
        std::sort(keys.begin() + cut[t], keys.begin() + cut[t + 1], less);
    });
    std::vector<Key> tmp((size_t)nc);
    for (int w = 1; w < nt; w *= 2) {                        // merge sorted runs pairwise, in parallel
        const int groups = (nt + 2 * w - 1) / (2 * w);
        pool.run(groups, [&](int g) {
            const int64_t lo = cut[std::min(nt, 2 * g * w)], mid = cut[std::min(nt, 2 * g * w + w)],
                          hi = cut[std::min(nt, 2 * g * w + 2 * w)];
            std::merge(keys.begin() + lo, keys.begin() + mid, keys.begin() + mid, keys.begin() + hi,
                       tmp.begin() + lo, less);
        });
        keys.swap(tmp);
    }
    // common prefixes of sorted neighbours (capped at 255: a restart column is a byte)
    std::vector<uint8_t> lcp((size_t)nc, 0);
    std::vector<std::vector<int64_t>> hist((size_t)nt, std::vector<int64_t>(256, 0));
    pool.run(nt, [&](int t) {
        for (int64_t p = std::max<int64_t>(1, cut[t]); p < cut[t + 1]; p++) {
            const int64_t a = keys[p - 1].idx, b = keys[p].idx;
            const int64_t lim = std::min<int64_t>(255, std::min(oc[a + 1] - oc[a], oc[b + 1] - oc[b]));
            const uint8_t *x = bc + oc[a], *y = bc + oc[b];
            int64_t l = 0;
            while (l < lim && x[l] == y[l]) l++;
            lcp[p] = (uint8_t)l;
            if (p % kPfxChain) hist[t][l]++;                  // a chain's first choice never restarts
        }
    });
    std::vector<int64_t> G(257, 0);                           // G[v] = restartable choices with lcp >= v
    for (int v = 255; v >= 0; v--) {
        int64_t h = 0;
        for (int t = 0; t < nt; t++) h += hist[t][v];
        G[v] = G[v + 1] + h;
    }
    int64_t best = 0;
    int c1 = 0, c2 = 0;
    for (int a = 1; a < 255; a++)
        for (int b = a + 1; b <= 255; b++) {
            const int64_t sv = (int64_t)a * (G[a] - G[b]) + (int64_t)b * G[b];
            if (sv > best) { best = sv; c1 = a; c2 = b; }
        }
    if ((double)best < kPfxMinSaving * (double)cols) return BLG_OK;
    // sorted order, restart columns, text word offsets (two characters per word)
    std::vector<int32_t> order((size_t)nc);
    std::vector<uint8_t> restart((size_t)nc);
    std::vector<int64_t> woff((size_t)nc + 1, 0);
    for (int64_t p = 0; p < nc; p++) {
        order[p] = keys[p].idx;
        restart[p] = (uint8_t)(p % kPfxChain == 0 ? 0 : lcp[p] >= c2 ? c2 : lcp[p] >= c1 ? c1 : 0);
        woff[p + 1] = woff[p] + (oc[keys[p].idx + 1] - oc[keys[p].idx] + 1) / 2;
    }
    auto up = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t words = (size_t)woff[nc] + kPfxTextSlack;
    const size_t o_order = 0, o_rs = up(4 * (size_t)nc), o_woff = o_rs + up((size_t)nc),
                 o_len = o_woff + up(8 * ((size_t)nc + 1)), o_sym = o_len + up(4 * (size_t)nc),
                 o_rowoff = o_sym + 256, o_text = o_rowoff + 512, o_work = o_text + up(4 * words),
                 total = o_work + 256;
    CK(dev_alloc(c, &s->pfx_mem, total), "cudaMallocAsync(prefix layout)");
    uint8_t *m = (uint8_t *)s->pfx_mem;
    CK(cudaMemcpyAsync(m + o_order, order.data(), 4 * (size_t)nc, cudaMemcpyHostToDevice, c->stream), "H2D order");
    CK(cudaMemcpyAsync(m + o_rs, restart.data(), (size_t)nc, cudaMemcpyHostToDevice, c->stream), "H2D restarts");
    CK(cudaMemcpyAsync(m + o_woff, woff.data(), 8 * ((size_t)nc + 1), cudaMemcpyHostToDevice, c->stream),
       "H2D word offsets");
    CK(cudaMemcpyAsync(m + o_sym, sym.data(), sym.size(), cudaMemcpyHostToDevice, c->stream), "H2D alphabet");
    CK(cudaMemcpyAsync(m + o_rowoff, rowoff.data(), 512, cudaMemcpyHostToDevice, c->stream), "H2D row offsets");
    CK(cudaMemsetAsync(m + o_text + 4 * (size_t)woff[nc], 0, 4 * kPfxTextSlack, c->stream), "memset slack");
    PrefixChoices &P = s->pd;
    P.text = (const uint32_t *)(m + o_text);
    P.woff = (const int64_t *)(m + o_woff);
    P.len = (const int32_t *)(m + o_len);
    P.orig = (const int32_t *)(m + o_order);
    P.restart = (const uint8_t *)(m + o_rs);
    P.sym = (const uint8_t *)(m + o_sym);
    P.nsym = (int)sym.size();
    P.n = nc;
    P.ck[0] = c1;
    P.ck[1] = c2;
    s->pfx_work = (unsigned long long *)(m + o_work);
    CK(launch(c, "prefix_text", [&] {
           return launch_prefix_text(c->stream, c->sms, s->c.d, P.orig, P.woff, (const uint16_t *)(m + o_rowoff),
                                     (uint32_t *)P.text, (int32_t *)P.len, c->d_status);
       }), "prefix_text");
    s->pfx_saving = (double)best / (double)cols;
    s->pfx = true;
    // the host vectors above are pageable: the copies completed before return
    return BLG_OK;
}

static int search_upload_choices(blg_ctx *c, const uint8_t *bc, const int64_t *oc, int64_t nc, blg_search *s,
                                 unsigned need = NEED_ALL, int32_t *perm_stage = nullptr) {
    s->nc = nc;
    int rc = upload_strings(c, bc, oc, nc, s->c);
    if (rc) return rc;
    // Choices sorted by length (a stable counting sort on the host's thread
    // pool, the byte gather on the device), when the length range is
    // moderate. Every string of a length bucket has the bucket's length, so
    // the sorted offsets follow from the bucket starts: the device computes
    // them, and only the permutation (pinned) and the bucket tables travel.
    if (nc > 0 && (need & NEED_SORTED) && nc < INT32_MAX) {
        LengthSort L;
        const int nt = nc >= (1 << 16) ? HostPool::get().size() : 1;
        int32_t *perm = nullptr;
        const int sorted = length_sort(oc, nc, nt, L, [&] {
            perm = perm_stage ? perm_stage : (int32_t *)host_stage(c, sizeof(int32_t) * (size_t)nc);
            return perm;
        });
        if (sorted < 0) return fail(c, BLG_ERR_ALLOC, "cudaHostAlloc(staging)");
        if (sorted) {
            const int64_t mn = L.mn, n_len = L.n_len, bytes = L.bytes;
            // one device block: perm | lstart, bucket starts | sorted offsets | sketches | sorted bytes
            auto up = [](size_t x) { return (x + 255) & ~size_t(255); };
            const size_t o_perm = 0, o_tab = up(sizeof(int32_t) * (size_t)nc),
                         o_soff = o_tab + up(sizeof(int64_t) * (size_t)(2 * n_len + 1)),
                         o_csk = o_soff + up(sizeof(int64_t) * (size_t)(nc + 1)),
                         o_ccnt = o_csk + up(sizeof(uint64_t) * (size_t)nc),
                         o_buf = o_ccnt + up(sizeof(uint4) * (size_t)nc),
                         total = o_buf + (size_t)bytes + kSlackBefore + kSlackAfter;
            CK(dev_alloc(c, &s->sorted_mem, total), "cudaMallocAsync(sorted choices)");
            uint8_t *m = (uint8_t *)s->sorted_mem;
            s->perm = (int32_t *)(m + o_perm);
            s->lstart = (int64_t *)(m + o_tab);
            int64_t *d_bstart = s->lstart + (n_len + 1);
            int64_t *d_soff = (int64_t *)(m + o_soff);
            s->csk = (uint64_t *)(m + o_csk);
            s->ccnt = (uint4 *)(m + o_ccnt);
            uint8_t *d_buf = m + o_buf;
            CK(cudaMemcpyAsync(s->perm, perm, sizeof(int32_t) * nc, cudaMemcpyHostToDevice, c->stream), "H2D perm");
            CK(cudaEventRecord(c->stage_done, c->stream), "event");
            std::vector<int64_t> tab(L.lstart);               // lstart then the bucket starts: one copy
            tab.insert(tab.end(), L.bstart.begin(), L.bstart.end());
            CK(cudaMemcpyAsync(s->lstart, tab.data(), sizeof(int64_t) * tab.size(), cudaMemcpyHostToDevice, c->stream),
               "H2D length tables");
            CK(launch(c, "sorted_offsets", [&] {
                   return launch_sorted_offsets(c->stream, c->sms, s->lstart, n_len, mn, d_bstart, nc, d_soff);
               }), "sorted_offsets");
            CK(cudaMemsetAsync(d_buf, 0, kSlackBefore, c->stream), "memset slack");
            CK(cudaMemsetAsync(d_buf + kSlackBefore + bytes, 0, kSlackAfter, c->stream), "memset slack");
            OwnedStrings &cs = s->cs;                          // owned by sorted_mem
            s->h_lstart = L.lstart;
            cs.d.buf = d_buf + kSlackBefore;
            cs.d.off = d_soff;
            cs.d.n = nc;
            cs.d.base = 0;
            cs.d.bytes = bytes;
            CK(launch(c, "gather_strings", [&] {
                   return launch_gather_strings(c->stream, c->sms, s->c.d, s->perm, cs.d.off,
                                                (uint8_t *)cs.d.buf, nc, c->d_status);
               }), "gather_strings");
            CK(launch(c, "sketch", [&] { return launch_sketch_strings(c->stream, c->sms, cs.d, s->csk, s->ccnt, c->d_status); }),
               "sketch");
            s->min_len = mn;
            s->n_len = n_len;
            s->lsorted = true;
        }
    }
    // Tile-transposed choices: padded size = sum over tiles of kTileCands x
    // the tile's longest choice; kept when at most twice the packed bytes
    // (plus 64 MiB), so a few long choices cannot blow up the copy.
    if (nc > 0 && (need & NEED_TT)) {
        const int64_t tiles = (nc + kTileCands - 1) / kTileCands;
        std::vector<int64_t> base(tiles + 1, 0);
        HostPool &pool = HostPool::get();
        const int nt = nc >= (1 << 16) ? pool.size() : 1;
        pool.run(nt, [&](int w) {                               // each tile's longest choice
            for (int64_t t = tiles * w / nt, te = tiles * (w + 1) / nt; t < te; t++) {
                int64_t mx = 0;
                const int64_t e = std::min(nc, (t + 1) * kTileCands);
                for (int64_t i = t * kTileCands; i < e; i++) mx = std::max(mx, oc[i + 1] - oc[i]);
                base[t + 1] = kTileCands * ((mx + 3) / 4);
            }
        });
        for (int64_t t = 0; t < tiles; t++) base[t + 1] += base[t];
        const int64_t bytes = oc[nc] - oc[0];
        if (base[tiles] * 4 <= 2 * bytes + (64ll << 20)) {
            // + kTtSlackRows rows: the search loop prefetches up to 4 words past a choice's end
            CK(dev_alloc(c, (void **)&s->tt_words,
                         sizeof(uint32_t) * ((size_t)base[tiles] + (size_t)kTtSlackRows * kTileCands)),
               "cudaMallocAsync(tt)");
            CK(dev_alloc(c, (void **)&s->tt_base, sizeof(int64_t) * (size_t)(tiles + 1)), "cudaMallocAsync(tt base)");
            CK(dev_alloc(c, (void **)&s->tt_len, sizeof(int32_t) * (size_t)nc), "cudaMallocAsync(tt len)");
            CK(cudaMemcpyAsync(s->tt_base, base.data(), sizeof(int64_t) * (tiles + 1), cudaMemcpyHostToDevice,
                               c->stream), "H2D tt base");
            CK(launch(c, "transpose_choices", [&] {
                   return launch_transpose_choices(c->stream, c->sms, s->c.d, s->tt_base, s->tt_words, s->tt_len,
                                                   c->d_status);
               }), "transpose_choices");
            s->tt = true;
        }
        if (need & NEED_PFX) {
            const int rc2 = search_build_prefix(c, bc, oc, nc, s);
            if (rc2) return rc2;
        }
    }
    // the host vectors above are pageable: the copies completed before return
    return BLG_OK;
}

static int search_run(blg_ctx *c, blg_search *s, int k, int dtype, void *d_out, int64_t q0 = 0,
                      int64_t q1 = -1);

// Queries into HBM, with their 4-gram sketches.
static int search_upload_queries(blg_ctx *c, const uint8_t *bq, const int64_t *oq, int64_t nq, blg_search *s) {
    s->nq = nq;
    int rc = upload_strings(c, bq, oq, nq, s->q);
    if (rc) return rc;
    // one block: the sketches (8 B each), then the 4-gram counts (16 B each, 16-byte aligned)
    const size_t nq1 = (size_t)std::max<int64_t>(nq, 1), o_cnt = (8 * nq1 + 15) & ~size_t(15);
    CK(dev_alloc(c, (void **)&s->qsk, o_cnt + 16 * nq1), "cudaMallocAsync(sketches)");
    s->sk_mem = s->qsk;
    s->qcnt = (uint4 *)((uint8_t *)s->qsk + o_cnt);
    CK(launch(c, "sketch", [&] { return launch_sketch_strings(c->stream, c->sms, s->q.d, s->qsk, s->qcnt, c->d_status); }),
       "sketch");
    return BLG_OK;
}

// One-call cdist with host results: queries in chunks of rows; the rows of
// chunk i go back (stream `down`) while chunk i+1 computes.
// d4 (optional): 4-bit results. The chunks then compute uint8 rows into
// d_out, pack them into d4 and copy back d4's bytes; chunk boundaries fall on
// even elements so no byte is shared by two chunks.
static int cdist_pipelined(blg_ctx *c, const uint8_t *bq, const int64_t *oq, int64_t nq, const uint8_t *bc,
                           const int64_t *oc, int64_t nc, int k, int dtype, void *out_host, void *d_out,
                           blg_search *s, void *d4) {
    const bool surv = k >= 0 && c->sched != BLG_SCHED_PLAIN;      // the survivor kernels run (search_run)
    int rc = search_upload_queries(c, bq, oq, nq, s);
    if (!rc) rc = search_upload_choices(c, bc, oc, nc, s, surv ? NEED_SORTED : NEED_TT);
    if (rc) return rc;
    const size_t row = dtype_size(dtype) * (size_t)nc;
    // Query chunks of relative sizes 4,4,4,4,4,4,4,2,1,1: the last chunk's
    // copy back is the part of the result stream no kernel hides, so the
    // tail chunks are small (1/32 of the rows instead of 1/8).
    static const int kWeights[] = {4, 4, 4, 4, 4, 4, 4, 2, 1, 1};
    std::vector<int64_t> cut{0};
    if (nq >= 32) {
        int acc = 0;
        for (int w : kWeights) cut.push_back(nq * (acc += w) / 32);
    } else {
        const int n8 = (int)std::min<int64_t>(8, nq);
        for (int i = 1; i <= n8; i++) cut.push_back(nq * i / n8);
    }
    if (d4 && (nc & 1)) {                               // even element boundaries: even rows
        std::vector<int64_t> even{0};
        for (size_t i = 1; i + 1 < cut.size(); i++)
            if ((cut[i] & ~int64_t(1)) > even.back()) even.push_back(cut[i] & ~int64_t(1));
        even.push_back(nq);
        cut.swap(even);
    }
    const int nch = (int)cut.size() - 1;
    std::vector<cudaEvent_t> ev(nch + 1, nullptr);
    for (auto &e : ev)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) rc = BLG_ERR_CUDA;
    auto fin = [&](int r) {
        cudaStreamSynchronize(c->down);
        cudaStreamSynchronize(c->stream);
        for (auto &e : ev)
            if (e) cudaEventDestroy(e);
        return r;
    };
    if (rc) return fin(fail(c, rc, "cudaEventCreate"));
    for (int ch = 0; ch <= nch && !rc; ch++) {
        if (ch < nch) {
            const int64_t q0 = cut[ch], q1 = cut[ch + 1];
            rc = search_build_classes(c, oq, q0, q1, s);
            if (!rc) rc = search_run(c, s, k, dtype, d_out, q0, q1);
            if (!rc && d4) rc = pack_u4(c, d_out, q0 * nc, q1 * nc, d4);
            if (!rc && cudaEventRecord(ev[ch], c->stream) != cudaSuccess) rc = fail(c, BLG_ERR_CUDA, "event");
            // exact runs: the host sorts the choices for the prefix-reuse
            // kernel while the first chunk computes on the tile-transposed
            // copy; the later chunks use it
            if (!rc && ch == 0 && k < 0 && nch > 1) rc = search_build_prefix(c, bc, oc, nc, s);
            if (rc) break;
        }
        if (ch >= 1) {
            const int64_t q0 = cut[ch - 1], q1 = cut[ch];
            if (cudaStreamWaitEvent(c->down, ev[ch - 1], 0) != cudaSuccess) { rc = fail(c, BLG_ERR_CUDA, "wait"); break; }
            const int64_t b0 = d4 ? q0 * nc / 2 : q0 * (int64_t)row, b1 = d4 ? (q1 * nc + 1) / 2 : q1 * (int64_t)row;
            cudaError_t e = cudaMemcpyAsync((uint8_t *)out_host + b0, (uint8_t *)(d4 ? d4 : d_out) + b0,
                                            (size_t)(b1 - b0), cudaMemcpyDeviceToHost, c->down);
            if (e != cudaSuccess) rc = cuda_fail(c, e, "D2H results");
        }
    }
    // frees on the context stream must follow the last copy back
    if (cudaEventRecord(ev[nch], c->down) == cudaSuccess) cudaStreamWaitEvent(c->stream, ev[nch], 0);
    return fin(rc);
}

static int search_upload(blg_ctx *c, const uint8_t *bq, const int64_t *oq, int64_t nq,
                         const uint8_t *bc, const int64_t *oc, int64_t nc, blg_search *s,
                         unsigned need = NEED_ALL, int32_t *perm_stage = nullptr) {
    int rc = search_upload_queries(c, bq, oq, nq, s);
    if (!rc && need == NEED_ALL && nq > 0) s->h_oq.assign(oq, oq + nq + 1);   // a resident search keeps them
    if (!rc) rc = search_upload_choices(c, bc, oc, nc, s, need, perm_stage);
    if (!rc) rc = search_build_classes(c, oq, 0, nq, s);
    return rc;
}

// Queries per CTA of the exact search: the autotuned value for this word
// count, else enough CTAs for 8 per SM, capped at 16.
static int pick_qpb(blg_ctx *c, int nw, int nq_cls, int64_t nc) {
    const int64_t tiles = (nc + 1023) / 1024;
    const int64_t target = (int64_t)c->sms * 8;
    int64_t qpb = (int64_t)nq_cls * tiles / target;
    if (qpb < 1) qpb = 1;
    if (qpb > 16) qpb = 16;
    if (nw >= 1 && nw <= 8 && c->tune.qpb[nw] > 0) qpb = std::min<int64_t>(c->tune.qpb[nw], std::max(1, nq_cls));
    const int64_t min_qpb = ((int64_t)nq_cls + 65534) / 65535;   // grid.y limit
    if (qpb < min_qpb) qpb = min_qpb;
    return (int)qpb;
}

// Launch the current classes' kernels; the max_dist fill covers rows [q0, q1)
// (all rows by default: the classes hold every query).
// Survivors per job of the thresholded search: the tuned size, halved
// (down to 1024) while the run would have fewer than 4 jobs per warp of the
// persistent grid, so small searches still spread over the GPU. The
// survivor count comes from the host copies of the length histogram.
static int survivor_job_size(blg_ctx *c, const blg_search *s, int k) {
    int64_t total = 0;
    const int64_t nl = s->n_len;
    for (auto &k_ : s->cls) {
        if (k_.lanes) continue;
        for (int32_t m : k_.h_qlen) {
            int64_t a = m - k - s->min_len, b = m + k - s->min_len + 1;
            a = std::max<int64_t>(0, std::min(a, nl));
            b = std::max<int64_t>(0, std::min(b, nl));
            if (b > a) total += s->h_lstart[b] - s->h_lstart[a];
        }
    }
    const int64_t warps = (int64_t)c->sms * surv_ctas(c, k) * 8;
    int job = c->tune.lpt_job;
    while (job > 1024 && total < 4 * warps * (int64_t)job) job >>= 1;
    return job;
}

// The sequential (not lane-spread) query classes of a search, for the
// survivor plan and kernels.
static SurvClasses seq_classes(blg_search *s) {
    SurvClasses C;
    for (auto &k_ : s->cls) {
        if (k_.lanes || C.n == kSurvClasses) continue;
        C.cls[C.n] = SearchClass{k_.nw, k_.nq, k_.qidx, k_.qlen, k_.peq};
        C.lo[C.n] = k_.lo;
        C.hi[C.n] = k_.hi;
        C.tile_start[C.n] = k_.tile_start;
        C.work[C.n] = k_.work;
        C.n++;
    }
    return C;
}

// Queries in the search's current classes (every query of the rows they
// were built for, empty ones included).
static int64_t class_queries(const blg_search *s) {
    int64_t n = 0;
    for (auto &k_ : s->cls) n += k_.nq;
    return n;
}

static int search_run(blg_ctx *c, blg_search *s, int k, int dtype, void *d_out, int64_t q0, int64_t q1) {
    if (!dtype_ok(dtype)) return fail(c, BLG_ERR_ARG, "dtype must be int32, uint16 or uint8");
    if (s->nq == 0 || s->nc == 0) return BLG_OK;
    if (q1 < 0) q1 = s->nq;
    // a class rebuild that an allocation failure cut short leaves queries
    // without a class: refuse to run rather than skip their rows
    if (class_queries(s) != q1 - q0)
        return fail(c, BLG_ERR_ALLOC, "the search's query classes are incomplete after an allocation failure");
    if (!d_out) return fail(c, BLG_ERR_ARG, "null output");
    const bool hask = k >= 0;
    const bool surv = hask && s->lsorted && c->sched != BLG_SCHED_PLAIN;
    if (surv) {
        // the sequential classes' survivor plans in one launch; max_dist <=
        // 31: their survivors in one more (lanes refilled as survivors
        // finish), which also fills the output with k+1 and defers its
        // results to the context's list (scattered after it; an in-place
        // repair launch runs only if the list ran full). max_dist > 31: the
        // fill kernel, then the full-word survivor kernels.
        const uint32_t fillv = (uint32_t)(dtype == BLG_UINT8 ? std::min(k + 1, 255)
                                          : dtype == BLG_UINT16 ? std::min(k + 1, 65535) : k + 1);
        const BatchFill whole{(uint8_t *)d_out + q0 * s->nc * (int64_t)dtype_size(dtype), (q1 - q0) * s->nc, dtype,
                              fillv};
        const SurvClasses C = seq_classes(s);
        const bool band = k <= 31 && C.n > 0;
        const int job = band ? survivor_job_size(c, s, k) : 1024;
        if (!band)
            CK(launch(c, "fill", [&] { return launch_fill(c->stream, c->sms, whole.out, whole.n, dtype, fillv); }),
               "fill");
        CK(launch(c, "surv_plan", [&] {
               return launch_surv_plan(c->stream, C, s->lstart, s->min_len, s->n_len, k, job);
           }), "surv_plan");
        if (band) {
            const ResultList L{c->rl_hdr + 2, c->rl_hdr, c->rl_cap};
            const FillItems F{nullptr, nullptr, 0, whole, fill_items_of(whole), c->rl_hdr + 1};
            CK(cudaMemsetAsync(c->rl_hdr, 0, 2 * sizeof(unsigned long long), c->stream), "clear list");
            CK(launch(c, "search_band", [&] {
                   return launch_search_band(c->stream, c->sms, surv_ctas(c, k), surv_round(c, k), job, C, s->cs.d,
                                             s->perm, s->ccnt, s->qcnt, k, dtype, d_out, s->nc, nullptr, &L, &F,
                                             c->d_status);
               }), "search_band");
            CK(launch(c, "list_scatter", [&] { return launch_list_scatter(c->stream, c->sms, L, C.work[0]); }),
               "list_scatter");
            CK(launch(c, "search_band_repair", [&] {
                   return launch_search_band(c->stream, c->sms, surv_ctas(c, k), surv_round(c, k), job, C, s->cs.d,
                                             s->perm, s->ccnt, s->qcnt, k, dtype, d_out, s->nc, nullptr, &L, nullptr,
                                             c->d_status);
               }), "search_band_repair");
        } else {
            for (int i = 0; i < C.n; i++)
                CK(launch(c, "search_surv", [&] {
                       return launch_search_surv(c->stream, c->sms, C.cls[i].nw, s->cs.d, s->perm, C.cls[i], C.lo[i],
                                                 C.hi[i], C.tile_start[i], C.work[i], k, dtype, d_out, s->nc,
                                                 c->d_status);
                   }), "search_surv");
        }
    }
    for (auto &k_ : s->cls) {
        SearchClass sc{k_.nw, k_.nq, k_.qidx, k_.qlen, k_.peq};
        if (surv && !k_.lanes) continue;
        if (k_.lanes) {
            CK(launch(c, "search_lanes", [&] {
                   return launch_search_lanes(c->stream, hask, s->c.d, sc, k_.nw, k, dtype, d_out,
                                              c->d_status);
               }), "search_lanes");
        } else {
            const int qpb = pick_qpb(c, k_.nw, k_.nq, s->nc);
            if (!hask && s->pfx && search_pfx_supported(k_.nw)) {
                // exact short queries over the prefix-sorted choices
                CK(cudaMemsetAsync(s->pfx_work, 0, sizeof(unsigned long long), c->stream), "reset work");
                CK(launch(c, "search_pfx", [&] {
                       return launch_search_pfx(c->stream, c->sms, 4, k_.nw, s->pd, sc, s->pfx_work, dtype, d_out);
                   }), "search_pfx");
            } else if (s->tt) {
                const TransposedChoices T{s->tt_words, s->tt_base, s->tt_len, s->nc};
                CK(launch(c, "search_tt", [&] {
                       return launch_search_tt(c->stream, k_.nw, hask, T, sc, qpb, k, dtype, d_out);
                   }), "search_tt");
            } else {
                CK(launch(c, "search_seq", [&] {
                       return launch_search_seq(c->stream, k_.nw, hask, s->c.d, sc, qpb, k, dtype, d_out,
                                                c->d_status);
                   }), "search_seq");
            }
        }
    }
    return BLG_OK;
}

// ---- matches-only search
// Dense scratch element type of a threshold k: the narrowest holding k + 1.
static int match_dtype(int k) { return k <= 254 ? BLG_UINT8 : k <= 65534 ? BLG_UINT16 : BLG_INT32; }

// Upper bound of the dense scratch of one query chunk: 1 GiB, or the
// environment's BLG_MATCH_SCRATCH_BYTES (a memory budget; at least one row).
static size_t match_scratch_bytes() {
    const char *e = getenv("BLG_MATCH_SCRATCH_BYTES");
    const long long v = e ? atoll(e) : 0;
    return v > 0 ? (size_t)v : (size_t(1) << 30);
}

// Rows [q0, q1) of search s (classes built for them) into the dense scratch
// (row q0 at its start), then the compaction: the chunk's match total comes
// back to the host (*total); up to `cap` records go to d_out (device) when
// d_out is given — or, when it is not, to a device buffer allocated for the
// chunk and copied to host_out. Synchronises once per call.
static int search_matches_rows(blg_ctx *c, blg_search *s, int k, int64_t q0, int64_t q1, void *scratch,
                               blg_match *d_out, blg_match *host_out, int64_t cap, int64_t *total) {
    const int sdt = match_dtype(k);
    const size_t es = dtype_size(sdt);
    const int64_t n = (q1 - q0) * s->nc;
    *total = 0;
    if (n <= 0) return BLG_OK;
    // the search writes absolute rows: offset the base so row q0 lands at the scratch's start
    uint8_t *base = (uint8_t *)scratch - (size_t)q0 * (size_t)s->nc * es;
    int rc = search_run(c, s, k, sdt, base, q0, q1);
    if (rc) return rc;
    int64_t *counts = nullptr;
    CK(dev_alloc(c, (void **)&counts, sizeof(int64_t) * (size_t)(match_blocks(n) + 1)), "cudaMallocAsync(match counts)");
    int64_t *d_total = counts + match_blocks(n);
    CK(launch(c, "match_count", [&] {
           return launch_match_compact(c->stream, c->sms, sdt, scratch, n, k, counts, d_total, s->nc, q0, nullptr, 0,
                                       false);
       }), "match_count");
    int64_t tot = 0;
    CK(cudaMemcpyAsync(&tot, d_total, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream), "D2H match total");
    CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    *total = tot;
    const int64_t m = std::min(tot, cap);
    if (m > 0) {
        blg_match *dst = d_out;
        if (!dst) CK(dev_alloc(c, (void **)&dst, sizeof(blg_match) * (size_t)m), "cudaMallocAsync(matches)");
        CK(launch(c, "match_emit", [&] {
               return launch_match_compact(c->stream, c->sms, sdt, scratch, n, k, counts, d_total, s->nc, q0, dst, m,
                                           true);
           }), "match_emit");
        if (!d_out) {
            CK(cudaMemcpyAsync(host_out, dst, sizeof(blg_match) * (size_t)m, cudaMemcpyDeviceToHost, c->stream),
               "D2H matches");
            dev_free(c, dst);
        }
    }
    dev_free(c, counts);
    return BLG_OK;
}

// LSD radix sort of list entries by their element index (entry >> 8), 8
// bits per pass over the index bytes that vary.
static void sort_by_index(std::vector<unsigned long long> &v) {
    if (v.size() < 2) return;
    unsigned long long top = 0;
    for (auto e : v) top |= e >> 8;
    std::vector<unsigned long long> tmp(v.size());
    for (int shift = 8; shift < 64 && (top >> (shift - 8)) != 0; shift += 8) {
        size_t cnt[257] = {0};
        for (auto e : v) cnt[((e >> shift) & 0xffu) + 1]++;
        for (int d = 0; d < 256; d++) cnt[d + 1] += cnt[d];
        for (auto e : v) tmp[cnt[(e >> shift) & 0xffu]++] = e;
        v.swap(tmp);
    }
}

// Matches of a thresholded search straight from the survivor kernel's result
// list, for runs on the survivor path with the banded loop (max_dist <= 31,
// choices length-sorted, a schedule other than plain, every query of the
// current classes in a sequential class). The kernel runs without an
// output and without a fill: it lists every result <= max_dist as its dense
// element index (base 0, one byte per element, so the listed address is
// row * nc + choice). The listed entries <= max_dist (an empty query lists
// min(n, max_dist + 1) for each survivor) are sorted by index on the host
// and become the records: no dense scratch, no compaction passes. *done =
// false, with nothing written, when the run does not qualify or the list
// ran full; the caller then takes the dense path.
static int search_matches_list(blg_ctx *c, blg_search *s, int k, blg_match *d_out, blg_match *host_out, int64_t cap,
                               int64_t *total, bool *done) {
    *done = false;
    *total = 0;
    if (k < 0 || k > 31 || !s->lsorted || c->sched == BLG_SCHED_PLAIN || !c->rl_hdr || c->rl_cap == 0)
        return BLG_OK;
    const SurvClasses C = seq_classes(s);
    if (C.n == 0 || C.n != (int)s->cls.size()) return BLG_OK;    // a lane-spread class: the dense path
    if (class_queries(s) != s->nq) return BLG_OK;                  // not every query's class: the dense path
    const int job = survivor_job_size(c, s, k);
    CK(launch(c, "surv_plan", [&] { return launch_surv_plan(c->stream, C, s->lstart, s->min_len, s->n_len, k, job); }),
       "surv_plan");
    const ResultList L{c->rl_hdr + 2, c->rl_hdr, c->rl_cap};
    const FillItems F{nullptr, nullptr, 0, BatchFill{nullptr, 0, BLG_UINT8, 0}, 0, c->rl_hdr + 1};
    CK(cudaMemsetAsync(c->rl_hdr, 0, 2 * sizeof(unsigned long long), c->stream), "clear list");
    CK(launch(c, "search_band_list", [&] {
           return launch_search_band(c->stream, c->sms, surv_ctas(c, k), surv_round(c, k), job, C, s->cs.d, s->perm,
                                     s->ccnt, s->qcnt, k, BLG_UINT8, nullptr, s->nc, nullptr, &L, &F, c->d_status);
       }), "search_band_list");
    unsigned long long cnt = 0;
    CK(cudaMemcpyAsync(&cnt, c->rl_hdr, sizeof(cnt), cudaMemcpyDeviceToHost, c->stream), "D2H list count");
    CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    if (cnt > c->rl_cap) return BLG_OK;                            // ran full: the dense path
    std::vector<unsigned long long> e(cnt);
    if (cnt) {
        CK(cudaMemcpyAsync(e.data(), c->rl_hdr + 2, sizeof(unsigned long long) * cnt, cudaMemcpyDeviceToHost,
                           c->stream), "D2H list");
        CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    }
    size_t keep = 0;
    for (auto x : e)
        if ((int)(x & 63u) <= k) e[keep++] = x;
    e.resize(keep);
    sort_by_index(e);
    const int64_t m = std::min<int64_t>((int64_t)keep, cap);
    std::vector<blg_match> staged;
    blg_match *rec = host_out;
    if (!rec && m > 0) {
        staged.resize((size_t)m);
        rec = staged.data();
    }
    for (int64_t i = 0; i < m; i++) {
        const int64_t idx = (int64_t)(e[(size_t)i] >> 8);
        rec[i].query = idx / s->nc;
        rec[i].choice = idx % s->nc;
        rec[i].dist = (int32_t)(e[(size_t)i] & 63u);
        rec[i].reserved = 0;
    }
    if (!host_out && m > 0) {
        CK(cudaMemcpyAsync(d_out, staged.data(), sizeof(blg_match) * (size_t)m, cudaMemcpyHostToDevice, c->stream),
           "H2D matches");
        CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    }
    *total = (int64_t)keep;
    *done = true;
    return BLG_OK;
}

static void search_release(blg_ctx *c, blg_search *s) {
    free_strings(c, s->q);
    free_strings(c, s->c);
    free_strings(c, s->cs);
    dev_free(c, s->sorted_mem);      // perm, lstart, sketches and the sorted copy live in it
    s->sorted_mem = nullptr;
    s->perm = nullptr;
    s->lstart = nullptr;
    s->csk = nullptr;
    s->lsorted = false;
    dev_free(c, s->tt_words);
    dev_free(c, s->tt_base);
    dev_free(c, s->tt_len);
    dev_free(c, s->pfx_mem);
    s->pfx_mem = nullptr;
    s->pfx_work = nullptr;
    s->pfx = false;
    dev_free(c, s->sk_mem);
    s->sk_mem = nullptr;
    s->csk = s->qsk = nullptr;
    s->ccnt = s->qcnt = nullptr;
    s->tt_words = nullptr;
    s->tt_base = nullptr;
    s->tt_len = nullptr;
    s->tt = false;
    free_classes(c, s);
}

// ------------------------------------------------------------ batches --
// A batch upload lays every problem out in two device blocks: `raw` (each
// problem's queries and choices as given, with slack) and `meta` (the rest,
// in three regions: A the choice permutations, copied from pinned memory in
// one copy; B the host-built tables -- length buckets, class query lists,
// launch descriptors, the jobs -- copied from the pinned arena in one copy;
// C what the device writes: sorted copies, offsets, sketches, Peq tables,
// survivor plans). The per-problem searches are views into those blocks.
struct blg_batch {
    std::vector<blg_search *> probs;
    std::vector<int> kk, dt;
    std::vector<void *> outs;
    std::vector<int> regular;         // problems outside the persistent kernel (long queries)
    void *d_raw = nullptr, *d_meta = nullptr;
    BatchJob *d_jobs = nullptr;       // views into d_meta
    int njobs = 0;
    int64_t *d_job_tiles = nullptr, *d_tile_base = nullptr;
    int32_t *d_work = nullptr;
    int nbanded = 0;
    BatchFill *d_fills = nullptr;
    int nfill = 0;
    int64_t max_fill = 0, pairs = 0;
    ResultList list{};                // the banded kernel's deferred results (list.item null: none)
    FillItems fill{};                 // the thresholded outputs as fill items of the banded kernel
    unsigned long long *hdr = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t graph_kernels = 0;
};

static void batch_release(blg_ctx *c, blg_batch *b) {
    for (auto *s : b->probs) {
        if (!s) continue;
        search_release(c, s);         // views: nothing of its own to free
        delete s;
    }
    b->probs.clear();
    dev_free(c, b->d_raw);
    dev_free(c, b->d_meta);
    b->d_raw = b->d_meta = nullptr;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

// Byte layout of a block: parts 256-byte aligned, in the order taken.
struct BlockLayout {
    size_t size = 0;
    size_t take(size_t bytes) {
        const size_t o = (size + 255) & ~size_t(255);
        size = o + bytes;
        return o;
    }
};

// The pinned arena of the context, at least `bytes` (null if it cannot be had).
static uint8_t *host_arena(blg_ctx *c, size_t bytes) {
    if (bytes > c->arena_bytes) {
        if (c->arena) cudaFreeHost(c->arena);
        c->arena = nullptr;
        c->arena_bytes = 0;
        if (cudaHostAlloc(&c->arena, bytes, cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        c->arena_bytes = bytes;
    }
    return (uint8_t *)c->arena;
}

// Problems are cut into up to kUploadGroups groups of similar byte counts.
// The choices stream in on the upload stream group by group (their bytes
// and offsets, two copies per problem); the host meanwhile finds each
// problem's length range and query classes and lays out the tables, with
// every problem's queries packed among them, which follow the first group's
// choices on the same stream in one copy. Each group's preparation kernels (length sort, sorted offsets,
// gather + sketches, Peq tables) start on the context stream once its
// strings have landed, so they overlap the next groups' copies.
constexpr int kUploadGroups = 8;

static int batch_upload_body(blg_ctx *c, const blg_problem *pr, int nprob, blg_batch *b,
                             std::vector<cudaEvent_t> &ev) {
    if (nprob < 0 || (nprob > 0 && !pr)) return fail(c, BLG_ERR_ARG, "bad problem list");
    auto pfail = [&](int i, const char *what) { return fail(c, BLG_ERR_ARG, "problem " + std::to_string(i) + ": " + what); };
    std::vector<char> work((size_t)nprob, 0);
    for (int i = 0; i < nprob; i++) {
        const blg_problem &p = pr[i];
        if (!dtype_ok(p.dtype)) return pfail(i, "bad dtype");
        if (p.nq < 0 || p.nc < 0) return pfail(i, "negative count");
        if (p.nq == 0 || p.nc == 0) continue;
        if (!p.d_out) return pfail(i, "null device output");
        int rc = check_offsets_host(c, p.off_q, p.nq);
        if (!rc) rc = check_offsets_host(c, p.off_c, p.nc);
        if (rc) return rc;
        if ((p.off_q[p.nq] > p.off_q[0] && !p.buf_q) || (p.off_c[p.nc] > p.off_c[0] && !p.buf_c))
            return pfail(i, "null buffer");
        work[i] = 1;
    }
    // ---- raw choices: one block; groups of contiguous problems with about
    // equal bytes. Queries: packed back to back (bytes at qpos, offsets at
    // qopos) into the tables' region, 16 zero bytes before them all and 48
    // after (a problem's neighbours are its slack).
    struct Raw { size_t c, coff; };
    std::vector<Raw> raw((size_t)nprob);
    std::vector<size_t> qpos((size_t)nprob, 0), qopos((size_t)nprob, 0);
    size_t qbytes = 0, qoffs = 0;
    BlockLayout rl;
    for (int i = 0; i < nprob; i++) {
        if (!work[i]) continue;
        const blg_problem &p = pr[i];
        raw[i].c = rl.take(kSlackBefore + (size_t)(p.off_c[p.nc] - p.off_c[0]) + kSlackAfter) + kSlackBefore;
        raw[i].coff = rl.take(8 * (size_t)(p.nc + 1));
        qpos[i] = qbytes;
        qopos[i] = qoffs;
        qbytes += (size_t)(p.off_q[p.nq] - p.off_q[0]);
        qoffs += (size_t)p.nq + 1;
    }
    std::vector<int> grp((size_t)nprob, 0);
    int G = 0;
    {
        size_t done = 0;
        for (int i = 0; i < nprob; i++) {
            if (!work[i]) continue;
            grp[i] = std::min(kUploadGroups - 1, (int)(done * kUploadGroups / std::max<size_t>(rl.size, 1)));
            done = raw[i].coff + 8 * (size_t)(pr[i].nc + 1);
            G = grp[i] + 1;
        }
    }
    // events: [0, G) each group's strings landed (group 0: and the tables);
    // [G] the strings' block allocated; [G + 1] the tables' block allocated
    for (int g = 0; g < G + 2; g++) {
        cudaEvent_t e;
        CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
        ev.push_back(e);
    }
    if (rl.size) CK(dev_alloc(c, &b->d_raw, rl.size), "cudaMallocAsync(batch strings)");
    CK(cudaEventRecord(ev[G], c->stream), "event");
    CK(cudaStreamWaitEvent(c->up, ev[G], 0), "wait");
    uint8_t *R = (uint8_t *)b->d_raw;
    for (int i = 0; i < nprob; i++) {
        const blg_problem &p = pr[i];
        blg_search *s = new (std::nothrow) blg_search();
        if (!s) return fail(c, BLG_ERR_ALLOC, "host allocation");
        b->probs.push_back(s);
        b->kk.push_back(p.max_dist < 0 ? -1 : p.max_dist);
        b->dt.push_back(p.dtype);
        b->outs.push_back(p.d_out);
        if (!work[i]) continue;
        s->nq = p.nq;
        s->nc = p.nc;
        auto view = [&](OwnedStrings &o, size_t at, size_t off_at, const int64_t *off, int64_t n) {
            o.d.buf = R + at;
            o.d.off = (const int64_t *)(R + off_at);
            o.d.n = n;
            o.d.base = off[0];
            o.d.bytes = off[n] - off[0];
        };
        view(s->c, raw[i].c, raw[i].coff, p.off_c, p.nc);
        b->pairs += p.nq * p.nc;
    }
    // the choices of problems [i0, i1) on the upload stream
    auto copy_raw = [&](int i0, int i1) -> cudaError_t {
        for (int i = i0; i < i1; i++) {
            if (!work[i]) continue;
            const blg_problem &p = pr[i];
            const DevStrings &d = b->probs[i]->c.d;
            cudaError_t e = cudaSuccess;
            if (d.bytes > 0)
                e = cudaMemcpyAsync((uint8_t *)d.buf, p.buf_c + p.off_c[0], (size_t)d.bytes, cudaMemcpyHostToDevice, c->up);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync((int64_t *)d.off, p.off_c, 8 * (size_t)(p.nc + 1), cudaMemcpyHostToDevice, c->up);
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    };
    int g0_end = 0;                           // the first problem after group 0
    while (g0_end < nprob && (!work[g0_end] || grp[g0_end] == 0)) g0_end++;
    CK(copy_raw(0, g0_end), "H2D batch strings");
    // ---- host, while group 0's strings fly: each problem's length range
    // (choices) and query classes, problems spread over the pool
    struct Prep {
        int64_t mn = 0, mx = 0;
        bool ok = true, neg = false;
        std::vector<QueryClass> cls;
    };
    std::vector<Prep> prep((size_t)nprob);
    std::vector<int> order;
    for (int i = 0; i < nprob; i++)
        if (work[i]) order.push_back(i);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return pr[x].nc > pr[y].nc; });
    std::atomic<size_t> next{0};
    HostPool::get().run(HostPool::get().size(), [&](int) {
        for (size_t t; (t = next++) < order.size();) {
            const int i = order[t];
            Prep &P = prep[i];
            const int64_t *oc = pr[i].off_c, *oq = pr[i].off_q;
            int64_t mn = INT64_MAX, mx = INT64_MIN;
            for (int64_t x = 0; x < pr[i].nc; x++) {
                const int64_t l = oc[x + 1] - oc[x];
                mn = std::min(mn, l);
                mx = std::max(mx, l);
            }
            for (int64_t x = 0; x < pr[i].nq; x++) P.neg |= oq[x + 1] < oq[x];
            P.mn = mn;
            P.mx = mx;
            P.neg |= mn < 0;
            P.ok = query_classes(oq, 0, pr[i].nq, P.cls);
        }
    });
    for (int i = 0; i < nprob; i++) {
        if (!work[i]) continue;
        if (prep[i].neg) return fail(c, BLG_ERR_ARG, "corrupt offsets (not monotone or out of range)");
        if (!prep[i].ok) return fail(c, BLG_ERR_ARG, "query longer than 2048 bytes is not supported");
    }
    // ---- which problems the persistent kernels take; the jobs and fills
    std::vector<char> sorted((size_t)nprob, 0), eligible((size_t)nprob, 0);
    int njobs = 0, nfill = 0, nclass = 0, nsorted = 0, nwork = 0;
    for (int i = 0; i < nprob; i++) {
        if (!work[i]) continue;
        nwork++;
        nclass += (int)prep[i].cls.size();
        sorted[i] = pr[i].nc < INT32_MAX && prep[i].mx - prep[i].mn < (1 << 22);
        nsorted += sorted[i];
        bool e = sorted[i];
        for (auto &q : prep[i].cls) e &= !q.lanes && q.nw <= kBatchMaxWords;
        eligible[i] = e;
        if (e) {
            njobs += (int)prep[i].cls.size();
            if (b->kk[i] >= 0) nfill++;
        } else {
            b->regular.push_back(i);
        }
    }
    // ---- the meta block: B host-built tables, then C device-written
    struct At {
        size_t hist = 0, tab = 0, perm = 0, soff = 0, csk = 0, ccnt = 0, sbuf = 0, qsk = 0, qcnt = 0;
        std::vector<size_t> both, lo, hi, wk, ts, peq;
    };
    std::vector<At> at((size_t)nprob);
    BlockLayout ml;
    const size_t b_begin = ml.take(0);
    const size_t b_qbytes = ml.take(kSlackBefore + qbytes + kSlackAfter), b_qoff = ml.take(8 * qoffs);
    for (int i = 0; i < nprob; i++)
        if (work[i])
            for (auto &q : prep[i].cls) at[i].both.push_back(ml.take(sizeof(int32_t) * 2 * q.idx.size()));
    const size_t b_ls = ml.take(sizeof(LenSortSet) * (size_t)nsorted),
                 b_ls_start = ml.take(sizeof(int64_t) * (size_t)(nsorted + 1)),
                 b_prep = ml.take(sizeof(UploadPrep) * (size_t)nwork),
                 b_prep_start = ml.take(sizeof(int64_t) * (size_t)(nwork + 1)),
                 b_sk = ml.take(sizeof(SketchSet) * (size_t)(nwork + nsorted)),
                 b_sk_start = ml.take(sizeof(int64_t) * (size_t)(nwork + nsorted + 1)),
                 b_peq = ml.take(sizeof(PeqSet) * (size_t)nclass),
                 b_peq_start = ml.take(sizeof(int64_t) * (size_t)(nclass + 1)),
                 b_jobs = ml.take(sizeof(BatchJob) * (size_t)njobs),
                 b_fills = ml.take(sizeof(BatchFill) * (size_t)nfill),
                 b_fstart = ml.take(sizeof(int64_t) * (size_t)(nfill + 1));
    const size_t b_end = ml.take(0);
    const size_t c_hist = ml.take(0);         // the count arrays, contiguous: one memset clears them
    for (int i = 0; i < nprob; i++)
        if (work[i] && sorted[i]) at[i].hist = ml.take(8 * (size_t)(prep[i].mx - prep[i].mn + 1));
    const size_t c_hist_end = ml.take(0);
    for (int i = 0; i < nprob; i++) {
        if (!work[i]) continue;
        const blg_problem &p = pr[i];
        if (sorted[i]) {
            const int64_t n_len = prep[i].mx - prep[i].mn + 1;
            at[i].tab = ml.take(sizeof(int64_t) * (size_t)(2 * n_len + 1));
            at[i].perm = ml.take(sizeof(int32_t) * (size_t)p.nc);
            at[i].soff = ml.take(sizeof(int64_t) * (size_t)(p.nc + 1));
            at[i].csk = ml.take(sizeof(uint64_t) * (size_t)p.nc);
            at[i].ccnt = ml.take(sizeof(uint4) * (size_t)p.nc);
            at[i].sbuf = ml.take(kSlackBefore + (size_t)b->probs[i]->c.d.bytes + kSlackAfter) + kSlackBefore;
        }
        at[i].qsk = ml.take(sizeof(uint64_t) * (size_t)p.nq);
        at[i].qcnt = ml.take(sizeof(uint4) * (size_t)p.nq);
        for (auto &q : prep[i].cls) {
            const size_t nq = q.idx.size();
            at[i].lo.push_back(ml.take(4 * nq));
            at[i].hi.push_back(ml.take(4 * nq));
            at[i].wk.push_back(ml.take(256));
            at[i].ts.push_back(ml.take(8 * (nq + 1)));
            at[i].peq.push_back(ml.take(sizeof(uint64_t) * 256 * (size_t)q.nw * nq));
        }
    }
    const size_t c_job_tiles = ml.take(sizeof(int64_t) * (size_t)std::max(njobs, 1)),
                 c_tile_base = ml.take(sizeof(int64_t) * (size_t)(njobs + 1)), c_work = ml.take(2 * sizeof(int32_t));
    // the banded kernel's deferred results: [count, fill items claimed], entries
    constexpr unsigned long long kBatchListCap = 1u << 20;
    const size_t c_list = ml.take(sizeof(unsigned long long) * (2 + kBatchListCap));
    CK(dev_alloc(c, &b->d_meta, ml.size), "cudaMallocAsync(batch tables)");
    CK(cudaEventRecord(ev[G + 1], c->stream), "event");
    uint8_t *M = (uint8_t *)b->d_meta;
    // ---- the problems' views, and region B built in the pinned arena
    const size_t b_bytes = b_end - b_begin;
    std::vector<uint8_t> pageable;
    uint8_t *H = host_arena(c, b_bytes);
    if (!H) {
        pageable.resize(b_bytes);
        H = pageable.data();
    }
    auto hb = [&](size_t off) { return H + (off - b_begin); };
    // the queries, packed (a problem's bytes and its offsets as given)
    {
        uint8_t *qb = hb(b_qbytes);
        memset(qb, 0, kSlackBefore);
        memset(qb + kSlackBefore + qbytes, 0, kSlackAfter);
        std::atomic<int> nx{0};
        HostPool::get().run(HostPool::get().size(), [&](int) {
            for (int i; (i = nx++) < nprob;) {
                if (!work[i]) continue;
                const blg_problem &p = pr[i];
                const size_t nb = (size_t)(p.off_q[p.nq] - p.off_q[0]);
                if (nb) memcpy(qb + kSlackBefore + qpos[i], p.buf_q + p.off_q[0], nb);
                memcpy(hb(b_qoff) + 8 * qopos[i], p.off_q, 8 * (size_t)(p.nq + 1));
            }
        });
    }
    LenSortSet *lss = (LenSortSet *)hb(b_ls);
    int64_t *lss_start = (int64_t *)hb(b_ls_start);
    UploadPrep *ups = (UploadPrep *)hb(b_prep);
    int64_t *ups_start = (int64_t *)hb(b_prep_start);
    SketchSet *sks = (SketchSet *)hb(b_sk);
    int64_t *sks_start = (int64_t *)hb(b_sk_start);
    PeqSet *pqs = (PeqSet *)hb(b_peq);
    int64_t *pqs_start = (int64_t *)hb(b_peq_start);
    BatchJob *jobs = (BatchJob *)hb(b_jobs);
    BatchFill *fills = (BatchFill *)hb(b_fills);
    int nl = 0, nu = 0, nsk = 0, npq = 0, nj = 0, nf = 0, max_nwc = 1;
    lss_start[0] = ups_start[0] = sks_start[0] = pqs_start[0] = 0;
    // each group's first set of every kind
    std::vector<int> gl((size_t)G + 1, 0), gu((size_t)G + 1, 0), gk((size_t)G + 1, 0), gq((size_t)G + 1, 0);
    for (int i = 0; i < nprob; i++) {
        if (!work[i]) continue;
        const blg_problem &p = pr[i];
        blg_search *s = b->probs[i];
        Prep &P = prep[i];
        for (int g = grp[i] + 1; g <= G; g++) {
            gl[g] = nl + (sorted[i] ? 1 : 0);
            gu[g] = nu + 1;
            gk[g] = nsk + 1 + (sorted[i] ? 1 : 0);
            gq[g] = npq + (int)P.cls.size();
        }
        s->q.d.buf = M + b_qbytes + kSlackBefore + qpos[i];
        s->q.d.off = (const int64_t *)(M + b_qoff) + qopos[i];
        s->q.d.n = p.nq;
        s->q.d.base = p.off_q[0];
        s->q.d.bytes = p.off_q[p.nq] - p.off_q[0];
        s->qsk = (uint64_t *)(M + at[i].qsk);
        s->qcnt = (uint4 *)(M + at[i].qcnt);
        UploadPrep u{};                          // (the packed queries' slack came with the tables)
        u.buf[1] = (uint8_t *)s->c.d.buf;
        u.bytes[1] = s->c.d.bytes;
        sks[nsk] = SketchSet{s->q.d, nullptr, nullptr, nullptr, s->qsk, s->qcnt, p.nq};
        sks_start[nsk + 1] = sks_start[nsk] + p.nq;
        nsk++;
        if (sorted[i]) {
            const int64_t n_len = P.mx - P.mn + 1;
            s->perm = (int32_t *)(M + at[i].perm);
            s->lstart = (int64_t *)(M + at[i].tab);
            s->csk = (uint64_t *)(M + at[i].csk);
            s->ccnt = (uint4 *)(M + at[i].ccnt);
            s->cs.d.buf = M + at[i].sbuf;
            s->cs.d.off = (const int64_t *)(M + at[i].soff);
            s->cs.d.n = p.nc;
            s->cs.d.base = 0;
            s->cs.d.bytes = s->c.d.bytes;
            s->min_len = P.mn;
            s->n_len = n_len;
            s->lsorted = true;
            lss[nl] = LenSortSet{s->c.d.off, p.nc, P.mn, n_len, (unsigned long long *)(M + at[i].hist), s->lstart,
                                 s->lstart + n_len + 1, s->perm};
            lss_start[nl + 1] = lss_start[nl] + p.nc;
            nl++;
            u.buf[2] = M + at[i].sbuf;
            u.bytes[2] = s->c.d.bytes;
            u.lstart = s->lstart;
            u.bstart = s->lstart + n_len + 1;
            u.n_len = n_len;
            u.min_len = P.mn;
            u.n_sorted = p.nc;
            u.soff = (int64_t *)(M + at[i].soff);
            sks[nsk] = SketchSet{s->c.d, s->perm, s->cs.d.off, M + at[i].sbuf, s->csk, s->ccnt, p.nc};
            sks_start[nsk + 1] = sks_start[nsk] + p.nc;
            nsk++;
        }
        ups[nu] = u;
        ups_start[nu + 1] = ups_start[nu] + u.n_sorted + 1;
        nu++;
        for (size_t x = 0; x < P.cls.size(); x++) {
            const QueryClass &q = P.cls[x];
            const size_t nq = q.idx.size();
            blg_search::Cls k{};
            k.lanes = q.lanes;
            k.nw = q.nw;
            k.nq = (int)nq;
            k.qidx = (int32_t *)(M + at[i].both[x]);
            k.qlen = k.qidx + nq;
            k.lo = (int32_t *)(M + at[i].lo[x]);
            k.hi = (int32_t *)(M + at[i].hi[x]);
            k.work = (int32_t *)(M + at[i].wk[x]);
            k.tile_start = (int64_t *)(M + at[i].ts[x]);
            k.peq = (uint64_t *)(M + at[i].peq[x]);
            k.mem = nullptr;
            k.h_qlen = q.len;
            int32_t *both = (int32_t *)hb(at[i].both[x]);
            std::copy(q.idx.begin(), q.idx.end(), both);
            std::copy(q.len.begin(), q.len.end(), both + nq);
            pqs[npq] = PeqSet{s->q.d, k.qidx, k.peq, k.nw};
            pqs_start[npq + 1] = pqs_start[npq] + (int64_t)nq;
            npq++;
            max_nwc = std::max(max_nwc, k.nw);
            s->cls.push_back(std::move(k));
        }
        if (!eligible[i]) continue;
        const int k = b->kk[i];
        for (auto &cl : s->cls) {
            BatchJob j{};
            j.CS = s->cs.d;
            j.perm = s->perm;
            j.lstart = s->lstart;
            j.min_len = s->min_len;
            j.n_len = s->n_len;
            j.cls = SearchClass{cl.nw, cl.nq, cl.qidx, cl.qlen, cl.peq};
            j.lo = cl.lo;
            j.hi = cl.hi;
            j.tile_start = cl.tile_start;
            j.nc = p.nc;
            j.k = k;
            j.dtype = p.dtype;
            j.nw = cl.nw;
            j.tile = 1024;                      // survivors per work unit (config 5: 0.99 ms per step; 1.30 with 4096)
            j.csk = s->csk;
            j.qsk = s->qsk;
            j.ccnt = s->ccnt;
            j.qcnt = s->qcnt;
            j.out = p.d_out;
            jobs[nj++] = j;
        }
        if (k >= 0) {
            const uint32_t v = (uint32_t)(p.dtype == BLG_UINT8 ? std::min(k + 1, 255)
                                          : p.dtype == BLG_UINT16 ? std::min(k + 1, 65535) : k + 1);
            fills[nf++] = BatchFill{p.d_out, p.nq * p.nc, p.dtype, v};
            b->max_fill = std::max(b->max_fill, p.nq * p.nc * (int64_t)dtype_size(p.dtype));
        }
    }
    // banded jobs first (they run in their own persistent kernel)
    std::stable_partition(jobs, jobs + nj, [](const BatchJob &j) { return j.k >= 0 && j.k <= 31; });
    b->nbanded = (int)std::count_if(jobs, jobs + nj, [](const BatchJob &j) { return j.k >= 0 && j.k <= 31; });
    b->njobs = nj;
    b->nfill = nf;
    b->d_jobs = (BatchJob *)(M + b_jobs);
    b->d_fills = (BatchFill *)(M + b_fills);
    b->d_job_tiles = (int64_t *)(M + c_job_tiles);
    b->d_tile_base = (int64_t *)(M + c_tile_base);
    b->d_work = (int32_t *)(M + c_work);
    int64_t *fstart = (int64_t *)hb(b_fstart);
    fstart[0] = 0;
    for (int f = 0; f < nf; f++) fstart[f + 1] = fstart[f] + fill_items_of(fills[f]);
    b->hdr = (unsigned long long *)(M + c_list);
    b->list = ResultList{b->hdr + 2, b->hdr, kBatchListCap};
    b->fill = FillItems{b->d_fills, (const int64_t *)(M + b_fstart), nf, BatchFill{}, fstart[nf], b->hdr + 1};
    // ---- the tables behind group 0's strings, then the other groups
    CK(cudaStreamWaitEvent(c->up, ev[G + 1], 0), "wait");
    CK(cudaMemcpyAsync(M + b_begin, H, b_bytes, cudaMemcpyHostToDevice, c->up), "H2D batch tables");
    if (G > 0) CK(cudaEventRecord(ev[0], c->up), "event");
    for (int g = 1; g < G; g++) {
        int i0 = 0, i1 = 0;
        while (i0 < nprob && (!work[i0] || grp[i0] < g)) i0++;
        i1 = i0;
        while (i1 < nprob && (!work[i1] || grp[i1] == g)) i1++;
        CK(copy_raw(i0, i1), "H2D batch strings");
        CK(cudaEventRecord(ev[g], c->up), "event");
    }
    if (c_hist_end > c_hist) CK(cudaMemsetAsync(M + c_hist, 0, c_hist_end - c_hist, c->stream), "memset counts");
    for (int g = 0; g < G; g++) {
        CK(cudaStreamWaitEvent(c->stream, ev[g], 0), "wait");
        const int l0 = gl[g], l1 = gl[g + 1], u0 = gu[g], u1 = gu[g + 1], k0 = gk[g], k1 = gk[g + 1], q0 = gq[g],
                  q1 = gq[g + 1];
        CK(launch(c, "length_sort", [&] {
               return launch_length_sort(c->stream, c->sms, (const LenSortSet *)(M + b_ls) + l0,
                                         (const int64_t *)(M + b_ls_start) + l0, l1 - l0, lss_start[l0],
                                         lss_start[l1] - lss_start[l0]);
           }), "length_sort");
        CK(launch(c, "upload_prep", [&] {
               return launch_upload_prep(c->stream, c->sms, (const UploadPrep *)(M + b_prep) + u0,
                                         (const int64_t *)(M + b_prep_start) + u0, u1 - u0, ups_start[u0],
                                         ups_start[u1] - ups_start[u0]);
           }), "upload_prep");
        CK(launch(c, "sketch_sets", [&] {
               return launch_sketch_sets(c->stream, c->sms, (const SketchSet *)(M + b_sk) + k0,
                                         (const int64_t *)(M + b_sk_start) + k0, k1 - k0, sks_start[k0],
                                         sks_start[k1] - sks_start[k0], c->d_status);
           }), "sketch_sets");
        CK(launch(c, "peq_sets", [&] {
               return launch_peq_sets(c->stream, (const PeqSet *)(M + b_peq) + q0, (const int64_t *)(M + b_peq_start) + q0,
                                      q1 - q0, pqs_start[q0], pqs_start[q1] - pqs_start[q0], max_nwc, c->d_status);
           }), "peq_sets");
    }
    CK(batch_set_attributes(), "kernel attributes");
    // the arena is read by the tables' copy; the context stream waited for
    // every group's strings
    CK(cudaStreamSynchronize(c->stream), "sync upload");
    // problems outside the persistent kernels plan their survivor jobs on
    // the host from the length buckets
    for (int i : b->regular) {
        blg_search *s = b->probs[i];
        if (!s->lsorted) continue;
        s->h_lstart.resize((size_t)s->n_len + 1);
        CK(cudaMemcpy(s->h_lstart.data(), s->lstart, 8 * (size_t)(s->n_len + 1), cudaMemcpyDeviceToHost),
           "D2H length buckets");
    }
    return BLG_OK;
}

static int batch_upload(blg_ctx *c, const blg_problem *pr, int nprob, blg_batch *b) {
    std::vector<cudaEvent_t> ev;
    const int rc = batch_upload_body(c, pr, nprob, b, ev);
    // after a failure, copies on the upload stream may still be in flight:
    // they end before the caller frees their destination
    cudaStreamSynchronize(c->up);
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
    return rc;
}

// First run: capture the batch's launches into one CUDA graph; every run
// then replays it on the context's stream.
static int batch_run(blg_ctx *c, blg_batch *b) {
    if (!b->exec) {
        const bool prof = c->prof;
        c->prof = false;                      // no per-launch events inside a capture
        const int64_t before = c->launches;
        CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed), "begin capture");
        BatchPlan plan{b->d_jobs, b->njobs, b->nbanded, b->d_job_tiles, b->d_tile_base, b->d_work, b->list,
                       b->fill, b->hdr};
        int nk = 0;
        cudaError_t e = launch_batch(c->stream, c->sms, plan, b->d_fills, b->nfill, b->max_fill, c->d_status, &nk);
        int rc = e == cudaSuccess ? BLG_OK : cuda_fail(c, e, "batch launch");
        for (int i : b->regular)
            if (!rc) rc = search_run(c, b->probs[i], b->kk[i], b->dt[i], b->outs[i]);
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(c->stream, &g);
        c->prof = prof;
        if (rc) { if (g) cudaGraphDestroy(g); return rc; }
        if (e != cudaSuccess) return cuda_fail(c, e, "end capture");
        e = cudaGraphInstantiate(&b->exec, g, 0);
        if (e != cudaSuccess) { cudaGraphDestroy(g); return cuda_fail(c, e, "graph instantiate"); }
        b->graph = g;
        b->graph_kernels = nk + (c->launches - before);
        c->launches = before;
    }
    CK(launch(c, "batch_graph", [&] { return cudaGraphLaunch(b->exec, c->stream); }), "graph launch");
    c->launches += b->graph_kernels - 1;
    return BLG_OK;
}

// ============================================================ autotuner ==
// Launch shapes are timed on synthetic inputs of each bucket (random DNA,
// fixed seed) and the fastest kept per device:
//   exact search:        queries per CTA, for queries of 1, 2 and 4 words
//                        (1024 queries x 65536 choices of the same length);
//   thresholded search:  CTAs per SM x columns per lane round, for max_dist
//                        <= 8 (1024 queries x 2^20 choices, lengths 100..256,
//                        5% planted near-copies, max_dist 4) and for 9..31
//                        (256 x 2^18, max_dist 16);
//   banded pairs solver: CTAs per SM (2^19 pairs, lengths 8..256, edit rates
//                        0..30%), for max_dist <= 15 (timed at 8) and 16..31
//                        (timed at 24);
//   short-pair tiles:    the staging shape (2^20 pairs of 32 bytes, 5%
//                        edits, exact).
// Results never depend on a shape; only time does.
namespace {

struct Rng {
    uint64_t s;
    uint32_t next() {
        s ^= s << 13;
        s ^= s >> 7;
        s ^= s << 17;
        return (uint32_t)(s >> 16);
    }
    double uni() { return (next() & 0xffffff) / 16777216.0; }
};

struct Packed {
    std::vector<uint8_t> buf;
    std::vector<int64_t> off{0};
    void add(const std::vector<uint8_t> &x) {
        buf.insert(buf.end(), x.begin(), x.end());
        off.push_back((int64_t)buf.size());
    }
    int64_t n() const { return (int64_t)off.size() - 1; }
    const uint8_t *data() const { return buf.empty() ? nullptr : buf.data(); }
};

// Random DNA, 16 bases per generator step.
std::vector<uint8_t> dna(Rng &r, int len) {
    static const uint8_t A[4] = {'A', 'C', 'G', 'T'};
    std::vector<uint8_t> x(len);
    uint32_t bits = 0;
    for (int i = 0; i < len; i++) {
        if ((i & 15) == 0) bits = r.next();
        x[i] = A[bits & 3];
        bits >>= 2;
    }
    return x;
}

std::vector<uint8_t> mutate(Rng &r, const std::vector<uint8_t> &a, double rate) {
    static const uint8_t A[4] = {'A', 'C', 'G', 'T'};
    std::vector<uint8_t> b;
    for (uint8_t ch : a) {
        if (r.uni() < rate) {
            const uint32_t op = r.next() % 3;
            if (op == 0) b.push_back(A[r.next() & 3]);                 // substitute
            else if (op == 1) { b.push_back(A[r.next() & 3]); b.push_back(ch); }   // insert before
            continue;                                                   // delete (op 2) or done
        }
        b.push_back(ch);
    }
    return b;
}

}  // namespace

// Event time (ms) of the fastest of `reps` runs of `fn` on the context stream.
template <typename F>
static int time_best(blg_ctx *c, int reps, F &&fn, float *best) {
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0), "event");
    CK(cudaEventCreate(&e1), "event");
    int rc = fn();                                      // warm-up
    *best = 1e30f;
    for (int r = 0; r < reps && !rc; r++) {
        cudaEventRecord(e0, c->stream);
        rc = fn();
        cudaEventRecord(e1, c->stream);
        if (cudaEventSynchronize(e1) != cudaSuccess) rc = fail(c, BLG_ERR_CUDA, "timing");
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        *best = std::min(*best, ms);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!rc) rc = sync_and_status(c);
    return rc;
}

static int tune_exact_search(blg_ctx *c, int nw) {
    Rng r{0x9E3779B97F4A7C15ull ^ (uint64_t)nw};
    Packed q, ch;
    const int len = 64 * nw;
    for (int i = 0; i < 1024; i++) q.add(dna(r, len));
    for (int i = 0; i < 65536; i++) ch.add(dna(r, len));
    blg_search s;
    int rc = search_upload(c, q.data(), q.off.data(), q.n(), ch.data(), ch.off.data(), ch.n(), &s);
    void *out = nullptr;
    if (!rc && dev_alloc(c, &out, sizeof(int32_t) * (size_t)q.n() * ch.n()) != cudaSuccess)
        rc = fail(c, BLG_ERR_ALLOC, "tuning output");
    float best_ms = 1e30f;
    int best = 0;
    for (int qpb : {4, 8, 16, 32, 64}) {
        if (rc) break;
        c->tune.qpb[nw] = qpb;
        float ms = 0.f;
        rc = time_best(c, 3, [&] { return search_run(c, &s, -1, BLG_INT32, out); }, &ms);
        if (!rc && ms < best_ms) { best_ms = ms; best = qpb; }
    }
    c->tune.qpb[nw] = rc ? 0 : best;
    dev_free(c, out);
    search_release(c, &s);
    return rc;
}

// The survivor kernel's CTAs per SM and columns per lane round for max_dist
// k, on a search big enough that the run-time job size (survivor_job_size)
// keeps the 4096-survivor jobs. k = 4 (the shapes of max_dist <= 8): 1024
// queries x 2^20 choices. Smaller searches misled it: 512 x 2^19 picked 3
// CTAs per SM in two runs of three, 7% slower at 1024 x 2^20 than the 4 it
// picks there (the output fill and the job tail weigh differently), and a
// still smaller one had its jobs halved at run time whatever the candidate.
// k = 16 (max_dist 9..31): 256 queries x 2^18 choices, where the wider band
// lets 4x more length candidates through the length filter and more of
// them past the 4-gram bound, and each passer runs longer.
static int tune_threshold_search(blg_ctx *c, int k) {
    Rng r{0x2545F4914F6CDD1Dull ^ (uint64_t)k};
    Packed q, ch;
    std::vector<std::vector<uint8_t>> qs;
    const int nq = k < kSurvWideK ? 1024 : 256, nc = k < kSurvWideK ? (1 << 20) : (1 << 18);
    for (int i = 0; i < nq; i++) {
        qs.push_back(dna(r, 100 + (int)(r.next() % 157)));
        q.add(qs.back());
    }
    for (int i = 0; i < nc; i++) {
        if (r.uni() < 0.05) ch.add(mutate(r, qs[r.next() % qs.size()], 0.05 * r.uni()));
        else ch.add(dna(r, 100 + (int)(r.next() % 157)));
    }
    blg_search s;
    int rc = search_upload(c, q.data(), q.off.data(), q.n(), ch.data(), ch.off.data(), ch.n(), &s);
    void *out = nullptr;
    if (!rc && dev_alloc(c, &out, (size_t)q.n() * ch.n()) != cudaSuccess) rc = fail(c, BLG_ERR_ALLOC, "tuning output");
    // The job size stays at its maximum, 4096: on 1024 x 2^20 it measured 8%
    // faster than 2048, while a search of this size cannot tell them apart;
    // smaller searches get smaller jobs at run time (survivor_job_size).
    // CTAs per SM x columns per lane round, set in the bucket k runs in
    int &ctas_t = k < kSurvWideK ? c->tune.lpt_ctas : c->tune.lpt_ctas_wide;
    int &round_t = k < kSurvWideK ? c->tune.surv_round : c->tune.surv_round_wide;
    float best_ms = 1e30f;
    int best_ctas = ctas_t, best_round = round_t;
    c->tune.lpt_job = 4096;
    for (int ctas : {2, 3, 4})
        for (int round : {8, 16, 32}) {
            if (rc) break;
            ctas_t = ctas;
            round_t = round;
            float ms = 0.f;
            rc = time_best(c, 5, [&] { return search_run(c, &s, k, BLG_UINT8, out); }, &ms);
            if (!rc && ms < best_ms) {
                best_ms = ms;
                best_ctas = ctas;
                best_round = round;
            }
        }
    ctas_t = best_ctas;
    round_t = best_round;
    dev_free(c, out);
    search_release(c, &s);
    return rc;
}

// CTAs per SM of the banded pairs solver for max_dist k (8: the shape of
// max_dist <= 15; 24: max_dist 16..31), on 2^19 pairs of lengths 8..256
// with edit rates 0..30%.
static int tune_band_pairs(blg_ctx *c, int k) {
    Rng r{0xD1B54A32D192ED03ull};
    Packed a, b;
    for (int i = 0; i < (1 << 19); i++) {
        std::vector<uint8_t> x = dna(r, 8 + (int)(r.next() % 249));
        b.add(mutate(r, x, 0.3 * r.uni()));
        a.add(x);
    }
    blg_pairs p;
    int rc = pairs_upload(c, a.data(), a.off.data(), b.data(), b.off.data(), a.n(), &p);
    void *out = nullptr;
    if (!rc && dev_alloc(c, &out, (size_t)a.n()) != cudaSuccess) rc = fail(c, BLG_ERR_ALLOC, "tuning output");
    if (!rc) rc = pairs_learn_alphabet(c, &p);
    const int sched = c->sched;
    c->sched = BLG_SCHED_AUTO;
    int &ctas_t = k < kBandWideK ? c->tune.band_ctas : c->tune.band_ctas_wide;
    float best_ms = 1e30f;
    int best = ctas_t;
    for (int ctas : {2, 3}) {
        if (rc) break;
        ctas_t = ctas;
        float ms = 0.f;
        rc = time_best(c, 3, [&] { return pairs_run(c, &p, k, BLG_UINT8, out); }, &ms);
        if (!rc && ms < best_ms) { best_ms = ms; best = ctas; }
    }
    c->sched = sched;
    ctas_t = best;
    dev_free(c, out);
    pairs_release(c, &p);
    return rc;
}

static int tune_tile_pairs(blg_ctx *c) {
    Rng r{0x5DEECE66Dull};
    Packed a, b;
    for (int i = 0; i < (1 << 20); i++) {
        std::vector<uint8_t> x = dna(r, 32);
        b.add(mutate(r, x, 0.05));
        a.add(x);
    }
    blg_pairs p;
    int rc = pairs_upload(c, a.data(), a.off.data(), b.data(), b.off.data(), a.n(), &p);
    void *out = nullptr;
    if (!rc && dev_alloc(c, &out, sizeof(int32_t) * (size_t)a.n()) != cudaSuccess) rc = fail(c, BLG_ERR_ALLOC, "tuning output");
    if (!rc) rc = pairs_learn_alphabet(c, &p);
    float best_ms = 1e30f;
    int best = c->tune.tile_shape;
    for (int shape : {1, 2, 3}) {
        if (rc) break;
        c->tune.tile_shape = shape;
        float ms = 0.f;
        rc = time_best(c, 5, [&] { return pairs_run(c, &p, -1, BLG_INT32, out); }, &ms);
        if (!rc && ms < best_ms) { best_ms = ms; best = shape; }
    }
    c->tune.tile_shape = best;
    dev_free(c, out);
    pairs_release(c, &p);
    return rc;
}

static std::string tuning_header(blg_ctx *c) {
    // the version tag changes whenever a tuned kernel's shape limits change
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, c->device);
    std::string name = prop.name;
    for (auto &ch : name)
        if (ch == ' ') ch = '_';
    return "BLGTUNE7 " + name + " sm" + std::to_string(prop.major * 10 + prop.minor) + " " + std::to_string(c->sms) +
           " " + std::to_string(blg_version());
}

static bool tuning_load(blg_ctx *c, const char *path) {
    FILE *f = fopen(path, "r");
    if (!f) return false;
    char line[256];
    bool ok = fgets(line, sizeof(line), f) && std::string(line) == tuning_header(c) + "\n";
    blg_tuning t;
    int fields = 0;
    while (ok && fgets(line, sizeof(line), f)) {
        char key[64];
        int v = 0;
        if (sscanf(line, "%63s %d", key, &v) != 2) continue;
        const std::string k = key;
        if (k.rfind("qpb", 0) == 0) {
            const int w = atoi(k.c_str() + 3);
            if (w >= 1 && w <= 8 && v >= 0 && v <= 4096) { t.qpb[w] = v; fields++; }
        } else if (k == "lpt_ctas" && v >= 1 && v <= 8) { t.lpt_ctas = v; fields++; }
        else if (k == "lpt_job" && v >= 256 && v <= 4096) { t.lpt_job = v; fields++; }
        else if (k == "surv_round" && (v == 8 || v == 16 || v == 32)) { t.surv_round = v; fields++; }
        else if (k == "lpt_ctas_wide" && v >= 1 && v <= 8) { t.lpt_ctas_wide = v; fields++; }
        else if (k == "surv_round_wide" && (v == 8 || v == 16 || v == 32)) { t.surv_round_wide = v; fields++; }
        else if (k == "band_ctas" && v >= 1 && v <= 3) { t.band_ctas = v; fields++; }
        else if (k == "band_ctas_wide" && v >= 1 && v <= 3) { t.band_ctas_wide = v; fields++; }
        else if (k == "tile_shape" && v >= 1 && v <= 3) { t.tile_shape = v; fields++; }
    }
    fclose(f);
    if (!ok || fields < 16) return false;
    t.tuned = 2;                                        // loaded from the cache
    c->tune = t;
    return true;
}

static void tuning_save(blg_ctx *c, const char *path) {
    FILE *f = fopen(path, "w");
    if (!f) return;
    fprintf(f, "%s\n", tuning_header(c).c_str());
    for (int w = 1; w <= 8; w++) fprintf(f, "qpb%d %d\n", w, c->tune.qpb[w]);
    fprintf(f, "lpt_ctas %d\nlpt_job %d\nsurv_round %d\nband_ctas %d\ntile_shape %d\n", c->tune.lpt_ctas,
            c->tune.lpt_job, c->tune.surv_round, c->tune.band_ctas, c->tune.tile_shape);
    fprintf(f, "lpt_ctas_wide %d\nsurv_round_wide %d\nband_ctas_wide %d\n", c->tune.lpt_ctas_wide,
            c->tune.surv_round_wide, c->tune.band_ctas_wide);
    fclose(f);
}

// ============================================================== C-ABI ==
extern "C" {

int blg_version(void) { return 100; }

int blg_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

int blg_init(int device, blg_ctx **out) {
    if (!out) return BLG_ERR_ARG;
    *out = nullptr;
    int n = blg_device_count();
    if (n <= 0) return BLG_ERR_NODEVICE;
    if (device < 0 || device >= n) return BLG_ERR_ARG;
    blg_ctx *c = new (std::nothrow) blg_ctx();
    if (!c) return BLG_ERR_ALLOC;
    c->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->up, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->down, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_status, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(c->d_status, 0, sizeof(uint32_t));
    // the survivor search's deferred results (8 MB): 2^20 entries, one per
    // result <= max_dist of a launch; more run the in-place repair launch
    if (e == cudaSuccess) e = cudaMalloc((void **)&c->rl_hdr, sizeof(unsigned long long) * (2 + (1u << 20)));
    if (e == cudaSuccess) c->rl_cap = 1u << 20;
    if (e == cudaSuccess) e = cudaEventCreate(&c->t0);
    if (e == cudaSuccess) e = cudaEventCreate(&c->t1);
    if (e == cudaSuccess) {
        // keep freed blocks in the stream-ordered pool instead of returning them
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
            uint64_t thr = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
        }
    }
    if (e != cudaSuccess) {
        blg_destroy(c);
        return e == cudaErrorMemoryAllocation ? BLG_ERR_ALLOC : BLG_ERR_CUDA;
    }
    *out = c;
    return BLG_OK;
}

void blg_destroy(blg_ctx *c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->up) cudaStreamSynchronize(c->up);
    if (c->down) cudaStreamSynchronize(c->down);
    for (auto &r : c->prof_recs) {
        cudaEventDestroy(r.e0);
        cudaEventDestroy(r.e1);
    }
    sched_model_free(c->model);
    c->model = nullptr;
    if (c->d_status) cudaFree(c->d_status);
    if (c->rl_hdr) cudaFree(c->rl_hdr);
    if (c->t0) cudaEventDestroy(c->t0);
    if (c->t1) cudaEventDestroy(c->t1);
    if (c->stage_done) cudaEventDestroy(c->stage_done);
    if (c->stage) cudaFreeHost(c->stage);
    if (c->arena) cudaFreeHost(c->arena);
    if (c->stream) cudaStreamDestroy(c->stream);
    if (c->up) cudaStreamDestroy(c->up);
    if (c->down) cudaStreamDestroy(c->down);
    delete c;
}

const char *blg_last_error(const blg_ctx *c) { return c ? c->err.c_str() : "no context"; }

#define ENTER(c)                                      \
    if (!(c)) return BLG_ERR_ARG;                     \
    std::lock_guard<std::mutex> lock_((c)->mu);       \
    (c)->err.clear();                                 \
    if (cudaSetDevice((c)->device) != cudaSuccess) return fail((c), BLG_ERR_CUDA, "cudaSetDevice")

int blg_pairs_upload(blg_ctx *c, const uint8_t *ba, const int64_t *oa, const uint8_t *bb,
                     const int64_t *ob, int64_t n, blg_pairs **out) {
    ENTER(c);
    if (!out) return fail(c, BLG_ERR_ARG, "null out");
    blg_pairs *p = new (std::nothrow) blg_pairs();
    if (!p) return fail(c, BLG_ERR_ALLOC, "host allocation");
    int rc = pairs_upload(c, ba, oa, bb, ob, n, p);
    // the bytes the set uses, once: they pick the pairs kernels' row layout.
    // The copies complete before the call returns (the alphabet's copy back
    // synchronises): the device copy is the data the host pass checked,
    // whatever the caller does with its buffers.
    if (!rc) rc = pairs_learn_alphabet(c, p);
    if (!rc && cudaStreamSynchronize(c->stream) != cudaSuccess) rc = fail(c, BLG_ERR_CUDA, "upload");
    if (rc) {
        pairs_release(c, p);
        delete p;
        return rc;
    }
    *out = p;
    return BLG_OK;
}

// A resident run as one CUDA graph launch. The first run with a new set of
// parameters runs directly (it also allocates the work plan); when the next
// run repeats them its launches (counter resets, prep, order, solve, or the
// tile kernel and its long-pair consumers) are captured into a graph, which
// later runs with the same parameters replay. Profiling and fault injection
// run directly (they change what a run records or does).
static int pairs_run_graph(blg_ctx *c, blg_pairs *p, int k, int dtype, void *d_out) {
    if (!dtype_ok(dtype)) return fail(c, BLG_ERR_ARG, "dtype must be int32, uint16 or uint8");
    if (p->n == 0) return BLG_OK;
    if (!d_out) return fail(c, BLG_ERR_ARG, "null output");
    if (c->prof || c->fault_alloc_after >= 0 || c->fault_wait_polls >= 0) {
        pairs_graph_drop(p);
        p->g_have_last = false;
        return pairs_run(c, p, k, dtype, d_out);
    }
    blg_pairs::GraphKey key;
    key.k = k < 0 ? -1 : k;
    key.dtype = dtype;
    key.sched = c->sched;
    key.learned = c->sched == BLG_SCHED_LEARNED && c->model && sched_model_trained(c->model);
    key.band_ctas = band_ctas(c, k);
    key.tile_shape = c->tune.tile_shape;
    key.out = d_out;
    if (p->gexec && p->g_key == key) {
        CK(cudaGraphLaunch(p->gexec, c->stream), "graph launch");
        c->launches += p->g_launches;
        return BLG_OK;
    }
    const bool repeat = p->g_have_last && p->g_last == key;
    p->g_last = key;
    p->g_have_last = true;
    if (!repeat) return pairs_run(c, p, k, dtype, d_out);
    pairs_graph_drop(p);
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed), "begin capture");
    const int64_t l0 = c->launches;
    const int rc = pairs_run(c, p, k, dtype, d_out);
    const cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    const int64_t nl = c->launches - l0;
    c->launches = l0;
    if (rc || e != cudaSuccess) {                      // run directly instead
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        if (rc) return rc;
        return pairs_run(c, p, k, dtype, d_out);
    }
    const cudaError_t e2 = cudaGraphInstantiate(&p->gexec, g, 0);
    cudaGraphDestroy(g);
    if (e2 != cudaSuccess) {
        p->gexec = nullptr;
        return cuda_fail(c, e2, "graph instantiate");
    }
    p->g_key = key;
    p->g_launches = nl;
    CK(cudaGraphLaunch(p->gexec, c->stream), "graph launch");
    c->launches += nl;
    return BLG_OK;
}

int blg_pairs_run(blg_ctx *c, blg_pairs *p, int32_t max_dist, int32_t dtype, void *d_out) {
    ENTER(c);
    if (!p) return fail(c, BLG_ERR_ARG, "null pairs");
    if (dtype != BLG_UINT4) return pairs_run_graph(c, p, max_dist, dtype, d_out);
    if (p->n == 0) return BLG_OK;
    if (!d_out) return fail(c, BLG_ERR_ARG, "null output");
    void *d8 = nullptr;                                 // uint8 results, then packed into d_out
    CK(dev_alloc(c, &d8, (size_t)p->n), "cudaMallocAsync(uint8 results)");
    int rc = pairs_run(c, p, max_dist, BLG_UINT8, d8);
    if (!rc) rc = pack_u4(c, d8, 0, p->n, d_out);
    dev_free(c, d8);
    return rc;
}

int blg_pairs_run_logged(blg_ctx *c, blg_pairs *p, int32_t max_dist, int32_t dtype, void *d_out,
                         int32_t *d_exit_cols) {
    ENTER(c);
    if (!p || !d_exit_cols) return fail(c, BLG_ERR_ARG, "null pairs or log");
    return pairs_run(c, p, max_dist, dtype, d_out, d_exit_cols);
}

int blg_sched_train(blg_ctx *c, blg_pairs *p, int32_t max_dist, int32_t epochs, float lr, int64_t max_rows,
                    float *loss_out) {
    ENTER(c);
    if (!p || p->n == 0) return fail(c, BLG_ERR_ARG, "empty training batch");
    if (epochs < 0 || max_rows <= 0 || !(lr > 0.f)) return fail(c, BLG_ERR_ARG, "bad training arguments");
    blg_sched_model *m = nullptr;
    int rc = sched_model_ensure(c, &m);
    if (rc) return rc;
    // 1. a logged run with features: labels = columns each pair's loop processed
    void *out = nullptr, *cols = nullptr, *x = nullptr, *y = nullptr, *nrows = nullptr;
    CK(dev_alloc(c, &out, sizeof(int32_t) * (size_t)p->n), "alloc");
    CK(dev_alloc(c, &cols, sizeof(int32_t) * (size_t)p->n), "alloc");
    rc = pairs_run_scheduled(c, p, p->a.d, p->b.d, max_dist, BLG_INT32, out, (int32_t *)cols, true);
    if (rc) return rc;
    // 2. rows (subsampled to at most max_rows)
    int64_t records = 0;
    for (int j = 0; j < kPairClasses; j++) records += p->pcap[j];
    int32_t counts[kPairClasses];
    CK(cudaMemcpyAsync(counts, p->plan_ctr, sizeof(counts), cudaMemcpyDeviceToHost, c->stream), "D2H counts");
    CK(cudaStreamSynchronize(c->stream), "sync");
    records = 0;
    for (int j = 0; j < kPairClasses; j++) records += std::min<int64_t>(counts[j], p->pcap[j]);
    const int64_t stride = std::max<int64_t>(1, (records + max_rows - 1) / max_rows);
    CK(dev_alloc(c, &x, sizeof(half) * kFeatures * (size_t)max_rows + 16), "alloc");
    CK(dev_alloc(c, &y, sizeof(float) * (size_t)max_rows + 16), "alloc");
    CK(dev_alloc(c, &nrows, sizeof(int64_t)), "alloc");
    const PairsPlan plan = plan_view(p);
    CK(launch(c, "collect_rows", [&] {
           return launch_collect_rows(c->stream, c->sms, plan, (const int32_t *)cols, stride, max_rows, (half *)x,
                                      (float *)y, (int64_t *)nrows);
       }), "collect_rows");
    int64_t rows = 0;
    CK(cudaMemcpyAsync(&rows, nrows, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream), "D2H rows");
    CK(cudaStreamSynchronize(c->stream), "sync");
    // 3. train
    rc = rows > 0 ? sched_train_rows(c, m, (half *)x, (float *)y, (const int64_t *)nrows, rows, epochs, lr, 4096,
                                     loss_out)
                  : fail(c, BLG_ERR_ARG, "no non-trivial pairs to learn from");
    dev_free(c, out);
    dev_free(c, cols);
    dev_free(c, x);
    dev_free(c, y);
    dev_free(c, nrows);
    const int rc2 = sync_and_status(c);
    return rc ? rc : rc2;
}

int blg_sched_train_search(blg_ctx *c, blg_search *s, int32_t max_dist, int32_t epochs, float lr, int64_t max_rows,
                           float *loss_out) {
    ENTER(c);
    if (!s || s->nq == 0 || s->nc == 0) return fail(c, BLG_ERR_ARG, "empty training search");
    if (!s->lsorted) return fail(c, BLG_ERR_ARG, "choice lengths too spread for the survivor plan");
    if (max_dist < 0 || max_dist > 31) return fail(c, BLG_ERR_ARG, "max_dist must be in 0..31");
    if (epochs < 0 || max_rows <= 0 || !(lr > 0.f)) return fail(c, BLG_ERR_ARG, "bad training arguments");
    blg_sched_model *m = nullptr;
    int rc = sched_model_ensure(c, &m);
    if (rc) return rc;
    // survivors of every sequential class (host estimate from the plans, for the row spacing)
    const SurvClasses C = seq_classes(s);
    CK(launch(c, "surv_plan", [&] {
           return launch_surv_plan(c->stream, C, s->lstart, s->min_len, s->n_len, max_dist, 1);
       }), "surv_plan");
    int64_t survivors = 0;
    for (int i = 0; i < C.n; i++) {
        int64_t t = 0;
        CK(cudaMemcpyAsync(&t, C.tile_start[i] + C.cls[i].nq, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream),
           "D2H");
        CK(cudaStreamSynchronize(c->stream), "sync");
        survivors += t;
    }
    if (survivors == 0) return fail(c, BLG_ERR_ARG, "no survivors to learn from");
    void *out = nullptr, *x = nullptr, *y = nullptr, *nrows = nullptr;
    CK(dev_alloc(c, &out, (size_t)s->nq * (size_t)s->nc), "alloc");
    CK(dev_alloc(c, &x, sizeof(half) * kFeatures * (size_t)max_rows + 16), "alloc");
    CK(dev_alloc(c, &y, sizeof(float) * (size_t)max_rows + 16), "alloc");
    CK(dev_alloc(c, &nrows, sizeof(int64_t)), "alloc");
    CK(cudaMemsetAsync(nrows, 0, sizeof(int64_t), c->stream), "memset");
    SurvRows R{(half *)x, (float *)y, max_rows, (int64_t *)nrows,
               (int)std::min<int64_t>(INT32_MAX, std::max<int64_t>(1, (survivors + max_rows - 1) / max_rows))};
    const int job = survivor_job_size(c, s, max_dist);
    CK(launch(c, "surv_plan", [&] {
           return launch_surv_plan(c->stream, C, s->lstart, s->min_len, s->n_len, max_dist, job);
       }), "surv_plan");
    CK(launch(c, "search_band_logged", [&] {
           return launch_search_band(c->stream, c->sms, surv_ctas(c, max_dist), surv_round(c, max_dist), job, C, s->cs.d,
                                     s->perm, s->ccnt, s->qcnt,
                                     max_dist, BLG_UINT8, out, s->nc, &R, nullptr, nullptr, c->d_status);
       }), "search_band_logged");
    int64_t rows = 0;
    CK(cudaMemcpyAsync(&rows, nrows, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream), "D2H rows");
    CK(cudaStreamSynchronize(c->stream), "sync");
    rows = std::min(rows, max_rows);
    CK(cudaMemcpyAsync(nrows, &rows, sizeof(int64_t), cudaMemcpyHostToDevice, c->stream), "H2D rows");
    rc = rows > 0 ? sched_train_rows(c, m, (half *)x, (float *)y, (const int64_t *)nrows, rows, epochs, lr, 4096,
                                     loss_out)
                  : fail(c, BLG_ERR_ARG, "no survivors to learn from");
    dev_free(c, out);
    dev_free(c, x);
    dev_free(c, y);
    dev_free(c, nrows);
    const int rc2 = sync_and_status(c);
    return rc ? rc : rc2;
}

void blg_pairs_free(blg_ctx *c, blg_pairs *p) {
    if (!c || !p) return;
    std::lock_guard<std::mutex> lock_(c->mu);
    cudaSetDevice(c->device);
    pairs_release(c, p);
    delete p;
}

int blg_search_upload(blg_ctx *c, const uint8_t *bq, const int64_t *oq, int64_t nq,
                      const uint8_t *bc, const int64_t *oc, int64_t nc, blg_search **out) {
    ENTER(c);
    if (!out) return fail(c, BLG_ERR_ARG, "null out");
    blg_search *s = new (std::nothrow) blg_search();
    if (!s) return fail(c, BLG_ERR_ALLOC, "host allocation");
    int rc = search_upload(c, bq, oq, nq, bc, oc, nc, s);
    if (rc) {
        search_release(c, s);
        delete s;
        return rc;
    }
    *out = s;
    return BLG_OK;
}

int blg_search_run(blg_ctx *c, blg_search *s, int32_t max_dist, int32_t dtype, void *d_out) {
    ENTER(c);
    if (!s) return fail(c, BLG_ERR_ARG, "null search");
    if (dtype != BLG_UINT4) return search_run(c, s, max_dist, dtype, d_out);
    const int64_t n = s->nq * s->nc;
    if (n == 0) return BLG_OK;
    if (!d_out) return fail(c, BLG_ERR_ARG, "null output");
    void *d8 = nullptr;                                 // uint8 results, then packed into d_out
    CK(dev_alloc(c, &d8, (size_t)n), "cudaMallocAsync(uint8 results)");
    int rc = search_run(c, s, max_dist, BLG_UINT8, d8);
    if (!rc) rc = pack_u4(c, d8, 0, n, d_out);
    dev_free(c, d8);
    return rc;
}

void blg_search_free(blg_ctx *c, blg_search *s) {
    if (!c || !s) return;
    std::lock_guard<std::mutex> lock_(c->mu);
    cudaSetDevice(c->device);
    search_release(c, s);
    delete s;
}

int blg_pairwise(blg_ctx *c, const uint8_t *ba, const int64_t *oa, const uint8_t *bb,
                 const int64_t *ob, int64_t n, int32_t max_dist, int32_t dtype, void *out_host,
                 void **out_device) {
    ENTER(c);
    if (!dtype_ok_out(dtype)) return fail(c, BLG_ERR_ARG, "dtype must be int32, uint16, uint8 or uint4");
    if (n < 0) return fail(c, BLG_ERR_ARG, "negative count");
    if (!out_device && n > 0 && !out_host) return fail(c, BLG_ERR_ARG, "null output");
    const bool u4 = dtype == BLG_UINT4;
    const size_t obytes = out_bytes(dtype, n);
    void *d_out = nullptr, *d8 = nullptr;
    CK(dev_alloc(c, &d_out, obytes), "cudaMallocAsync(out)");
    if (u4 && dev_alloc(c, &d8, (size_t)n) != cudaSuccess) {   // uint8 results before packing
        dev_free(c, d_out);
        return fail(c, BLG_ERR_ALLOC, "cudaMallocAsync(uint8 results)");
    }
    blg_pairs p;
    int rc = check_offsets_host(c, oa, n);
    if (!rc) rc = check_offsets_host(c, ob, n);
    // host results of a large set: chunks overlap copies and kernels (4-bit
    // results: one pass, their copy back is small)
    const bool pipe = !rc && !out_device && !u4 && n >= (1 << 18);
    if (pipe) {
        rc = alloc_strings(c, ba, oa, n, p.a);
        if (!rc) rc = alloc_strings(c, bb, ob, n, p.b);
        if (!rc) rc = pairwise_pipelined(c, ba, oa, bb, ob, n, max_dist, dtype, out_host, d_out, &p);
    } else {
        if (!rc) rc = pairs_classify(c, oa, ob, n, &p);
        if (!rc) rc = upload_strings(c, ba, oa, n, p.a);
        if (!rc) rc = upload_strings(c, bb, ob, n, p.b);
        if (!rc) rc = pairs_run(c, &p, max_dist, u4 ? BLG_UINT8 : dtype, u4 ? d8 : d_out);
        if (!rc && u4 && n > 0) rc = pack_u4(c, d8, 0, n, d_out);
    }
    if (!rc && !pipe && !out_device && n > 0) {
        cudaError_t e = cudaMemcpyAsync(out_host, d_out, obytes, cudaMemcpyDeviceToHost, c->stream);
        if (e != cudaSuccess) rc = cuda_fail(c, e, "D2H results");
    }
    pairs_release(c, &p);
    dev_free(c, d8);
    if (rc || !out_device) dev_free(c, d_out);
    const int rc2 = sync_and_status(c);
    if (rc) return rc;
    if (rc2) {
        if (out_device) dev_free(c, d_out);
        return rc2;
    }
    if (out_device) *out_device = d_out;
    return BLG_OK;
}

int blg_cdist(blg_ctx *c, const uint8_t *bq, const int64_t *oq, int64_t nq, const uint8_t *bc,
              const int64_t *oc, int64_t nc, int32_t max_dist, int32_t dtype, void *out_host,
              void **out_device) {
    ENTER(c);
    if (!dtype_ok_out(dtype)) return fail(c, BLG_ERR_ARG, "dtype must be int32, uint16, uint8 or uint4");
    if (nq < 0 || nc < 0) return fail(c, BLG_ERR_ARG, "negative count");
    const bool u4 = dtype == BLG_UINT4;
    const int64_t n = nq * nc;
    const size_t obytes = out_bytes(dtype, n);
    if (!out_device && obytes > 0 && !out_host) return fail(c, BLG_ERR_ARG, "null output");
    void *d_out = nullptr, *d8 = nullptr;
    CK(dev_alloc(c, &d_out, obytes), "cudaMallocAsync(out)");
    if (u4 && dev_alloc(c, &d8, (size_t)n) != cudaSuccess) {   // uint8 results before packing
        dev_free(c, d_out);
        return fail(c, BLG_ERR_ALLOC, "cudaMallocAsync(uint8 results)");
    }
    blg_search s;
    int rc = BLG_OK;
    if (nq > 0 && nc > 0) {
        // a result matrix of 64 MiB or more going to the host (32 MiB of
        // 4-bit results): query chunks, each chunk's rows copied back while
        // the next chunk computes
        const bool pipe = !out_device && nq >= 2 && obytes >= (u4 ? (32u << 20) : (64u << 20));
        if (!pipe) {
            rc = search_upload(c, bq, oq, nq, bc, oc, nc, &s);
            if (!rc) rc = search_run(c, &s, max_dist, u4 ? BLG_UINT8 : dtype, u4 ? d8 : d_out);
            if (!rc && u4) rc = pack_u4(c, d8, 0, n, d_out);
            if (!rc && !out_device) {
                cudaError_t e = cudaMemcpyAsync(out_host, d_out, obytes, cudaMemcpyDeviceToHost, c->stream);
                if (e != cudaSuccess) rc = cuda_fail(c, e, "D2H results");
            }
        } else {
            rc = cdist_pipelined(c, bq, oq, nq, bc, oc, nc, max_dist, u4 ? BLG_UINT8 : dtype, out_host,
                                 u4 ? d8 : d_out, &s, u4 ? d_out : nullptr);
        }
        search_release(c, &s);
    }
    dev_free(c, d8);
    if (rc || !out_device) dev_free(c, d_out);
    const int rc2 = sync_and_status(c);
    if (rc) return rc;
    if (rc2) {
        if (out_device) dev_free(c, d_out);
        return rc2;
    }
    if (out_device) *out_device = d_out;
    return BLG_OK;
}

int blg_search_matches(blg_ctx *c, blg_search *s, int32_t max_dist, blg_match *d_out, int64_t capacity,
                       int64_t *count) {
    ENTER(c);
    if (!s || !count) return fail(c, BLG_ERR_ARG, "null search or count");
    if (max_dist < 0) return fail(c, BLG_ERR_ARG, "matches need max_dist >= 0");
    if (capacity < 0 || (capacity > 0 && !d_out)) return fail(c, BLG_ERR_ARG, "bad match buffer");
    *count = 0;
    if (s->nq == 0 || s->nc == 0) return BLG_OK;
    {   // the survivor kernel's result list, where the run qualifies
        bool listed = false;
        int64_t t = 0;
        const int rc = search_matches_list(c, s, max_dist, d_out, nullptr, capacity, &t, &listed);
        if (rc) return rc;
        if (listed) {
            const int rc2 = sync_and_status(c);
            if (rc2) return rc2;
            *count = t;
            return BLG_OK;
        }
    }
    // else query rows in chunks whose dense scratch stays within the budget
    // (1 GiB); the all-query classes are rebuilt afterwards for the
    // search's other runs
    const size_t row = dtype_size(match_dtype(max_dist)) * (size_t)s->nc;
    const int64_t rows = std::max<int64_t>(1, std::min<int64_t>(s->nq, (int64_t)(match_scratch_bytes() / row)));
    const bool chunked = rows < s->nq && (int64_t)s->h_oq.size() == s->nq + 1;
    const int64_t step = chunked ? rows : s->nq;
    void *scratch = nullptr;
    CK(dev_alloc(c, &scratch, row * (size_t)step), "cudaMallocAsync(match scratch)");
    int64_t total = 0;
    int rc = BLG_OK;
    for (int64_t q0 = 0; q0 < s->nq && !rc; q0 += step) {
        const int64_t q1 = std::min(s->nq, q0 + step);
        if (chunked) rc = search_build_classes(c, s->h_oq.data(), q0, q1, s);
        int64_t t = 0;
        const int64_t written = std::min(total, capacity);
        if (!rc) rc = search_matches_rows(c, s, max_dist, q0, q1, scratch, d_out ? d_out + written : nullptr,
                                          nullptr, capacity - written, &t);
        total += t;
    }
    if (chunked) {      // the all-query classes back for the search's other runs, after an error too
        const int rc3 = search_build_classes(c, s->h_oq.data(), 0, s->nq, s);
        if (!rc) rc = rc3;
    }
    dev_free(c, scratch);
    const int rc2 = sync_and_status(c);
    if (rc) return rc;
    if (rc2) return rc2;
    *count = total;
    return BLG_OK;
}

int blg_cdist_matches(blg_ctx *c, const uint8_t *bq, const int64_t *oq, int64_t nq, const uint8_t *bc,
                      const int64_t *oc, int64_t nc, int32_t max_dist, blg_match *out, int64_t capacity,
                      int64_t *count) {
    ENTER(c);
    if (!count) return fail(c, BLG_ERR_ARG, "null count");
    if (max_dist < 0) return fail(c, BLG_ERR_ARG, "matches need max_dist >= 0");
    if (nq < 0 || nc < 0) return fail(c, BLG_ERR_ARG, "negative count");
    if (capacity < 0 || (capacity > 0 && !out)) return fail(c, BLG_ERR_ARG, "bad match buffer");
    *count = 0;
    if (nq == 0 || nc == 0) return BLG_OK;
    blg_search s;
    const bool surv = c->sched != BLG_SCHED_PLAIN;
    int rc = search_upload_queries(c, bq, oq, nq, &s);
    if (!rc) rc = search_upload_choices(c, bc, oc, nc, &s, surv ? NEED_SORTED : NEED_TT);
    // the survivor kernel's result list, where the run qualifies
    int64_t total = 0;
    bool listed = false;
    if (!rc && surv && max_dist <= 31) {
        rc = search_build_classes(c, oq, 0, nq, &s);
        if (!rc) rc = search_matches_list(c, &s, max_dist, nullptr, out, capacity, &total, &listed);
    }
    // else query rows in chunks whose dense scratch stays within the budget
    // (1 GiB)
    const size_t row = dtype_size(match_dtype(max_dist)) * (size_t)nc;
    const int64_t rows = std::max<int64_t>(1, std::min<int64_t>(nq, (int64_t)(match_scratch_bytes() / row)));
    void *scratch = nullptr;
    if (!rc && !listed && dev_alloc(c, &scratch, row * (size_t)rows) != cudaSuccess)
        rc = fail(c, BLG_ERR_ALLOC, "cudaMallocAsync(match scratch)");
    for (int64_t q0 = 0; q0 < nq && !rc && !listed; q0 += rows) {
        const int64_t q1 = std::min(nq, q0 + rows);
        rc = search_build_classes(c, oq, q0, q1, &s);
        int64_t t = 0;
        const int64_t written = std::min(total, capacity);
        if (!rc) rc = search_matches_rows(c, &s, max_dist, q0, q1, scratch, nullptr, out + written,
                                          capacity - written, &t);
        total += t;
    }
    dev_free(c, scratch);
    search_release(c, &s);
    const int rc2 = sync_and_status(c);
    if (rc) return rc;
    if (rc2) return rc2;
    *count = total;
    return BLG_OK;
}

int blg_batch_upload(blg_ctx *c, const blg_problem *probs, int32_t nprob, blg_batch **out) {
    ENTER(c);
    if (!out) return fail(c, BLG_ERR_ARG, "null out");
    blg_batch *b = new (std::nothrow) blg_batch();
    if (!b) return fail(c, BLG_ERR_ALLOC, "host allocation");
    int rc = batch_upload(c, probs, nprob, b);
    if (rc) {
        batch_release(c, b);
        delete b;
        return rc;
    }
    *out = b;
    return BLG_OK;
}

int blg_batch_run(blg_ctx *c, blg_batch *b) {
    ENTER(c);
    if (!b) return fail(c, BLG_ERR_ARG, "null batch");
    return batch_run(c, b);
}

int64_t blg_batch_pairs(const blg_batch *b) { return b ? b->pairs : 0; }

void blg_batch_free(blg_ctx *c, blg_batch *b) {
    if (!c || !b) return;
    std::lock_guard<std::mutex> lock_(c->mu);
    cudaSetDevice(c->device);
    batch_release(c, b);
    delete b;
}

int blg_cdist_batch(blg_ctx *c, const blg_problem *probs, int32_t nprob) {
    blg_batch *b = nullptr;
    int rc = blg_batch_upload(c, probs, nprob, &b);
    if (rc) return rc;
    rc = blg_batch_run(c, b);
    if (!rc) rc = blg_synchronize(c);
    blg_batch_free(c, b);
    return rc;
}

int blg_malloc(blg_ctx *c, size_t bytes, void **d_ptr) {
    ENTER(c);
    if (!d_ptr) return fail(c, BLG_ERR_ARG, "null out");
    CK(dev_alloc(c, d_ptr, bytes), "cudaMallocAsync");
    CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    return BLG_OK;
}

int blg_free(blg_ctx *c, void *d_ptr) {
    ENTER(c);
    dev_free(c, d_ptr);
    return BLG_OK;
}

int blg_host_alloc(blg_ctx *c, size_t bytes, void **h_ptr) {
    ENTER(c);
    if (!h_ptr) return fail(c, BLG_ERR_ARG, "null out");
    *h_ptr = nullptr;
    CK(cudaMallocHost(h_ptr, bytes ? bytes : 16), "cudaMallocHost");
    return BLG_OK;
}

int blg_host_free(blg_ctx *c, void *h_ptr) {
    ENTER(c);
    if (h_ptr) CK(cudaFreeHost(h_ptr), "cudaFreeHost");
    return BLG_OK;
}

int blg_memcpy_h2d(blg_ctx *c, void *d_dst, const void *h_src, size_t bytes) {
    ENTER(c);
    if (bytes == 0) return BLG_OK;
    CK(cudaMemcpyAsync(d_dst, h_src, bytes, cudaMemcpyHostToDevice, c->stream), "H2D");
    CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    return BLG_OK;
}

int blg_memcpy_d2h(blg_ctx *c, void *h_dst, const void *d_src, size_t bytes) {
    ENTER(c);
    if (bytes == 0) return BLG_OK;
    CK(cudaMemcpyAsync(h_dst, d_src, bytes, cudaMemcpyDeviceToHost, c->stream), "D2H");
    CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    return BLG_OK;
}

int blg_memset(blg_ctx *c, void *d_dst, int value, size_t bytes) {
    ENTER(c);
    if (bytes == 0) return BLG_OK;
    CK(cudaMemsetAsync(d_dst, value, bytes, c->stream), "memset");
    return BLG_OK;
}

int blg_synchronize(blg_ctx *c) {
    ENTER(c);
    return sync_and_status(c);
}

int blg_timer_start(blg_ctx *c) {
    ENTER(c);
    CK(cudaEventRecord(c->t0, c->stream), "cudaEventRecord");
    return BLG_OK;
}

int blg_timer_stop(blg_ctx *c, float *ms) {
    ENTER(c);
    CK(cudaEventRecord(c->t1, c->stream), "cudaEventRecord");
    CK(cudaEventSynchronize(c->t1), "cudaEventSynchronize");
    float v = 0.f;
    CK(cudaEventElapsedTime(&v, c->t0, c->t1), "cudaEventElapsedTime");
    if (ms) *ms = v;
    return BLG_OK;
}

int64_t blg_launch_count(const blg_ctx *c) { return c ? c->launches : 0; }

int blg_autotune(blg_ctx *c, const char *cache_path) {
    ENTER(c);
    if (cache_path && *cache_path && tuning_load(c, cache_path)) return BLG_OK;
    const int sched = c->sched;
    c->sched = BLG_SCHED_AUTO;
    int rc = BLG_OK;
    for (int nw : {1, 2, 4})
        if (!rc) rc = tune_exact_search(c, nw);
    if (!rc) {
        // word counts not timed take the nearest timed one
        c->tune.qpb[3] = c->tune.qpb[4];
        for (int w = 5; w <= 8; w++) c->tune.qpb[w] = c->tune.qpb[4];
        // the max_dist axis: the survivor search at max_dist 4 and 16, the
        // banded pairs solver at 8 and 24 (each sets its own bucket)
        rc = tune_threshold_search(c, 4);
        if (!rc) rc = tune_threshold_search(c, 16);
    }
    if (!rc) rc = tune_band_pairs(c, 8);
    if (!rc) rc = tune_band_pairs(c, 24);
    if (!rc) rc = tune_tile_pairs(c);
    c->sched = sched;
    if (rc) {
        c->tune = blg_tuning();                         // keep the defaults on any failure
        return rc;
    }
    c->tune.tuned = 1;
    if (cache_path && *cache_path) tuning_save(c, cache_path);
    return BLG_OK;
}

int blg_get_tuning(blg_ctx *c, int32_t *values, int n) {
    ENTER(c);
    if (!values || n < 14) return fail(c, BLG_ERR_ARG, "need at least 14 values");
    for (int w = 1; w <= 8; w++) values[w - 1] = c->tune.qpb[w];
    values[8] = c->tune.lpt_ctas;
    values[9] = c->tune.lpt_job;
    values[10] = c->tune.band_ctas;
    values[11] = c->tune.tuned;
    values[12] = c->tune.tile_shape;
    values[13] = c->tune.surv_round;
    if (n >= 17) {                                      // the shapes of the wide max_dist buckets
        values[14] = c->tune.lpt_ctas_wide;
        values[15] = c->tune.surv_round_wide;
        values[16] = c->tune.band_ctas_wide;
    }
    return BLG_OK;
}

int blg_set_schedule(blg_ctx *c, int mode) {
    ENTER(c);
    if (mode < BLG_SCHED_AUTO || mode > BLG_SCHED_LENSORT) return fail(c, BLG_ERR_ARG, "unknown schedule");
    c->sched = mode;
    return BLG_OK;
}

int blg_set_fault_injection(blg_ctx *c, int64_t alloc_fail_after, int32_t wait_polls) {
    ENTER(c);
    c->fault_alloc_after = alloc_fail_after < 0 ? -1 : alloc_fail_after;
    c->fault_wait_polls = wait_polls < 0 ? -1 : wait_polls;
    return BLG_OK;
}

int blg_profile_enable(blg_ctx *c, int on) {
    ENTER(c);
    c->prof = on != 0;
    return BLG_OK;
}

int blg_profile_report(blg_ctx *c, char *buf, size_t cap) {
    ENTER(c);
    CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    for (auto &r : c->prof_recs) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, r.e0, r.e1);
        auto &a = c->prof_acc[r.name];
        a.first += 1;
        a.second += ms;
        cudaEventDestroy(r.e0);
        cudaEventDestroy(r.e1);
    }
    c->prof_recs.clear();
    std::string s;
    for (auto &kv : c->prof_acc) {
        char line[256];
        snprintf(line, sizeof(line), "%s %lld %.6f\n", kv.first.c_str(), (long long)kv.second.first,
                 kv.second.second);
        s += line;
    }
    c->prof_acc.clear();
    if (buf && cap) {
        const size_t nb = std::min(cap - 1, s.size());
        memcpy(buf, s.data(), nb);
        buf[nb] = 0;
    }
    return BLG_OK;
}

}  // extern "C"
