/*
 * bitlev_gb300.h — C-ABI of the GB300 bit-parallel Levenshtein engine.
 *
 * Drop-in for the GPU path of karims/editdist-bench's `bitlev` library:
 * bitlev.gpu.pairwise / bitlev.gpu.cdist (bitlev/gpu.py:71-138) and the
 * resident-state launch helpers its benchmark uses (bench/cudamyers.py:
 * 83-174). The library is loaded through ctypes by the Python layer
 * (editdist_bench_gb300/gpu.py); plain pointers and sizes only.
 *
 * Inputs are bitlev's packed layout (csrc/edpy.c:200-224, `_edpy.pack`):
 * one byte buffer and int64 offsets off[0..n], string i = buf[off[i] ..
 * off[i+1]). Distances are exact unit-cost Levenshtein distances; with
 * max_dist = k >= 0 the result is min(d, k + 1) (csrc/myers.c:101-143);
 * max_dist < 0 means exact. Narrow dtypes saturate at their maximum
 * (bitlev/_common.py:25-29). Every string length is computed on the GPU:
 * there is no CPU fallback (the reference sends strings longer than
 * 256/512 to its CPU path, bitlev/gpu.py:97-101,131-136).
 *
 * Return codes (bitlev raises the Python equivalents):
 *   BLG_OK 0, BLG_ERR_ALLOC -1 (MemoryError), BLG_ERR_ARG -2 (ValueError),
 *   BLG_ERR_CUDA -3, BLG_ERR_TIMEOUT -4, BLG_ERR_NODEVICE -5 (RuntimeError).
 * blg_last_error() gives the message of the last failing call.
 *
 * Threading: one context per device and process is enough; calls on one
 * context are serialised by a mutex; work runs on the context's stream.
 */
#ifndef BITLEV_GB300_H
#define BITLEV_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BLG_OK 0
#define BLG_ERR_ALLOC (-1)
#define BLG_ERR_ARG (-2)
#define BLG_ERR_CUDA (-3)
#define BLG_ERR_TIMEOUT (-4)
#define BLG_ERR_NODEVICE (-5)

/* dtype codes: bitlev's DTYPES (bitlev/_common.py:7) */
#define BLG_INT32 0
#define BLG_UINT16 1
#define BLG_UINT8 2
/* 4-bit results, two per byte (element 2i in the low nibble of byte i, 2i+1
 * in the high nibble), saturating at 15: for max_dist <= 14 every result is
 * exact, and the device -> host copy is half of uint8's. No counterpart in
 * the reference, which names narrower results as the way to cut the search's
 * result stream (README.md:319-321). Accepted by blg_pairwise, blg_cdist,
 * blg_pairs_run and blg_search_run; an output of n results is (n + 1) / 2
 * bytes. */
#define BLG_UINT4 3

typedef struct blg_ctx blg_ctx;
typedef struct blg_pairs blg_pairs;   /* resident pairs  (bench/cudamyers.py:83-114 PairsState) */
typedef struct blg_search blg_search; /* resident search (bench/cudamyers.py:139-152 CrossState) */

/* Library ABI version (major*100 + minor). */
int blg_version(void);

/* Number of visible CUDA devices (0 when none). Replaces bitlev.gpu.available()'s
 * CuPy device query (bitlev/gpu.py:36-41). */
int blg_device_count(void);

/* Create a context on `device` (own stream, status word, allocator pool).
 * Replaces the lazily built CuPy RawModule (bitlev/gpu.py:44-51). */
int blg_init(int device, blg_ctx **out);
void blg_destroy(blg_ctx *ctx);
const char *blg_last_error(const blg_ctx *ctx);

/* out[i] = d(a_i, b_i) — bitlev.gpu.pairwise (bitlev/gpu.py:71-103).
 * Host inputs; n >= 0. When out_device is NULL the results are written to
 * out_host (n elements of `dtype`); otherwise a device buffer is allocated,
 * filled and returned in *out_device (free with blg_free) — return_device. */
int blg_pairwise(blg_ctx *ctx, const uint8_t *buf_a, const int64_t *off_a, const uint8_t *buf_b,
                 const int64_t *off_b, int64_t n, int32_t max_dist, int32_t dtype, void *out_host,
                 void **out_device);

/* out[i*nc + j] = d(q_i, c_j) — bitlev.gpu.cdist (bitlev/gpu.py:106-138). */
int blg_cdist(blg_ctx *ctx, const uint8_t *buf_q, const int64_t *off_q, int64_t nq,
              const uint8_t *buf_c, const int64_t *off_c, int64_t nc, int32_t max_dist,
              int32_t dtype, void *out_host, void **out_device);

/* Resident pairs: upload once, run many times with results left in HBM —
 * the "kernel-only" protocol of bench/cudamyers.py:83-136 (PairsState +
 * pairs()). d_out must hold n elements of dtype (device memory). The run
 * is stream-ordered and does not synchronise. */
int blg_pairs_upload(blg_ctx *ctx, const uint8_t *buf_a, const int64_t *off_a, const uint8_t *buf_b,
                     const int64_t *off_b, int64_t n, blg_pairs **out);
int blg_pairs_run(blg_ctx *ctx, blg_pairs *p, int32_t max_dist, int32_t dtype, void *d_out);
void blg_pairs_free(blg_ctx *ctx, blg_pairs *p);
/* blg_pairs_run that also records, per pair, how many text columns its
 * column loop processed before the max_dist exit fired (0 for pairs settled
 * by the length gap or an empty pattern; the text length when no exit) —
 * the labels the work-order scheduler is trained on. d_exit_cols: int32[n]. */
int blg_pairs_run_logged(blg_ctx *ctx, blg_pairs *p, int32_t max_dist, int32_t dtype, void *d_out,
                         int32_t *d_exit_cols);

/* Resident search (bench/cudamyers.py:139-174, CrossState + cross()):
 * d_out holds nq*nc elements of dtype, row-major. */
int blg_search_upload(blg_ctx *ctx, const uint8_t *buf_q, const int64_t *off_q, int64_t nq,
                      const uint8_t *buf_c, const int64_t *off_c, int64_t nc, blg_search **out);
int blg_search_run(blg_ctx *ctx, blg_search *s, int32_t max_dist, int32_t dtype, void *d_out);
void blg_search_free(blg_ctx *ctx, blg_search *s);

/* Matches-only thresholded search: every (query, choice) with distance
 * <= max_dist, as records sorted by (query, choice), instead of the dense
 * nq*nc matrix. No counterpart in the reference, which names it as what
 * fuzzy search usually wants (README.md:319-321). max_dist >= 0 (a dense
 * result is the exact case). At most `capacity` records are written; *count
 * receives the total number of matches either way, so a caller whose buffer
 * was too small can call again with *count records of room.
 * blg_cdist_matches: host inputs, records in host memory (`out`).
 * blg_search_matches: a resident search, records in device memory (`d_out`);
 * synchronises (the count comes back to the host). */
typedef struct {
    int64_t query;
    int64_t choice;
    int32_t dist;
    int32_t reserved;      /* 0 */
} blg_match;
int blg_cdist_matches(blg_ctx *ctx, const uint8_t *buf_q, const int64_t *off_q, int64_t nq,
                      const uint8_t *buf_c, const int64_t *off_c, int64_t nc, int32_t max_dist,
                      blg_match *out, int64_t capacity, int64_t *count);
int blg_search_matches(blg_ctx *ctx, blg_search *s, int32_t max_dist, blg_match *d_out, int64_t capacity,
                       int64_t *count);

/* Many independent cdist problems (host inputs, device outputs — the
 * return_device form), run by one persistent kernel that pulls
 * (problem, query, 1024-choice) tiles from a device work counter; the batch's
 * launches are captured into one CUDA graph on the first run and replayed.
 * No counterpart in the reference (one bitlev.gpu.cdist call per problem,
 * bitlev/gpu.py:106-138). d_out: nq*nc elements of dtype, row-major. */
typedef struct {
    const uint8_t *buf_q;
    const int64_t *off_q;
    int64_t nq;
    const uint8_t *buf_c;
    const int64_t *off_c;
    int64_t nc;
    int32_t max_dist;   /* < 0: exact */
    int32_t dtype;
    void *d_out;
} blg_problem;
typedef struct blg_batch blg_batch;
int blg_batch_upload(blg_ctx *ctx, const blg_problem *probs, int32_t nprob, blg_batch **out);
int blg_batch_run(blg_ctx *ctx, blg_batch *b);         /* stream-ordered, no sync */
int64_t blg_batch_pairs(const blg_batch *b);          /* sum of nq*nc */
void blg_batch_free(blg_ctx *ctx, blg_batch *b);
/* upload + run + synchronise + free */
int blg_cdist_batch(blg_ctx *ctx, const blg_problem *probs, int32_t nprob);

/* cdist with every buffer already in device memory and NO device allocation:
 * no counterpart in the reference (bitlev.gpu always allocates through CuPy).
 * For callers that cannot call cudaMalloc — plugins of an engine that owns
 * the GPU's memory, or request paths that must not block on or fail in an
 * allocation. The only scratch (per-query Peq tables) is a fixed 2 MiB
 * array inside the library, per device, for the life of the process.
 * Limits: every query at most 256 bytes (longer -> BLG_ERR_ARG after the
 * call; that row is not written); string buffers 16-byte aligned, offset
 * arrays 8-byte aligned, the output aligned to its element size (checked
 * before anything runs: BLG_ERR_ARG); offsets relative to each buffer's
 * start; q_bytes/c_bytes are the readable sizes of the byte buffers and must
 * leave 16 bytes after the last string. The first call on a device looks up
 * the scratch address and, with CUDA's lazy module loading, loads the
 * library's kernels and the 2 MiB array onto the device: make one small
 * call at start-up (before any stream capture), so that later calls allocate
 * nothing. Not usable after a device reset (cudaDeviceReset) in the same
 * process. All calls share the scratch: calls whose work overlaps on the GPU
 * (other contexts or threads on the same device) race; calls on one context
 * are ordered. Returns after the results are complete (synchronises). */
int blg_cdist_noalloc(blg_ctx *ctx, const uint8_t *d_buf_q, size_t q_bytes, const int64_t *d_off_q,
                      int64_t nq, const uint8_t *d_buf_c, size_t c_bytes, const int64_t *d_off_c,
                      int64_t nc, int32_t max_dist, int32_t dtype, void *d_out);

/* Work order of thresholded (max_dist >= 0) runs. Results never depend on it.
 *  AUTO    — survivor compaction: choices kept length-sorted, only pairs whose
 *            lengths are within max_dist run the column loop, the rest of the
 *            output is filled with max_dist+1;
 *  PLAIN   — every (query, choice) / pair in natural order, one thread each
 *            (the reference's schedule, csrc/gpu_kernels.cu:6-69);
 *  LEARNED — AUTO plus survivors ordered by the scheduler network's
 *            predicted exit column;
 *  LENSORT — AUTO with the work ordered by length difference alone, equal
 *            lengths first (an ablation: survivors of a search, records of
 *            the pairs plan). */
#define BLG_SCHED_AUTO 0
#define BLG_SCHED_PLAIN 1
#define BLG_SCHED_LEARNED 2
#define BLG_SCHED_LENSORT 3
int blg_set_schedule(blg_ctx *ctx, int mode);

/* The work-order scheduler (BLG_SCHED_LEARNED): a 7 -> 32 -> 32 -> 1 MLP
 * (FP16 weights, FP32 sums) that predicts the fraction of a pair's text its
 * column loop processes before the max_dist exit. No counterpart in the
 * reference. blg_sched_train runs a logged pass over the batch (features:
 * trimmed and untrimmed lengths, length gap, max_dist, 4-gram sketch distance;
 * label: logged exit column / text length), keeps at most max_rows rows and
 * trains the context's network for `epochs` epochs on the GPU (momentum
 * SGD, minibatches of 4096, one epoch captured as a CUDA graph); *loss_out
 * = last epoch's mean squared error. */
int blg_sched_train(blg_ctx *ctx, blg_pairs *p, int32_t max_dist, int32_t epochs, float lr,
                    int64_t max_rows, float *loss_out);
/* The same network for a thresholded search (max_dist <= 31): a logged run of
 * the survivor kernel over the resident search `s` collects rows (features:
 * query and choice lengths, length gap, max_dist, 4-gram sketch distance;
 * label: the banded loop's exit column / choice length) from every survivor
 * spaced to keep at most max_rows, then trains as above. Under
 * BLG_SCHED_LEARNED the survivor kernel then orders each job of survivors by
 * the network's predicted work (longest first). */
int blg_sched_train_search(blg_ctx *ctx, blg_search *s, int32_t max_dist, int32_t epochs, float lr,
                           int64_t max_rows, float *loss_out);
/* 1345 FP32 master weights: W1[32][7], b1[32], W2[32][32], b2[32], W3[32], b3. */
int blg_sched_set_weights(blg_ctx *ctx, const float *w, int n);
int blg_sched_get_weights(blg_ctx *ctx, float *w, int n);
/* Mean-squared-error gradient at the current weights over host rows
 * (x: rows x 7 IEEE halves, y: targets) without updating the weights. */
int blg_sched_gradient(blg_ctx *ctx, const uint16_t *x_half, const float *y, int rows, float *grad_out,
                       float *loss_out);
int blg_sched_predict(blg_ctx *ctx, const uint16_t *x_half, int64_t rows, float *out);
/* Versioned checkpoint ("BLGMLP02", count, FP32 weights). */
int blg_sched_save(blg_ctx *ctx, const char *path);
int blg_sched_load(blg_ctx *ctx, const char *path);

/* Autotuner: times candidate launch shapes on synthetic inputs of each
 * length bucket and max_dist kind and keeps the fastest for this context:
 * queries per CTA of the exact search (by query word count), CTAs per SM and
 * columns per lane round of the thresholded search's survivor kernel (one
 * shape for max_dist <= 8, tuned at 4, one for 9..31, tuned at 16), CTAs
 * per SM of the banded pairs solver (max_dist <= 15, tuned at 8; 16..31,
 * tuned at 24), the staging shape of the short-pair tile kernel. With a cache path, a cache written for the same device model,
 * SM count and library version is loaded instead of timing, and a fresh
 * result is written there. No counterpart in the reference (fixed launch
 * geometry, bitlev/gpu.py:90-96,121-130). Results never depend on it. */
int blg_autotune(blg_ctx *ctx, const char *cache_path);
/* values[n >= 14]: qpb for 1..8 query words (0 = heuristic), CTAs per SM
 * (max_dist <= 8) and survivors per job of the thresholded search, CTAs per
 * SM of the banded solver (max_dist <= 15), 0 (defaults) / 1 (timed) / 2
 * (loaded from a cache), the staging shape of the short-pair tile kernel
 * (1: one stage of 512 pairs, 2: two stages of 512, 3: two stages of 256),
 * and the columns per lane round of the thresholded search's survivor
 * kernel (8, 16 or 32; max_dist <= 8). With n >= 17 also the wide max_dist
 * buckets: the survivor kernel's CTAs per SM and columns per round for
 * max_dist 9..31 and the banded solver's CTAs per SM for 16..31. */
int blg_get_tuning(blg_ctx *ctx, int32_t *values, int n);

/* Device memory and stream helpers (the parts of CuPy bitlev.gpu used:
 * cp.empty / .get() / Device().synchronize(), bitlev/gpu.py:59-68,102). */
int blg_malloc(blg_ctx *ctx, size_t bytes, void **d_ptr);
int blg_free(blg_ctx *ctx, void *d_ptr);
int blg_memcpy_h2d(blg_ctx *ctx, void *d_dst, const void *h_src, size_t bytes);
int blg_memcpy_d2h(blg_ctx *ctx, void *h_dst, const void *d_src, size_t bytes);
int blg_memset(blg_ctx *ctx, void *d_dst, int value, size_t bytes);
/* Page-locked host memory (cudaMallocHost), for inputs and results that move
 * between host and device at full link speed: the one-call entry points
 * overlap their copies with the kernels when the host buffers are pinned.
 * The counterpart of cupyx.empty_pinned for callers of the CuPy path. */
int blg_host_alloc(blg_ctx *ctx, size_t bytes, void **h_ptr);
int blg_host_free(blg_ctx *ctx, void *h_ptr);
/* Wait for the context's stream and report any status a kernel raised. */
int blg_synchronize(blg_ctx *ctx);

/* Fault injection for tests of the error paths; no counterpart in the
 * reference, whose one failure mode besides bad arguments is an allocation
 * failure (csrc/myers.c:162-164 returns -1, bench/cmyers.py:82-84 raises
 * MemoryError). alloc_fail_after >= 0: after that many more device
 * allocations of this context succeed, the next one fails as if the device
 * were out of memory (BLG_ERR_ALLOC); the hook is then spent. -1: off.
 * wait_polls >= 0: the short-pair tile kernel's bounded wait for its staged
 * strings gives up after that many polls instead of its normal bound, so the
 * call ends with BLG_ERR_TIMEOUT (the kernel still waits, at the normal
 * bound, for its copies in flight before it returns). -1: normal bound.
 * Nothing here faults, traps or hangs the GPU; the context stays usable. */
int blg_set_fault_injection(blg_ctx *ctx, int64_t alloc_fail_after, int32_t wait_polls);

/* Timing on the context's stream with CUDA events (ms between start/stop). */
int blg_timer_start(blg_ctx *ctx);
int blg_timer_stop(blg_ctx *ctx, float *ms);
/* Kernels launched by this context so far. */
int64_t blg_launch_count(const blg_ctx *ctx);
/* Per-kernel event timing of every launch while enabled (bench roofline). */
int blg_profile_enable(blg_ctx *ctx, int on);
/* Writes "name launches total_ms\n" lines (after synchronising) into buf. */
int blg_profile_report(blg_ctx *ctx, char *buf, size_t cap);

#ifdef __cplusplus
}
#endif

#endif /* BITLEV_GB300_H */
