// Descriptors of a multi-problem batch (shared by kernels and host runtime).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "blg_internal.h"

namespace blg {

constexpr int kBatchMaxWords = 4;   // batched queries up to 256 bytes; longer ones run per problem

// One (problem, query word-class): everything the persistent kernel needs.
struct BatchJob {
    DevStrings CS;             // its choices, length-sorted
    const int32_t *perm;       // sorted -> original choice index
    const int64_t *lstart;     // first sorted index per length
    int64_t min_len, n_len;
    SearchClass cls;           // the class's queries and Peq tables
    int32_t *lo, *hi;          // survivor range per query
    int64_t *tile_start;       // tile prefix per query (nq + 1)
    int64_t nc;
    int k, dtype, nw;
    int tile;                  // survivors per work unit: 4096 (banded survivor jobs) or 1024
    const uint64_t *csk;       // 4-gram sketches of the sorted choices
    const uint64_t *qsk;       // 4-gram sketches of the queries (by query row)
    const uint4 *ccnt;         // binned 4-gram counts of the sorted choices
    const uint4 *qcnt;         // binned 4-gram counts of the queries (by query row)
    void *out;
};

struct BatchPlan {
    const BatchJob *jobs;      // device array; banded jobs (0 <= k <= 31) first
    int njobs;
    int nbanded;               // jobs [0, nbanded) run in the banded survivor kernel (k_batch_band)
    int64_t *job_tiles;        // [njobs]
    int64_t *tile_base;        // [njobs + 1]
    int32_t *work;             // persistent-kernel counters: [0] banded jobs, [1] the others
    // with list.item: the banded kernel fills every thresholded output itself
    // (fill items) and defers its results to the list; hdr = [list count,
    // fill items claimed], cleared by the run
    ResultList list;
    FillItems fill;
    unsigned long long *hdr;
};

// ---- batch upload: each kind of preparation runs once per group of
// problems. Sets are addressed through a prefix over their item counts: a
// launch covers items [first, first + total) of sets [0, nsets) of its
// arrays (start[0] = first), and item J belongs to the last set s with
// start[s] <= J.

// One problem's choices sorted by length on the device (items: its n
// choices): counts per length into hist, then per set (one block each)
// bucket starts lstart / bstart with hist turned into bucket cursors, then
// each choice's slot taken from its bucket's cursor. The order inside a
// bucket is the order the slots were taken in: results never depend on it.
struct LenSortSet {
    const int64_t *off;                // the raw choices' offsets (n + 1)
    int64_t n, min_len, n_len;
    unsigned long long *hist;          // [n_len], zero before the count
    int64_t *lstart;                   // [n_len + 1] first sorted index per length
    int64_t *bstart;                   // [n_len] first sorted byte per length
    int32_t *perm;                     // [n] sorted -> raw index
};

// One problem's slack and sorted offsets (items: n_sorted + 1).
struct UploadPrep {
    uint8_t *buf[3];                   // raw queries, raw choices, sorted choices (null: absent)
    int64_t bytes[3];
    const int64_t *lstart, *bstart;    // length buckets of the sorted copy (n_sorted > 0)
    int64_t n_len, min_len, n_sorted;
    int64_t *soff;                     // sorted offsets [n_sorted + 1]
};

// One string set to sketch (items: n): output string i is src string
// perm[i] (perm null: string i, nothing copied), copied to dst + dst_off[i].
struct SketchSet {
    DevStrings src;
    const int32_t *perm;
    const int64_t *dst_off;
    uint8_t *dst;
    uint64_t *sketch;
    uint4 *counts;
    int64_t n;
};

// One query class's Peq tables (items: its queries; one CTA each).
struct PeqSet {
    DevStrings Q;
    const int32_t *qidx;
    uint64_t *peq;                     // [nq][256][nwc]
    int nwc;
};

cudaError_t launch_length_sort(cudaStream_t st, int sms, const LenSortSet *sets, const int64_t *start, int nsets,
                               int64_t first, int64_t total);
cudaError_t launch_upload_prep(cudaStream_t st, int sms, const UploadPrep *sets, const int64_t *start, int nsets,
                               int64_t first, int64_t total);
cudaError_t launch_sketch_sets(cudaStream_t st, int sms, const SketchSet *sets, const int64_t *start, int nsets,
                               int64_t first, int64_t total, uint32_t *status);
cudaError_t launch_peq_sets(cudaStream_t st, const PeqSet *sets, const int64_t *start, int nsets, int64_t first,
                            int64_t total, int max_nwc, uint32_t *status);

cudaError_t batch_set_attributes();
cudaError_t launch_batch(cudaStream_t st, int sms, const BatchPlan &plan, const BatchFill *fills, int nfill,
                         int64_t max_fill, uint32_t *status, int *kernels);
cudaError_t launch_list_scatter(cudaStream_t st, int sms, const ResultList &L, int32_t *work);

}  // namespace blg
