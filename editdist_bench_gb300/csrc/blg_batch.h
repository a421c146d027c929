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

struct BatchFill {
    void *out;
    int64_t n;
    int dtype;
    uint32_t value;
};

struct BatchPlan {
    const BatchJob *jobs;      // device array; banded jobs (0 <= k <= 31) first
    int njobs;
    int nbanded;               // jobs [0, nbanded) run in the banded survivor kernel (k_batch_band)
    int64_t *job_tiles;        // [njobs]
    int64_t *tile_base;        // [njobs + 1]
    int32_t *work;             // persistent-kernel counters: [0] banded jobs, [1] the others
};

cudaError_t batch_set_attributes();
cudaError_t launch_batch(cudaStream_t st, int sms, const BatchPlan &plan, const BatchFill *fills, int nfill,
                         int64_t max_fill, uint32_t *status);

}  // namespace blg
