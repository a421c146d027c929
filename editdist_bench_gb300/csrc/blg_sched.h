// Work plans of the scheduled paths (shared by kernels and host runtime).
#pragma once
#include <cuda_fp16.h>
#include <stdint.h>

#include "blg_internal.h"

namespace blg {

constexpr int kPairClasses = 6;      // 0: pattern <= 64 (one thread); 1..5: 2..32 lanes
constexpr int kCostBuckets = 256;    // counting-sort keys (log-spaced cost or predicted work)
constexpr int kFeatures = 7;         // scheduler network inputs per record

// Pairwise plan: records of non-trivial pairs per class, before (raw) and
// after (sorted, per 1024-record segment) ordering, their keys, optional
// feature rows, counters.
struct PairsPlan {
    LongItem *raw[kPairClasses];
    LongItem *sorted[kPairClasses];
    uint8_t *key[kPairClasses];
    half *feat[kPairClasses];        // kFeatures halves per record (learned schedule)
    int64_t cap[kPairClasses];
    int32_t *count;                  // [kPairClasses]
    int32_t *head;                   // [kPairClasses]
};

// Logged rows of the learned scheduler from the thresholded search (features,
// label = exit column / text length) for every `stride`-th survivor, up to
// `cap` rows; `count` counts the rows written.
struct SurvRows {
    half *x;
    float *y;
    int64_t cap;
    int64_t *count;
    int stride;
};


}  // namespace blg
