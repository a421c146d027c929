// Internal types shared by the kernels (blg_kernels.cu) and the host
// runtime (blg_api.cu). Not part of the public C-ABI.
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>

namespace blg {

// A packed string set resident in HBM: bytes of string i are
// buf[off[i] - base, off[i+1] - base). The byte buffer carries 16 bytes of
// slack before and 48 after the data, so the kernels' aligned window loads
// and read-ahead cursors never leave the allocation; `buf` points 16 bytes
// into it.
constexpr int kSlackBefore = 16, kSlackAfter = 48;
struct DevStrings {
    const uint8_t *buf = nullptr;
    const int64_t *off = nullptr;
    int64_t n = 0;
    int64_t base = 0;       // off[0] on the host
    int64_t bytes = 0;      // off[n] - off[0]
};

// Status bits raised by kernels (atomicOr into a device word).
enum : uint32_t {
    ST_BAD_OFFSETS = 1u << 0,   // offsets not monotone / out of range
    ST_TOO_LONG = 1u << 1,      // pattern longer than the lane-spread limit
    ST_QUEUE_TIMEOUT = 1u << 2, // a bounded device wait gave up
    ST_QUEUE_OVERFLOW = 1u << 3,
};

// Long pairs (trimmed pattern longer than 64) are queued by the pairs kernel
// and solved lane-spread: one 64-bit pattern word per lane, LANES lanes per
// pair, classes LANES = 2, 4, 8, 16, 32.
constexpr int kLongClasses = 5;
constexpr int kMaxLanePattern = 64 * 32;

struct LongItem {
    const uint8_t *pat;
    const uint8_t *txt;
    int32_t m, n;
    int64_t idx;
};

struct LongQueue {
    LongItem *items[kLongClasses];   // one region per class
    int64_t cap[kLongClasses];       // capacity of each region (pairs that may land there)
    int32_t *counts;                 // kLongClasses producers' counters
    int32_t *heads;                  // kLongClasses consumers' counters
};

// Choices in tile-transposed form (exact search): tiles of kTileCands
// consecutive choices; word w (bytes 4w..4w+3) of choice c of tile T sits at
// words[base[T] + w * kTileCands + (c - T * kTileCands)], so the 32 lanes of
// a warp reading their choices' word w touch one 128-byte line. base[T+1] -
// base[T] = kTileCands * ceil(longest choice of T / 4); len[c] = length.
constexpr int kTileCands = 1024;

// Rows of words allocated past the last tile of transposed choices, so the
// search loop may prefetch up to this many words beyond any choice's end.
constexpr int kTtSlackRows = 4;

struct TransposedChoices {
    const uint32_t *words = nullptr;
    const int64_t *base = nullptr;    // [tiles + 1]
    const int32_t *len = nullptr;     // [n]
    int64_t n = 0;
};

// Choices sorted lexicographically for the exact search with prefix reuse
// (k_search_pfx). A warp's 32 lanes hold different queries and share one
// choice at a time, so the text, its length and its restart column are the
// same on every lane. Each warp walks a chain of consecutive sorted choices
// (kPfxChain, or a divisor of it when a launch has few queries); a choice
// restarts at the largest checkpoint column not above its common prefix with
// the previous sorted choice (0 at a chain start), from the column state that
// choice's run saved there.
// Text: sorted choice p occupies words text[woff[p] ..] with two characters
// per 32-bit word, each character stored as its shared-memory Peq row offset
// (alphabet index x kPfxRowBytes, 16 bits), so a column's Peq address needs
// no byte extraction or scaling. The alphabet is the set of bytes that occur
// in the choices (at most kPfxMaxSymbols).
constexpr int kPfxChain = 32;
constexpr int kPfxWarps = 8;                         // warps per CTA; a work item = kPfxWarps chains
constexpr int kPfxCheckpoints = 2;
constexpr int kPfxMaxSymbols = 32;
constexpr int kPfxRowBytes = 1024;                   // one symbol's Peq entries: 32 lanes x QI x NW x 8 B
constexpr int kPfxTextSlack = 8;                     // words readable past the last choice (prefetch)

struct PrefixChoices {
    const uint32_t *text = nullptr;   // row offsets, 2 per word
    const int64_t *woff = nullptr;    // [n + 1] first word of sorted choice p
    const int32_t *len = nullptr;     // [n] length of sorted choice p
    const int32_t *orig = nullptr;    // [n] original index of sorted choice p
    const uint8_t *restart = nullptr; // [n] first column to compute for sorted choice p
    const uint8_t *sym = nullptr;     // [nsym] the byte of each alphabet index
    int nsym = 0;
    int64_t n = 0;
    int ck[kPfxCheckpoints] = {0, 0};
};

// Per-query-class search launch description.
struct SearchClass {
    int nw;                 // pattern words (sequential kernels) or 0 for lane-spread
    int nq;                 // queries in this class
    const int32_t *qidx;    // device: query row per class entry
    const int32_t *qlen;    // device: query length per class entry
    const uint64_t *peq;    // device: [nq][256][nw] Peq tables
};

// Pair sets using at most kBandSymbols distinct bytes run the pairs kernels'
// one-row-per-byte pattern tables (row kBandSymbols stays empty for the
// bytes outside the set); larger alphabets use nibble rows.
constexpr int kBandSymbols = 15;

// Query word classes of the sequential search kernels (patterns of 1..8
// 64-bit words); longer queries run lane-spread. A thresholded run plans and
// solves the survivors of all its sequential classes in one launch each.
constexpr int kSurvClasses = 8;

struct SurvClasses {
    int n = 0;                                 // classes
    SearchClass cls[kSurvClasses];
    int32_t *lo[kSurvClasses];                 // survivor range per query
    int32_t *hi[kSurvClasses];
    int64_t *tile_start[kSurvClasses];         // job prefix per query (nq + 1)
    int32_t *work[kSurvClasses];               // job counters (cleared by the plan)
};

// An output array to fill with one value (dtype-sized elements).
struct BatchFill {
    void *out;
    int64_t n;
    int dtype;
    uint32_t value;
};

// Results <= k deferred by a survivor kernel that fills its own output:
// entries (element address << 8 | dtype << 6 | value), count (may pass cap:
// the list ran full).
struct ResultList {
    unsigned long long *item;
    unsigned long long *count;
    unsigned long long cap;
};

// Output arrays to fill, as work items of kFillChunk bytes (whole elements).
constexpr int64_t kFillChunk = 65536;

struct FillItems {
    const BatchFill *fills;       // the arrays (null: the one array `one`)
    const int64_t *start;         // [nfill + 1] first item of each array
    int nfill;
    BatchFill one;
    int64_t total;                // items
    unsigned long long *ctr;      // items claimed, zero before the launch
};

// element bytes of a result dtype (0 int32, 1 uint16, 2 uint8)
__host__ __device__ inline int elem_bytes(int dtype) { return dtype == 2 ? 1 : dtype == 1 ? 2 : 4; }

__host__ __device__ inline int64_t fill_items_of(const BatchFill &f) {
    return (f.n * elem_bytes(f.dtype) + kFillChunk - 1) / kFillChunk;
}

}  // namespace blg
