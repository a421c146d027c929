// The library context shared by the host translation units of the C-ABI.
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <string>
#include <vector>

struct blg_sched_model;   // the work-order scheduler network (blg_mlp.cu)

// Launch shapes chosen by the autotuner (blg_autotune); the defaults are the
// hand-picked shapes used before any tuning. The banded kernels' shapes have
// a max_dist axis: one shape for small max_dist, one for the rest up to 31
// (kSurvWideK, kBandWideK): a wider band keeps more survivors alive for
// more columns, which moves the best occupancy / round length.
constexpr int kSurvWideK = 9;     // thresholded search: max_dist 9..31 take the *_wide shapes (tuned at 16)
constexpr int kBandWideK = 16;    // banded pairs solver: max_dist 16..31 take band_ctas_wide (tuned at 24)
struct blg_tuning {
    int qpb[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};   // exact search: queries per CTA by query words (0: heuristic)
    int lpt_ctas = 4;                            // thresholded search, max_dist <= 8: CTAs per SM
    int lpt_job = 4096;                          // thresholded search: survivors per job
    int surv_round = 16;                         // thresholded search, max_dist <= 8: columns per lane round (8, 16, 32)
    int lpt_ctas_wide = 4;                       // thresholded search, max_dist 9..31: CTAs per SM
    int surv_round_wide = 16;                    // thresholded search, max_dist 9..31: columns per lane round
    int band_ctas = 3;                           // banded pairs solver, max_dist <= 15: CTAs per SM
    int band_ctas_wide = 3;                      // banded pairs solver, max_dist 16..31: CTAs per SM
    int tile_shape = 1;                          // short-pair tile kernel: 1 = one stage of 512 pairs, 2 = two of 512,
                                                 // 3 = two of 256 (1M pairs of 32 bytes: 61, 79, 76 us)
    int tuned = 0;
};

struct blg_ctx {
    struct ProfRec {
        const char *name;
        cudaEvent_t e0, e1;
    };
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;     // kernels (and every resident-state call)
    cudaStream_t up = nullptr;         // host -> device copies of the one-call pipelines
    cudaStream_t down = nullptr;       // device -> host copies of the one-call pipelines
    uint32_t *d_status = nullptr;      // status bits raised by kernels (blg::ST_*)
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    std::mutex mu;                     // serialises calls on one context
    std::string err;
    int64_t launches = 0;
    int sched = 0;                     // BLG_SCHED_* (work order of thresholded runs)
    blg_sched_model *model = nullptr;  // trained/loaded scheduler network, if any
    blg_tuning tune;                   // launch shapes (autotuned or defaults)
    bool prof = false;
    // fault injection for tests of the error paths (blg_set_fault_injection):
    // the device allocation after `fault_alloc_after` more successes fails
    // (-1: off); the short-pair tile kernel's first bounded copy wait gives
    // up after `fault_wait_polls` polls (-1: the normal bound)
    int64_t fault_alloc_after = -1;
    int32_t fault_wait_polls = -1;
    // pinned host staging for arrays the host builds and copies (grown on
    // demand; stage_done marks the end of the last copy out of it)
    void *stage = nullptr;
    // pinned room for a batch upload's small host-built tables (HostArena)
    void *arena = nullptr;
    size_t arena_bytes = 0;
    // the survivor search's deferred results: header [count, fill items
    // claimed], then rl_cap entries (allocated at init)
    unsigned long long *rl_hdr = nullptr;
    unsigned long long rl_cap = 0;
    size_t stage_bytes = 0;
    cudaEvent_t stage_done = nullptr;
    std::vector<ProfRec> prof_recs;
    std::map<std::string, std::pair<int64_t, double>> prof_acc;
};

// Record an error message and return `code`.
int fail(blg_ctx *c, int code, const std::string &msg);
// Map a CUDA error to BLG_ERR_ALLOC / BLG_ERR_CUDA with a message.
int cuda_fail(blg_ctx *c, cudaError_t e, const char *what);
// Synchronise the context stream, read and clear the kernels' status word.
int sync_and_status(blg_ctx *c);
void sched_model_free(blg_sched_model *m);

// Return the mapped error from the enclosing function (its context is `c`).
#define CK(call, what)                                        \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return cuda_fail(c, e_, what); \
    } while (0)
