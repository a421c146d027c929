// The work-order scheduler network: a 7 -> 32 -> 32 -> 1 MLP that predicts,
// for each work record of the scheduled pairwise path, the fraction of its
// text the column loop will process before the max_dist exit fires. The
// prediction times the pair's size (columns x words) becomes the record's
// counting-sort key, so warps take pairs that finish together. It only
// changes the order in which pairs are computed, never which pairs or
// their values.
//
// Weights are FP16 (the form inference and the training forward pass use),
// with an FP32 master copy for the SGD update; all sums accumulate in FP32.
// Training kernels: k_collect_rows (features + logged exit columns ->
// rows), k_mlp_grad (forward + backward of a minibatch, per-block gradient
// sums as small outer products over rows staged in shared memory),
// k_mlp_sgd (momentum SGD, FP16 refresh). One epoch is captured into a CUDA
// graph once and replayed per epoch.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/bitlev_gb300.h"
#include "blg_context.h"
#include "blg_kernels.cuh"
#include "blg_sched.h"

namespace blg {

constexpr int kH = 32;                                   // hidden width
constexpr int kOffW1 = 0, kOffB1 = kOffW1 + kH * kFeatures, kOffW2 = kOffB1 + kH, kOffB2 = kOffW2 + kH * kH,
              kOffW3 = kOffB2 + kH, kOffB3 = kOffW3 + kH, kParams = kOffB3 + 1;   // 1345
constexpr int kRowsPerBlock = 128;
constexpr int kRowFloats = kFeatures + 1 + 4 * kH + 1;  // x, target, h1, h2, dh1, dh2, d

struct MlpRows {
    half *x;        // [rows][kFeatures]
    float *y;       // [rows] target fraction in [0, 1]
    int64_t rows;
};

// Forward pass of one row with weights already in shared memory (FP32
// values of the FP16 weights). Returns the prediction; fills h1/h2.
__device__ __forceinline__ float mlp_forward(const float *w, const float *x, float *h1, float *h2) {
#pragma unroll 4
    for (int j = 0; j < kH; j++) {
        float s = w[kOffB1 + j];
#pragma unroll
        for (int i = 0; i < kFeatures; i++) s = fmaf(w[kOffW1 + j * kFeatures + i], x[i], s);
        h1[j] = s > 0.f ? s : 0.f;
    }
#pragma unroll 4
    for (int j = 0; j < kH; j++) {
        float s = w[kOffB2 + j];
#pragma unroll 8
        for (int i = 0; i < kH; i++) s = fmaf(w[kOffW2 + j * kH + i], h1[i], s);
        h2[j] = s > 0.f ? s : 0.f;
    }
    float y = w[kOffB3];
#pragma unroll 8
    for (int i = 0; i < kH; i++) y = fmaf(w[kOffW3 + i], h2[i], y);
    return y;
}

__device__ __forceinline__ void load_weights(const half *w16, float *w) {
    for (int x = threadIdx.x; x < kParams; x += blockDim.x) w[x] = __half2float(w16[x]);
}

// rows[r] = (features of record r, logged columns / text length), over all
// classes in class order; `stride` subsamples when there are too many records.
__global__ void __launch_bounds__(256) k_collect_rows(PairsPlan plan, const int32_t *cols, int64_t stride,
                                                      int64_t max_rows, MlpRows rows, int64_t *n_rows) {
    int64_t before = 0;
    for (int cls = 0; cls < kPairClasses; cls++) {
        const int64_t cnt = min((int64_t)plan.count[cls], plan.cap[cls]);
        for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r * stride < cnt;
             r += (int64_t)gridDim.x * blockDim.x) {
            const int64_t dst = before + r;
            if (dst >= max_rows) break;
            const int64_t src = r * stride;
            const LongItem it = plan.raw[cls][src];
            const half *f = plan.feat[cls] + src * kFeatures;
#pragma unroll
            for (int i = 0; i < kFeatures; i++) rows.x[dst * kFeatures + i] = f[i];
            rows.y[dst] = it.n > 0 ? (float)cols[it.idx] / (float)it.n : 0.f;
        }
        before += (cnt + stride - 1) / stride;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *n_rows = before < max_rows ? before : max_rows;
}

// Forward + backward of rows [r0, r0 + B); gradients of the mean squared
// error summed per block into `grad` (FP32), loss sum into loss[0].
__global__ void __launch_bounds__(kRowsPerBlock) k_mlp_grad(const half *w16, MlpRows rows, const int64_t *n_rows,
                                                            int64_t r0, int B, float *grad, float *loss) {
    extern __shared__ float sm[];
    float *w = sm;                                       // kParams
    float *rb = sm + ((kParams + 3) & ~3);               // kRowsPerBlock x kRowFloats
    load_weights(w16, w);
    __syncthreads();
    const int64_t nr = *n_rows;
    const int64_t r = r0 + (int64_t)blockIdx.x * kRowsPerBlock + threadIdx.x;
    const int64_t rend = min(r0 + (int64_t)B, nr);
    float *my = rb + threadIdx.x * kRowFloats;
    float *x = my, *h1 = my + kFeatures + 1, *h2 = h1 + kH, *dh1 = h2 + kH, *dh2 = dh1 + kH;
    float &dslot = my[kRowFloats - 1];
    float sq = 0.f;
    if (r < rend) {
#pragma unroll
        for (int i = 0; i < kFeatures; i++) x[i] = __half2float(rows.x[r * kFeatures + i]);
        const float t = rows.y[r];
        const float y = mlp_forward(w, x, h1, h2);
        const float e = y - t;
        sq = e * e;
        const float d = 2.f * e / (float)B;
        dslot = d;
#pragma unroll 8
        for (int i = 0; i < kH; i++) dh2[i] = h2[i] > 0.f ? d * w[kOffW3 + i] : 0.f;
#pragma unroll 4
        for (int i = 0; i < kH; i++) {
            float s = 0.f;
#pragma unroll 8
            for (int j = 0; j < kH; j++) s = fmaf(w[kOffW2 + j * kH + i], dh2[j], s);
            dh1[i] = h1[i] > 0.f ? s : 0.f;
        }
    } else {
        for (int i = 0; i < kRowFloats; i++) my[i] = 0.f;
    }
    // loss: warp sum, one atomic per warp
    for (int o = 16; o; o >>= 1) sq += __shfl_down_sync(kFull, sq, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, sq);
    __syncthreads();
    // parameter gradients: each thread owns a strided set of parameters and
    // sums its outer-product term over the block's rows
    for (int p = threadIdx.x; p < kParams; p += blockDim.x) {
        float g = 0.f;
        for (int q = 0; q < kRowsPerBlock; q++) {
            const float *row = rb + q * kRowFloats;
            const float *qx = row, *qh1 = row + kFeatures + 1, *qh2 = qh1 + kH, *qdh1 = qh2 + kH,
                        *qdh2 = qdh1 + kH;
            const float qd = row[kRowFloats - 1];
            if (p < kOffB1) g = fmaf(qdh1[p / kFeatures], qx[p % kFeatures], g);
            else if (p < kOffW2) g += qdh1[p - kOffB1];
            else if (p < kOffB2) g = fmaf(qdh2[(p - kOffW2) / kH], qh1[(p - kOffW2) % kH], g);
            else if (p < kOffW3) g += qdh2[p - kOffB2];
            else if (p < kOffB3) g = fmaf(qd, qh2[p - kOffW3], g);
            else g += qd;
        }
        atomicAdd(&grad[p], g);
    }
}

// Momentum SGD on the FP32 master, FP16 refresh, gradient reset.
__global__ void __launch_bounds__(256) k_mlp_sgd(float *master, float *mom, float *grad, half *w16, float lr,
                                                 float beta) {
    for (int p = threadIdx.x; p < kParams; p += blockDim.x) {
        const float v = beta * mom[p] + grad[p];
        mom[p] = v;
        master[p] -= lr * v;
        w16[p] = __float2half(master[p]);
        grad[p] = 0.f;
    }
}

// Inference weights in shared memory, laid out for 16-byte loads:
//   W1p[32][8]  row j = W1[j][0..6], b1[j]   (input 7 is a constant 1)
//   W2[32][32], b2[32], W3[32], b3
constexpr int kInfW1 = 0, kInfW2 = kInfW1 + kH * 8, kInfB2 = kInfW2 + kH * kH, kInfW3 = kInfB2 + kH,
              kInfB3 = kInfW3 + kH, kInfFloats = kInfB3 + 4;

__device__ __forceinline__ void load_inference_weights(const half *w16, float *w) {
    for (int x = threadIdx.x; x < kInfFloats; x += blockDim.x) {
        float v = 0.f;
        if (x < kInfW2) {
            const int j = x >> 3, i = x & 7;
            v = __half2float(w16[i < kFeatures ? kOffW1 + j * kFeatures + i : kOffB1 + j]);
        } else if (x < kInfB2) v = __half2float(w16[kOffW2 + (x - kInfW2)]);
        else if (x < kInfW3) v = __half2float(w16[kOffB2 + (x - kInfB2)]);
        else if (x < kInfB3) v = __half2float(w16[kOffW3 + (x - kInfW3)]);
        else if (x == kInfB3) v = __half2float(w16[kOffB3]);
        w[x] = v;
    }
}

// 16-byte shared load the compiler may not hoist out of the row loop (the
// 1345 weights would not fit in registers).
__device__ __forceinline__ float4 lds4(const float *p) {
    float4 v;
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "r"((uint32_t)__cvta_generic_to_shared(p)));
    return v;
}

// Forward pass of two rows at once (each weight load feeds both), every
// activation in registers. FP16 weights held as FP32, FP32 sums.
__device__ __forceinline__ void mlp_forward2(const float *w, const float (&x0)[8], const float (&x1)[8], float &y0,
                                             float &y1) {
    float h0[kH], h1[kH];
#pragma unroll
    for (int j = 0; j < kH; j++) {
        const float4 a = lds4(w + kInfW1 + j * 8), b = lds4(w + kInfW1 + j * 8 + 4);
        float s0 = a.x * x0[0], s1 = a.x * x1[0];
        s0 = fmaf(a.y, x0[1], s0); s1 = fmaf(a.y, x1[1], s1);
        s0 = fmaf(a.z, x0[2], s0); s1 = fmaf(a.z, x1[2], s1);
        s0 = fmaf(a.w, x0[3], s0); s1 = fmaf(a.w, x1[3], s1);
        s0 = fmaf(b.x, x0[4], s0); s1 = fmaf(b.x, x1[4], s1);
        s0 = fmaf(b.y, x0[5], s0); s1 = fmaf(b.y, x1[5], s1);
        s0 = fmaf(b.z, x0[6], s0); s1 = fmaf(b.z, x1[6], s1);
        h0[j] = fmaxf(s0 + b.w, 0.f);
        h1[j] = fmaxf(s1 + b.w, 0.f);
    }
    const float4 bb3 = lds4(w + kInfB3);
    y0 = bb3.x;
    y1 = bb3.x;
#pragma unroll
    for (int j = 0; j < kH; j++) {
        float s0 = 0.f, s1 = 0.f;
#pragma unroll
        for (int i = 0; i < kH; i += 4) {
            const float4 a = lds4(w + kInfW2 + j * kH + i);
            s0 = fmaf(a.x, h0[i], s0); s1 = fmaf(a.x, h1[i], s1);
            s0 = fmaf(a.y, h0[i + 1], s0); s1 = fmaf(a.y, h1[i + 1], s1);
            s0 = fmaf(a.z, h0[i + 2], s0); s1 = fmaf(a.z, h1[i + 2], s1);
            s0 = fmaf(a.w, h0[i + 3], s0); s1 = fmaf(a.w, h1[i + 3], s1);
        }
        const float4 bw = lds4(w + ((j & ~3) + kInfB2)), ww = lds4(w + ((j & ~3) + kInfW3));
        const float b2j = (j & 3) == 0 ? bw.x : (j & 3) == 1 ? bw.y : (j & 3) == 2 ? bw.z : bw.w;
        const float w3j = (j & 3) == 0 ? ww.x : (j & 3) == 1 ? ww.y : (j & 3) == 2 ? ww.z : ww.w;
        y0 = fmaf(w3j, fmaxf(s0 + b2j, 0.f), y0);
        y1 = fmaf(w3j, fmaxf(s1 + b2j, 0.f), y1);
    }
}

__device__ __forceinline__ void read_features(const PairsPlan &plan, int cls, int i, int cnt, float (&x)[8]) {
#pragma unroll
    for (int q = 0; q < 8; q++) x[q] = 0.f;
    if (i < cnt) {
        const half *f = plan.feat[cls] + (size_t)i * kFeatures;
#pragma unroll
        for (int q = 0; q < kFeatures; q++) x[q] = __half2float(f[q]);
    }
    x[7] = 1.f;
}

__device__ __forceinline__ void write_key(const PairsPlan &plan, int cls, int i, float y, int band) {
    y = y < 0.f ? 0.f : (y > 1.f ? 1.f : y);
    const LongItem it = plan.raw[cls][i];
    const float work = band ? y * (float)it.n + 16.f : (y * (float)it.n + 1.f) * (float)((it.m + 63) >> 6);
    int b = (int)(__log2f(work) * 8.f) + 1;
    plan.key[cls][i] = (uint8_t)(b < 0 ? 0 : (b > kCostBuckets - 1 ? kCostBuckets - 1 : b));
}

// Inference: record -> predicted fraction of its text -> cost key. The
// banded solver's work is the exit column plus a window fill of about 16
// steps whatever the pattern length; the word solvers' work is columns x
// pattern words. Two records per thread.
__global__ void __launch_bounds__(256) k_mlp_keys(const half *w16, PairsPlan plan, int band) {
    __shared__ __align__(16) float w[kInfFloats];
    load_inference_weights(w16, w);
    __syncthreads();
    for (int cls = 0; cls < kPairClasses; cls++) {
        const int cnt = min(plan.count[cls], (int)plan.cap[cls]);
        const int stride = 2 * gridDim.x * blockDim.x;
        for (int i = 2 * (blockIdx.x * blockDim.x) + threadIdx.x; i < cnt; i += stride) {
            float x0[8], x1[8], y0, y1;
            read_features(plan, cls, i, cnt, x0);
            read_features(plan, cls, i + blockDim.x, cnt, x1);
            mlp_forward2(w, x0, x1, y0, y1);
            write_key(plan, cls, i, y0, band);
            if (i + (int)blockDim.x < cnt) write_key(plan, cls, i + blockDim.x, y1, band);
        }
    }
}

// Predictions for given rows (diagnostics and tests).
__global__ void __launch_bounds__(256) k_mlp_predict(const half *w16, const half *x, int64_t rows, float *out) {
    __shared__ float w[kParams];
    load_weights(w16, w);
    __syncthreads();
    float h1[kH], h2[kH], xx[kFeatures];
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int q = 0; q < kFeatures; q++) xx[q] = __half2float(x[r * kFeatures + q]);
        out[r] = mlp_forward(w, xx, h1, h2);
    }
}

}  // namespace blg

// ============================================================== host ==
using namespace blg;

struct blg_sched_model {
    float *master = nullptr, *mom = nullptr, *grad = nullptr, *loss = nullptr;
    half *w16 = nullptr;
    bool trained = false;
};

namespace {

// Deterministic initial weights: He-style uniform from a fixed LCG.
void init_weights(std::vector<float> &w, uint32_t seed) {
    uint32_t s = seed * 2654435761u + 12345u;
    auto uni = [&]() {
        s = s * 1664525u + 1013904223u;
        return ((s >> 8) * (1.0f / 16777216.0f)) * 2.f - 1.f;
    };
    w.assign(kParams, 0.f);
    for (int i = 0; i < kH * kFeatures; i++) w[kOffW1 + i] = uni() * 0.9f;    // sqrt(6/7)
    for (int i = 0; i < kH * kH; i++) w[kOffW2 + i] = uni() * 0.43f;          // sqrt(6/32)
    for (int i = 0; i < kH; i++) w[kOffW3 + i] = uni() * 0.43f;
    for (int i = 0; i < kH; i++) { w[kOffB1 + i] = 0.01f; w[kOffB2 + i] = 0.01f; }
    w[kOffB3] = 0.5f;
}

}  // namespace

int sched_model_ensure(blg_ctx *c, blg_sched_model **out) {
    if (!c->model) {
        blg_sched_model *m = new (std::nothrow) blg_sched_model();
        if (!m) return fail(c, BLG_ERR_ALLOC, "host allocation");
        cudaError_t e = cudaMalloc(&m->master, sizeof(float) * kParams);
        if (e == cudaSuccess) e = cudaMalloc(&m->mom, sizeof(float) * kParams);
        if (e == cudaSuccess) e = cudaMalloc(&m->grad, sizeof(float) * kParams);
        if (e == cudaSuccess) e = cudaMalloc(&m->loss, sizeof(float) * 2);
        if (e == cudaSuccess) e = cudaMalloc(&m->w16, sizeof(half) * kParams);
        if (e != cudaSuccess) {
            cudaFree(m->master); cudaFree(m->mom); cudaFree(m->grad); cudaFree(m->loss); cudaFree(m->w16);
            delete m;
            return cuda_fail(c, e, "model allocation");
        }
        c->model = m;
    }
    *out = c->model;
    return BLG_OK;
}

bool sched_model_trained(const blg_sched_model *m) { return m && m->trained; }

void sched_model_free(blg_sched_model *m) {
    if (!m) return;
    cudaFree(m->master); cudaFree(m->mom); cudaFree(m->grad); cudaFree(m->loss); cudaFree(m->w16);
    delete m;
}

static int set_weights(blg_ctx *c, blg_sched_model *m, const std::vector<float> &w) {
    std::vector<half> h(kParams);
    for (int i = 0; i < kParams; i++) h[i] = __float2half(w[i]);
    CK(cudaMemcpyAsync(m->master, w.data(), sizeof(float) * kParams, cudaMemcpyHostToDevice, c->stream), "H2D master");
    CK(cudaMemcpyAsync(m->w16, h.data(), sizeof(half) * kParams, cudaMemcpyHostToDevice, c->stream), "H2D w16");
    CK(cudaMemsetAsync(m->mom, 0, sizeof(float) * kParams, c->stream), "zero momentum");
    CK(cudaMemsetAsync(m->grad, 0, sizeof(float) * kParams, c->stream), "zero grad");
    CK(cudaStreamSynchronize(c->stream), "sync");
    return BLG_OK;
}

// Host-side pieces the runtime (blg_api.cu) calls.
cudaError_t launch_mlp_keys(cudaStream_t st, int sms, const blg_sched_model *m, const PairsPlan &plan, bool band) {
    k_mlp_keys<<<sms * 4, 256, 0, st>>>(m->w16, plan, band ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_collect_rows(cudaStream_t st, int sms, const PairsPlan &plan, const int32_t *cols,
                                int64_t stride, int64_t max_rows, half *x, float *y, int64_t *n_rows) {
    MlpRows rows{x, y, max_rows};
    k_collect_rows<<<sms * 4, 256, 0, st>>>(plan, cols, stride, max_rows, rows, n_rows);
    return cudaGetLastError();
}

// Train for `epochs` over rows already on the device (x: [rows][7] half,
// y: [rows] float). One epoch = ceil(rows / batch) (grad, sgd) launches,
// captured once into a CUDA graph and replayed.
int sched_train_rows(blg_ctx *c, blg_sched_model *m, half *x, float *y, const int64_t *d_rows, int64_t rows,
                     int epochs, float lr, int batch, float *loss_out) {
    if (!m->trained) {
        std::vector<float> w;
        init_weights(w, 2003u);
        int rc = set_weights(c, m, w);
        if (rc) return rc;
    }
    const size_t smem = sizeof(float) * (((kParams + 3) & ~3) + kRowsPerBlock * kRowFloats);
    CK(cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "smem attr");
    MlpRows R{x, y, rows};
    const int64_t nb = (rows + batch - 1) / batch;
    const int blocks = (batch + kRowsPerBlock - 1) / kRowsPerBlock;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    for (int64_t bi = 0; bi < nb; bi++) {
        k_mlp_grad<<<blocks, kRowsPerBlock, smem, c->stream>>>(m->w16, R, d_rows, bi * batch, batch, m->grad, m->loss);
        k_mlp_sgd<<<1, 256, 0, c->stream>>>(m->master, m->mom, m->grad, m->w16, lr, 0.9f);
    }
    cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
    if (e != cudaSuccess) return cuda_fail(c, e, "end capture");
    e = cudaGraphInstantiate(&exec, graph, 0);
    if (e != cudaSuccess) { cudaGraphDestroy(graph); return cuda_fail(c, e, "graph instantiate"); }
    float last = 0.f;
    for (int ep = 0; ep < epochs; ep++) {
        cudaMemsetAsync(m->loss, 0, sizeof(float), c->stream);
        e = cudaGraphLaunch(exec, c->stream);
        if (e != cudaSuccess) break;
        c->launches += 2 * nb;
        float l = 0.f;
        cudaMemcpyAsync(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost, c->stream);
        cudaStreamSynchronize(c->stream);
        last = rows > 0 ? l / (float)rows : 0.f;
    }
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(c, e, "graph launch");
    m->trained = true;
    if (loss_out) *loss_out = last;
    return BLG_OK;
}

extern "C" {

int blg_sched_set_weights(blg_ctx *c, const float *w, int n) {
    if (!c) return BLG_ERR_ARG;
    std::lock_guard<std::mutex> lock(c->mu);
    c->err.clear();
    if (n != kParams || !w) return fail(c, BLG_ERR_ARG, "expected 1345 weights");
    cudaSetDevice(c->device);
    blg_sched_model *m = nullptr;
    int rc = sched_model_ensure(c, &m);
    if (rc) return rc;
    std::vector<float> v(w, w + n);
    rc = set_weights(c, m, v);
    if (!rc) m->trained = true;
    return rc;
}

int blg_sched_get_weights(blg_ctx *c, float *w, int n) {
    if (!c) return BLG_ERR_ARG;
    std::lock_guard<std::mutex> lock(c->mu);
    c->err.clear();
    if (n != kParams || !w) return fail(c, BLG_ERR_ARG, "expected 1345 weights");
    if (!c->model || !c->model->trained) return fail(c, BLG_ERR_ARG, "no trained scheduler");
    cudaSetDevice(c->device);
    CK(cudaMemcpyAsync(w, c->model->master, sizeof(float) * kParams, cudaMemcpyDeviceToHost, c->stream), "D2H");
    CK(cudaStreamSynchronize(c->stream), "sync");
    return BLG_OK;
}

// Gradient of the mean squared error over `rows` host rows at the current
// weights (FP16 forward, FP32 sums), without updating them: the hook the
// gradient check against the CPU restatement uses.
int blg_sched_gradient(blg_ctx *c, const uint16_t *x_half, const float *y, int rows, float *grad_out,
                       float *loss_out) {
    if (!c) return BLG_ERR_ARG;
    std::lock_guard<std::mutex> lock(c->mu);
    c->err.clear();
    if (rows <= 0 || !x_half || !y || !grad_out) return fail(c, BLG_ERR_ARG, "bad arguments");
    if (!c->model || !c->model->trained) return fail(c, BLG_ERR_ARG, "set weights first");
    cudaSetDevice(c->device);
    blg_sched_model *m = c->model;
    half *dx = nullptr;
    float *dy = nullptr;
    int64_t *dn = nullptr;
    CK(cudaMalloc(&dx, sizeof(half) * kFeatures * rows), "malloc");
    CK(cudaMalloc(&dy, sizeof(float) * rows), "malloc");
    CK(cudaMalloc(&dn, sizeof(int64_t)), "malloc");
    const int64_t r64 = rows;
    cudaMemcpyAsync(dx, x_half, sizeof(half) * kFeatures * rows, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(dy, y, sizeof(float) * rows, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(dn, &r64, sizeof(int64_t), cudaMemcpyHostToDevice, c->stream);
    cudaMemsetAsync(m->grad, 0, sizeof(float) * kParams, c->stream);
    cudaMemsetAsync(m->loss, 0, sizeof(float), c->stream);
    const size_t smem = sizeof(float) * (((kParams + 3) & ~3) + kRowsPerBlock * kRowFloats);
    cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    MlpRows R{dx, dy, rows};
    k_mlp_grad<<<(rows + kRowsPerBlock - 1) / kRowsPerBlock, kRowsPerBlock, smem, c->stream>>>(
        m->w16, R, dn, 0, rows, m->grad, m->loss);
    c->launches++;
    cudaMemcpyAsync(grad_out, m->grad, sizeof(float) * kParams, cudaMemcpyDeviceToHost, c->stream);
    float l = 0.f;
    cudaMemcpyAsync(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    cudaMemsetAsync(m->grad, 0, sizeof(float) * kParams, c->stream);
    const cudaError_t e = cudaStreamSynchronize(c->stream);
    cudaFree(dx);
    cudaFree(dy);
    cudaFree(dn);
    if (e != cudaSuccess) return cuda_fail(c, e, "gradient");
    if (loss_out) *loss_out = l / (float)rows;
    return BLG_OK;
}

// Predictions for host rows (diagnostics).
int blg_sched_predict(blg_ctx *c, const uint16_t *x_half, int64_t rows, float *out) {
    if (!c) return BLG_ERR_ARG;
    std::lock_guard<std::mutex> lock(c->mu);
    c->err.clear();
    if (rows <= 0 || !x_half || !out) return fail(c, BLG_ERR_ARG, "bad arguments");
    if (!c->model || !c->model->trained) return fail(c, BLG_ERR_ARG, "no trained scheduler");
    cudaSetDevice(c->device);
    half *dx = nullptr;
    float *dout = nullptr;
    CK(cudaMalloc(&dx, sizeof(half) * kFeatures * rows), "malloc");
    CK(cudaMalloc(&dout, sizeof(float) * rows), "malloc");
    cudaMemcpyAsync(dx, x_half, sizeof(half) * kFeatures * rows, cudaMemcpyHostToDevice, c->stream);
    k_mlp_predict<<<c->sms * 4, 256, 0, c->stream>>>(c->model->w16, dx, rows, dout);
    c->launches++;
    cudaMemcpyAsync(out, dout, sizeof(float) * rows, cudaMemcpyDeviceToHost, c->stream);
    const cudaError_t e = cudaStreamSynchronize(c->stream);
    cudaFree(dx);
    cudaFree(dout);
    if (e != cudaSuccess) return cuda_fail(c, e, "predict");
    return BLG_OK;
}

// Versioned binary checkpoint: "BLGMLP02", int32 count, FP32 master weights.
int blg_sched_save(blg_ctx *c, const char *path) {
    std::vector<float> w(kParams);
    int rc = blg_sched_get_weights(c, w.data(), kParams);
    if (rc) return rc;
    FILE *f = fopen(path, "wb");
    if (!f) return fail(c, BLG_ERR_ARG, std::string("cannot write ") + path);
    const int32_t n = kParams;
    const bool ok = fwrite("BLGMLP02", 1, 8, f) == 8 && fwrite(&n, 4, 1, f) == 1 &&
                    fwrite(w.data(), sizeof(float), kParams, f) == (size_t)kParams;
    fclose(f);
    return ok ? BLG_OK : fail(c, BLG_ERR_ARG, "short write");
}

int blg_sched_load(blg_ctx *c, const char *path) {
    if (!c) return BLG_ERR_ARG;
    FILE *f = fopen(path, "rb");
    if (!f) return fail(c, BLG_ERR_ARG, std::string("cannot read ") + path);
    char magic[8];
    int32_t n = 0;
    std::vector<float> w(kParams);
    const bool ok = fread(magic, 1, 8, f) == 8 && memcmp(magic, "BLGMLP02", 8) == 0 && fread(&n, 4, 1, f) == 1 &&
                    n == kParams && fread(w.data(), sizeof(float), kParams, f) == (size_t)kParams;
    fclose(f);
    if (!ok) return fail(c, BLG_ERR_ARG, "not a scheduler checkpoint (BLGMLP02, 1345 weights)");
    return blg_sched_set_weights(c, w.data(), kParams);
}

}  // extern "C"
