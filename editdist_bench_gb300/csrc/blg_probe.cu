// Integer-pipe throughput probe: the denominator of the integer roofline.
//
// Measures, on the running GPU, how many 32-bit integer lane-operations per
// second the SMs sustain on the instruction mix bit-parallel Levenshtein
// uses: LOP3 (3-input logic), IADD3 and shifts. Every thread runs 8
// independent dependency chains (enough ILP to hide ALU latency at full
// occupancy); the result is folded into one store so nothing is dead code.
// Separate library (libblg_probe.so): a measurement tool, not part of the
// Levenshtein C-ABI.
#include <cuda_runtime.h>
#include <stdint.h>

namespace {

__device__ __forceinline__ uint32_t lop3_96(uint32_t a, uint32_t b, uint32_t c) {
    uint32_t r;
    asm volatile("lop3.b32 %0, %1, %2, %3, 0x96;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
    return r;
}
__device__ __forceinline__ uint32_t lop3_e8(uint32_t a, uint32_t b, uint32_t c) {
    uint32_t r;
    asm volatile("lop3.b32 %0, %1, %2, %3, 0xe8;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
    return r;
}
__device__ __forceinline__ uint32_t add3(uint32_t a, uint32_t b, uint32_t c) {
    uint32_t r;
    asm volatile("add.u32 %0, %1, %2;\n\tadd.u32 %0, %0, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
    return r;
}

// mode 0: logic only (LOP3 stream); mode 1: logic + adds (2 LOP3 : 1 3-input add)
template <int MODE>
__global__ void __launch_bounds__(256) k_int_peak(uint32_t *out, int iters, uint32_t seed) {
    uint32_t x[8];
#pragma unroll
    for (int c = 0; c < 8; c++) x[c] = seed * (threadIdx.x + 1) + 0x9e3779b9u * (c + 1) + blockIdx.x;
    const uint32_t k1 = seed ^ 0x85ebca6bu, k2 = seed ^ 0xc2b2ae35u;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int r = 0; r < 4; r++) {
#pragma unroll
            for (int c = 0; c < 8; c++) {
                if (MODE == 0) {
                    x[c] = lop3_96(x[c], k1, x[(c + 1) & 7]);
                    x[c] = lop3_e8(x[c], k2, x[(c + 3) & 7]);
                } else {
                    x[c] = lop3_96(x[c], k1, x[(c + 1) & 7]);
                    x[c] = add3(x[c], k2, x[(c + 3) & 7]);
                }
            }
        }
    }
    uint32_t acc = 0;
#pragma unroll
    for (int c = 0; c < 8; c++) acc ^= x[c];
    if (acc == 0x12345678u) out[0] = acc;   // practically never; keeps the chains live
}

}  // namespace

extern "C" {

// Runs the probe on `device`; returns 0 and the 32-bit lane-instructions per
// second of each mode (MODE 0: 2 LOP3 per chain step; MODE 1: one LOP3 and
// one 3-input add, which ptxas emits as a single IADD3).
int blg_probe_int_peak(int device, int iters, double *logic_ops_per_s, double *mixed_ops_per_s) {
    if (cudaSetDevice(device) != cudaSuccess) return -3;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    uint32_t *d = nullptr;
    if (cudaMalloc(&d, 64) != cudaSuccess) return -1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = sms * 8, threads = 256;
    const double lane_steps = (double)blocks * threads * iters * 4 * 8;
    double best[2] = {0, 0};
    for (int mode = 0; mode < 2; mode++) {
        for (int rep = 0; rep < 4; rep++) {
            cudaEventRecord(e0);
            if (mode == 0) k_int_peak<0><<<blocks, threads>>>(d, iters, 0x1234u + rep);
            else k_int_peak<1><<<blocks, threads>>>(d, iters, 0x1234u + rep);
            cudaEventRecord(e1);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            const double ops = lane_steps * 2.0;   // two SASS instructions per chain step
            if (rep > 0 && ms > 0) best[mode] = ops / (ms * 1e-3) > best[mode] ? ops / (ms * 1e-3) : best[mode];
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    if (cudaGetLastError() != cudaSuccess) return -3;
    if (logic_ops_per_s) *logic_ops_per_s = best[0];
    if (mixed_ops_per_s) *mixed_ops_per_s = best[1];
    return 0;
}

// SM count and maximum SM clock (kHz) of `device`: the issue-slot
// denominator of the per-kernel utilisation figure (4 warp instructions per
// SM per clock).
int blg_probe_device_info(int device, int *sms, int *clock_khz) {
    if (cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return -3;
    if (cudaDeviceGetAttribute(clock_khz, cudaDevAttrClockRate, device) != cudaSuccess) return -3;
    return 0;
}

}  // extern "C"
