// probe.cu -- measured integer issue peaks of a GPU, the denominators of the
// DP kernels' roofline (the measured peaks on file cover HBM and bf16 only).
// Benchmark tooling: built into its own library, not the alignment path's.  Each probe thread runs 8 independent dependency chains of one
// instruction kind, long enough that issue, not latency, is the limit; the
// result is lane-operations per second (a 16x2 operation counts once per
// 32-bit lane: it updates two 16-bit values).
#include <cuda_runtime.h>

#include <cstdint>

#include "esp_workloads.h"

namespace {

constexpr int kChains = 8;
constexpr int kIters = 4096;

template <int KIND>
__global__ void __launch_bounds__(256) int_probe(uint32_t seed, uint32_t *sink) {
    uint32_t x[kChains];
    const uint32_t y = seed * 0x9E3779B9u + threadIdx.x, z = seed ^ 0x7F4A7C15u;
#pragma unroll
    for (int c = 0; c < kChains; c++) x[c] = threadIdx.x * (c + 1) + blockIdx.x;
#pragma unroll 1
    for (int it = 0; it < kIters; it++) {
#pragma unroll
        for (int c = 0; c < kChains; c++) {
            if (KIND == 0) {  // 3-input logic
                asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(x[c]) : "r"(y), "r"(z));
            } else if (KIND == 1) {  // integer max
                asm volatile("max.s32 %0, %0, %1;" : "+r"(x[c]) : "r"(y + c));
            } else if (KIND == 2) {  // integer add
                asm volatile("add.u32 %0, %0, %1;" : "+r"(x[c]) : "r"(y));
            } else if (KIND == 3) {  // integer multiply-add
                asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(x[c]) : "r"(y | 1u), "r"(z));
            } else if (KIND == 4) {  // 16x2 add-then-max (two 16-bit lanes)
                x[c] = __viaddmax_s16x2(x[c], y, z + c);
            } else {  // 16x2 three-way max
                x[c] = __vimax3_s16x2(x[c], y, z + c);
            }
        }
    }
    uint32_t acc = 0;
#pragma unroll
    for (int c = 0; c < kChains; c++) acc ^= x[c];
    if (acc == seed) sink[0] = acc;  // keeps the chains live
}

template <int KIND>
int run(int sms, cudaStream_t st, uint32_t *sink, double *out) {
    const int blocks = sms * 8, threads = 256;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    int_probe<KIND><<<blocks, threads, 0, st>>>(1u, sink);  // warm-up
    cudaEventRecord(a, st);
    const int reps = 5;
    for (int r = 0; r < reps; r++) int_probe<KIND><<<blocks, threads, 0, st>>>(r + 2u, sink);
    cudaEventRecord(b, st);
    cudaError_t e = cudaEventSynchronize(b);
    float ms = 0;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (e != cudaSuccess || ms <= 0) return ESP_ECUDA;
    double ops = (double)reps * blocks * threads * kChains * kIters;
    *out = ops / (ms * 1e-3);
    return ESP_OK;
}

using ProbeFn = int (*)(int, cudaStream_t, uint32_t *, double *);

// Runs the probes `fns` on `device`, one result each.
int run_probes(int device, int n, const ProbeFn *fns, double **out) {
    if (cudaSetDevice(device) != cudaSuccess) return ESP_ECUDA;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        return ESP_ECUDA;
    cudaStream_t st = nullptr;
    uint32_t *sink = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return ESP_ECUDA;
    int rc = cudaMalloc((void **)&sink, 4) == cudaSuccess ? ESP_OK : ESP_ECUDA;
    for (int k = 0; k < n && rc == ESP_OK; k++) rc = fns[k](sms, st, sink, out[k]);
    cudaFree(sink);
    cudaStreamDestroy(st);
    return rc;
}

}  // namespace

extern "C" int esp_probe_simd16_peaks(int device, double *addmax, double *max3) {
    if (!addmax || !max3) return ESP_EINVAL;
    const ProbeFn fns[2] = {run<4>, run<5>};
    double *out[2] = {addmax, max3};
    return run_probes(device, 2, fns, out);
}

extern "C" int esp_probe_int_peaks(int device, double *lop3, double *imnmx, double *iadd,
                                   double *imad) {
    if (!lop3 || !imnmx || !iadd || !imad) return ESP_EINVAL;
    const ProbeFn fns[4] = {run<0>, run<1>, run<2>, run<3>};
    double *out[4] = {lop3, imnmx, iadd, imad};
    return run_probes(device, 4, fns, out);
}
