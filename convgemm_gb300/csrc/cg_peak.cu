// Measurement of the FP32 FMA (SIMT) peak that the FP32 plain form's roofline is quoted
// against: every thread runs eight independent FMA chains, enough to cover the FMA latency
// on all four schedulers of every SM, with no memory traffic inside the loop.
#include "../../include/convgemm_gpu.h"
#include "cg_internal.h"

namespace {

__global__ void __launch_bounds__(256) ffma_peak_kernel(int iters, float seed, float *out) {
    float a[8];
#pragma unroll
    for (int j = 0; j < 8; j++) a[j] = seed + 0.001f * (float) (threadIdx.x + j);
    const float m = 0.9999f, c = 1e-6f;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 16; u++) {
#pragma unroll
            for (int j = 0; j < 8; j++) a[j] = fmaf(a[j], m, c);
        }
    }
    float s = 0.0f;
#pragma unroll
    for (int j = 0; j < 8; j++) s += a[j];
    if (s == 12345.678f) out[0] = s;   // never true for these inputs: keeps the chains live
}

}  // namespace

extern "C" convgemm_status_t convgemm_measure_ffma(int iters, float *out, double *flops, void *stream) {
    if (iters < 1 || !out || !flops)
        return cg_set_error(CONVGEMM_ERROR_INVALID_VALUE, "convgemm_measure_ffma: bad argument");
    int dev = 0, sms = 0;
    if (convgemm_status_t e = cg_cuda_check(cudaGetDevice(&dev), "cudaGetDevice")) return e;
    if (convgemm_status_t e =
            cg_cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count"))
        return e;
    const int blocks = sms * 8;   // 2048 threads per SM
    ffma_peak_kernel<<<blocks, 256, 0, (cudaStream_t) stream>>>(iters, 1.0f, out);
    cg_note_launch();
    *flops = 2.0 * 8 * 16 * (double) iters * blocks * 256;
    return cg_cuda_check(cudaGetLastError(), "FMA peak launch");
}
