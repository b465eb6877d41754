// Throughput probe of the FP32 FMA pipe, used as the roofline denominator of
// the FP32-bound FMM stages (M2L, P2P).  Each thread runs 8 independent FMA
// chains so that issue, not latency, limits the rate.
#include "edfmm_internal.cuh"

namespace edfmm {
namespace {

__global__ void __launch_bounds__(256) k_fma_probe(int iters, float seed, float *sink) {
    float a0 = seed + threadIdx.x, a1 = a0 + 1.f, a2 = a0 + 2.f, a3 = a0 + 3.f;
    float a4 = a0 + 4.f, a5 = a0 + 5.f, a6 = a0 + 6.f, a7 = a0 + 7.f;
    const float b = 0.999999f, c = 1e-7f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            a0 = fmaf(a0, b, c);
            a1 = fmaf(a1, b, c);
            a2 = fmaf(a2, b, c);
            a3 = fmaf(a3, b, c);
            a4 = fmaf(a4, b, c);
            a5 = fmaf(a5, b, c);
            a6 = fmaf(a6, b, c);
            a7 = fmaf(a7, b, c);
        }
    }
    const float r = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (r == 1234.5678f) sink[threadIdx.x] = r;  // keeps the chains alive
}

}  // namespace
}  // namespace edfmm

using namespace edfmm;

extern "C" EDFMM_API int edfmm_measure_fp32_peak(int iters, void *stream, double *tflops_out) {
    if (!tflops_out || iters <= 0) return fail(EDFMM_ERR_ARG, "bad arguments");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int dev = 0, sms = 0;
    EDFMM_CUDA_TRY(cudaGetDevice(&dev));
    EDFMM_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    DevBuf sink;
    if (int rc = sink.reserve(256 * sizeof(float))) return rc;
    const int blocks = sms * 8;
    cudaEvent_t e0, e1;
    EDFMM_CUDA_TRY(cudaEventCreate(&e0));
    EDFMM_CUDA_TRY(cudaEventCreate(&e1));
    k_fma_probe<<<blocks, 256, 0, s>>>(iters / 8 + 1, 1.0f, dptr<float>(sink));  // warm-up
    EDFMM_LAUNCH_CHECK("k_fma_probe");
    EDFMM_CUDA_TRY(cudaEventRecord(e0, s));
    k_fma_probe<<<blocks, 256, 0, s>>>(iters, 1.0f, dptr<float>(sink));
    EDFMM_LAUNCH_CHECK("k_fma_probe");
    EDFMM_CUDA_TRY(cudaEventRecord(e1, s));
    EDFMM_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.f;
    EDFMM_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double fmas = (double)blocks * 256.0 * (double)iters * 16.0 * 8.0;
    *tflops_out = 2.0 * fmas / (ms * 1e-3) / 1e12;
    return EDFMM_OK;
}
