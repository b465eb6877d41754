// Throughput probes of the FP32 and FP64 FMA pipes, used as the roofline
// denominators of the FP32-bound FMM stages (M2L, P2P) and the FP64 dense
// operator.  Each thread runs 8 independent FMA chains so that issue, not
// latency, limits the rate.
#include "edfmm_internal.cuh"

namespace edfmm {
namespace {

template <typename T>
__global__ void __launch_bounds__(256) k_fma_probe(int iters, T seed, T *sink) {
    T a0 = seed + T(threadIdx.x), a1 = a0 + T(1), a2 = a0 + T(2), a3 = a0 + T(3);
    T a4 = a0 + T(4), a5 = a0 + T(5), a6 = a0 + T(6), a7 = a0 + T(7);
    const T b = T(0.999999), c = T(1e-7);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            a0 = fma(a0, b, c);
            a1 = fma(a1, b, c);
            a2 = fma(a2, b, c);
            a3 = fma(a3, b, c);
            a4 = fma(a4, b, c);
            a5 = fma(a5, b, c);
            a6 = fma(a6, b, c);
            a7 = fma(a7, b, c);
        }
    }
    const T r = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (r == T(1234.5678)) sink[threadIdx.x] = r;  // keeps the chains alive
}

template <typename T>
int measure_peak(int iters, void *stream, double *tflops_out) {
    if (!tflops_out || iters <= 0) return fail(EDFMM_ERR_ARG, "bad arguments");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int dev = 0, sms = 0;
    EDFMM_CUDA_TRY(cudaGetDevice(&dev));
    EDFMM_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    DevBuf sink;
    if (int rc = sink.reserve(256 * sizeof(T))) return rc;
    const int blocks = sms * 8;
    cudaEvent_t e0, e1;
    EDFMM_CUDA_TRY(cudaEventCreate(&e0));
    EDFMM_CUDA_TRY(cudaEventCreate(&e1));
    k_fma_probe<T><<<blocks, 256, 0, s>>>(iters / 8 + 1, T(1), dptr<T>(sink));  // warm-up
    EDFMM_LAUNCH_CHECK("k_fma_probe");
    EDFMM_CUDA_TRY(cudaEventRecord(e0, s));
    k_fma_probe<T><<<blocks, 256, 0, s>>>(iters, T(1), dptr<T>(sink));
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

}  // namespace
}  // namespace edfmm

using namespace edfmm;

extern "C" EDFMM_API int edfmm_measure_fp32_peak(int iters, void *stream, double *tflops_out) {
    return measure_peak<float>(iters, stream, tflops_out);
}

extern "C" EDFMM_API int edfmm_measure_fp64_peak(int iters, void *stream, double *tflops_out) {
    return measure_peak<double>(iters, stream, tflops_out);
}
