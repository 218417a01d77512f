// probe.cu -- gpss_measure_fma_rate: the FMA throughput of the current device,
// the compute roof that the roofline reports of the FP64 kernels and of the
// compensated FP32 passes (both bound by their FMA pipe, not by HBM) are
// measured against.
#include <cuda_runtime.h>
#include "../../include/gpss.h"

namespace {

// every thread runs 8 independent FMA chains (enough to cover the pipe
// latency); the sums are written so that nothing is eliminated
template <typename T> __global__ void k_fma_rate(T *out, T a, T b, int iters)
{
    T x[8];
#pragma unroll
    for (int i = 0; i < 8; i++) x[i] = (T)(threadIdx.x + i) * (T)1e-3;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int i = 0; i < 8; i++) x[i] = fma(x[i], a, b);
    }
    T s = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) s += x[i];
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T> int rate(double *tflops)
{
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return GPSS_ECUDA;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return GPSS_ECUDA;
    const int threads = 256, blocks = nsm * 8;
    T *out = nullptr;
    if (cudaMalloc(&out, sizeof(T) * (size_t)threads * blocks) != cudaSuccess) return GPSS_ENOMEM;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = GPSS_OK;
    float ms = 0.f;
    int iters = sizeof(T) == 4 ? 4096 : 128;
    const T a = (T)0.999999, b = (T)1e-7;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) rc = GPSS_ECUDA;
    for (int trial = 0; rc == GPSS_OK && trial < 4; trial++) {
        k_fma_rate<T><<<blocks, threads>>>(out, a, b, iters);  // warm-up
        cudaEventRecord(e0);
        k_fma_rate<T><<<blocks, threads>>>(out, a, b, iters);
        cudaEventRecord(e1);
        if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
            rc = GPSS_ECUDA;
            break;
        }
        if (ms >= 2.0f) break;  // long enough to time
        iters *= 4;
    }
    if (rc == GPSS_OK && cudaGetLastError() != cudaSuccess) rc = GPSS_ECUDA;
    if (rc == GPSS_OK) *tflops = 2.0 * 8.0 * iters * (double)threads * blocks / (ms * 1e-3) / 1e12;
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(out);
    return rc;
}

}  // namespace

extern "C" int gpss_measure_fma_rate(int precision, double *tflops)
{
    if (!tflops || (precision != GPSS_FP32 && precision != GPSS_FP64)) return GPSS_EINVAL;
    return precision == GPSS_FP32 ? rate<float>(tflops) : rate<double>(tflops);
}
