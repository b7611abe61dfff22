// peaks.cu -- measured FMA throughput of this GPU's FP64 and FP32 pipes, the
// denominators of the roofline of kernels bound by arithmetic rather than by
// memory: the FP64 drop-in's pair kernels (GB300 runs FP64 at a small fraction
// of the FP32 rate) and the double-word refinement on the FP32 pipe.
//
// Every thread runs kChains independent multiply-add chains for `iters`
// rounds, so the pipe, not the dependency latency, sets the rate; the chains'
// results are summed into one value per thread and written out so the
// compiler keeps the work.  Timed with CUDA events around one launch after an
// untimed warm-up launch.
#include <cuda_runtime.h>

#include "host_common.h"

namespace {

constexpr int kChains = 8;

template <typename T>
__global__ void __launch_bounds__(256) fma_loop(T *out, int iters, T a, T b) {
    T x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) x[c] = (T)(threadIdx.x + c) * (T)1e-3;
    for (int k = 0; k < iters; k++) {
#pragma unroll
        for (int c = 0; c < kChains; c++) x[c] = x[c] * a + b;
    }
    T s = 0;
#pragma unroll
    for (int c = 0; c < kChains; c++) s += x[c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T>
int measure(int iters, double *tflops, double *ms_out) {
    int dev = 0, sms = 0;
    DPG_CK(cudaGetDevice(&dev));
    DPG_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = sms * 8, threads = 256;
    T *out = nullptr;
    DPG_CK(cudaMalloc((void **)&out, sizeof(T) * (size_t)blocks * threads));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    // a = 1 - 2^-20, b = 2^-21: the chains stay bounded and normal
    const T a = (T)(1.0 - 1.0 / (1 << 20)), b = (T)(1.0 / (1 << 21));
    fma_loop<T><<<blocks, threads>>>(out, iters / 8 + 1, a, b);
    cudaEventRecord(e0);
    fma_loop<T><<<blocks, threads>>>(out, iters, a, b);
    cudaEventRecord(e1);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) return dpg::set_error(DPG_ERR_CUDA, "fma peak: %s", cudaGetErrorString(e));
    const double flops = 2.0 * kChains * (double)iters * blocks * threads;
    *tflops = flops / (ms * 1e-3) / 1e12;
    if (ms_out) *ms_out = ms;
    return DPG_OK;
}

}  // namespace

extern "C" int dpg_measure_fma_peak(int fp64, int iters, double *tflops, double *ms) {
    if (!tflops || iters <= 0) return dpg::set_error(DPG_ERR_ARG, "dpg_measure_fma_peak: bad argument");
    return fp64 ? measure<double>(iters, tflops, ms) : measure<float>(iters, tflops, ms);
}
