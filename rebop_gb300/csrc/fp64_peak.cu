// FP64 pipe throughput probe: the roofline denominator of the SSA kernels.
//
// The direct method's per-event work is a chain of binary64 multiplies, adds,
// compares and one divide; no HBM or tensor-core roofline bounds it.  This
// kernel measures how many binary64 FMA instructions per second the GPU
// retires: every thread runs 8 independent DFMA chains so the pipe, not
// latency, is the limit.  Timed with CUDA events on the caller's stream.
#include <cuda_runtime.h>

#include <cstdint>

namespace rbg {

__global__ void __launch_bounds__(256) fp64_fma_probe(double *sink, int iters, double a, double b) {
    double x0 = threadIdx.x * 1e-9, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
    double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            x0 = __fma_rn(x0, a, b);
            x1 = __fma_rn(x1, a, b);
            x2 = __fma_rn(x2, a, b);
            x3 = __fma_rn(x3, a, b);
            x4 = __fma_rn(x4, a, b);
            x5 = __fma_rn(x5, a, b);
            x6 = __fma_rn(x6, a, b);
            x7 = __fma_rn(x7, a, b);
        }
    }
    double s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == 12345.678) sink[0] = s;  // keeps the chains live
}

}  // namespace rbg

// Returns DFMA instructions retired per second (0 on failure).
extern "C" double rbg_internal_fp64_fma_rate(void *stream) {
    using namespace rbg;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0.0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    double *sink = nullptr;
    if (cudaMalloc(&sink, sizeof(double)) != cudaSuccess) return 0.0;
    const int block = 256, grid = sms * 8, iters = 2048;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fp64_fma_probe<<<grid, block, 0, st>>>(sink, 64, 0.999999, 1e-7);  // warm-up
    cudaEventRecord(e0, st);
    fp64_fma_probe<<<grid, block, 0, st>>>(sink, iters, 0.999999, 1e-7);
    cudaEventRecord(e1, st);
    float ms = 0.f;
    double rate = 0.0;
    if (cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess && ms > 0)
        rate = (double)grid * block * iters * 32.0 / (ms * 1e-3);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    return rate;
}
