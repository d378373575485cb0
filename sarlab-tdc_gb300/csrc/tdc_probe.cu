// tdc_probe.cu -- throughput probes used as roofline denominators by the
// benchmark: the FP32 FFMA rate of the SIMT pipe (the bound of the focus
// kernels) and the FP64 DFMA rate (why range and phase use double-float).
// No reference counterpart.
#include <cuda_runtime.h>

#include "tdc_gb300.h"

namespace {

constexpr int kChains = 16;  // independent FMA chains per thread (hides the 4-cycle latency)

template <typename T>
__global__ void __launch_bounds__(256) fma_probe_kernel(int iters, T seed, T *__restrict__ out)
{
    T a[kChains];
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = seed + (T)(threadIdx.x + k);
    const T m = (T)0.999999, c = (T)1e-7;
#pragma unroll 1
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int r = 0; r < 8; ++r) {
#pragma unroll
            for (int k = 0; k < kChains; ++k) a[k] = a[k] * m + c;
        }
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < kChains; ++k) s += a[k];
    if (s == (T)-1) out[blockIdx.x] = s;  // never true; keeps the chains live
}

}  // namespace

extern "C" {

// Launch `blocks` x 256 threads of `iters` x 128 FMAs (FP32 when fp64 == 0, else FP64).
// Returns the FLOP count (2 per FMA) through *flops. Time it with events on `stream`.
int tdc_probe_fma(int fp64, int blocks, int iters, void *scratch_dev, double *flops, void *stream)
{
    if (blocks <= 0 || iters <= 0 || !scratch_dev) return TDC_ERR_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (fp64) {
        fma_probe_kernel<double><<<blocks, 256, 0, st>>>(iters, 1.0, static_cast<double *>(scratch_dev));
    } else {
        fma_probe_kernel<float><<<blocks, 256, 0, st>>>(iters, 1.0f, static_cast<float *>(scratch_dev));
    }
    if (flops) *flops = 2.0 * 8.0 * kChains * (double)iters * (double)blocks * 256.0;
    return cudaGetLastError() == cudaSuccess ? TDC_OK : TDC_ERR_CUDA;
}

}  // extern "C"
