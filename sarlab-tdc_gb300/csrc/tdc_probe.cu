// tdc_probe.cu -- throughput probes used as roofline denominators by the
// benchmark: the FP32 FFMA rate of the SIMT pipe (the bound of the focus
// kernels) and the FP64 DFMA rate (why range and phase use double-float);
// and the self-test of the kernels' bounded waits. No reference counterpart.
#include <cuda_runtime.h>

#include <string>

#include "tdc_device.cuh"
#include "tdc_gb300.h"
#include "tdc_internal.h"

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

// One CTA waits, with the focus kernels' bounded wait, on an mbarrier phase that nothing
// completes (no thread arrives, no copy is issued), then reports the timeout in the status
// word the way the focus kernels do and returns.
__global__ void wait_timeout_probe_kernel(uint64_t limit_ns, int *__restrict__ status)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        tdc::mbar_init(&bar, 1);
        tdc::fence_barrier_init();
    }
    __syncthreads();
    const bool ok = tdc::mbar_wait_bounded(&bar, 0u, limit_ns);
    if (__syncthreads_or(!ok) && threadIdx.x == 0) atomicOr(status, tdc::kStatusTimeout);
}

}  // namespace

extern "C" {

int tdc_selftest_wait_timeout(int device, int limit_us, int *timed_out, double *elapsed_ms)
{
    if (limit_us <= 0 || limit_us > 2000000 || !timed_out)
        return tdc::set_last_error(TDC_ERR_INVALID_ARGUMENT, "limit_us must be in (0, 2e6] and timed_out non-null");
    *timed_out = 0;
    if (cudaSetDevice(device) != cudaSuccess) return tdc::set_last_error(TDC_ERR_CUDA, "cudaSetDevice failed");
    int *status = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaMalloc(&status, sizeof(int));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) e = cudaMemsetAsync(status, 0, sizeof(int), st);
    if (e == cudaSuccess) e = cudaEventRecord(e0, st);
    if (e == cudaSuccess) {
        wait_timeout_probe_kernel<<<1, 32, 0, st>>>((uint64_t)limit_us * 1000u, status);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1, st);
    int h = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, status, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    float ms = 0.f;
    if (e == cudaSuccess && elapsed_ms) {
        e = cudaEventElapsedTime(&ms, e0, e1);
        *elapsed_ms = ms;
    }
    if (e1) cudaEventDestroy(e1);
    if (e0) cudaEventDestroy(e0);
    if (st) cudaStreamDestroy(st);
    if (status) cudaFree(status);
    if (e != cudaSuccess) return tdc::set_last_error(TDC_ERR_CUDA, std::string("self-test: ") + cudaGetErrorString(e));
    *timed_out = (h & tdc::kStatusTimeout) ? 1 : 0;
    return TDC_OK;
}

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
