// tdc_prep.cu -- per-acquisition preparation kernels of the GB300 TDC engine:
// the range window (tdc-lib/src/tdckernels.cu:32-64), its application to the
// raw chirps once per start() instead of once per pixel, focus-grid layout
// conversion and per-chirp position offsets (autofocus).
#include <cuda_runtime.h>
#include <stdint.h>

#include "tdc_device.cuh"
#include "tdc_internal.h"

namespace tdc {

namespace {

// w[n] = a - (1 - a) cos(2 pi n / N) (periodic), a = 25/46, or all ones.
__global__ void range_window_kernel(float *__restrict__ w, int n, int apply)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    w[i] = apply ? kRangeA - (1.0f - kRangeA) * cospif(2.0f * (float)i / (float)n) : 1.0f;
}

// In place on rows of s_pad complex samples (first S valid): x *= w[s]; padding -> 0.
__global__ void prewindow_kernel(float2 *__restrict__ xw, const float *__restrict__ w, int C, int S, int s_pad)
{
    const long long total = (long long)C * s_pad;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int s = (int)(idx % s_pad);
        float2 v = make_float2(0.f, 0.f);
        if (s < S) {
            const float ws = w[s];
            const float2 x = xw[idx];
            v = make_float2(x.x * ws, x.y * ws);
        }
        xw[idx] = v;
    }
}

// Range-windowed, zero-padded rows from a source the device can read directly
// (device memory, or pageable host memory on a system with coherent host access).
__global__ void prewindow_from_kernel(const float2 *__restrict__ src, const float *__restrict__ w, int C, int S,
                                      int s_pad, float2 *__restrict__ xw)
{
    const long long total = (long long)C * s_pad;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long c = idx / s_pad;
        const int s = (int)(idx - c * s_pad);
        float2 v = make_float2(0.f, 0.f);
        if (s < S) {
            const float2 x = src[c * S + s];
            const float ws = w[s];
            v = make_float2(x.x * ws, x.y * ws);
        }
        xw[idx] = v;
    }
}

// flag |= 1 when any sample of a chirp differs (bitwise) from the chirp's first sample;
// a is [C][S][k] floats.
__global__ void rows_differ_kernel(const unsigned int *__restrict__ a, int C, int S, int k, int *__restrict__ flag)
{
    const long long per = (long long)S * k;
    const long long total = (long long)C * per;
    bool differ = false;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long c = idx / per;
        const long long r = idx - c * per;
        differ |= a[idx] != a[c * per + (r % k)];
    }
    if (__syncthreads_or(differ) && threadIdx.x == 0) atomicOr(flag, 1);
}

// The same test reading 16 bytes per load (a 16-byte aligned, C x S x k < 2^31 elements):
// the arrays usually sit in the caller's host memory, where wide loads move them faster.
__global__ void rows_differ_vec_kernel(const uint4 *__restrict__ a4, unsigned int total, unsigned int per,
                                       unsigned int k, int *__restrict__ flag)
{
    const unsigned int *a = reinterpret_cast<const unsigned int *>(a4);
    const unsigned int n4 = total / 4;
    bool differ = false;
    for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += gridDim.x * blockDim.x) {
        const uint4 v = a4[i];
        const unsigned int w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const unsigned int e = 4 * i + q;
            const unsigned int c = e / per;
            const unsigned int r = e - c * per;
            differ |= w[q] != a[c * per + r % k];
        }
    }
    for (unsigned int e = 4 * n4 + blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        const unsigned int c = e / per;
        const unsigned int r = e - c * per;
        differ |= a[e] != a[c * per + r % k];
    }
    if (__syncthreads_or(differ) && threadIdx.x == 0) atomicOr(flag, 1);
}

// out[c][s] = s * rows[c][s]: rows pre-scaled by the sample index (the adjoint's B = sum_s s x_s z^s).
__global__ void scale_rows_kernel(const float2 *__restrict__ rows, long long total, int s_pad, float2 *__restrict__ out)
{
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const float s = (float)(idx % s_pad);
        const float2 x = rows[idx];
        out[idx] = make_float2(s * x.x, s * x.y);
    }
}

// Bounding box of the grid's high floats: out = (min x, min y, min z, max x, max y, max z),
// each as an order-preserving int (see float_key); out must start at (INT_MAX x3, INT_MIN x3).
__device__ __forceinline__ int float_key(float f)
{
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}

__global__ void grid_bbox_kernel(const float4 *__restrict__ hi, long long P, int *__restrict__ out)
{
    int mn[3] = {0x7fffffff, 0x7fffffff, 0x7fffffff}, mx[3] = {(int)0x80000000, (int)0x80000000, (int)0x80000000};
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < P; p += (long long)gridDim.x * blockDim.x) {
        const float4 v = hi[p];
        const int k[3] = {float_key(v.x), float_key(v.y), float_key(v.z)};
        for (int d = 0; d < 3; ++d) {
            mn[d] = min(mn[d], k[d]);
            mx[d] = max(mx[d], k[d]);
        }
    }
    for (int d = 0; d < 3; ++d) {
        for (int off = 16; off > 0; off >>= 1) {
            mn[d] = min(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], off));
            mx[d] = max(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], off));
        }
        if ((threadIdx.x & 31) == 0) {
            atomicMin(&out[d], mn[d]);
            atomicMax(&out[3 + d], mx[d]);
        }
    }
}

__global__ void grid_f32_kernel(const float *__restrict__ g, long long P, float4 *__restrict__ hi)
{
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    hi[p] = make_float4(g[3 * p], g[3 * p + 1], g[3 * p + 2], 0.f);
}

__device__ __forceinline__ void split_dd(double v, float &h, float &l)
{
    h = (float)v;
    l = (float)(v - (double)h);
}

__global__ void grid_f64_kernel(const double *__restrict__ g, long long P, float4 *__restrict__ hi,
                                float4 *__restrict__ lo)
{
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    float h[3], l[3];
    for (int k = 0; k < 3; ++k) split_dd(g[3 * p + k], h[k], l[k]);
    hi[p] = make_float4(h[0], h[1], h[2], 0.f);
    lo[p] = make_float4(l[0], l[1], l[2], 0.f);
}

// recs[c].p = base[c] + off[c] as double-float pairs (off may be null).
__global__ void chirp_positions_kernel(ChirpRec *__restrict__ recs, const double *__restrict__ base,
                                       const double *__restrict__ off, int C)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    float h[3], l[3];
    for (int k = 0; k < 3; ++k) {
        const double v = base[3 * c + k] + (off ? off[3 * c + k] : 0.0);
        split_dd(v, h[k], l[k]);
    }
    ChirpRec r = recs[c];
    r.p_hi = make_float4(h[0], h[1], h[2], r.p_hi.w);
    r.p_lo = make_float4(l[0], l[1], l[2], 0.f);
    recs[c] = r;
}

}  // namespace

cudaError_t launch_range_window(float *w, int n, int apply, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    range_window_kernel<<<(n + 127) / 128, 128, 0, st>>>(w, n, apply);
    return cudaGetLastError();
}

cudaError_t launch_prewindow(float2 *xw, const float *w, int C, int S, int s_pad, cudaStream_t st)
{
    const long long total = (long long)C * s_pad;
    if (total <= 0) return cudaSuccess;
    long long blocks = (total + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    prewindow_kernel<<<(unsigned)blocks, 256, 0, st>>>(xw, w, C, S, s_pad);
    return cudaGetLastError();
}

cudaError_t launch_prewindow_from(const float2 *src, const float *w, int C, int S, int s_pad, float2 *xw,
                                  cudaStream_t st)
{
    const long long total = (long long)C * s_pad;
    if (total <= 0) return cudaSuccess;
    long long blocks = (total + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    prewindow_from_kernel<<<(unsigned)blocks, 256, 0, st>>>(src, w, C, S, s_pad, xw);
    return cudaGetLastError();
}

cudaError_t launch_rows_differ(const float *a, int C, int S, int k, int *flag, cudaStream_t st)
{
    const long long total = (long long)C * S * k;
    if (total <= 0) return cudaSuccess;
    if ((reinterpret_cast<uintptr_t>(a) & 15u) == 0 && total < (1LL << 31)) {
        long long blocks = (total / 4 + 255) / 256;
        if (blocks > 152 * 16) blocks = 152 * 16;
        if (blocks < 1) blocks = 1;
        rows_differ_vec_kernel<<<(unsigned)blocks, 256, 0, st>>>(reinterpret_cast<const uint4 *>(a),
                                                                (unsigned)total, (unsigned)((long long)S * k),
                                                                (unsigned)k, flag);
        return cudaGetLastError();
    }
    long long blocks = (total + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    rows_differ_kernel<<<(unsigned)blocks, 256, 0, st>>>(reinterpret_cast<const unsigned int *>(a), C, S, k, flag);
    return cudaGetLastError();
}

cudaError_t launch_scale_rows(const float2 *rows, int C, int s_pad, float2 *rows_out, cudaStream_t st)
{
    const long long total = (long long)C * s_pad;
    if (total <= 0) return cudaSuccess;
    long long blocks = (total + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    scale_rows_kernel<<<(unsigned)blocks, 256, 0, st>>>(rows, total, s_pad, rows_out);
    return cudaGetLastError();
}

cudaError_t launch_grid_bbox(const float4 *hi, long long P, int *out, cudaStream_t st)
{
    if (P <= 0) return cudaSuccess;
    long long blocks = (P + 255) / 256;
    if (blocks > 152 * 8) blocks = 152 * 8;
    grid_bbox_kernel<<<(unsigned)blocks, 256, 0, st>>>(hi, P, out);
    return cudaGetLastError();
}

cudaError_t launch_grid_from_f32(const float *grid, long long P, float4 *hi, cudaStream_t st)
{
    if (P <= 0) return cudaSuccess;
    grid_f32_kernel<<<(unsigned)((P + 255) / 256), 256, 0, st>>>(grid, P, hi);
    return cudaGetLastError();
}

cudaError_t launch_grid_from_f64(const double *grid, long long P, float4 *hi, float4 *lo, cudaStream_t st)
{
    if (P <= 0) return cudaSuccess;
    grid_f64_kernel<<<(unsigned)((P + 255) / 256), 256, 0, st>>>(grid, P, hi, lo);
    return cudaGetLastError();
}

cudaError_t launch_chirp_positions(ChirpRec *recs, const double *base, const double *off, int C, cudaStream_t st)
{
    if (C <= 0) return cudaSuccess;
    chirp_positions_kernel<<<(C + 127) / 128, 128, 0, st>>>(recs, base, off, C);
    return cudaGetLastError();
}

}  // namespace tdc
