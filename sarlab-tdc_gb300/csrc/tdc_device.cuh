// tdc_device.cuh -- device helpers of the GB300 TDC engine: double-float range
// and phase arithmetic, the FP32 Doppler window of the reference, and the
// mbarrier / bulk-copy primitives (inline PTX, sm_90+ forms valid on sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "tdc_internal.h"

namespace tdc {

constexpr float kTwoPiF = 6.28318530717958647692f;
constexpr float kPiF = 3.14159265358979323846f;

// Pixel of slot `slot` (0 .. kFocusTile-1) of tile `t`, or -1 where the slot lies outside
// the grid (see FocusJob::tile_cols).
__device__ __forceinline__ long long tile_pixel(int tile_cols, int grid_cols, long long P, int t, int slot)
{
    if (tile_cols <= 0) {
        const long long p = (long long)t * kFocusTile + slot;
        return p < P ? p : -1;
    }
    const int n_tc = (grid_cols + tile_cols - 1) / tile_cols;
    const int tr = t / n_tc;
    const int col = (t - tr * n_tc) * tile_cols + slot % tile_cols;
    const long long row = (long long)tr * (kFocusTile / tile_cols) + slot / tile_cols;
    const long long p = row * grid_cols + col;
    return col < grid_cols && p < P ? p : -1;
}

// ---------------------------------------------------------------------------
// Error-free transformations (Knuth two-sum, FMA two-product).

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// Double-float difference (ah + al) - (bh + bl) -> (h, l), |l| small relative to h
// unless the difference cancels to (near) zero.
__device__ __forceinline__ void dd_sub(float ah, float al, float bh, float bl, float &h, float &l)
{
    float e;
    two_sum(ah, -bh, h, e);
    l = e + (al - bl);
}

// Range R = |d| with d = (dx, dy, dz) as double-float pairs. Returns (r_hi, r_lo)
// with r_hi + r_lo accurate to ~1e-14 relative, and rs = 1/sqrt(D) (inf at D = 0).
// D = |d|^2 is summed exactly from two-products of the high parts; the square
// root takes one Newton step on the double-float residual D - r_hi^2.
__device__ __forceinline__ void dd_range(float dxh, float dxl, float dyh, float dyl, float dzh, float dzl,
                                         float &r_hi, float &r_lo, float &rs, float &d_hi)
{
    const float ax = dxh * dxh, ex = fmaf(dxh, dxh, -ax);
    const float ay = dyh * dyh, ey = fmaf(dyh, dyh, -ay);
    const float az = dzh * dzh, ez = fmaf(dzh, dzh, -az);
    float s1, e1, s2, e2;
    two_sum(ax, ay, s1, e1);
    two_sum(s1, az, s2, e2);
    float lo = (ex + ey) + (ez + e1) + e2;
    lo = fmaf(2.0f * dxh, dxl, lo);
    lo = fmaf(2.0f * dyh, dyl, lo);
    lo = fmaf(2.0f * dzh, dzl, lo);
    const float dh = s2 + lo;
    const float dl = lo - (dh - s2);
    rs = rsqrtf(dh);
    float r1 = dh * rs;
    const float res = fmaf(-r1, r1, dh) + dl;
    float r2 = res * (0.5f * rs);
    if (!(dh > 0.0f)) {  // antenna exactly on the pixel: R = 0 (the window is NaN -> 0 there)
        r1 = 0.0f;
        r2 = 0.0f;
    }
    r_hi = r1;
    r_lo = r2;
    d_hi = dh;
}

// Fractional cycles of (g_hi + g_lo) * (r_hi + r_lo), in [-0.5, 0.5] up to rounding.
__device__ __forceinline__ float dd_frac_mul(float g_hi, float g_lo, float r_hi, float r_lo)
{
    const float ph = g_hi * r_hi;
    float pl = fmaf(g_hi, r_hi, -ph);
    pl = fmaf(g_hi, r_lo, pl);
    pl = fmaf(g_lo, r_hi, pl);
    const float n = rintf(ph);
    return (ph - n) + pl;
}

// (cos t, sin t) for |t| <= 0.8 by their Taylor series to t^8 / t^9 (error < 3e-8).
__device__ __forceinline__ float2 sincos_small(float t)
{
    const float t2 = t * t;
    const float c = fmaf(-0.5f * t2, fmaf(-t2 * (1.0f / 12.0f), fmaf(-t2, 1.0f / 30.0f, 1.0f), 1.0f), 1.0f);
    const float s = t * fmaf(-t2 * (1.0f / 6.0f), fmaf(-t2 * (1.0f / 20.0f), fmaf(-t2, 1.0f / 42.0f, 1.0f), 1.0f),
                             1.0f);
    return make_float2(c, s);
}

// ---------------------------------------------------------------------------
// FP32 Doppler window, windowing.h:29-58 semantics: inclusive |df| <= B/2,
// NaN -> 0, taper a - (1-a) cos(2 pi df / B - pi) or rectangular.
__device__ __forceinline__ float doppler_window(float fdop, float fdc, float half_bw, float inv_bw, bool taper,
                                               float a)
{
    const float df = fdop - fdc;
    if (!(fabsf(df) <= half_bw)) return 0.0f;
    if (!taper) return 1.0f;
    return a - (1.0f - a) * __cosf(kTwoPiF * df * inv_bw - kPiF);
}

// fDop = 2/lambda * v.(T - P) / |T - P|  (windowing.h:29-37) with d = P - T, rs = 1/|d|.
__device__ __forceinline__ float doppler_freq(float two_over_lambda, float vx, float vy, float vz, float dx,
                                              float dy, float dz, float rs)
{
    const float dotv = -(vx * dx + vy * dy + vz * dz);
    return two_over_lambda * dotv * rs;
}

// Skip test of tdcprocessor.cpp:347-383 for one pixel and one chunk: min over
// the 9 points of |fDop - centre| (std::min_element keeps a NaN first element,
// never picks a later NaN), then <= B/2.
__device__ __forceinline__ bool chunk_is_nonzero(const SkipPoint *__restrict__ pts, float tx, float ty, float tz,
                                                 float two_over_lambda, float half_bw)
{
    float m = 0.0f;
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const float4 pf = __ldg(&pts[i].pos_fdc);
        const float4 v = __ldg(&pts[i].vel);
        const float dx = pf.x - tx, dy = pf.y - ty, dz = pf.z - tz;
        const float rs = rsqrtf(dx * dx + dy * dy + dz * dz);
        const float val = fabsf(doppler_freq(two_over_lambda, v.x, v.y, v.z, dx, dy, dz, rs) - pf.w);
        if (i == 0) {
            m = val;
        } else if (val < m) {
            m = val;
        }
    }
    return m <= half_bw;
}

// ---------------------------------------------------------------------------
// mbarrier + bulk copy (PTX ISA 8.0, sm_90+).

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_barrier_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// Global -> shared bulk copy completing on `bar`. dst, src 16-byte aligned, bytes % 16 == 0.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Wait for phase `parity` of `bar` to complete, giving up after `limit_ns`.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint64_t limit_ns)
{
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (uint32_t it = 0;; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 63u) == 63u && global_ns() - t0 > limit_ns) return false;
    }
}

constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s: far above any healthy copy

}  // namespace tdc
