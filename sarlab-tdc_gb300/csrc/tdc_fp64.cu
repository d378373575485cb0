// tdc_fp64.cu -- plain all-FP64-phase focus kernel of the GB300 TDC engine.
//
// Same decomposition (pixel tile x chirp group units, Kahan per pixel across
// chirps, FP64 reduce of group partials) and the same window and skip-test
// semantics as the FP32-bulk kernel, but the phase of every sample is formed
// in FP64: R in FP64, cycles = R * (2 f_s / c0) in FP64, reduced modulo one in
// FP64, then sin/cos and the complex multiply-accumulate in FP32.
//
// Two roles:
//   * the comparator "plain all-FP64-phase kernel of the same method";
//   * the general path for inputs the FP32-bulk kernel does not take:
//     per-sample antenna trajectories (a ChirpRec per (chirp, sample), as the
//     reference's tdckernels.cu:204-208 reads position[elementIdx]) and
//     non-uniform sample times (the 2 f_s / c0 table is per sample).
// Samples and records are read through the read-only cache; this kernel is
// bound by the FP64 pipe, not by data movement.
#include <cuda_runtime.h>
#include <stdint.h>

#include "tdc_device.cuh"
#include "tdc_internal.h"

namespace tdc {

namespace {

constexpr int kPT = kFocusPT;
constexpr int kThreads = kFocusThreads;

__device__ __forceinline__ double to_d(float h, float l) { return (double)h + (double)l; }

template <bool PER_SAMPLE>
__global__ void __launch_bounds__(kThreads) focus_fp64_kernel(const FocusJob *__restrict__ jobs,
                                                                 const FocusUnit *__restrict__ units)
{
    const FocusUnit un = units[blockIdx.x];
    const FocusJob &J = jobs[un.job];
    const int tid = threadIdx.x;
    const long long P = J.P;
    const int c0 = un.group * J.chirps_per_group;
    const int c1 = min(J.C, c0 + J.chirps_per_group);
    const int S = J.S, s_pad = J.s_pad;
    const bool taper = (J.flags & kFlagTaper) != 0;
    const bool skip_test = (J.flags & kFlagSkipTest) != 0;
    const float tol = J.two_over_lambda, half_bw = J.half_bw, inv_bw = J.inv_bw, az_a = J.az_a;
    const double *__restrict__ gs = J.gs;
    const float4 *__restrict__ xw = J.xw;

    double tx[kPT], ty[kPT], tz[kPT];
    float txh[kPT], tyh[kPT], tzh[kPT];
#pragma unroll
    for (int i = 0; i < kPT; ++i) {
        const long long p = tile_pixel(J.tile_cols, J.grid_cols, P, un.tile, i * kThreads + tid);
        float4 hi = make_float4(0.f, 0.f, 0.f, 0.f), lo = hi;
        if (p >= 0) {
            hi = __ldg(&J.grid_hi[p]);
            if (J.grid_lo) lo = __ldg(&J.grid_lo[p]);
        }
        tx[i] = to_d(hi.x, lo.x);
        ty[i] = to_d(hi.y, lo.y);
        tz[i] = to_d(hi.z, lo.z);
        txh[i] = hi.x;
        tyh[i] = hi.y;
        tzh[i] = hi.z;
    }

    float2 sum[kPT], comp[kPT];
    float wskip[kPT];
#pragma unroll
    for (int i = 0; i < kPT; ++i) {
        sum[i] = make_float2(0.f, 0.f);
        comp[i] = make_float2(0.f, 0.f);
        wskip[i] = 1.0f;
    }
    int cur_chunk = -1;

    for (int c = c0; c < c1; ++c) {
        if (skip_test) {
            const int k = c / J.chunk;
            if (k != cur_chunk) {
                cur_chunk = k;
#pragma unroll
                for (int i = 0; i < kPT; ++i)
                    wskip[i] = chunk_is_nonzero(J.skip + (size_t)k * 9, txh[i], tyh[i], tzh[i], tol, half_bw)
                                   ? 1.0f
                                   : 0.0f;
            }
        }
        float2 acc[kPT];
        double r[kPT];
        float w[kPT];
#pragma unroll
        for (int i = 0; i < kPT; ++i) acc[i] = make_float2(0.f, 0.f);

        bool live = false;
        if (PER_SAMPLE) {
#pragma unroll
            for (int i = 0; i < kPT; ++i) live |= wskip[i] != 0.0f;
        } else {
            const ChirpRec rec = J.chirps[c];
            const double px = to_d(rec.p_hi.x, rec.p_lo.x), py = to_d(rec.p_hi.y, rec.p_lo.y),
                         pz = to_d(rec.p_hi.z, rec.p_lo.z);
#pragma unroll
            for (int i = 0; i < kPT; ++i) {
                const double dx = px - tx[i], dy = py - ty[i], dz = pz - tz[i];
                r[i] = sqrt(dx * dx + dy * dy + dz * dz);
                const float fdx = (float)dx, fdy = (float)dy, fdz = (float)dz;
                const float rs = rsqrtf(fdx * fdx + fdy * fdy + fdz * fdz);
                const float fd = doppler_freq(tol, rec.vel.x, rec.vel.y, rec.vel.z, fdx, fdy, fdz, rs);
                w[i] = wskip[i] * doppler_window(fd, rec.p_hi.w, half_bw, inv_bw, taper, az_a);
                live |= w[i] != 0.0f;
            }
        }
        // a chirp whose weight is zero for every pixel of the warp contributes nothing
        if (!__any_sync(0xffffffffu, live)) continue;

        const float4 *__restrict__ row = xw + (size_t)c * (s_pad / 2);
        for (int s2 = 0; s2 < (S + 1) / 2; ++s2) {
            const float4 xv = __ldg(&row[s2]);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int s = 2 * s2 + h;
                if (s >= S) break;
                const double g = __ldg(&gs[s]);
                const float xr = h ? xv.z : xv.x, xi = h ? xv.w : xv.y;
                if (PER_SAMPLE) {
                    const ChirpRec rec = J.chirps[(size_t)c * S + s];
                    const double px = to_d(rec.p_hi.x, rec.p_lo.x), py = to_d(rec.p_hi.y, rec.p_lo.y),
                                 pz = to_d(rec.p_hi.z, rec.p_lo.z);
#pragma unroll
                    for (int i = 0; i < kPT; ++i) {
                        const double dx = px - tx[i], dy = py - ty[i], dz = pz - tz[i];
                        const double rr = sqrt(dx * dx + dy * dy + dz * dz);
                        const float fdx = (float)dx, fdy = (float)dy, fdz = (float)dz;
                        const float rs = rsqrtf(fdx * fdx + fdy * fdy + fdz * fdz);
                        const float fd = doppler_freq(tol, rec.vel.x, rec.vel.y, rec.vel.z, fdx, fdy, fdz, rs);
                        const float ws = wskip[i] * doppler_window(fd, rec.p_hi.w, half_bw, inv_bw, taper, az_a);
                        const double cyc = rr * g;
                        const float fr = (float)(cyc - rint(cyc));
                        float sn, cs;
                        __sincosf(kTwoPiF * fr, &sn, &cs);
                        const float wr = ws * xr, wi = ws * xi;
                        acc[i].x = fmaf(wr, cs, fmaf(-wi, sn, acc[i].x));
                        acc[i].y = fmaf(wr, sn, fmaf(wi, cs, acc[i].y));
                    }
                } else {
#pragma unroll
                    for (int i = 0; i < kPT; ++i) {
                        const double cyc = r[i] * g;
                        const float fr = (float)(cyc - rint(cyc));
                        float sn, cs;
                        __sincosf(kTwoPiF * fr, &sn, &cs);
                        acc[i].x = fmaf(xr, cs, fmaf(-xi, sn, acc[i].x));
                        acc[i].y = fmaf(xr, sn, fmaf(xi, cs, acc[i].y));
                    }
                }
            }
        }

#pragma unroll
        for (int i = 0; i < kPT; ++i) {
            const float2 v = PER_SAMPLE ? acc[i] : make_float2(w[i] * acc[i].x, w[i] * acc[i].y);
            const float yr = v.x - comp[i].x, yi = v.y - comp[i].y;
            const float tr = sum[i].x + yr, ti = sum[i].y + yi;
            comp[i].x = (tr - sum[i].x) - yr;
            comp[i].y = (ti - sum[i].y) - yi;
            sum[i].x = tr;
            sum[i].y = ti;
        }
    }

    float4 *__restrict__ part = J.partial + (size_t)un.group * P;
#pragma unroll
    for (int i = 0; i < kPT; ++i) {
        const long long pidx = tile_pixel(J.tile_cols, J.grid_cols, P, un.tile, i * kThreads + tid);
        if (pidx >= 0) part[pidx] = make_float4(sum[i].x, sum[i].y, comp[i].x, comp[i].y);
    }
}

}  // namespace

cudaError_t launch_focus_fp64(const FocusJob *jobs_dev, const FocusUnit *units_dev, int n_units, int *status_dev,
                              int per_sample, cudaStream_t st)
{
    (void)status_dev;
    if (n_units <= 0) return cudaSuccess;
    if (per_sample) {
        focus_fp64_kernel<true><<<n_units, kThreads, 0, st>>>(jobs_dev, units_dev);
    } else {
        focus_fp64_kernel<false><<<n_units, kThreads, 0, st>>>(jobs_dev, units_dev);
    }
    return cudaGetLastError();
}

}  // namespace tdc
