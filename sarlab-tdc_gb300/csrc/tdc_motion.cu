// tdc_motion.cu -- FP32 focus kernel for per-sample antenna positions that move
// smoothly within each chirp.
//
// The reference reads position[c][s] per element (tdc-lib/src/tdckernels.cu:204-208),
// so an antenna that keeps moving during a chirp changes the range, and the phase,
// of every sample. When every chirp's positions follow a polynomial in the sample
// index to within the rounding of their FP32 values -- an antenna moving with some
// velocity and acceleration during the chirp -- the host fits, per chirp,
//     P[c, s] = P0_c + V1_c s + V2_c s^2        (P0 as a double-float pair)
// and this kernel forms the phase (cycles) of sample s at pixel T as
//     g_s R_s = (g0 + g1 s) R0 + psi(s),   psi(s) = g_s (R_s - R0),
// with R0 = |P0 - T| in double-float as in the FP32-bulk kernel and
//     R_s - R0 = (N / 2R0) f(N / R0^2),  N = 2 (P0 - T).D_s + |D_s|^2,  D_s = V1 s + V2 s^2,
//     f(e) = 2 / (1 + sqrt(1 + e)) = 1 - e/4 + e^2/8 - ...   (host bound |e| <= 0.02).
// psi is smooth in s. Over segments of M samples (a power of two the host chooses
// from a bound on psi's curvature) it is replaced by its chord plus the mean of the
// chord's deviation, -c2 (M^2 - 1) / 6 for curvature c2 = psi''/2, so a segment's
// phase is linear in s and its sum goes through the bulk kernel's blocked Horner
// recurrence with a phasor table for the segment's own per-sample step
// beta + sigma_m (sigma_m the chord's slope). Segments chain in one Horner state,
// last first: the chord of segment m ends where segment m+1's begins, so entering
// segment m the carried sum needs only the factor e^{j 2 pi (off_{m+1} - off_m)}
// (the beta M and chord terms cancel against QL_m^{M/L}).
//
// Cost per correlation: the 4-FFMA complex multiply-accumulate; per (pixel,
// segment): one evaluation of psi, one sincos and the 8-entry table (~55
// instructions, ~0.9 per correlation at M = 64). Staging, work units, skip test,
// Kahan accumulation and the FP64 group reduction are the bulk kernel's.
#include <cuda_runtime.h>
#include <stdint.h>

#include "tdc_device.cuh"
#include "tdc_internal.h"

namespace tdc {

namespace {

#ifndef TDC_MOTION_MINB
#define TDC_MOTION_MINB 3
#endif

constexpr int kL = 8;  // in-block phasor table length (the bulk kernel's)

struct MotionShared {
    float t[kFocusPT * 6][kFocusThreads];  // (x_hi, y_hi, z_hi, x_lo, y_lo, z_lo) per pixel slot
};

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

// One Horner block for one pixel: H <- H * ql + sum_{k<L} x_k p_k (p_0 = 1).
__device__ __forceinline__ float2 horner_block(float2 h, float2 ql, const float2 (&p)[kL - 1],
                                               const float4 (&xv)[kL / 2])
{
    float tr = fmaf(h.x, ql.x, xv[0].x);
    tr = fmaf(-h.y, ql.y, tr);
    float ti = fmaf(h.x, ql.y, xv[0].y);
    ti = fmaf(h.y, ql.x, ti);
#pragma unroll
    for (int k = 1; k < kL; ++k) {
        const float xr = (k & 1) ? xv[k >> 1].z : xv[k >> 1].x;
        const float xi = (k & 1) ? xv[k >> 1].w : xv[k >> 1].y;
        tr = fmaf(xr, p[k - 1].x, tr);
        tr = fmaf(-xi, p[k - 1].y, tr);
        ti = fmaf(xr, p[k - 1].y, ti);
        ti = fmaf(xi, p[k - 1].x, ti);
    }
    return make_float2(tr, ti);
}

// Per-(pixel, chirp) coefficients of psi: N(s) = s (n1 + s (n2 + s (k3 + s k4))), the
// range change d = (N ia) f(N ib), ia = 1/(2 R0), ib = 1/R0^2, and g_s = g0 + g1 s.
struct PsiCoef {
    float n1, n2, ia, ib;
};

__device__ __forceinline__ float motion_psi(float s, const PsiCoef &q, float k3, float k4, float g0, float g1)
{
    const float n = s * fmaf(s, fmaf(s, fmaf(s, k4, k3), q.n2), q.n1);
    const float e = n * q.ib;
    const float f = fmaf(fmaf(e, 0.125f, -0.25f), e, 1.0f);
    return fmaf(g1, s, g0) * ((n * q.ia) * f);
}

template <bool SKIP_ZERO>
__global__ void __launch_bounds__(kFocusThreads, TDC_MOTION_MINB)
    focus_motion_kernel(const FocusJob *__restrict__ jobs, const FocusUnit *__restrict__ units, int n_units,
                        int *__restrict__ counter, int *__restrict__ status, int stage_bytes)
{
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t full_bar[kFocusStages];
    __shared__ int s_unit;
    __shared__ FocusJob sJ;

    MotionShared &sp = *reinterpret_cast<MotionShared *>(smem + kFocusStages * stage_bytes);
    const int tid = threadIdx.x;

    if (tid == 0) {
        for (int i = 0; i < kFocusStages; ++i) mbar_init(&full_bar[i], 1);
        fence_barrier_init();
    }
    __syncthreads();

    uint32_t n_issued = 0;    // producer (thread 0) only
    uint32_t n_consumed = 0;  // uniform across the CTA

    for (;;) {
        if (tid == 0) s_unit = atomicAdd(counter, 1);
        __syncthreads();
        const int u = s_unit;
        if (u >= n_units) break;
        const FocusUnit un = units[u];
        if (tid < (int)(sizeof(FocusJob) / sizeof(int)))
            reinterpret_cast<int *>(&sJ)[tid] = reinterpret_cast<const int *>(&jobs[un.job])[tid];
        __syncthreads();

        const int C = sJ.C;
        const int c0 = un.group * sJ.chirps_per_group;
        const int c1 = min(C, c0 + sJ.chirps_per_group);
        const int CB = sJ.stage_chirps;
        const int nblk = (c1 - c0 + CB - 1) / CB;
        const int s_pad = sJ.s_pad;
        const uint32_t row_bytes = static_cast<uint32_t>(s_pad) * 8u;
        const float4 *__restrict__ xw = sJ.xw;
        const MotionRec *__restrict__ mrecs = reinterpret_cast<const MotionRec *>(sJ.chirps);

        auto issue = [&](int j) {
            const int cb0 = c0 + j * CB;
            const int cnt = min(CB, c1 - cb0);
            const int st = n_issued % kFocusStages;
            unsigned char *base = smem + st * stage_bytes;
            const uint32_t bx = cnt * row_bytes, br = cnt * (uint32_t)sizeof(MotionRec);
            mbar_arrive_expect_tx(&full_bar[st], bx + br);
            bulk_g2s(base, xw + (size_t)cb0 * (s_pad / 2), bx, &full_bar[st]);
            bulk_g2s(base + CB * row_bytes, mrecs + cb0, br, &full_bar[st]);
            ++n_issued;
        };
        if (tid == 0) {
            fence_proxy_async_smem();
            const int npro = nblk < kFocusStages ? nblk : kFocusStages;
            for (int j = 0; j < npro; ++j) issue(j);
        }

        const long long P = sJ.P;
#pragma unroll
        for (int i = 0; i < kFocusPT; ++i) {
            const long long p = tile_pixel(sJ.tile_cols, sJ.grid_cols, P, un.tile, i * kFocusThreads + tid);
            float4 hi = make_float4(0.f, 0.f, 0.f, 0.f), lo = hi;
            if (p >= 0) {
                hi = __ldg(&sJ.grid_hi[p]);
                if (sJ.grid_lo) lo = __ldg(&sJ.grid_lo[p]);
            }
            sp.t[i * 6 + 0][tid] = hi.x;
            sp.t[i * 6 + 1][tid] = hi.y;
            sp.t[i * 6 + 2][tid] = hi.z;
            sp.t[i * 6 + 3][tid] = lo.x;
            sp.t[i * 6 + 4][tid] = lo.y;
            sp.t[i * 6 + 5][tid] = lo.z;
        }

        const float g0h = sJ.g0_hi, g0l = sJ.g0_lo, g1 = sJ.g1, g1l = sJ.g1_lo;
        const float g0f = g0h + g0l;
        const float tol = sJ.two_over_lambda, half_bw = sJ.half_bw, inv_bw = sJ.inv_bw, az_a = sJ.az_a;
        const bool taper = (sJ.flags & kFlagTaper) != 0;
        const bool skip_test = (sJ.flags & kFlagSkipTest) != 0;
        const bool exact_ql = (sJ.flags & kFlagMotionExactQL) != 0;
        const int chunk = sJ.chunk;
        const SkipPoint *__restrict__ skip = sJ.skip;
        // segments: M samples (a power of two >= kL), the last one s_pad - (nseg - 1) M
        const int M = sJ.seg_len;
        const int nseg = (s_pad + M - 1) / M;
        const int len_last = s_pad - (nseg - 1) * M;
        const float inv_m = 1.0f / (float)M, inv_last = 1.0f / (float)len_last;
        const float mean_m = ((float)M * (float)M - 1.0f) * (1.0f / 6.0f);
        const float mean_last = ((float)len_last * (float)len_last - 1.0f) * (1.0f / 6.0f);

        float2 sum[kFocusPT], comp[kFocusPT];
        float wskip[kFocusPT];
#pragma unroll
        for (int i = 0; i < kFocusPT; ++i) {
            sum[i] = make_float2(0.f, 0.f);
            comp[i] = make_float2(0.f, 0.f);
            wskip[i] = 1.0f;
        }
        int cur_chunk = -1;
        bool timed_out = false;

        for (int j = 0; j < nblk; ++j) {
            const int st = n_consumed % kFocusStages;
            const uint32_t parity = (n_consumed / kFocusStages) & 1u;
            const bool ok = mbar_wait_bounded(&full_bar[st], parity, kWaitLimitNs);
            if (__syncthreads_or(!ok)) {
                timed_out = true;
                break;
            }
            const unsigned char *base = smem + st * stage_bytes;
            const float4 *xs_stage = reinterpret_cast<const float4 *>(base);
            const MotionRec *recs = reinterpret_cast<const MotionRec *>(base + CB * row_bytes);
            const int cb0 = c0 + j * CB;
            const int cnt = min(CB, c1 - cb0);

            for (int cc = 0; cc < cnt; ++cc) {
                const int c = cb0 + cc;
                if (skip_test) {
                    const int k = c / chunk;
                    if (k != cur_chunk) {
                        cur_chunk = k;
#pragma unroll
                        for (int i = 0; i < kFocusPT; ++i) {
                            wskip[i] = chunk_is_nonzero(skip + (size_t)k * 9, sp.t[i * 6 + 0][tid],
                                                        sp.t[i * 6 + 1][tid], sp.t[i * 6 + 2][tid], tol,
                                                        half_bw)
                                           ? 1.0f
                                           : 0.0f;
                        }
                    }
                }
                const float4 *xs = xs_stage + (size_t)cc * (s_pad / 2);
                const float4 ph = recs[cc].p_hi, pl = recs[cc].p_lo;

                // ---- per (pixel, chirp): range, window, beta, psi's coefficients ----
                float rh[kFocusPT], rl[kFocusPT], w[kFocusPT], rs[kFocusPT];
                bool live = false;
#pragma unroll
                for (int i = 0; i < kFocusPT; ++i) {
                    float dxh, dxl, dyh, dyl, dzh, dzl;
                    dd_sub(ph.x, pl.x, sp.t[i * 6 + 0][tid], sp.t[i * 6 + 3][tid], dxh, dxl);
                    dd_sub(ph.y, pl.y, sp.t[i * 6 + 1][tid], sp.t[i * 6 + 4][tid], dyh, dyl);
                    dd_sub(ph.z, pl.z, sp.t[i * 6 + 2][tid], sp.t[i * 6 + 5][tid], dzh, dzl);
                    float dh;
                    dd_range(dxh, dxl, dyh, dyl, dzh, dzl, rh[i], rl[i], rs[i], dh);
                    const float4 v = recs[cc].vel;
                    const float fd = doppler_freq(tol, v.x, v.y, v.z, dxh, dyh, dzh, rs[i]);
                    w[i] = wskip[i] * doppler_window(fd, ph.w, half_bw, inv_bw, taper, az_a);
                    live |= w[i] != 0.0f;
                }
                // a chirp whose window (Doppler band, skip test) is zero for every pixel of the
                // warp contributes nothing
                if (SKIP_ZERO && !__any_sync(0xffffffffu, live)) continue;

                const float4 v1 = recs[cc].v1, v2 = recs[cc].v2;
                const float k3 = recs[cc].vel.w, k4 = v2.w;
                float bh[kFocusPT], bl[kFocusPT], dq[kFocusPT];
                float2 q0[kFocusPT], qlb[kFocusPT], h[kFocusPT];
                PsiCoef pc[kFocusPT];
                float psi_e[kFocusPT];
#pragma unroll
                for (int i = 0; i < kFocusPT; ++i) {
                    // beta = (g1 + g1l) (rh + rl) cycles per sample, reduced modulo 1
                    float b0 = g1 * rh[i];
                    float b1 = fmaf(g1, rh[i], -b0);
                    b1 = fmaf(g1, rl[i], b1);
                    b1 = fmaf(g1l, rh[i], b1);
                    b0 -= rintf(b0);
                    bh[i] = b0;
                    bl[i] = b1;
                    const float lbh = (float)kL * b0;  // exact
                    const float lfr = (lbh - rintf(lbh)) + (float)kL * b1;
                    float sl, cl;
                    sincospif(2.0f * lfr, &sl, &cl);
                    qlb[i] = make_float2(cl, sl);
                    // psi's coefficients: (P0 - T).V1, (P0 - T).V2 from the high parts
                    const float dx = ph.x - sp.t[i * 6 + 0][tid], dy = ph.y - sp.t[i * 6 + 1][tid],
                                dz = ph.z - sp.t[i * 6 + 2][tid];
                    const float a1 = fmaf(dx, v1.x, fmaf(dy, v1.y, dz * v1.z));
                    const float a2 = fmaf(dx, v2.x, fmaf(dy, v2.y, dz * v2.z));
                    pc[i].n1 = 2.0f * a1;
                    pc[i].n2 = fmaf(2.0f, a2, v1.w);
                    pc[i].ia = 0.5f * rs[i];
                    pc[i].ib = rs[i] * rs[i];
                    // curvature c2 = psi''/2 = g0 d2 + g1 d1 with d1 = n1 / 2R0,
                    // d2 = n2 / 2R0 - n1^2 / 8R0^3; mean chord deviation -c2 (len^2 - 1) / 6
                    const float d1 = pc[i].n1 * pc[i].ia;
                    const float d2 = fmaf(-0.25f * pc[i].n1 * pc[i].n1, pc[i].ia * pc[i].ib, pc[i].n2 * pc[i].ia);
                    const float c2 = fmaf(g0f, d2, g1 * d1);
                    const float off0 = -c2 * (nseg > 1 ? mean_m : mean_last);
                    dq[i] = kTwoPiF * c2 * (mean_m - mean_last);  // 2 pi (off_last - off_full)
                    const float alpha = dd_frac_mul(g0h, g0l, rh[i], rl[i]);
                    float sa, ca;
                    __sincosf(kTwoPiF * (alpha + off0), &sa, &ca);
                    q0[i] = make_float2(w[i] * ca, w[i] * sa);
                    h[i] = make_float2(0.f, 0.f);
                    psi_e[i] = motion_psi((float)s_pad, pc[i], k3, k4, g0f, g1);
                }

                // ---- segments, last first ----
                for (int m = nseg - 1; m >= 0; --m) {
                    const int s0 = m * M;
                    const bool last = m == nseg - 1;
                    const float inv_len = last ? inv_last : inv_m;
                    float2 p[kFocusPT][kL - 1], ql[kFocusPT];
#pragma unroll
                    for (int i = 0; i < kFocusPT; ++i) {
                        const float psi0 = motion_psi((float)s0, pc[i], k3, k4, g0f, g1);
                        const float sg = (psi_e[i] - psi0) * inv_len;  // chord slope [cycles / sample]
                        psi_e[i] = psi0;
                        float s1, c1s;
                        __sincosf(kTwoPiF * (bh[i] + (bl[i] + sg)), &s1, &c1s);
                        p[i][0] = make_float2(c1s, s1);
#pragma unroll
                        for (int k = 1; k < kL - 1; ++k) p[i][k] = cmul(p[i][k - 1], p[i][0]);
                        if (exact_ql) {
                            // L (beta + sigma) = frac(L bh) + L (bl + sigma) cycles: exact terms
                            const float lbh = (float)kL * bh[i];
                            const float lfr = (lbh - rintf(lbh)) + (float)kL * (bl[i] + sg);
                            float sl, cl;
                            sincospif(2.0f * lfr, &sl, &cl);
                            ql[i] = make_float2(cl, sl);
                        } else {
                            ql[i] = cmul(qlb[i], sincos_small(kTwoPiF * (float)kL * sg));
                        }
                        if (m == nseg - 2) {
                            // entering the first full segment after the (shorter) last one
                            const float2 r = make_float2(fmaf(-0.5f * dq[i], dq[i], 1.0f), dq[i]);
                            h[i] = cmul(h[i], r);
                        }
                    }
                    const float4 *xseg = xs + s0 / 2;
                    const int nb = (last ? len_last : M) / kL;
#pragma unroll 8
                    for (int b = nb - 1; b >= 0; --b) {
                        float4 xv[kL / 2];
#pragma unroll
                        for (int q = 0; q < kL / 2; ++q) xv[q] = xseg[b * (kL / 2) + q];
#pragma unroll
                        for (int i = 0; i < kFocusPT; ++i) h[i] = horner_block(h[i], ql[i], p[i], xv);
                    }
                }

#pragma unroll
                for (int i = 0; i < kFocusPT; ++i) {
                    const float2 v = cmul(q0[i], h[i]);
                    // Kahan: comp carries the rounding error of the running sum (true = sum - comp).
                    const float yr = v.x - comp[i].x, yi = v.y - comp[i].y;
                    const float tr = sum[i].x + yr, ti = sum[i].y + yi;
                    comp[i].x = (tr - sum[i].x) - yr;
                    comp[i].y = (ti - sum[i].y) - yi;
                    sum[i].x = tr;
                    sum[i].y = ti;
                }
            }

            __syncthreads();  // every thread is done with this stage
            ++n_consumed;
            if (tid == 0 && j + kFocusStages < nblk) {
                fence_proxy_async_smem();
                issue(j + kFocusStages);
            }
        }

        if (timed_out) {
            // Let the copies still in flight land before the CTA exits, then report.
            if (tid == 0) {
                for (uint32_t k = n_consumed; k < n_issued; ++k)
                    mbar_wait_bounded(&full_bar[k % kFocusStages], (k / kFocusStages) & 1u, kWaitLimitNs);
                atomicOr(status, kStatusTimeout);
            }
            __syncthreads();
            return;
        }

        float4 *__restrict__ part = sJ.partial + (size_t)un.group * P;
#pragma unroll
        for (int i = 0; i < kFocusPT; ++i) {
            const long long pidx = tile_pixel(sJ.tile_cols, sJ.grid_cols, P, un.tile, i * kFocusThreads + tid);
            if (pidx >= 0) part[pidx] = make_float4(sum[i].x, sum[i].y, comp[i].x, comp[i].y);
        }
        __syncthreads();  // sJ / sp are rewritten by the next unit
    }
}

}  // namespace

int focus_motion_smem_bytes(int stage_bytes)
{
    return kFocusStages * stage_bytes + (int)sizeof(MotionShared);
}

int focus_motion_blocks_per_sm(int stage_bytes)
{
    const int smem = focus_motion_smem_bytes(stage_bytes);
    int best = 1 << 30;
    for (auto fn : {focus_motion_kernel<false>, focus_motion_kernel<true>}) {
        int blocks = 0;
        if (allow_max_dynamic_smem(fn) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, kFocusThreads, smem) != cudaSuccess)
            return 0;
        best = blocks < best ? blocks : best;
    }
    return best;
}

cudaError_t launch_focus_motion(const FocusJob *jobs_dev, const FocusUnit *units_dev, int n_units, int *counter_dev,
                                int *status_dev, int stage_bytes, int grid_ctas, bool skip_zero, cudaStream_t st)
{
    const int smem = focus_motion_smem_bytes(stage_bytes);
    const auto fn = skip_zero ? focus_motion_kernel<true> : focus_motion_kernel<false>;
    cudaError_t e = allow_max_dynamic_smem(fn);
    if (e != cudaSuccess) return e;
    fn<<<grid_ctas, kFocusThreads, smem, st>>>(jobs_dev, units_dev, n_units, counter_dev, status_dev, stage_bytes);
    return cudaGetLastError();
}

}  // namespace tdc
