// tdc_general.cu -- FP32 general focus kernel of the GB300 TDC engine: the
// inputs the FP32-bulk kernel does not take, at FP32-bulk-like accuracy.
//
//   * per-sample antenna positions (position[c][s] varies within a chirp, as the
//     reference's tdckernels.cu:204-208 reads it per element);
//   * per-sample Doppler windows (velocity / attitude varying within a chirp,
//     tdckernels.cu:106-130 evaluates the window per element);
//   * non-uniform sample times (2 f_s / c0 not affine in s).
//
// Phase of sample s of chirp c at pixel T, in cycles:
//   g_s R_s,  R_s = |P[c,s] - T|,  g_s = 2 f_s / c0.
// Split about sample 0 (R0 = |P[c,0] - T| in double-float, as in the bulk kernel)
// and the affine fit g_s = g0 + g1 s + r_s:
//   g_s R_s = (g0 + g1 s) R0  +  r_s R0  +  g_s d_s,   d_s = R_s - R0.
// The first term is the bulk kernel's alpha + beta s, evaluated with the same
// blocked Horner recurrence (H <- H QL + sum_k x'_k p_k). The rest, psi_s, is a
// per-(pixel, sample) correction folded into the sample: x'_s = x_s w_s e^{j 2 pi psi_s}.
// d_s comes without cancellation from the per-sample offset D_s = P[c,s] - P[c,0]
// (host table: D_s and |D_s|^2 per (chirp, sample)):
//   N = 2 (P0 - T).D + |D|^2 = R_s^2 - R0^2,   d_s = N / (R0 + R_s) = (N / 2R0) f(N / R0^2),
//   f(e) = 2 / (1 + sqrt(1 + e)) = 1 - e/4 + e^2/8 - 5e^3/64 + 7e^4/128 - ...,
// the series taken to e^2 when the host bounds |e| <= 0.02 and |psi| <= 4 cycles (then
// the sincos takes psi unreduced: its argument scaling adds < 2e-6 rad), else to e^4 with
// psi reduced modulo one cycle ("wide" variants, which also carry the non-uniform
// sampling residual; the host routes |e| > 0.1 to the FP64 kernel; at 0.1 the
// truncation is 4e-7 of d_s).
//
// Same unit decomposition, staging (cp.async.bulk + mbarrier pipeline), skip test,
// Kahan accumulation and FP64 group reduction as the bulk kernel; a chirp whose
// chirp-level weight is zero for every pixel of a warp skips the Horner loop. The
// per-sample window works in band units, q = (fDop - centre) / B, from a table of
// velocities pre-scaled by -2 / (lambda B) and centres by 1 / B.
#include <cuda_runtime.h>
#include <stdint.h>

#include "tdc_device.cuh"
#include "tdc_internal.h"

namespace tdc {

namespace {

#ifndef TDC_GENERAL_MINB
#define TDC_GENERAL_MINB 2
#endif

constexpr int kL = 8;                   // in-block phasor table length
constexpr int kPT = kGeneralPT;         // pixels per thread
constexpr int kT = kFocusTile / kPT;    // threads per CTA (a CTA covers one 512-pixel tile)
constexpr int kTile = kT * kPT;
// Double buffering: a chirp row takes tens of microseconds of arithmetic per CTA, far
// longer than its copy, and the smaller footprint keeps two CTAs resident per SM.
constexpr int kStages = 2;
static_assert(kTile == kFocusTile, "work units tile the grid like the FP32-bulk kernel");

struct GenShared {
    float t[kPT * 6][kT];  // (x_hi, y_hi, z_hi, x_lo, y_lo, z_lo) per pixel slot
};

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

// Nearest integer for |v| < 2^22 without a conversion instruction.
__device__ __forceinline__ float round_small(float v)
{
    constexpr float kMagic = 12582912.0f;  // 1.5 x 2^23
    return (v + kMagic) - kMagic;
}

// The window-and-residual variant without per-sample positions keeps more samples in
// flight than 128 registers hold: it runs one CTA per SM instead of spilling.
//
// Stages: rows of job.seg_len samples. When a whole row fits (seg_len = s_pad) a stage
// holds stage_chirps chirps; otherwise each chirp's row is staged in segments, last
// segment first, and the chirp's Horner state carries from segment to segment. Stage
// layout: [x rows][trajectory rows][window rows][window-offset rows][residual r_s][g_s]
// [records], the per-sample tables only where the variant reads them.
template <bool TRAJ, bool WIN, bool WIDE>
__global__ void __launch_bounds__(kT, (!TRAJ && WIN && WIDE) ? 1 : TDC_GENERAL_MINB)
    focus_general_kernel(const FocusJob *__restrict__ jobs, const FocusUnit *__restrict__ units, int n_units,
                         int *__restrict__ counter, int *__restrict__ status, int stage_bytes)
{
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t full_bar[kStages];
    __shared__ int s_unit;
    __shared__ FocusJob sJ;

    GenShared &sp = *reinterpret_cast<GenShared *>(smem + kStages * stage_bytes);

    constexpr bool TW = TRAJ && WIN;  // per-sample positions and windows: window-offset rows staged
    const int tid = threadIdx.x;
    if (tid == 0) {
        for (int i = 0; i < kStages; ++i) mbar_init(&full_bar[i], 1);
        fence_barrier_init();
    }
    __syncthreads();

    uint32_t n_issued = 0;
    uint32_t n_consumed = 0;

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
        const int s_pad = sJ.s_pad;
        const int seg = sJ.seg_len;  // samples per staged row segment (multiple of 16)
        const int nseg = (s_pad + seg - 1) / seg;
        const int CB = nseg == 1 ? sJ.stage_chirps : 1;
        const int nblk = nseg == 1 ? (c1 - c0 + CB - 1) / CB : (c1 - c0) * nseg;
        const uint32_t xrow = static_cast<uint32_t>(seg) * 8u;
        const uint32_t arow = static_cast<uint32_t>(seg) * 16u;
        const uint32_t grow = static_cast<uint32_t>(seg) * 4u;
        const uint32_t off_a = CB * xrow;
        const uint32_t off_b = off_a + (TRAJ ? CB * arow : 0u);
        const uint32_t off_w = off_b + (WIN ? CB * arow : 0u);
        const uint32_t off_g = off_w + (TW ? CB * grow : 0u);
        const uint32_t off_r = off_g + (WIDE ? grow : 0u) + (TRAJ ? grow : 0u);
        const float4 *__restrict__ xw = sJ.xw;
        const float4 *__restrict__ traj = sJ.traj;
        const float4 *__restrict__ wins = sJ.wins;
        const float *__restrict__ wdot = sJ.wdot;
        const float *__restrict__ gres = sJ.gres;
        const float *__restrict__ gsam = sJ.gsam;
        const ChirpRec *__restrict__ chirps = sJ.chirps;

        // stage j -> first chirp, chirps, segment, sample offset, samples
        auto stage_of = [&](int j, int &cb0, int &cnt, int &sg, int &off, int &len) {
            if (nseg == 1) {
                cb0 = c0 + j * CB;
                cnt = min(CB, c1 - cb0);
                sg = 0;
            } else {
                cb0 = c0 + j / nseg;
                cnt = 1;
                sg = nseg - 1 - j % nseg;
            }
            off = sg * seg;
            len = min(seg, s_pad - off);
        };

        auto issue = [&](int j) {
            int cb0, cnt, sg, off, len;
            stage_of(j, cb0, cnt, sg, off, len);
            const int st = n_issued % kStages;
            unsigned char *base = smem + st * stage_bytes;
            const uint32_t lx = static_cast<uint32_t>(len) * 8u, la = static_cast<uint32_t>(len) * 16u,
                           lg = static_cast<uint32_t>(len) * 4u;
            uint32_t total =
                cnt * (lx + (TRAJ ? la : 0u) + (WIN ? la : 0u) + (TW ? lg : 0u) + (uint32_t)sizeof(ChirpRec));
            if (WIDE) total += lg;
            if (TRAJ) total += lg;
            mbar_arrive_expect_tx(&full_bar[st], total);
            for (int cc = 0; cc < cnt; ++cc) {
                const size_t row = (size_t)(cb0 + cc) * s_pad + off;
                bulk_g2s(base + cc * xrow, xw + row / 2, lx, &full_bar[st]);
                if (TRAJ) bulk_g2s(base + off_a + cc * arow, traj + row, la, &full_bar[st]);
                if (WIN) bulk_g2s(base + off_b + cc * arow, wins + row, la, &full_bar[st]);
                if (TW) bulk_g2s(base + off_w + cc * grow, wdot + row, lg, &full_bar[st]);
            }
            uint32_t og = off_g;
            if (WIDE) {
                bulk_g2s(base + og, gres + off, lg, &full_bar[st]);
                og += grow;
            }
            if (TRAJ) bulk_g2s(base + og, gsam + off, lg, &full_bar[st]);
            bulk_g2s(base + off_r, chirps + cb0, cnt * (uint32_t)sizeof(ChirpRec), &full_bar[st]);
            ++n_issued;
        };

        if (tid == 0) {
            fence_proxy_async_smem();
            const int npro = nblk < kStages ? nblk : kStages;
            for (int j = 0; j < npro; ++j) issue(j);
        }

        const long long P = sJ.P;
#pragma unroll
        for (int i = 0; i < kPT; ++i) {
            const long long p = tile_pixel(sJ.tile_cols, sJ.grid_cols, P, un.tile, i * kT + tid);
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
        const float tol = sJ.two_over_lambda, half_bw = sJ.half_bw, inv_bw = sJ.inv_bw, az_a = sJ.az_a;
        const bool taper = (sJ.flags & kFlagTaper) != 0;
        const bool skip_test = (sJ.flags & kFlagSkipTest) != 0;
        const int chunk = sJ.chunk;
        const SkipPoint *__restrict__ skip = sJ.skip;

        float2 sum[kPT], comp[kPT];
        float wskip[kPT];
#pragma unroll
        for (int i = 0; i < kPT; ++i) {
            sum[i] = make_float2(0.f, 0.f);
            comp[i] = make_float2(0.f, 0.f);
            wskip[i] = 1.0f;
        }
        // per-(pixel, chirp) state, carried across the segments of a chirp
        float2 p[kPT][kL - 1];
        float2 ql[kPT], q0[kPT], h[kPT];
        float t2x[kPT], t2y[kPT], t2z[kPT];
        float r0[kPT], a2[kPT], b2[kPT];  // R0, 1/2R0, 1/R0^2
        float r0sq[kPT];                   // R0^2 (per-sample positions and windows)
        bool live = true;
        int cur_chunk = -1;
        bool timed_out = false;

        for (int j = 0; j < nblk; ++j) {
            const int st = n_consumed % kStages;
            const uint32_t parity = (n_consumed / kStages) & 1u;
            const bool ok = mbar_wait_bounded(&full_bar[st], parity, kWaitLimitNs);
            if (__syncthreads_or(!ok)) {
                timed_out = true;
                break;
            }
            const unsigned char *base = smem + st * stage_bytes;
            const ChirpRec *recs = reinterpret_cast<const ChirpRec *>(base + off_r);
            const float *sgr = reinterpret_cast<const float *>(base + off_g);           // r_s of the segment
            const float *sgg = sgr + (WIDE ? seg : 0);                                  // g_s of the segment
            int cb0, cnt, sg, off, len;
            stage_of(j, cb0, cnt, sg, off, len);

            for (int cc = 0; cc < cnt; ++cc) {
                const int c = cb0 + cc;
                const float4 *xs = reinterpret_cast<const float4 *>(base) + (size_t)cc * (seg / 2);
                const float4 *as = reinterpret_cast<const float4 *>(base + off_a) + (size_t)cc * seg;
                const float4 *bs = reinterpret_cast<const float4 *>(base + off_b) + (size_t)cc * seg;
                const float *us = reinterpret_cast<const float *>(base + off_w) + (size_t)cc * seg;

                if (sg == nseg - 1) {
                    // first staged segment of the chirp: skip weight, range, phase set-up
                    if (skip_test) {
                        const int k = c / chunk;
                        if (k != cur_chunk) {
                            cur_chunk = k;
#pragma unroll
                            for (int i = 0; i < kPT; ++i)
                                wskip[i] = chunk_is_nonzero(skip + (size_t)k * 9, sp.t[i * 6 + 0][tid],
                                                            sp.t[i * 6 + 1][tid], sp.t[i * 6 + 2][tid], tol,
                                                            half_bw)
                                               ? 1.0f
                                               : 0.0f;
                        }
                    }
                    const ChirpRec r = recs[cc];
                    bool any = false;
#pragma unroll
                    for (int i = 0; i < kPT; ++i) {
                        float dxh, dxl, dyh, dyl, dzh, dzl;
                        dd_sub(r.p_hi.x, r.p_lo.x, sp.t[i * 6 + 0][tid], sp.t[i * 6 + 3][tid], dxh, dxl);
                        dd_sub(r.p_hi.y, r.p_lo.y, sp.t[i * 6 + 1][tid], sp.t[i * 6 + 4][tid], dyh, dyl);
                        dd_sub(r.p_hi.z, r.p_lo.z, sp.t[i * 6 + 2][tid], sp.t[i * 6 + 5][tid], dzh, dzl);
                        float rh, rl, rs, dh;
                        dd_range(dxh, dxl, dyh, dyl, dzh, dzl, rh, rl, rs, dh);
                        const float alpha = dd_frac_mul(g0h, g0l, rh, rl);
                        float bh = g1 * rh;
                        float bl = fmaf(g1, rh, -bh);
                        bl = fmaf(g1, rl, bl);
                        bl = fmaf(g1l, rh, bl);
                        bh -= rintf(bh);
                        float s1, c1s;
                        __sincosf(kTwoPiF * (bh + bl), &s1, &c1s);
                        p[i][0] = make_float2(c1s, s1);
#pragma unroll
                        for (int k = 1; k < kL - 1; ++k) p[i][k] = cmul(p[i][k - 1], p[i][0]);
                        const float lbh = (float)kL * bh;
                        const float lfr = (lbh - rintf(lbh)) + (float)kL * bl;
                        float sl, cl;
                        sincospif(2.0f * lfr, &sl, &cl);
                        ql[i] = make_float2(cl, sl);
                        float w = wskip[i];
                        if (!WIN) {
                            const float fd = doppler_freq(tol, r.vel.x, r.vel.y, r.vel.z, dxh, dyh, dzh, rs);
                            w *= doppler_window(fd, r.p_hi.w, half_bw, inv_bw, taper, az_a);
                        }
                        any |= w != 0.0f;
                        float sa, ca;
                        __sincosf(kTwoPiF * alpha, &sa, &ca);
                        q0[i] = make_float2(w * ca, w * sa);
                        h[i] = make_float2(0.f, 0.f);
                        // TRAJ: 2 (P0 - T) for the range change; else the unit vector (P0 - T) / R0
                        // of the per-sample window
                        const float sc = TRAJ ? 2.0f : rs;
                        t2x[i] = sc * dxh;
                        t2y[i] = sc * dyh;
                        t2z[i] = sc * dzh;
                        r0[i] = rh;
                        a2[i] = 0.5f * rs;  // 1 / 2R0
                        b2[i] = rs * rs;    // 1 / R0^2
                        if (TW) r0sq[i] = rh * rh;
                    }
                    // a chirp whose chirp-level weight (skip test, and the window unless it is
                    // per sample) is zero for every pixel of the warp contributes nothing
                    live = __any_sync(0xffffffffu, any);
                }
                if (!live) continue;

                // Horner over this segment's blocks, last block first; each sample corrected per pixel.
                for (int b = len / kL - 1; b >= 0; --b) {
                    float2 acc[kPT];
#pragma unroll
                    for (int i = 0; i < kPT; ++i) acc[i] = cmul(h[i], ql[i]);
#pragma unroll
                    for (int k = 0; k < kL; ++k) {
                        const int s = b * kL + k;  // sample within the segment
                        const float4 xv = xs[s >> 1];
                        const float xr = (k & 1) ? xv.z : xv.x;
                        const float xi = (k & 1) ? xv.w : xv.y;
                        float4 av = make_float4(0.f, 0.f, 0.f, 0.f), bv = av;
                        if (TRAJ) av = as[s];
                        if (WIN) bv = bs[s];
                        const float uD = TW ? us[s] : 0.0f;
                        const float res = WIDE ? sgr[s] : 0.0f;
                        const float gsv = TRAJ ? sgg[s] : 0.0f;
#pragma unroll
                        for (int i = 0; i < kPT; ++i) {
                            float yr = xr, yi = xi;
                            float n = 0.0f;  // N = 2 (P0 - T).D + |D|^2 = |P0 - T + D|^2 - R0^2
                            if (TRAJ || WIDE) {
                                float psi = 0.0f;
                                if (TRAJ) {
                                    // |D|^2 from the table
                                    n = fmaf(t2x[i], av.x, fmaf(t2y[i], av.y, fmaf(t2z[i], av.z, av.w)));
                                    const float e = n * b2[i];
                                    float f;
                                    if (WIDE) {
                                        f = fmaf(e, 7.0f / 128.0f, -5.0f / 64.0f);
                                        f = fmaf(f, e, 0.125f);
                                        f = fmaf(f, e, -0.25f);
                                    } else {
                                        f = fmaf(e, 0.125f, -0.25f);
                                    }
                                    f = fmaf(f, e, 1.0f);
                                    psi = (gsv * a2[i]) * (n * f);  // g_s d_s (radians when narrow)
                                }
                                if (WIDE) {
                                    psi = fmaf(res, r0[i], psi);
                                    psi -= round_small(psi);
                                    psi *= kTwoPiF;
                                }
                                float sn, cs;
                                __sincosf(psi, &sn, &cs);
                                yr = fmaf(xr, cs, -xi * sn);
                                yi = fmaf(xr, sn, xi * cs);
                            }
                            if (WIN) {
                                // per-sample window at P[c,s] (d = P0 - T + D_s) in band units:
                                // q = (fDop - centre) / B from the table's velocity scaled by
                                // -2/(lambda B) and centre / B; in band for |q| <= 1/2, taper
                                // a - (1-a) cos(2 pi q - pi) = a + (1-a) cos(2 pi q)
                                // (with moving positions: u.d = (u/2).2(P0 - T) + u.D, the second
                                // term from the table, and |d|^2 = R0^2 + N)
                                float q;
                                if (TRAJ) {
                                    const float ud = fmaf(bv.x, t2x[i], fmaf(bv.y, t2y[i], fmaf(bv.z, t2z[i], uD)));
                                    q = fmaf(ud, rsqrtf(r0sq[i] + n), -bv.w);
                                } else {
                                    q = fmaf(bv.x, t2x[i], fmaf(bv.y, t2y[i], fmaf(bv.z, t2z[i], -bv.w)));
                                }
                                float w = taper ? fmaf(1.0f - az_a, __cosf(kTwoPiF * q), az_a) : 1.0f;
                                w = fabsf(q) <= 0.5f ? w : 0.0f;
                                yr *= w;
                                yi *= w;
                            }
                            if (k == 0) {
                                acc[i].x += yr;
                                acc[i].y += yi;
                            } else {
                                acc[i].x = fmaf(yr, p[i][k - 1].x, acc[i].x);
                                acc[i].x = fmaf(-yi, p[i][k - 1].y, acc[i].x);
                                acc[i].y = fmaf(yr, p[i][k - 1].y, acc[i].y);
                                acc[i].y = fmaf(yi, p[i][k - 1].x, acc[i].y);
                            }
                        }
                    }
#pragma unroll
                    for (int i = 0; i < kPT; ++i) h[i] = acc[i];
                }

                if (sg == 0) {
#pragma unroll
                    for (int i = 0; i < kPT; ++i) {
                        const float2 v = cmul(q0[i], h[i]);
                        const float yr = v.x - comp[i].x, yi = v.y - comp[i].y;
                        const float tr = sum[i].x + yr, ti = sum[i].y + yi;
                        comp[i].x = (tr - sum[i].x) - yr;
                        comp[i].y = (ti - sum[i].y) - yi;
                        sum[i].x = tr;
                        sum[i].y = ti;
                    }
                }
            }

            __syncthreads();
            ++n_consumed;
            if (tid == 0 && j + kStages < nblk) {
                fence_proxy_async_smem();
                issue(j + kStages);
            }
        }

        if (timed_out) {
            if (tid == 0) {
                for (uint32_t k = n_consumed; k < n_issued; ++k)
                    mbar_wait_bounded(&full_bar[k % kStages], (k / kStages) & 1u, kWaitLimitNs);
                atomicOr(status, kStatusTimeout);
            }
            __syncthreads();
            return;
        }

        float4 *__restrict__ part = sJ.partial + (size_t)un.group * P;
#pragma unroll
        for (int i = 0; i < kPT; ++i) {
            const long long pidx = tile_pixel(sJ.tile_cols, sJ.grid_cols, P, un.tile, i * kT + tid);
            if (pidx >= 0) part[pidx] = make_float4(sum[i].x, sum[i].y, comp[i].x, comp[i].y);
        }
        __syncthreads();
    }
}

template <bool TRAJ, bool WIN, bool WIDE>
struct GeneralKernel {
    static constexpr auto fn = focus_general_kernel<TRAJ, WIN, WIDE>;
};

using KernelFn = void (*)(const FocusJob *, const FocusUnit *, int, int *, int *, int);

KernelFn select_kernel(int variant)
{
    switch (variant & 7) {
        case 1: return GeneralKernel<true, false, false>::fn;
        case 2: return GeneralKernel<false, true, false>::fn;
        case 3: return GeneralKernel<true, true, false>::fn;
        case 4: return GeneralKernel<false, false, true>::fn;
        case 5: return GeneralKernel<true, false, true>::fn;
        case 6: return GeneralKernel<false, true, true>::fn;
        case 7: return GeneralKernel<true, true, true>::fn;
        default: return nullptr;
    }
}

}  // namespace

int focus_general_smem_bytes(int stage_bytes)
{
    return kStages * stage_bytes + (int)sizeof(GenShared);
}

int focus_general_blocks_per_sm(int variant, int stage_bytes)
{
    KernelFn fn = select_kernel(variant);
    if (!fn) return 0;
    const int smem = focus_general_smem_bytes(stage_bytes);
    if (allow_max_dynamic_smem(fn) != cudaSuccess) return 0;
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, kT, smem) != cudaSuccess) return 0;
    return blocks;
}

cudaError_t launch_focus_general(int variant, const FocusJob *jobs_dev, const FocusUnit *units_dev, int n_units,
                                 int *counter_dev, int *status_dev, int stage_bytes, int grid_ctas, cudaStream_t st)
{
    KernelFn fn = select_kernel(variant);
    if (!fn) return cudaErrorInvalidValue;
    const int smem = focus_general_smem_bytes(stage_bytes);
    cudaError_t e = allow_max_dynamic_smem(fn);
    if (e != cudaSuccess) return e;
    fn<<<grid_ctas, kT, smem, st>>>(jobs_dev, units_dev, n_units, counter_dev, status_dev, stage_bytes);
    return cudaGetLastError();
}

}  // namespace tdc
