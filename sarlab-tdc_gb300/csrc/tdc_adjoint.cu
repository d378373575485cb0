// tdc_adjoint.cu -- adjoint of the focus with respect to per-chirp antenna
// position offsets (autofocus). No reference counterpart.
//
// Forward (tdc_focus.cu): I(T) = sum_c q0_c(T) A_c(T), q0 = w e^{j 2 pi alpha},
// A = sum_s x_s z^s, z = e^{j 2 pi beta}, phase of sample s = 2 pi g_s R,
// g_s = g0 + s g1. With R = |P_c + d_c - T|:
//   dI/dR_c = j 2 pi q0 (g0 A + g1 B),  B = sum_s s x_s z^s,
//   dL/dd_c = sum_T Re(conj(G_T) dI/dR_c) (P_c + d_c - T) / R,
// where G_T = dL/dRe I + j dL/dIm I is the incoming image gradient. The Doppler
// window and the skip test are held fixed (not differentiated).
//
// A and B come from one pass over the samples with the forward's blocked
// Horner scheme: over blocks b (last first), with y_b = sum_k x_{bL+k} p_k and
// y'_b = sum_k k x_{bL+k} p_k,
//   A <- A QL + y_b,     B <- (B + L A_old) QL + y'_b,
// i.e. 8 FFMA per correlation. With the forward's sums A stored per (chirp, pixel)
// (the storing focus instance) and the rows staged pre-scaled by the sample index,
// x'_s = s x_s, B is the forward's own recurrence over x' (B <- B QL + sum_k x'_k p_k,
// 8-entry table): 4 FFMA per correlation, and A is read back. Either way the
// reference response is recomputed per tile and never stored. Per chirp the CTA
// reduces its pixels' contributions (warp shuffles + shared memory) into one float4
// per (tile, chirp); an FP64 kernel sums the tiles in order, so the gradient is
// deterministic.
#include <cuda_runtime.h>
#include <stdint.h>

#include "tdc_device.cuh"
#include "tdc_internal.h"

namespace tdc {

namespace {

constexpr int kLA = 4;  // in-block table length of the coupled recurrence (two tables per pixel)
constexpr int kLS = 8;  // in-block table length with stored sums (one table, as in the forward)
#ifndef TDC_ADJOINT_UNROLL
#define TDC_ADJOINT_UNROLL 8
#endif
constexpr int kAdjUnroll = TDC_ADJOINT_UNROLL;  // Horner blocks unrolled in the stored-sums recurrence
#ifndef TDC_ADJOINT_UNROLL_COUPLED
#define TDC_ADJOINT_UNROLL_COUPLED 4
#endif
constexpr int kAdjUnrollCoupled = TDC_ADJOINT_UNROLL_COUPLED;  // ... and in the coupled one

struct AdjShared {
    float t[kFocusPT * 6][kFocusThreads];  // pixel coordinates (hi xyz, lo xyz)
    float2 g[kFocusPT][kFocusThreads];     // incoming image gradient per pixel slot
};

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

template <bool STORED>
__global__ void __launch_bounds__(kFocusThreads, 3)
    adjoint_fp32_kernel(const FocusJob *__restrict__ jobs, const FocusUnit *__restrict__ units, int n_units,
                        int *__restrict__ counter, int *__restrict__ status, int stage_bytes,
                        const float2 *__restrict__ gimg, float4 *__restrict__ gpart)
{
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t full_bar[kFocusStages];
    __shared__ int s_unit;
    __shared__ FocusJob sJ;

    AdjShared &sp = *reinterpret_cast<AdjShared *>(smem + kFocusStages * stage_bytes);
    float *sred = reinterpret_cast<float *>(smem + kFocusStages * stage_bytes + sizeof(AdjShared));
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    if (tid == 0) {
        for (int i = 0; i < kFocusStages; ++i) mbar_init(&full_bar[i], 1);
        fence_barrier_init();
    }
    __syncthreads();

    uint32_t n_issued = 0, n_consumed = 0;

    for (;;) {
        if (tid == 0) s_unit = atomicAdd(counter, 1);
        __syncthreads();
        const int u = s_unit;
        if (u >= n_units) break;
        const FocusUnit un = units[u];
        if (tid < (int)(sizeof(FocusJob) / sizeof(int))) {
            reinterpret_cast<int *>(&sJ)[tid] = reinterpret_cast<const int *>(&jobs[un.job])[tid];
        }
        __syncthreads();

        const int C = sJ.C;
        const int c0 = un.group * sJ.chirps_per_group;
        const int c1 = min(C, c0 + sJ.chirps_per_group);
        const int CB = sJ.stage_chirps;
        const int nblk = (c1 - c0 + CB - 1) / CB;
        const int s_pad = sJ.s_pad;
        const uint32_t row_bytes = static_cast<uint32_t>(s_pad) * 8u;
        const float4 *__restrict__ xw = sJ.xw;
        const ChirpRec *__restrict__ chirps = sJ.chirps;

        if (tid == 0) {
            const int npro = nblk < kFocusStages ? nblk : kFocusStages;
            for (int j = 0; j < npro; ++j) {
                const int cb0 = c0 + j * CB;
                const int cnt = min(CB, c1 - cb0);
                const int st = n_issued % kFocusStages;
                unsigned char *base = smem + st * stage_bytes;
                const uint32_t bx = cnt * row_bytes, br = cnt * (uint32_t)sizeof(ChirpRec);
                mbar_arrive_expect_tx(&full_bar[st], bx + br);
                bulk_g2s(base, xw + (size_t)cb0 * (s_pad / 2), bx, &full_bar[st]);
                bulk_g2s(base + CB * row_bytes, chirps + cb0, br, &full_bar[st]);
                ++n_issued;
            }
        }

        const long long tile_base = (long long)un.tile * kFocusTile;
        const long long P = sJ.P;
#pragma unroll
        for (int i = 0; i < kFocusPT; ++i) {
            const long long p = tile_base + i * kFocusThreads + tid;
            float4 hi = make_float4(0.f, 0.f, 0.f, 0.f), lo = hi;
            float2 g = make_float2(0.f, 0.f);
            if (p < P) {
                hi = __ldg(&sJ.grid_hi[p]);
                if (sJ.grid_lo) lo = __ldg(&sJ.grid_lo[p]);
                g = gimg[p];
            }
            sp.t[i * 6 + 0][tid] = hi.x;
            sp.t[i * 6 + 1][tid] = hi.y;
            sp.t[i * 6 + 2][tid] = hi.z;
            sp.t[i * 6 + 3][tid] = lo.x;
            sp.t[i * 6 + 4][tid] = lo.y;
            sp.t[i * 6 + 5][tid] = lo.z;
            sp.g[i][tid] = g;
        }

        const float g0h = sJ.g0_hi, g0l = sJ.g0_lo, g1 = sJ.g1, g1l = sJ.g1_lo;
        const float g0f = g0h + g0l;
        const float tol = sJ.two_over_lambda, half_bw = sJ.half_bw, inv_bw = sJ.inv_bw, az_a = sJ.az_a;
        const bool taper = (sJ.flags & kFlagTaper) != 0;
        const bool skip_test = (sJ.flags & kFlagSkipTest) != 0;
        const int chunk = sJ.chunk;
        const SkipPoint *__restrict__ skip = sJ.skip;
        constexpr int kL = STORED ? kLS : kLA;
        const int nb = s_pad / kL;
        const float2 *__restrict__ sums = sJ.chirp_sums;

        float wskip[kFocusPT];
#pragma unroll
        for (int i = 0; i < kFocusPT; ++i) wskip[i] = 1.0f;
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
            const ChirpRec *recs = reinterpret_cast<const ChirpRec *>(base + CB * row_bytes);
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
                const ChirpRec r = recs[cc];
                const float4 *xs = xs_stage + (size_t)cc * (s_pad / 2);

                float2 p[kFocusPT][kL - 1], kp[kFocusPT][STORED ? 1 : kLA - 1];
                float2 ql[kFocusPT], q0[kFocusPT], A[kFocusPT], B[kFocusPT];
                float ux[kFocusPT], uy[kFocusPT], uz[kFocusPT];
#pragma unroll
                for (int i = 0; i < kFocusPT; ++i) {
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
                    if (!STORED) {
#pragma unroll
                        for (int k = 0; k < kLA - 1; ++k)
                            kp[i][k] = make_float2((float)(k + 1) * p[i][k].x, (float)(k + 1) * p[i][k].y);
                    }
                    const float lbh = (float)kL * bh;
                    const float lfr = (lbh - rintf(lbh)) + (float)kL * bl;
                    float sl, cl;
                    sincospif(2.0f * lfr, &sl, &cl);
                    ql[i] = make_float2(cl, sl);
                    const float fd = doppler_freq(tol, r.vel.x, r.vel.y, r.vel.z, dxh, dyh, dzh, rs);
                    const float w = wskip[i] * doppler_window(fd, r.p_hi.w, half_bw, inv_bw, taper, az_a);
                    float sa, ca;
                    __sincosf(kTwoPiF * alpha, &sa, &ca);
                    q0[i] = make_float2(w * ca, w * sa);
                    const float rsu = dh > 0.0f ? rs : 0.0f;  // unit vector (P - T) / R, 0 at R = 0
                    ux[i] = dxh * rsu;
                    uy[i] = dyh * rsu;
                    uz[i] = dzh * rsu;
                    A[i] = make_float2(0.f, 0.f);
                    B[i] = make_float2(0.f, 0.f);
                }

                if (STORED) {
                    // B = sum_s x'_s z^s over the pre-scaled rows, the forward's recurrence
#pragma unroll kAdjUnroll
                    for (int b = nb - 1; b >= 0; --b) {
                        float4 xv[kLS / 2];
#pragma unroll
                        for (int m = 0; m < kLS / 2; ++m) xv[m] = xs[b * (kLS / 2) + m];
#pragma unroll
                        for (int i = 0; i < kFocusPT; ++i) {
                            float br = fmaf(B[i].x, ql[i].x, xv[0].x);
                            br = fmaf(-B[i].y, ql[i].y, br);
                            float bi = fmaf(B[i].x, ql[i].y, xv[0].y);
                            bi = fmaf(B[i].y, ql[i].x, bi);
#pragma unroll
                            for (int k = 1; k < kLS; ++k) {
                                const float xr = (k & 1) ? xv[k >> 1].z : xv[k >> 1].x;
                                const float xi = (k & 1) ? xv[k >> 1].w : xv[k >> 1].y;
                                br = fmaf(xr, p[i][k - 1].x, br);
                                br = fmaf(-xi, p[i][k - 1].y, br);
                                bi = fmaf(xr, p[i][k - 1].y, bi);
                                bi = fmaf(xi, p[i][k - 1].x, bi);
                            }
                            B[i] = make_float2(br, bi);
                        }
                    }
                    // A as the forward computed it (zero where its window vote skipped the chirp)
#pragma unroll
                    for (int i = 0; i < kFocusPT; ++i) {
                        const long long px = tile_base + i * kFocusThreads + tid;
                        A[i] = px < P ? sums[(size_t)c * P + px] : make_float2(0.f, 0.f);
                    }
                }
#pragma unroll kAdjUnrollCoupled
                for (int b = STORED ? -1 : nb - 1; b >= 0; --b) {
                    const float4 xa = xs[b * 2], xb = xs[b * 2 + 1];
                    const float xr[kLA] = {xa.x, xa.z, xb.x, xb.z};
                    const float xi[kLA] = {xa.y, xa.w, xb.y, xb.w};
#pragma unroll
                    for (int i = 0; i < kFocusPT; ++i) {
                        // B <- (B + L A) QL + sum_{k>=1} k x_k p_k  (uses A before its update)
                        const float2 tb = make_float2(fmaf((float)kLA, A[i].x, B[i].x),
                                                      fmaf((float)kLA, A[i].y, B[i].y));
                        float br = fmaf(tb.x, ql[i].x, -tb.y * ql[i].y);
                        float bi = fmaf(tb.x, ql[i].y, tb.y * ql[i].x);
                        // A <- A QL + x_0 + sum_{k>=1} x_k p_k
                        float ar = fmaf(A[i].x, ql[i].x, xr[0]);
                        ar = fmaf(-A[i].y, ql[i].y, ar);
                        float ai = fmaf(A[i].x, ql[i].y, xi[0]);
                        ai = fmaf(A[i].y, ql[i].x, ai);
#pragma unroll
                        for (int k = 1; k < kLA; ++k) {
                            ar = fmaf(xr[k], p[i][STORED ? 0 : k - 1].x, ar);
                            ar = fmaf(-xi[k], p[i][STORED ? 0 : k - 1].y, ar);
                            ai = fmaf(xr[k], p[i][STORED ? 0 : k - 1].y, ai);
                            ai = fmaf(xi[k], p[i][STORED ? 0 : k - 1].x, ai);
                            br = fmaf(xr[k], kp[i][STORED ? 0 : k - 1].x, br);
                            br = fmaf(-xi[k], kp[i][STORED ? 0 : k - 1].y, br);
                            bi = fmaf(xr[k], kp[i][STORED ? 0 : k - 1].y, bi);
                            bi = fmaf(xi[k], kp[i][STORED ? 0 : k - 1].x, bi);
                        }
                        A[i] = make_float2(ar, ai);
                        B[i] = make_float2(br, bi);
                    }
                }

                float gx = 0.f, gy = 0.f, gz = 0.f;
#pragma unroll
                for (int i = 0; i < kFocusPT; ++i) {
                    // S = g0 A + g1 B ; T = q0 S ; dI/dR = j 2 pi T
                    const float2 s = make_float2(fmaf(g0f, A[i].x, g1 * B[i].x), fmaf(g0f, A[i].y, g1 * B[i].y));
                    const float2 t = cmul(q0[i], s);
                    const float2 g = sp.g[i][tid];
                    // Re(conj(G) * j 2 pi T) = 2 pi (G.im T.re - G.re T.im)
                    const float dldr = kTwoPiF * (g.y * t.x - g.x * t.y);
                    gx = fmaf(dldr, ux[i], gx);
                    gy = fmaf(dldr, uy[i], gy);
                    gz = fmaf(dldr, uz[i], gz);
                }
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) {
                    gx += __shfl_xor_sync(0xffffffffu, gx, off);
                    gy += __shfl_xor_sync(0xffffffffu, gy, off);
                    gz += __shfl_xor_sync(0xffffffffu, gz, off);
                }
                if (lane == 0) {
                    sred[(cc * 4 + warp) * 3 + 0] = gx;
                    sred[(cc * 4 + warp) * 3 + 1] = gy;
                    sred[(cc * 4 + warp) * 3 + 2] = gz;
                }
            }

            __syncthreads();  // stage consumed; per-chirp warp sums in sred
            if (tid < cnt) {
                float v[3];
#pragma unroll
                for (int k = 0; k < 3; ++k)
                    v[k] = (sred[(tid * 4 + 0) * 3 + k] + sred[(tid * 4 + 1) * 3 + k]) +
                           (sred[(tid * 4 + 2) * 3 + k] + sred[(tid * 4 + 3) * 3 + k]);
                gpart[(size_t)un.tile * C + cb0 + tid] = make_float4(v[0], v[1], v[2], 0.f);
            }
            ++n_consumed;
            if (tid == 0 && j + kFocusStages < nblk) {
                const int jn = j + kFocusStages;
                const int cb0n = c0 + jn * CB;
                const int cntn = min(CB, c1 - cb0n);
                const int stn = n_issued % kFocusStages;
                unsigned char *basen = smem + stn * stage_bytes;
                const uint32_t bx = cntn * row_bytes, br = cntn * (uint32_t)sizeof(ChirpRec);
                fence_proxy_async_smem();
                mbar_arrive_expect_tx(&full_bar[stn], bx + br);
                bulk_g2s(basen, xw + (size_t)cb0n * (s_pad / 2), bx, &full_bar[stn]);
                bulk_g2s(basen + CB * row_bytes, chirps + cb0n, br, &full_bar[stn]);
                ++n_issued;
            }
        }

        if (timed_out) {
            if (tid == 0) {
                for (uint32_t k = n_consumed; k < n_issued; ++k) {
                    mbar_wait_bounded(&full_bar[k % kFocusStages], (k / kFocusStages) & 1u, kWaitLimitNs);
                }
                atomicOr(status, kStatusTimeout);
            }
            __syncthreads();
            return;
        }
        __syncthreads();  // sJ / sp / sred are rewritten by the next unit
    }
}

// grad[c] = sum over tiles of gpart[tile][c], in FP64, tile order.
__global__ void adjoint_reduce_kernel(const float4 *__restrict__ gpart, int n_tiles, int C, double *__restrict__ grad)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    double x = 0.0, y = 0.0, z = 0.0;
    for (int t = 0; t < n_tiles; ++t) {
        const float4 v = gpart[(size_t)t * C + c];
        x += v.x;
        y += v.y;
        z += v.z;
    }
    grad[3 * c + 0] = x;
    grad[3 * c + 1] = y;
    grad[3 * c + 2] = z;
}

}  // namespace

int adjoint_fp32_smem_bytes(int stage_bytes, int stage_chirps)
{
    return kFocusStages * stage_bytes + (int)sizeof(AdjShared) + stage_chirps * 4 * 3 * (int)sizeof(float);
}

int adjoint_fp32_blocks_per_sm(int stage_bytes, int stage_chirps, bool stored)
{
    const int smem = adjoint_fp32_smem_bytes(stage_bytes, stage_chirps);
    auto fn = stored ? adjoint_fp32_kernel<true> : adjoint_fp32_kernel<false>;
    if (allow_max_dynamic_smem(fn) != cudaSuccess) return 0;
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, kFocusThreads, smem) != cudaSuccess) return 0;
    return blocks;
}

cudaError_t launch_adjoint_fp32(const FocusJob *jobs_dev, const FocusUnit *units_dev, int n_units, int *counter_dev,
                                int *status_dev, int stage_bytes, int stage_chirps, int grid_ctas,
                                const float2 *gimg, float4 *gpart, bool stored, cudaStream_t st)
{
    const int smem = adjoint_fp32_smem_bytes(stage_bytes, stage_chirps);
    auto fn = stored ? adjoint_fp32_kernel<true> : adjoint_fp32_kernel<false>;
    cudaError_t e = allow_max_dynamic_smem(fn);
    if (e != cudaSuccess) return e;
    fn<<<grid_ctas, kFocusThreads, smem, st>>>(jobs_dev, units_dev, n_units, counter_dev, status_dev, stage_bytes,
                                               gimg, gpart);
    return cudaGetLastError();
}

cudaError_t launch_adjoint_reduce(const float4 *gpart, int n_tiles, int C, double *grad, cudaStream_t st)
{
    if (C <= 0) return cudaSuccess;
    adjoint_reduce_kernel<<<(C + 127) / 128, 128, 0, st>>>(gpart, n_tiles, C, grad);
    return cudaGetLastError();
}

}  // namespace tdc
