// tdc_focus.cu -- FP32-bulk fused focus kernel of the GB300 TDC engine.
//
// Replaces the reference's per-(chunk, pixel) sequence createWindowKernel ->
// referenceResponseKernel -> correlateWithReference -> nppsSum_32fc -> addToImage
// (tdc-lib/src/tdckernels.cu:70-315, driven from tdcprocessor.cpp:77-156) with one
// persistent launch over work units (pixel tile x chirp group):
//
//   I(T) = sum_c w_az(T, c) * sum_s xw[c, s] * exp(+j 2 pi (2 R_c(T) f_s / c0)),
//   xw = range-windowed raw samples, f_s = f_0 + s df (uniform sample spacing).
//
// Per (pixel, chirp): R in double-float, phase at sample 0 (alpha) reduced
// modulo one cycle in double-float, per-sample step beta. Per sample the
// phasor is exp(j 2 pi (alpha + (bL + k) beta)) = e^{j2pi alpha} QL^b p_k, with
// p_k = e^{j 2 pi k beta} (k < L) kept in registers and QL = e^{j 2 pi L beta}.
// The chirp sum is evaluated by Horner's rule over the blocks b (last block
// first): H <- H * QL + sum_k x_{bL+k} p_k, so every sample costs exactly one
// complex multiply-add (4 FFMA) and no separate phasor advance. Block phasors
// never accumulate more than S/L rotations of an accurately computed QL.
// Chirp sums are accumulated per pixel with Kahan compensation; partial sums
// per chirp group are combined in FP64 by focus_reduce_kernel in a fixed order,
// so results do not depend on scheduling.
//
// Chirp sample rows and trajectory records are staged global->shared with
// cp.async.bulk on an mbarrier pipeline (kFocusStages deep) and read back as
// broadcast 128-bit shared loads shared by all 512 pixels of the tile.
//
// Two variations planned by the host: focus_fp32_anchored_kernel forms the range in
// double-float once per 32 pixels and chirp and each pixel's difference from it in FP32
// (short rows, unbounded band); under a finite band a work unit may cover only the chirps
// of its group that its tile can see in band (FocusUnit::span).
#include <cuda_runtime.h>
#include <stdint.h>

#include "tdc_device.cuh"
#include "tdc_internal.h"

namespace tdc {

namespace {

#ifndef TDC_FOCUS_L
#define TDC_FOCUS_L 8
#endif
#ifndef TDC_FOCUS_MINB
#define TDC_FOCUS_MINB 3
#endif
#ifndef TDC_FOCUS_UNROLL
#define TDC_FOCUS_UNROLL 8
#endif
#ifndef TDC_FOCUS_SWAP
#define TDC_FOCUS_SWAP 0
#endif

constexpr int kL = TDC_FOCUS_L;  // in-block phasor table length
constexpr int kUnrollBlocks = TDC_FOCUS_UNROLL;
// Finite-band instance: vote on the chirp-level windows before the phase set-up (1) or
// after it (0).
#ifndef TDC_FOCUS_EARLY_VOTE
#define TDC_FOCUS_EARLY_VOTE 1
#endif
constexpr bool kEarlyVote = TDC_FOCUS_EARLY_VOTE != 0;
// Anchored instance: chirp sums into a per-stage sum, the stage sums into the Kahan sum (1),
// or every chirp sum into the Kahan sum (0).
#ifndef TDC_ANCHOR_STAGE_SUM
#define TDC_ANCHOR_STAGE_SUM 1
#endif
constexpr bool kAnchorStageSums = TDC_ANCHOR_STAGE_SUM != 0;

struct SharedPixel {
    float t[kFocusPT * 6][kFocusThreads];  // (x_hi, y_hi, z_hi, x_lo, y_lo, z_lo) per pixel slot
};

// Anchored ranges (flat tiles, unbounded band). The 32 consecutive pixels of one warp and
// slot share an anchor pixel, their 17th (or their last inside the grid). Per chirp, one lane
// forms the anchor's range R0, start phase alpha0 = frac(g0 R0), per-sample step
// beta0 = frac(g1 R0) and block step QL0 = e^{j 2 pi L beta0} in double-float (a stage's
// 4 slots x chirps anchor records take one or two passes of the warp's lanes); a pixel then
// needs only its range difference dR = R - R0 = d.(d - 2e) / (R0 + R) in FP32 (d = pixel -
// anchor, e = antenna - anchor: no cancellation, |dR| <= |d|) and small corrections
// alpha0 + g0 dR, beta0 + g1 dR, QL0 e^{j 2 pi L g1 dR} (|2 pi L g1 dR| <= 0.25 by the host's
// bound). With an unbounded band and finite velocities and window centres, a chirp's window
// weight is 1 (0 where the antenna sits on the pixel: NaN Doppler), so this instance forms no
// Doppler frequency. Its chirp sums q0 H go into a per-stage sum by complex FMA, and the stage
// sums into the Kahan-compensated sum.
constexpr int kAnchorRecs = kFocusPT * kAnchorMaxStageChirps;  // anchor records per warp and stage
struct SharedAnchor {
    float4 d[kFocusPT][kFocusThreads];              // pixel - anchor per slot (x, y, z, 0)
    float anc[kFocusThreads / 32][kFocusPT][6];      // anchor per (warp, slot): hi xyz, lo xyz
    float4 rec[kFocusThreads / 32][kAnchorRecs][2];  // per (chirp, slot): (e, R0), (alpha0, beta0, QL0)
};

// (cos t, sin t) for |t| <= 0.25 (the anchored block-step correction, host-bounded) by their
// Taylor series to t^6 / t^5 (error < 2e-8).
__device__ __forceinline__ float2 sincos_anchor(float t)
{
    const float t2 = t * t;
    const float c = fmaf(t2, fmaf(t2, fmaf(t2, -1.0f / 720.0f, 1.0f / 24.0f), -0.5f), 1.0f);
    const float s = t * fmaf(t2, fmaf(t2, 1.0f / 120.0f, -1.0f / 6.0f), 1.0f);
    return make_float2(c, s);
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

// Kahan: comp carries the rounding error of the running sum (true = sum - comp).
__device__ __forceinline__ void kahan_add(float2 &sum, float2 &comp, float2 v)
{
    const float yr = v.x - comp.x, yi = v.y - comp.y;
    const float tr = sum.x + yr, ti = sum.y + yi;
    comp.x = (tr - sum.x) - yr;
    comp.y = (ti - sum.y) - yi;
    sum.x = tr;
    sum.y = ti;
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
#if TDC_FOCUS_SWAP
        tr = fmaf(p[k - 1].x, xr, tr);
        ti = fmaf(p[k - 1].y, xr, ti);
        tr = fmaf(p[k - 1].y, -xi, tr);
        ti = fmaf(p[k - 1].x, xi, ti);
#else
        tr = fmaf(xr, p[k - 1].x, tr);
        tr = fmaf(-xi, p[k - 1].y, tr);
        ti = fmaf(xr, p[k - 1].y, ti);
        ti = fmaf(xi, p[k - 1].x, ti);
#endif
    }
    return make_float2(tr, ti);
}

// Range of one (pixel, chirp) in double-float and its chirp-level weight: the skip weight
// times the Doppler window at the chirp's record.
__device__ __forceinline__ void chirp_range(const ChirpRec &r, float txh, float tyh, float tzh, float txl, float tyl,
                                            float tzl, float wskip, float tol, float half_bw, float inv_bw,
                                            bool taper, float az_a, float &rh, float &rl, float &w)
{
    float dxh, dxl, dyh, dyl, dzh, dzl;
    dd_sub(r.p_hi.x, r.p_lo.x, txh, txl, dxh, dxl);
    dd_sub(r.p_hi.y, r.p_lo.y, tyh, tyl, dyh, dyl);
    dd_sub(r.p_hi.z, r.p_lo.z, tzh, tzl, dzh, dzl);
    float rs, dh;
    dd_range(dxh, dxl, dyh, dyl, dzh, dzl, rh, rl, rs, dh);
    const float fd = doppler_freq(tol, r.vel.x, r.vel.y, r.vel.z, dxh, dyh, dzh, rs);
    w = wskip * doppler_window(fd, r.p_hi.w, half_bw, inv_bw, taper, az_a);
}

// Phase terms of one (pixel, chirp) from its double-float range R = rh + rl: the in-block
// phasors p_k = e^{j 2 pi k beta} (k = 1..L-1, beta = g1 R cycles per sample, reduced
// modulo 1), the block step QL = e^{j 2 pi L beta} from an accurate sincospif, and the
// weighted start phasor q0 = w e^{j 2 pi alpha}, alpha = frac(g0 R).
__device__ __forceinline__ void chirp_phasors(float rh, float rl, float g0h, float g0l, float g1, float g1l, float w,
                                              float2 (&p)[kL - 1], float2 &ql, float2 &q0)
{
    const float alpha = dd_frac_mul(g0h, g0l, rh, rl);
    float bh = g1 * rh;
    float bl = fmaf(g1, rh, -bh);
    bl = fmaf(g1, rl, bl);
    bl = fmaf(g1l, rh, bl);
    bh -= rintf(bh);
    float s1, c1s;
    __sincosf(kTwoPiF * (bh + bl), &s1, &c1s);
    p[0] = make_float2(c1s, s1);
#pragma unroll
    for (int k = 1; k < kL - 1; ++k) p[k] = cmul(p[k - 1], p[0]);
    const float lbh = (float)kL * bh;  // exact
    const float lfr = (lbh - rintf(lbh)) + (float)kL * bl;
    float sl, cl;
    sincospif(2.0f * lfr, &sl, &cl);
    ql = make_float2(cl, sl);
    float sa, ca;
    __sincosf(kTwoPiF * alpha, &sa, &ca);
    q0 = make_float2(w * ca, w * sa);
}

// Anchor record of one (chirp, anchor): e = antenna - anchor, R0 (both rounded to FP32),
// alpha0 = frac(g0 R0), beta0 = frac(g1 R0) and QL0 = e^{j 2 pi L beta0}, from double-float R0.
__device__ __forceinline__ void anchor_record(const ChirpRec &r, const float *A, float g0h, float g0l, float g1,
                                              float g1l, float4 &rec0, float4 &rec1)
{
    float exh, exl, eyh, eyl, ezh, ezl;
    dd_sub(r.p_hi.x, r.p_lo.x, A[0], A[3], exh, exl);
    dd_sub(r.p_hi.y, r.p_lo.y, A[1], A[4], eyh, eyl);
    dd_sub(r.p_hi.z, r.p_lo.z, A[2], A[5], ezh, ezl);
    float rh, rl, rs, dh;
    dd_range(exh, exl, eyh, eyl, ezh, ezl, rh, rl, rs, dh);
    const float alpha0 = dd_frac_mul(g0h, g0l, rh, rl);
    float bh = g1 * rh;
    float bl = fmaf(g1, rh, -bh);
    bl = fmaf(g1, rl, bl);
    bl = fmaf(g1l, rh, bl);
    bh -= rintf(bh);
    const float lbh = (float)kL * bh;  // exact
    const float lfr = (lbh - rintf(lbh)) + (float)kL * bl;
    float sl, cl;
    sincospif(2.0f * lfr, &sl, &cl);
    rec0 = make_float4(exh + exl, eyh + eyl, ezh + ezl, rh + rl);
    rec1 = make_float4(alpha0, bh + bl, cl, sl);
}

// Pixel of a unit's slot (valid when unit_pixel_ok). Block tiles come with a finite band,
// i.e. with the SKIP_ZERO instances; the unbounded-band instances map slots to flat tiles
// only (p >= P past the grid's end).
template <bool BLOCK_TILES>
__device__ __forceinline__ long long unit_pixel(const FocusJob &J, long long P, int tile, int slot)
{
    if (BLOCK_TILES) return tile_pixel(J.tile_cols, J.grid_cols, P, tile, slot);
    return (long long)tile * kFocusTile + slot;
}

template <bool BLOCK_TILES>
__device__ __forceinline__ bool unit_pixel_ok(long long p, long long P)
{
    return BLOCK_TILES ? p >= 0 : p < P;
}

// SKIP_ZERO: chirps whose window is zero for a whole warp skip the Horner loop (launched
// when a job's Doppler band is finite; with an unbounded band no window is zero, and the
// plain instance keeps the hot loop's schedule).
// STORE: also write each (pixel, chirp) sum A = sum_s x_s z^s (before the start phasor q0) to
// job.chirp_sums[c][p], zero for chirps skipped by the window vote (the adjoint reads them).
// ANCHOR: anchored ranges (SharedAnchor); flat tiles and an unbounded band only, stages of at
// most kAnchorMaxStageChirps chirps, pixels within the host's anchor distance bound.
template <bool SKIP_ZERO, bool STORE, bool ANCHOR>
__device__ __forceinline__ void focus_fp32_body(const FocusJob *__restrict__ jobs, const FocusUnit *__restrict__ units,
                                                int n_units, int *__restrict__ counter, int *__restrict__ status,
                                                int stage_bytes)
{
    static_assert(!ANCHOR || (!SKIP_ZERO && !STORE), "anchored ranges: plain instance only");
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t full_bar[kFocusStages];
    __shared__ int s_unit;
    __shared__ FocusJob sJ;

    SharedPixel &sp = *reinterpret_cast<SharedPixel *>(smem + kFocusStages * stage_bytes);
    SharedAnchor &sa = *reinterpret_cast<SharedAnchor *>(smem + kFocusStages * stage_bytes);

    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;

    if (tid == 0) {
        for (int i = 0; i < kFocusStages; ++i) mbar_init(&full_bar[i], 1);
        fence_barrier_init();
    }
    __syncthreads();

    uint32_t n_issued = 0;    // producer (thread 0) only
    uint32_t n_consumed = 0;  // uniform across the CTA

    for (;;) {
        if (tid == 0) {
            s_unit = atomicAdd(counter, 1);
        }
        __syncthreads();
        const int u = s_unit;
        if (u >= n_units) break;
        const FocusUnit un = units[u];
        if (tid < (int)(sizeof(FocusJob) / sizeof(int))) {
            reinterpret_cast<int *>(&sJ)[tid] = reinterpret_cast<const int *>(&jobs[un.job])[tid];
        }
        __syncthreads();

        const int C = sJ.C;
        int c0 = un.group * sJ.chirps_per_group;
        int c1 = min(C, c0 + sJ.chirps_per_group);
        if (!STORE && un.span) {
            // the chirps of the group that the tile may see in band (the rest are out of band
            // for all its pixels; the storing instance writes every chirp's sum, so it takes all)
            c1 = min(c1, c0 + unit_span_hi(un.span));
            c0 += unit_span_lo(un.span);
        }
        const int CB = sJ.stage_chirps;
        const int nblk = c1 > c0 ? (c1 - c0 + CB - 1) / CB : 0;
        const int s_pad = sJ.s_pad;
        const uint32_t row_bytes = static_cast<uint32_t>(s_pad) * 8u;
        const float4 *__restrict__ xw = sJ.xw;
        const ChirpRec *__restrict__ chirps = sJ.chirps;

        if (ANCHOR && kFocusPT * CB > kAnchorRecs) {
            // more anchor records a stage than the shared buffer holds (the host never plans
            // this): report, before any copy of this unit is issued
            if (tid == 0) atomicOr(status, kStatusBadJob);
            break;
        }

        // Producer: issue the first stages of this unit (every warp is past the previous
        // unit's last stage: the buffers are free).
        if (tid == 0) {
            fence_proxy_async_smem();
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

        const long long P = sJ.P;
        if constexpr (ANCHOR) {
            // Anchor of slot i (lane i): the 17th pixel of the warp's 32, or the last inside the
            // grid; none for 32 pixels wholly past the grid's end.
            if (lane < kFocusPT) {
                const int i = lane;
                const long long base = (long long)un.tile * kFocusTile + i * kFocusThreads + warp * 32;
                const long long n_valid = min(32LL, P - base);
                float4 hi = make_float4(0.f, 0.f, 0.f, 0.f), lo = hi;
                if (n_valid > 0) {
                    const long long a = base + min(16LL, n_valid - 1);
                    hi = __ldg(&sJ.grid_hi[a]);
                    if (sJ.grid_lo) lo = __ldg(&sJ.grid_lo[a]);
                }
                float *A = sa.anc[warp][lane];
                A[0] = hi.x;
                A[1] = hi.y;
                A[2] = hi.z;
                A[3] = lo.x;
                A[4] = lo.y;
                A[5] = lo.z;
            }
            __syncwarp();
#pragma unroll
            for (int i = 0; i < kFocusPT; ++i) {
                const long long p = (long long)un.tile * kFocusTile + i * kFocusThreads + tid;
                float4 dv = make_float4(0.f, 0.f, 0.f, 0.f);
                if (p < P) {
                    const float4 hi = __ldg(&sJ.grid_hi[p]);
                    const float4 lo = sJ.grid_lo ? __ldg(&sJ.grid_lo[p]) : make_float4(0.f, 0.f, 0.f, 0.f);
                    const float *A = sa.anc[warp][i];
                    dv = make_float4((hi.x - A[0]) + (lo.x - A[3]), (hi.y - A[1]) + (lo.y - A[4]),
                                     (hi.z - A[2]) + (lo.z - A[5]), 0.f);
                }
                sa.d[i][tid] = dv;
            }
        } else {
            // Pixel coordinates of this thread's PT slots -> shared (own column).
#pragma unroll
            for (int i = 0; i < kFocusPT; ++i) {
                const long long p = unit_pixel<SKIP_ZERO>(sJ, P, un.tile, i * kFocusThreads + tid);
                float4 hi = make_float4(0.f, 0.f, 0.f, 0.f), lo = hi;
                if (unit_pixel_ok<SKIP_ZERO>(p, P)) {
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
        }

        const float g0h = sJ.g0_hi, g0l = sJ.g0_lo, g1 = sJ.g1;
        const float g1l = sJ.g1_lo;
        const float kql = kTwoPiF * (float)kL * g1;  // block step phase per metre of dR (anchored)
        const float tol = sJ.two_over_lambda, half_bw = sJ.half_bw, inv_bw = sJ.inv_bw, az_a = sJ.az_a;
        const bool taper = (sJ.flags & kFlagTaper) != 0;
        const bool skip_test = (sJ.flags & kFlagSkipTest) != 0;
        const int chunk = sJ.chunk;
        const SkipPoint *__restrict__ skip = sJ.skip;
        const int nb = s_pad / kL;

        float2 sum[kFocusPT], comp[kFocusPT];
        float wskip[kFocusPT];
#pragma unroll
        for (int i = 0; i < kFocusPT; ++i) {
            sum[i] = make_float2(0.f, 0.f);
            comp[i] = make_float2(0.f, 0.f);
            wskip[i] = 1.0f;
        }
        static_assert(kFocusPT == 4, "store_sums takes four pixel slots");
        auto store_sums = [&](int c, float2 a0, float2 a1, float2 a2, float2 a3) {
            const float2 a[4] = {a0, a1, a2, a3};
            float2 *__restrict__ out = sJ.chirp_sums + (size_t)c * P;
#pragma unroll
            for (int i = 0; i < kFocusPT; ++i) {
                const long long px = unit_pixel<SKIP_ZERO>(sJ, P, un.tile, i * kFocusThreads + tid);
                if (unit_pixel_ok<SKIP_ZERO>(px, P)) out[px] = a[i];
            }
        };
        int chunk_end = 0;  // first chirp past the skip-test chunk of wskip
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
            float2 ssum[kFocusPT];  // this stage's chirp sums (anchored instance)
#pragma unroll
            for (int i = 0; i < kFocusPT; ++i) ssum[i] = make_float2(0.f, 0.f);

            if constexpr (ANCHOR) {
                // The stage's anchor records for this warp, record k = chirp x 4 + slot, from the
                // staged chirp records. (Forming several stages' records at a time from the
                // records in global memory measured 2-3.5% slower, every warp of the CTA waiting
                // on those loads; one warp in turn forming the whole CTA's a stage ahead did not
                // make rows of 1-2 chirps a stage pay either.)
                for (int k = lane; k < kFocusPT * cnt; k += 32)
                    anchor_record(recs[k >> 2], sa.anc[warp][k & (kFocusPT - 1)], g0h, g0l, g1, g1l,
                                  sa.rec[warp][k][0], sa.rec[warp][k][1]);
                __syncwarp();
            }

            for (int cc = 0; cc < cnt; ++cc) {
                const int c = cb0 + cc;
                if (skip_test && c >= chunk_end) {
                    // (chirps of a unit come in increasing order)
                    const int k = c / chunk;
                    chunk_end = (k + 1) * chunk;
                    {
#pragma unroll
                        for (int i = 0; i < kFocusPT; ++i) {
                            float tx, ty, tz;
                            if constexpr (ANCHOR) {
                                // (the anchored instance keeps no pixel coordinates in shared memory)
                                const long long px = (long long)un.tile * kFocusTile + i * kFocusThreads + tid;
                                const float4 hi = px < P ? __ldg(&sJ.grid_hi[px]) : make_float4(0.f, 0.f, 0.f, 0.f);
                                tx = hi.x;
                                ty = hi.y;
                                tz = hi.z;
                            } else {
                                tx = sp.t[i * 6 + 0][tid];
                                ty = sp.t[i * 6 + 1][tid];
                                tz = sp.t[i * 6 + 2][tid];
                            }
                            wskip[i] = chunk_is_nonzero(skip + (size_t)k * 9, tx, ty, tz, tol, half_bw) ? 1.0f : 0.0f;
                        }
                    }
                }
                const ChirpRec r = recs[cc];
                const float4 *xs = xs_stage + (size_t)cc * (s_pad / 2);

                float2 p[kFocusPT][kL - 1];
                float2 ql[kFocusPT], q0[kFocusPT], h[kFocusPT];
                if constexpr (ANCHOR) {
#pragma unroll
                    for (int i = 0; i < kFocusPT; ++i) {
                        const float4 dd = sa.d[i][tid];
                        const int k = cc * kFocusPT + i;
                        const float4 e = sa.rec[warp][k][0], a1 = sa.rec[warp][k][1];
                        // antenna - pixel, and R^2 - R0^2 = d.(d - 2e)
                        const float dvx = e.x - dd.x, dvy = e.y - dd.y, dvz = e.z - dd.z;
                        float num = dd.x * fmaf(-2.0f, e.x, dd.x);
                        num = fmaf(dd.y, fmaf(-2.0f, e.y, dd.y), num);
                        num = fmaf(dd.z, fmaf(-2.0f, e.z, dd.z), num);
                        const float r2 = fmaf(dvx, dvx, fmaf(dvy, dvy, dvz * dvz));
                        const float rs = rsqrtf(r2);
                        const float rr = r2 > 0.0f ? r2 * rs : 0.0f;
                        const float den = e.w + rr;
                        const float dr = den > 0.0f ? __fdividef(num, den) : 0.0f;
                        const float w = r2 > 0.0f ? wskip[i] : 0.0f;
                        // start phase alpha0 + g0 dR modulo one cycle: g0h dR less its nearest integer
                        // in one rounding (|.| <= 1/2), then alpha0 and g0's low part
                        float a = fmaf(g0h, dr, -rintf(g0h * dr)) + a1.x;
                        a = fmaf(g0l, dr, a);
                        a -= rintf(a);
                        float sa0, ca0;
                        __sincosf(kTwoPiF * a, &sa0, &ca0);
                        q0[i] = make_float2(w * ca0, w * sa0);
                        float s1, c1s;
                        __sincosf(kTwoPiF * fmaf(g1, dr, a1.y), &s1, &c1s);
                        p[i][0] = make_float2(c1s, s1);
#pragma unroll
                        for (int q = 1; q < kL - 1; ++q) p[i][q] = cmul(p[i][q - 1], p[i][0]);
                        ql[i] = cmul(make_float2(a1.z, a1.w), sincos_anchor(kql * dr));
                        h[i] = make_float2(0.f, 0.f);
                    }
                } else if (SKIP_ZERO && kEarlyVote) {
                    // Ranges and windows first: a chirp whose window (Doppler band, skip test) is
                    // zero for every pixel of the warp contributes nothing, and skips the phase
                    // set-up as well as the Horner loop.
                    float rh[kFocusPT], rl[kFocusPT], w[kFocusPT];
                    bool live = false;
#pragma unroll
                    for (int i = 0; i < kFocusPT; ++i) {
                        chirp_range(r, sp.t[i * 6 + 0][tid], sp.t[i * 6 + 1][tid], sp.t[i * 6 + 2][tid],
                                    sp.t[i * 6 + 3][tid], sp.t[i * 6 + 4][tid], sp.t[i * 6 + 5][tid], wskip[i],
                                    tol, half_bw, inv_bw, taper, az_a, rh[i], rl[i], w[i]);
                        live |= w[i] != 0.0f;
                    }
                    if (!__any_sync(0xffffffffu, live)) {
                        if (STORE) store_sums(c, make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f),
                                              make_float2(0.f, 0.f));
                        continue;
                    }
#pragma unroll
                    for (int i = 0; i < kFocusPT; ++i) {
                        chirp_phasors(rh[i], rl[i], g0h, g0l, g1, g1l, w[i], p[i], ql[i], q0[i]);
                        h[i] = make_float2(0.f, 0.f);
                    }
                } else {
                    // One pass per pixel, in this order (the unbounded-band instance's schedule:
                    // other orders of the same operations measured 0.5-3% slower).
                    bool live = false;
#pragma unroll
                    for (int i = 0; i < kFocusPT; ++i) {
                        float dxh, dxl, dyh, dyl, dzh, dzl;
                        dd_sub(r.p_hi.x, r.p_lo.x, sp.t[i * 6 + 0][tid], sp.t[i * 6 + 3][tid], dxh, dxl);
                        dd_sub(r.p_hi.y, r.p_lo.y, sp.t[i * 6 + 1][tid], sp.t[i * 6 + 4][tid], dyh, dyl);
                        dd_sub(r.p_hi.z, r.p_lo.z, sp.t[i * 6 + 2][tid], sp.t[i * 6 + 5][tid], dzh, dzl);
                        float rh, rl, rs, dh;
                        dd_range(dxh, dxl, dyh, dyl, dzh, dzl, rh, rl, rs, dh);
                        const float alpha = dd_frac_mul(g0h, g0l, rh, rl);
                        // beta = (g1 + g1l) * (rh + rl) cycles per sample, reduced modulo 1.
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
                        const float lbh = (float)kL * bh;  // exact
                        const float lfr = (lbh - rintf(lbh)) + (float)kL * bl;
                        float sl, cl;
                        sincospif(2.0f * lfr, &sl, &cl);
                        ql[i] = make_float2(cl, sl);
                        const float fd = doppler_freq(tol, r.vel.x, r.vel.y, r.vel.z, dxh, dyh, dzh, rs);
                        const float w = wskip[i] * doppler_window(fd, r.p_hi.w, half_bw, inv_bw, taper, az_a);
                        if (SKIP_ZERO) live |= w != 0.0f;
                        float sa, ca;
                        __sincosf(kTwoPiF * alpha, &sa, &ca);
                        q0[i] = make_float2(w * ca, w * sa);
                        h[i] = make_float2(0.f, 0.f);
                    }
                    if (SKIP_ZERO && !__any_sync(0xffffffffu, live)) {
                        if (STORE) store_sums(c, make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f),
                                              make_float2(0.f, 0.f));
                        continue;
                    }
                }

                // Horner over blocks, last block first.
#pragma unroll kUnrollBlocks
                for (int b = nb - 1; b >= 0; --b) {
                    float4 xv[kL / 2];
#pragma unroll
                    for (int m = 0; m < kL / 2; ++m) xv[m] = xs[b * (kL / 2) + m];
#pragma unroll
                    for (int i = 0; i < kFocusPT; ++i) h[i] = horner_block(h[i], ql[i], p[i], xv);
                }

                if (STORE) store_sums(c, h[0], h[1], h[2], h[3]);
                if constexpr (ANCHOR && kAnchorStageSums) {
#pragma unroll
                    for (int i = 0; i < kFocusPT; ++i) {
                        ssum[i].x = fmaf(q0[i].x, h[i].x, ssum[i].x);
                        ssum[i].x = fmaf(-q0[i].y, h[i].y, ssum[i].x);
                        ssum[i].y = fmaf(q0[i].x, h[i].y, ssum[i].y);
                        ssum[i].y = fmaf(q0[i].y, h[i].x, ssum[i].y);
                    }
                } else {
#pragma unroll
                    for (int i = 0; i < kFocusPT; ++i) kahan_add(sum[i], comp[i], cmul(q0[i], h[i]));
                }
            }
            if constexpr (ANCHOR && kAnchorStageSums) {
#pragma unroll
                for (int i = 0; i < kFocusPT; ++i) kahan_add(sum[i], comp[i], ssum[i]);
            }

            __syncthreads();  // every thread is done with this stage
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
            // Let the copies still in flight land before the CTA exits, then report.
            if (tid == 0) {
                for (uint32_t k = n_consumed; k < n_issued; ++k) {
                    mbar_wait_bounded(&full_bar[k % kFocusStages], (k / kFocusStages) & 1u, kWaitLimitNs);
                }
                atomicOr(status, kStatusTimeout);
            }
            __syncthreads();
            return;
        }

        float4 *__restrict__ part = sJ.partial + (size_t)un.group * P;
#pragma unroll
        for (int i = 0; i < kFocusPT; ++i) {
            const long long pidx = unit_pixel<SKIP_ZERO>(sJ, P, un.tile, i * kFocusThreads + tid);
            if (unit_pixel_ok<SKIP_ZERO>(pidx, P)) part[pidx] = make_float4(sum[i].x, sum[i].y, comp[i].x, comp[i].y);
        }
        __syncthreads();  // sJ / sp are rewritten by the next unit
    }
}

template <bool SKIP_ZERO, bool STORE>
__global__ void __launch_bounds__(kFocusThreads, TDC_FOCUS_MINB)
    focus_fp32_kernel(const FocusJob *__restrict__ jobs, const FocusUnit *__restrict__ units, int n_units,
                      int *__restrict__ counter, int *__restrict__ status, int stage_bytes)
{
    focus_fp32_body<SKIP_ZERO, STORE, false>(jobs, units, n_units, counter, status, stage_bytes);
}

// The anchored-range instance is a kernel of its own, so that its register budget can be set
// apart from the others' (TDC_ANCHOR_MAXNREG > 0: at most that many registers a thread).
#ifndef TDC_ANCHOR_MAXNREG
#define TDC_ANCHOR_MAXNREG 0
#endif
#if TDC_ANCHOR_MAXNREG > 0
__global__ void __maxnreg__(TDC_ANCHOR_MAXNREG)
#else
__global__ void __launch_bounds__(kFocusThreads, TDC_FOCUS_MINB)
#endif
    focus_fp32_anchored_kernel(const FocusJob *__restrict__ jobs, const FocusUnit *__restrict__ units, int n_units,
                               int *__restrict__ counter, int *__restrict__ status, int stage_bytes)
{
    focus_fp32_body<false, false, true>(jobs, units, n_units, counter, status, stage_bytes);
}

// Long chirps: the same focus with a chirp's samples staged in segments of
// job.seg_len samples (a row longer than the pipeline stages hold). Stages walk each
// chirp's segments last first, so the Horner state of the chirp carries from one
// segment to the next; the per-(pixel, chirp) set-up runs at the chirp's first staged
// segment, the Kahan accumulation after its segment 0.
template <bool SKIP_ZERO>
__global__ void __launch_bounds__(kFocusThreads, TDC_FOCUS_MINB)
    focus_fp32_seg_kernel(const FocusJob *__restrict__ jobs, const FocusUnit *__restrict__ units, int n_units,
                          int *__restrict__ counter, int *__restrict__ status, int stage_bytes)
{
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t full_bar[kFocusStages];
    __shared__ int s_unit;
    __shared__ FocusJob sJ;

    SharedPixel &sp = *reinterpret_cast<SharedPixel *>(smem + kFocusStages * stage_bytes);
    const int tid = threadIdx.x;
    if (tid == 0) {
        for (int i = 0; i < kFocusStages; ++i) mbar_init(&full_bar[i], 1);
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
        const int seg = sJ.seg_len;                 // samples per segment (multiple of 16)
        const int nseg = (s_pad + seg - 1) / seg;
        const int nstage = (c1 - c0) * nseg;
        const uint32_t seg_bytes = static_cast<uint32_t>(seg) * 8u;
        const float4 *__restrict__ xw = sJ.xw;
        const ChirpRec *__restrict__ chirps = sJ.chirps;

        // stage j: chirp c0 + j / nseg, segment nseg - 1 - j % nseg
        auto issue = [&](int j) {
            const int c = c0 + j / nseg;
            const int sg = nseg - 1 - j % nseg;
            const int off = sg * seg;
            const int len = min(seg, s_pad - off);
            const int st = n_issued % kFocusStages;
            unsigned char *base = smem + st * stage_bytes;
            const uint32_t bx = static_cast<uint32_t>(len) * 8u, br = (uint32_t)sizeof(ChirpRec);
            mbar_arrive_expect_tx(&full_bar[st], bx + br);
            bulk_g2s(base, xw + ((size_t)c * s_pad + off) / 2, bx, &full_bar[st]);
            bulk_g2s(base + seg_bytes, chirps + c, br, &full_bar[st]);
            ++n_issued;
        };
        if (tid == 0) {
            fence_proxy_async_smem();
            const int npro = nstage < kFocusStages ? nstage : kFocusStages;
            for (int j = 0; j < npro; ++j) issue(j);
        }

        const long long P = sJ.P;
#pragma unroll
        for (int i = 0; i < kFocusPT; ++i) {
            const long long p = unit_pixel<SKIP_ZERO>(sJ, P, un.tile, i * kFocusThreads + tid);
            float4 hi = make_float4(0.f, 0.f, 0.f, 0.f), lo = hi;
            if (unit_pixel_ok<SKIP_ZERO>(p, P)) {
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

        float2 sum[kFocusPT], comp[kFocusPT];
        float wskip[kFocusPT];
#pragma unroll
        for (int i = 0; i < kFocusPT; ++i) {
            sum[i] = make_float2(0.f, 0.f);
            comp[i] = make_float2(0.f, 0.f);
            wskip[i] = 1.0f;
        }
        float2 p[kFocusPT][kL - 1];
        float2 ql[kFocusPT], q0[kFocusPT], h[kFocusPT];
        bool live = true;
        int cur_chunk = -1;
        bool timed_out = false;

        for (int j = 0; j < nstage; ++j) {
            const int st = n_consumed % kFocusStages;
            const uint32_t parity = (n_consumed / kFocusStages) & 1u;
            const bool ok = mbar_wait_bounded(&full_bar[st], parity, kWaitLimitNs);
            if (__syncthreads_or(!ok)) {
                timed_out = true;
                break;
            }
            const unsigned char *base = smem + st * stage_bytes;
            const float4 *xs = reinterpret_cast<const float4 *>(base);
            const int c = c0 + j / nseg;
            const int sg = nseg - 1 - j % nseg;
            const int len = min(seg, s_pad - sg * seg);

            if (sg == nseg - 1) {
                // first staged segment of the chirp: skip weight, range, phase set-up
                if (skip_test) {
                    const int k = c / chunk;
                    if (k != cur_chunk) {
                        cur_chunk = k;
#pragma unroll
                        for (int i = 0; i < kFocusPT; ++i)
                            wskip[i] = chunk_is_nonzero(skip + (size_t)k * 9, sp.t[i * 6 + 0][tid],
                                                        sp.t[i * 6 + 1][tid], sp.t[i * 6 + 2][tid], tol, half_bw)
                                           ? 1.0f
                                           : 0.0f;
                    }
                }
                const ChirpRec r = *reinterpret_cast<const ChirpRec *>(base + seg_bytes);
                // (the phase terms are set up for every chirp: the state carried across a long
                // row's segments leaves no registers for voting before them)
                bool any = false;
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
                    const float lbh = (float)kL * bh;
                    const float lfr = (lbh - rintf(lbh)) + (float)kL * bl;
                    float sl, cl;
                    sincospif(2.0f * lfr, &sl, &cl);
                    ql[i] = make_float2(cl, sl);
                    const float fd = doppler_freq(tol, r.vel.x, r.vel.y, r.vel.z, dxh, dyh, dzh, rs);
                    const float w = wskip[i] * doppler_window(fd, r.p_hi.w, half_bw, inv_bw, taper, az_a);
                    any |= w != 0.0f;
                    float sa, ca;
                    __sincosf(kTwoPiF * alpha, &sa, &ca);
                    q0[i] = make_float2(w * ca, w * sa);
                    h[i] = make_float2(0.f, 0.f);
                }
                live = !SKIP_ZERO || __any_sync(0xffffffffu, any);
            }

            if (live) {
                // Horner over this segment's blocks, last block first
                for (int b = len / kL - 1; b >= 0; --b) {
                    float4 xv[kL / 2];
#pragma unroll
                    for (int m = 0; m < kL / 2; ++m) xv[m] = xs[b * (kL / 2) + m];
#pragma unroll
                    for (int i = 0; i < kFocusPT; ++i) h[i] = horner_block(h[i], ql[i], p[i], xv);
                }
                if (sg == 0) {
#pragma unroll
                    for (int i = 0; i < kFocusPT; ++i) {
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

            __syncthreads();  // every thread is done with this stage
            ++n_consumed;
            if (tid == 0 && j + kFocusStages < nstage) {
                fence_proxy_async_smem();
                issue(j + kFocusStages);
            }
        }

        if (timed_out) {
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
            const long long pidx = unit_pixel<SKIP_ZERO>(sJ, P, un.tile, i * kFocusThreads + tid);
            if (unit_pixel_ok<SKIP_ZERO>(pidx, P)) part[pidx] = make_float4(sum[i].x, sum[i].y, comp[i].x, comp[i].y);
        }
        __syncthreads();
    }
}

// image[p] = sum over groups of (sum - comp), added in FP64 in group order.
__global__ void focus_reduce_kernel(const float4 *__restrict__ partial, int n_groups, long long P,
                                    float2 *__restrict__ image)
{
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    double re = 0.0, im = 0.0;
    for (int g = 0; g < n_groups; ++g) {
        const float4 v = partial[(size_t)g * P + p];
        re += (double)v.x - (double)v.z;
        im += (double)v.y - (double)v.w;
    }
    image[p] = make_float2((float)re, (float)im);
}

}  // namespace

int focus_fp32_smem_bytes(int stage_bytes, bool anchored)
{
    return kFocusStages * stage_bytes + (int)(anchored ? sizeof(SharedAnchor) : sizeof(SharedPixel));
}

int focus_fp32_anchor_blocks_per_sm(int stage_bytes)
{
    const int smem = focus_fp32_smem_bytes(stage_bytes, true);
    int blocks = 0;
    if (allow_max_dynamic_smem(focus_fp32_anchored_kernel) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, focus_fp32_anchored_kernel, kFocusThreads,
                                                      smem) != cudaSuccess)
        return 0;
    return blocks;
}

int focus_fp32_blocks_per_sm(int stage_bytes)
{
    const int smem = focus_fp32_smem_bytes(stage_bytes, false);
    int best = 1 << 30;
    for (auto fn : {focus_fp32_kernel<false, false>, focus_fp32_kernel<true, false>, focus_fp32_kernel<false, true>,
                    focus_fp32_kernel<true, true>}) {
        int blocks = 0;
        if (allow_max_dynamic_smem(fn) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, kFocusThreads, smem) != cudaSuccess)
            return 0;
        best = blocks < best ? blocks : best;
    }
    return best;
}

cudaError_t launch_focus_fp32(const FocusJob *jobs_dev, const FocusUnit *units_dev, int n_units, int *counter_dev,
                              int *status_dev, int stage_bytes, int grid_ctas, bool skip_zero, bool store_sums,
                              bool anchored, cudaStream_t st)
{
    if (anchored && (skip_zero || store_sums)) return cudaErrorInvalidValue;
    const int smem = focus_fp32_smem_bytes(stage_bytes, anchored);
    using Fn = void (*)(const FocusJob *, const FocusUnit *, int, int *, int *, int);
    const Fn fn = anchored    ? focus_fp32_anchored_kernel
                  : skip_zero ? (store_sums ? focus_fp32_kernel<true, true> : focus_fp32_kernel<true, false>)
                              : (store_sums ? focus_fp32_kernel<false, true> : focus_fp32_kernel<false, false>);
    cudaError_t e = allow_max_dynamic_smem(fn);
    if (e != cudaSuccess) return e;
    fn<<<grid_ctas, kFocusThreads, smem, st>>>(jobs_dev, units_dev, n_units, counter_dev, status_dev, stage_bytes);
    return cudaGetLastError();
}

int focus_fp32_seg_blocks_per_sm(int stage_bytes)
{
    const int smem = focus_fp32_smem_bytes(stage_bytes, false);
    int blocks = 0, blocks_skip = 0;
    if (allow_max_dynamic_smem(focus_fp32_seg_kernel<false>) != cudaSuccess ||
        allow_max_dynamic_smem(focus_fp32_seg_kernel<true>) != cudaSuccess)
        return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, focus_fp32_seg_kernel<false>, kFocusThreads, smem) !=
            cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_skip, focus_fp32_seg_kernel<true>, kFocusThreads,
                                                      smem) != cudaSuccess)
        return 0;
    return blocks < blocks_skip ? blocks : blocks_skip;
}

cudaError_t launch_focus_fp32_seg(const FocusJob *jobs_dev, const FocusUnit *units_dev, int n_units,
                                  int *counter_dev, int *status_dev, int stage_bytes, int grid_ctas, bool skip_zero,
                                  cudaStream_t st)
{
    const int smem = focus_fp32_smem_bytes(stage_bytes, false);
    cudaError_t e = skip_zero ? allow_max_dynamic_smem(focus_fp32_seg_kernel<true>)
                              : allow_max_dynamic_smem(focus_fp32_seg_kernel<false>);
    if (e != cudaSuccess) return e;
    if (skip_zero)
        focus_fp32_seg_kernel<true><<<grid_ctas, kFocusThreads, smem, st>>>(jobs_dev, units_dev, n_units,
                                                                             counter_dev, status_dev, stage_bytes);
    else
        focus_fp32_seg_kernel<false><<<grid_ctas, kFocusThreads, smem, st>>>(jobs_dev, units_dev, n_units,
                                                                              counter_dev, status_dev, stage_bytes);
    return cudaGetLastError();
}

cudaError_t launch_focus_reduce(const float4 *partial, int n_groups, long long P, float2 *image, cudaStream_t st)
{
    if (P <= 0) return cudaSuccess;
    const int threads = 256;
    const long long blocks = (P + threads - 1) / threads;
    focus_reduce_kernel<<<(unsigned)blocks, threads, 0, st>>>(partial, n_groups, P, image);
    return cudaGetLastError();
}

}  // namespace tdc
