// tdc_capi.cpp -- host side of the GB300 TDC engine behind the C ABI of
// include/tdc_gb300.h: the processor (TdcProcessor's contract,
// tdc-lib/src/tdcprocessor.cpp:39-243), input analysis, the device-resident
// acquisition, work planning and kernel launches.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <string>
#include <thread>
#include <vector>

#include "tdc_gb300.h"
#include "tdc_internal.h"
#include "tdc_processor_impl.h"

using namespace tdc;

namespace tdc {
namespace impl {

thread_local std::string g_err;

int fail(int code, const std::string &msg)
{
    g_err = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char *what)
{
    return fail(e == cudaErrorMemoryAllocation ? TDC_ERR_NO_MEMORY : TDC_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}





// ---- host FP32 math with the reference's semantics (gpumath.h, windowing.h) ----
// Quaternions (a, b, c, d) = (w, x, y, z).
void q_prod_f(const float *a, const float *b, float *o)
{
    const float r0 = (a[0] * b[0]) - (a[1] * b[1]) - (a[2] * b[2]) - (a[3] * b[3]);
    const float r1 = (a[0] * b[1]) + (a[1] * b[0]) + (a[2] * b[3]) - (a[3] * b[2]);
    const float r2 = (a[0] * b[2]) - (a[1] * b[3]) + (a[2] * b[0]) + (a[3] * b[1]);
    const float r3 = (a[0] * b[3]) + (a[1] * b[2]) - (a[2] * b[1]) + (a[3] * b[0]);
    o[0] = r0;
    o[1] = r1;
    o[2] = r2;
    o[3] = r3;
}

void q_rot_f(const float *q, const float *v, float *o)
{
    const float vq[4] = {0.f, v[0], v[1], v[2]};
    const float qc[4] = {q[0], -q[1], -q[2], -q[3]};
    float t[4], r[4];
    q_prod_f(q, vq, t);
    q_prod_f(t, qc, r);
    o[0] = r[1];
    o[1] = r[2];
    o[2] = r[3];
}

// Doppler window centre of one trajectory sample (tdckernels.cu:114-122).
float window_centre(const float *vel, const float *att, const float *bore, float lambda, bool centroid,
                    float fixed_centre)
{
    if (!centroid) return fixed_centre;
    float ant[3];
    q_rot_f(att, bore, ant);
    return 2.0f / lambda * ((vel[0] * ant[0]) + (vel[1] * ant[1]) + (vel[2] * ant[2]));
}



// Phase tolerance for treating the sample frequencies as affine in the sample index.
constexpr double kUniformPhaseTolRad = 1e-4;
// FP32 general kernel: largest |(R_s^2 - R0^2) / R0^2| its range-change series takes, and
// the bytes of chirp rows per pipeline stage it aims for.
constexpr double kGeneralMaxEps = 0.1;
constexpr double kGeneralNarrowEps = 0.02;
constexpr double kGeneralNarrowCycles = 4.0;
// Smooth-motion kernel: largest deviation of the per-sample phase correction from its
// per-segment linear model (chord + mean offset) [rad].
constexpr double kMotionTolRad = 2e-3;
// Work of one unit (tile x chirp group) the planner aims at in long launches [correlations]:
// a few milliseconds of a CTA's time (measured: 16-64 units per slot take 533 ms instead of
// 538.6 ms on 1024^2 x 4096 x 1024; at 4.5 ms launches more units cost 2-8%).
constexpr double kUnitTargetCorr = 64e6;
// Block tiles: kFocusTile / kBlockTileCols grid rows x kBlockTileCols columns.
#ifndef TDC_BLOCK_TILES
#define TDC_BLOCK_TILES 1
#endif
constexpr int kBlockTileCols = 16;
#ifndef TDC_GENERAL_STAGE_TARGET
#define TDC_GENERAL_STAGE_TARGET 32768
#endif
// 1: stage general-kernel rows in segments whenever a row exceeds the stage target (tuning)
#ifndef TDC_GENERAL_ALWAYS_SEGMENT
#define TDC_GENERAL_ALWAYS_SEGMENT 0
#endif
constexpr int kGeneralStageTarget = TDC_GENERAL_STAGE_TARGET;
// Long chirps: samples per staged segment when a whole row does not fit the bulk kernel's stages.
constexpr int kSegmentSamples = 2048;

}  // namespace impl
}  // namespace tdc

using namespace tdc::impl;


namespace tdc {
namespace impl {

int check_proc(const tdc_processor *p)
{
    if (!p) return fail(TDC_ERR_INVALID_ARGUMENT, "null processor");
    return TDC_OK;
}

// Trajectory constant within every chirp (bitwise), per array.
bool rows_constant(const float *a, int C, int S, int k)
{
    if (!a) return true;
    for (int c = 0; c < C; ++c) {
        const float *row = a + (size_t)c * S * k;
        for (int s = 1; s < S; ++s) {
            if (std::memcmp(row, row + (size_t)s * k, sizeof(float) * k) != 0) return false;
        }
    }
    return true;
}

// Least-squares affine fit f_s ~ F0 + F1 s of f_s = f0 + K t_s (FP64 on the FP32 inputs).
void fit_frequencies(const float *t, int S, float f0, float K, double &F0, double &F1, double &resid)
{
    std::vector<double> f(S);
    for (int s = 0; s < S; ++s) f[s] = (double)f0 + (double)K * (double)t[s];
    if (S == 1) {
        F0 = f[0];
        F1 = 0.0;
        resid = 0.0;
        return;
    }
    const double sm = 0.5 * (S - 1);
    double fm = 0.0;
    for (int s = 0; s < S; ++s) fm += f[s];
    fm /= S;
    double num = 0.0, den = 0.0;
    for (int s = 0; s < S; ++s) {
        num += (s - sm) * (f[s] - fm);
        den += (s - sm) * (s - sm);
    }
    F1 = num / den;
    F0 = fm - F1 * sm;
    resid = 0.0;
    for (int s = 0; s < S; ++s) resid = std::max(resid, std::fabs(f[s] - (F0 + F1 * s)));
}

double max_range(const double *amin, const double *amax, const double *gmin, const double *gmax)
{
    double r2 = 0.0;
    for (int k = 0; k < 3; ++k) {
        const double d = std::max(std::fabs(amax[k] - gmin[k]), std::fabs(gmax[k] - amin[k]));
        r2 += d * d;
    }
    return std::sqrt(r2);
}

void stats_reset(tdc_processor *p) { std::memset(&p->stats, 0, sizeof(p->stats)); }

// fn(thread, begin, end) over chirps [0, n) on up to 16 host threads, about 1M elements
// (chirps x per_item) or more per thread; returns the number of threads used.
template <class F>
int parallel_chirps(int n, long long per_item, F fn)
{
    const long long total = (long long)n * std::max(1LL, per_item);
    const long long hw = std::max(1u, std::min(std::thread::hardware_concurrency(), 16u));
    const int nt = (int)std::max(1LL, std::min({hw, total >> 20, (long long)n}));
    if (nt <= 1) {
        fn(0, 0, n);
        return 1;
    }
    std::vector<std::thread> pool;
    pool.reserve(nt);
    for (int t = 0; t < nt; ++t)
        pool.emplace_back(fn, t, (int)((long long)n * t / nt), (int)((long long)n * (t + 1) / nt));
    for (std::thread &th : pool) th.join();
    return nt;
}

const float kZero3[3] = {0.f, 0.f, 0.f};
const float kQId[4] = {1.f, 0.f, 0.f, 0.f};

// Trajectory record of (chirp c, sample s): position (double-float when FP64 positions
// are set), window centre, velocity.
ChirpRec make_record(const tdc_processor *p, int c, int s, bool centroid, float center)
{
    const size_t te = p->traj_per_chirp ? (size_t)c : (size_t)c * p->S + s;
    const float *vl = p->vel ? p->vel + 3 * te : kZero3;
    const float *at = p->att ? p->att + 4 * te : kQId;
    const float fdc = window_centre(vl, at, p->bore, p->lambda, centroid, center);
    float h[3], l[3];
    for (int k = 0; k < 3; ++k) {
        if (p->pos64) {
            split_dd(p->pos64[3 * (size_t)c + k], h[k], l[k]);
        } else {
            h[k] = p->pos[3 * te + k];
            l[k] = 0.f;
        }
    }
    ChirpRec r;
    r.p_hi = make_float4(h[0], h[1], h[2], fdc);
    r.p_lo = make_float4(l[0], l[1], l[2], 0.f);
    r.vel = make_float4(vl[0], vl[1], vl[2], 0.f);
    return r;
}

// Upload + prepare the acquisition for the given start() options.
int prepare(tdc_processor *p, const StartOpts &o, int &launches)
{
    NvtxRange nvtx("tdc prepare");
    if (!p->has_raw) return fail(TDC_ERR_STATE, "setRawData must be called before start()");
    const int C = p->C, S = p->S;
    TDC_CK(cudaSetDevice(p->device), "cudaSetDevice");
    const int s_pad = (int)round_up((size_t)S, kSampleAlign);
    cudaStream_t st = p->stream;

    // Where the device reads the caller's buffers in place, the raw rows are windowed
    // and padded on the GPU while the host analyses the trajectory (launched right
    // after the trajectory scan, which the host waits for through an event).
    auto window_raw_in_place = [&]() -> int {
        TDC_CK(p->xw.ensure((size_t)C * s_pad * 8), "alloc samples");
        TDC_CK(p->wr.ensure((size_t)S * 4), "alloc range window");
        TDC_CK(launch_range_window(p->wr.as<float>(), S, o.range_win, st), "range window kernel");
        TDC_CK(launch_prewindow_from(reinterpret_cast<const float2 *>(p->raw), p->wr.as<float>(), C, S, s_pad,
                                     p->xw.as<float2>(), st),
               "prewindow kernel");
        launches += 2;
        return TDC_OK;
    };

    // ---- host analysis ----
    // Trajectory element of (chirp c, sample s): per-sample arrays, or one row per chirp.
    const bool tpc = p->traj_per_chirp;
    auto ti = [tpc, S](long c, long s) -> size_t { return tpc ? (size_t)c : (size_t)c * S + s; };
    bool pos_differ = false, motion_differ = false;
    bool raw_windowed = false;
    if (tpc) {
        p->per_chirp = true;
    } else if (p->host_reads) {
        // The device reads the caller's per-sample arrays in place (coherent host access)
        // and reports whether any chirp's samples differ: flag[0] positions, flag[1] velocity
        // or attitude.
        TDC_CK(p->flag.ensure(64), "alloc flag");
        int *flag = p->flag.as<int>();
        TDC_CK(cudaMemsetAsync(flag, 0, 8, p->stream), "reset flag");
        if (!p->pos64) TDC_CK(launch_rows_differ(p->pos, C, S, 3, flag, p->stream), "scan kernel");
        if (p->vel) TDC_CK(launch_rows_differ(p->vel, C, S, 3, flag + 1, p->stream), "scan kernel");
        if (p->att) TDC_CK(launch_rows_differ(p->att, C, S, 4, flag + 1, p->stream), "scan kernel");
        int differ[2] = {0, 0};
        TDC_CK(cudaMemcpyAsync(differ, flag, 8, cudaMemcpyDeviceToHost, p->stream), "read flag");
        TDC_CK(cudaEventRecord(p->ev[5], p->stream), "event");
        if (int rc = window_raw_in_place()) return rc;
        raw_windowed = true;
        TDC_CK(cudaEventSynchronize(p->ev[5]), "scan sync");
        pos_differ = differ[0] != 0;
        motion_differ = differ[1] != 0;
        launches += (!p->pos64) + (p->vel != nullptr) + (p->att != nullptr);
    } else {
        pos_differ = !p->pos64 && !rows_constant(p->pos, C, S, 3);
        motion_differ = !rows_constant(p->vel, C, S, 3) || !rows_constant(p->att, C, S, 4);
    }
    if (!tpc) p->per_chirp = !pos_differ && !motion_differ;
    if (p->host_reads && !raw_windowed)
        if (int rc = window_raw_in_place()) return rc;
    fit_frequencies(p->sample_times, S, p->start_freq, p->mod_rate, p->F0, p->F1, p->resid_hz);
    for (int k = 0; k < 3; ++k) {
        p->ant_min[k] = std::numeric_limits<double>::infinity();
        p->ant_max[k] = -std::numeric_limits<double>::infinity();
    }
    std::vector<double> base((size_t)C * 3);
    for (int c = 0; c < C; ++c) {
        for (int k = 0; k < 3; ++k) {
            const double v = p->pos64 ? p->pos64[3 * (size_t)c + k] : (double)p->pos[3 * ti(c, 0) + k];
            base[3 * (size_t)c + k] = v;
            p->ant_min[k] = std::min(p->ant_min[k], v);
            p->ant_max[k] = std::max(p->ant_max[k], v);
        }
    }
    if (!p->per_chirp && p->pos && !p->pos64) {
        std::vector<double> box(16 * 6);
        const int nt = parallel_chirps(C, S, [&](int t, int c0, int c1) {
            double *b = &box[6 * t];
            for (int k = 0; k < 3; ++k) {
                b[k] = std::numeric_limits<double>::infinity();
                b[3 + k] = -std::numeric_limits<double>::infinity();
            }
            for (size_t i = (size_t)c0 * S; i < (size_t)c1 * S; ++i)
                for (int k = 0; k < 3; ++k) {
                    b[k] = std::min(b[k], (double)p->pos[3 * i + k]);
                    b[3 + k] = std::max(b[3 + k], (double)p->pos[3 * i + k]);
                }
        });
        for (int t = 0; t < nt; ++t)
            for (int k = 0; k < 3; ++k) {
                p->ant_min[k] = std::min(p->ant_min[k], box[6 * t + k]);
                p->ant_max[k] = std::max(p->ant_max[k], box[6 * t + 3 + k]);
            }
    }

    // ---- trajectory records: one per chirp (the record of sample 0 when the trajectory
    // varies within chirps; the FP64 general kernel's per-sample records are built only
    // when that kernel runs, see sample_records) ----
    std::vector<ChirpRec> recs(C);
    parallel_chirps(C, 1, [&](int, int cb, int ce) {
        for (int c = cb; c < ce; ++c) recs[c] = make_record(p, c, 0, o.centroid != 0, o.center);
    });
    p->sample_recs_ready = false;
    p->rec_host = recs;
    p->rec_finite = true;
    for (int c = 0; c < C; ++c)
        p->rec_finite = p->rec_finite && std::isfinite(recs[c].vel.x) && std::isfinite(recs[c].vel.y) &&
                        std::isfinite(recs[c].vel.z) && std::isfinite(recs[c].p_hi.w);
    {
        double v[3] = {0.0, 0.0, 0.0};
        for (int c = 0; c < C; ++c) {
            v[0] += recs[c].vel.x;
            v[1] += recs[c].vel.y;
            v[2] += recs[c].vel.z;
        }
        const double n = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        for (int k = 0; k < 3; ++k) p->vel_dir[k] = n > 0.0 ? v[k] / n : 0.0;
    }

    // ---- FP32 general path tables (per-sample trajectories / windows, non-uniform sampling) ----
    const double g0 = 2.0 * p->F0 / kC0, g1 = 2.0 * p->F1 / kC0;
    std::vector<float> gres(3 * (size_t)s_pad, 0.f);  // residuals, 2 f_s / c0, 2 pi x 2 f_s / c0
    for (int s = 0; s < S; ++s) {
        const double gsv = 2.0 * ((double)p->start_freq + (double)p->mod_rate * (double)p->sample_times[s]) / kC0;
        gres[s] = (float)(gsv - (g0 + g1 * s));
        gres[(size_t)s_pad + s] = (float)gsv;
        gres[2 * (size_t)s_pad + s] = (float)(2.0 * M_PI * gsv);
    }
    std::vector<float4> traj, wins;
    std::vector<float> wdot;
    p->traj_varies = pos_differ;
    p->delta_max = 0.0;
    bool any_velocity = false;
    if (!p->per_chirp && p->vel) {
        const size_t n = (size_t)C * (p->traj_per_chirp ? 1 : S) * 3;
        for (size_t i = 0; i < n && !any_velocity; ++i) any_velocity = p->vel[i] != 0.f;
    }
    // The window can change within a chirp when the band is finite and either the motion
    // varies per sample or a moving antenna's direction to the pixel does.
    p->win_varies = !p->per_chirp && std::isfinite(o.bw) && (motion_differ || (pos_differ && any_velocity));
    if (p->traj_varies) {
        traj.assign((size_t)C * s_pad, make_float4(0.f, 0.f, 0.f, 0.f));
        std::vector<double> d2(16, 0.0);
        const int nt = parallel_chirps(C, S, [&](int t, int cb, int ce) {
            double m = 0.0;
            for (int c = cb; c < ce; ++c) {
                const float *p0 = p->pos + 3 * ti(c, 0);
                for (int s = 0; s < S; ++s) {
                    const float *ps = p->pos + 3 * ti(c, s);
                    const double dx = (double)ps[0] - p0[0], dy = (double)ps[1] - p0[1], dz = (double)ps[2] - p0[2];
                    m = std::max(m, dx * dx + dy * dy + dz * dz);
                    traj[(size_t)c * s_pad + s] =
                        make_float4((float)dx, (float)dy, (float)dz, (float)(dx * dx + dy * dy + dz * dz));
                }
            }
            d2[t] = m;
        });
        p->delta_max = std::sqrt(*std::max_element(d2.begin(), d2.begin() + nt));
    }
    if (p->win_varies) {
        // In band units: velocity x (-2 / lambda) / B and window centre / B, so the kernel forms
        // (fDop - centre) / B with one dot product and one fused multiply-add. With positions
        // moving within chirps the kernel dots the velocity with 2 (P0 - T) and adds the
        // pixel-independent part u . D_s from its own table, so u is stored halved.
        const bool with_traj = p->traj_varies;
        wins.assign((size_t)C * s_pad, make_float4(0.f, 0.f, 0.f, 0.f));
        if (with_traj) wdot.assign((size_t)C * s_pad, 0.f);
        const double vs = -2.0 / (double)p->lambda / (double)o.bw, cs = 1.0 / (double)o.bw;
        const double us = with_traj ? 0.5 : 1.0;
        parallel_chirps(C, S, [&](int, int cb, int ce) {
            for (int c = cb; c < ce; ++c)
                for (int s = 0; s < S; ++s) {
                    const size_t i = (size_t)c * s_pad + s;
                    const ChirpRec r = make_record(p, c, s, o.centroid != 0, o.center);
                    const double ux = r.vel.x * vs, uy = r.vel.y * vs, uz = r.vel.z * vs;
                    wins[i] = make_float4((float)(us * ux), (float)(us * uy), (float)(us * uz), (float)(r.p_hi.w * cs));
                    if (with_traj) wdot[i] = (float)(ux * traj[i].x + uy * traj[i].y + uz * traj[i].z);
                }
        });
    }

    // ---- smooth intra-chirp motion (the smooth-motion kernel) ----
    // Least-squares fit of each chirp's D_s = P[c,s] - P[c,0] by V0 + V1 s + V2 s^2 (orthogonal
    // polynomials in the centred index); accepted when every sample's residual stays within two
    // ulp of the chirp's largest FP32 coordinate on that axis, i.e. what remains is the rounding
    // of the input (up to half an ulp per sample, spread a little further by the fit).
    std::vector<MotionRec> mrecs;
    p->motion_fit_ok = false;
    p->motion_v1max = p->motion_v2max = 0.0;
    if (p->traj_varies && !p->win_varies && S >= 3) {
        mrecs.resize(C);
        const double hs = 0.5 * (S - 1);
        double sxx = 0.0, m2 = 0.0, sqq = 0.0;
        for (int s = 0; s < S; ++s) m2 += (s - hs) * (s - hs);
        m2 /= S;
        for (int s = 0; s < S; ++s) {
            const double x = s - hs, q = x * x - m2;
            sxx += x * x;
            sqq += q * q;
        }
        std::vector<double> vmax(3 * 16, 0.0);
        std::vector<char> bad(16, 0);
        const int nt = parallel_chirps(C, S, [&](int t, int cb, int ce) {
            double v1m = 0.0, v2m = 0.0;
            bool fail_fit = false;
            for (int c = cb; c < ce && !fail_fit; ++c) {
                const float *p0 = p->pos + 3 * ti(c, 0);
                double V0[3], V1[3], V2[3];
                for (int k = 0; k < 3; ++k) {
                    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
                    for (int s = 0; s < S; ++s) {
                        const double y = (double)p->pos[3 * ti(c, s) + k] - (double)p0[k];
                        const double x = s - hs;
                        a0 += y;
                        a1 += y * x;
                        a2 += y * (x * x - m2);
                    }
                    a0 /= S;
                    a1 /= sxx;
                    a2 /= sqq;
                    V0[k] = a0 - a1 * hs + a2 * (hs * hs - m2);
                    V1[k] = a1 - 2.0 * a2 * hs;
                    V2[k] = a2;
                    float vmag = 0.f;
                    for (int s = 0; s < S; ++s) vmag = std::max(vmag, std::fabs(p->pos[3 * ti(c, s) + k]));
                    const double ulp = vmag > 0.f ? std::ldexp(1.0, std::ilogb(vmag) - 23) : 1e-38;
                    for (int s = 0; s < S && !fail_fit; ++s) {
                        const double y = (double)p->pos[3 * ti(c, s) + k] - (double)p0[k];
                        const double r = y - (V0[k] + s * (V1[k] + s * V2[k]));
                        if (!(std::fabs(r) <= 2.0 * ulp)) fail_fit = true;
                    }
                }
                if (fail_fit) break;
                const ChirpRec r0 = make_record(p, c, 0, o.centroid != 0, o.center);
                float h[3], l[3];
                for (int k = 0; k < 3; ++k) split_dd((double)p0[k] + V0[k], h[k], l[k]);
                MotionRec &m = mrecs[c];
                const double n1 = std::sqrt(V1[0] * V1[0] + V1[1] * V1[1] + V1[2] * V1[2]);
                const double n2 = std::sqrt(V2[0] * V2[0] + V2[1] * V2[1] + V2[2] * V2[2]);
                m.p_hi = make_float4(h[0], h[1], h[2], r0.p_hi.w);
                m.p_lo = make_float4(l[0], l[1], l[2], 0.f);
                m.vel = make_float4(r0.vel.x, r0.vel.y, r0.vel.z,
                                    (float)(2.0 * (V1[0] * V2[0] + V1[1] * V2[1] + V1[2] * V2[2])));
                m.v1 = make_float4((float)V1[0], (float)V1[1], (float)V1[2], (float)(n1 * n1));
                m.v2 = make_float4((float)V2[0], (float)V2[1], (float)V2[2], (float)(n2 * n2));
                v1m = std::max(v1m, n1);
                v2m = std::max(v2m, n2);
            }
            vmax[3 * t] = v1m;
            vmax[3 * t + 1] = v2m;
            bad[t] = fail_fit ? 1 : 0;
        });
        bool ok = true;
        for (int t = 0; t < nt; ++t) {
            ok = ok && !bad[t];
            p->motion_v1max = std::max(p->motion_v1max, vmax[3 * t]);
            p->motion_v2max = std::max(p->motion_v2max, vmax[3 * t + 1]);
        }
        p->motion_fit_ok = ok;
        if (!ok) mrecs.clear();
    }

    // ---- skip-test points (tdcprocessor.cpp:347-383, stale staging rows included) ----
    const int n_chunks = (C + kChunk - 1) / kChunk;
    std::vector<SkipPoint> skip((size_t)n_chunks * 9);
    {
        int rows[3], samples[3];
        for (int i = 0; i < 3; ++i) {
            rows[i] = std::max(i * (kChunk / 2) - 1, 0);
            samples[i] = std::max(i * (S / 2) - 1, 0);
        }
        for (int k = 0; k < n_chunks; ++k) {
            const long base_pri = (long)k * kChunk;
            const long valid = std::min<long>(kChunk, C - base_pri);
            for (int i = 0; i < 3; ++i) {
                long pri;
                if (rows[i] < valid) pri = base_pri + rows[i];
                else if (k == 0) pri = -1;  // never-written staging row: zeros
                else pri = base_pri - kChunk + rows[i];
                for (int j = 0; j < 3; ++j) {
                    SkipPoint sp;
                    if (pri < 0) {
                        const float zq[4] = {0.f, 0.f, 0.f, 0.f};
                        const float fdc = window_centre(kZero3, zq, p->bore, p->lambda, o.centroid != 0, o.center);
                        sp.pos_fdc = make_float4(0.f, 0.f, 0.f, fdc);
                        sp.vel = make_float4(0.f, 0.f, 0.f, 0.f);
                    } else {
                        const size_t e = ti(pri, samples[j]);
                        const float *ps = p->pos + 3 * e;
                        const float *vl = p->vel ? p->vel + 3 * e : kZero3;
                        const float *at = p->att ? p->att + 4 * e : kQId;
                        const float fdc = window_centre(vl, at, p->bore, p->lambda, o.centroid != 0, o.center);
                        sp.pos_fdc = make_float4(ps[0], ps[1], ps[2], fdc);
                        sp.vel = make_float4(vl[0], vl[1], vl[2], 0.f);
                    }
                    skip[(size_t)k * 9 + i * 3 + j] = sp;
                }
            }
        }
    }

    // ---- per-sample 2 f_s / c0 table (FP64 kernels) ----
    std::vector<double> gs(S);
    for (int s = 0; s < S; ++s)
        gs[s] = 2.0 * ((double)p->start_freq + (double)p->mod_rate * (double)p->sample_times[s]) / kC0;

    // ---- device buffers ----
    p->s_pad = s_pad;
    p->n_chunks = n_chunks;
    TDC_CK(p->xw.ensure((size_t)C * s_pad * 8), "alloc samples");
    TDC_CK(p->wr.ensure((size_t)S * 4), "alloc range window");
    // sample-0 records go to gen_rec when the trajectory varies within chirps (chirps then
    // holds the per-sample records of the FP64 general kernel, built on demand)
    DevBuf &rec_buf = p->per_chirp ? p->chirps : p->gen_rec;
    TDC_CK(rec_buf.ensure((size_t)C * sizeof(ChirpRec)), "alloc chirp records");
    TDC_CK(p->skip.ensure(skip.size() * sizeof(SkipPoint)), "alloc skip table");
    TDC_CK(p->gs.ensure((size_t)S * 8), "alloc frequency table");
    TDC_CK(p->pos_base.ensure((size_t)C * 3 * 8), "alloc base positions");

    if (!p->host_reads) {
        TDC_CK(cudaMemcpy2DAsync(p->xw.p, (size_t)s_pad * 8, p->raw, (size_t)S * 8, (size_t)S * 8, C,
                                 cudaMemcpyHostToDevice, st),
               "copy raw data");
    }
    TDC_CK(p->gres.ensure(gres.size() * 4), "alloc per-sample frequency tables");
    {
        // The small per-acquisition tables go through one pinned staging buffer, so their
        // copies are asynchronous DMA instead of staged pageable copies.
        struct Piece {
            void *dst;
            const void *src;
            size_t bytes;
        };
        const Piece pieces[] = {{rec_buf.p, recs.data(), (size_t)C * sizeof(ChirpRec)},
                                {p->skip.p, skip.data(), skip.size() * sizeof(SkipPoint)},
                                {p->gs.p, gs.data(), (size_t)S * 8},
                                {p->pos_base.p, base.data(), (size_t)C * 24},
                                {p->gres.p, gres.data(), gres.size() * 4}};
        size_t total = 0;
        for (const Piece &pc : pieces) total += round_up(pc.bytes, 256);
        TDC_CK(p->table_host.ensure(total), "alloc pinned table staging");
        unsigned char *h = static_cast<unsigned char *>(p->table_host.p);
        for (const Piece &pc : pieces) {
            std::memcpy(h, pc.src, pc.bytes);
            TDC_CK(cudaMemcpyAsync(pc.dst, h, pc.bytes, cudaMemcpyHostToDevice, st), "copy acquisition tables");
            h += round_up(pc.bytes, 256);
        }
    }
    if (!traj.empty()) {
        TDC_CK(p->traj.ensure(traj.size() * sizeof(float4)), "alloc per-sample offsets");
        TDC_CK(cudaMemcpyAsync(p->traj.p, traj.data(), traj.size() * sizeof(float4), cudaMemcpyHostToDevice, st),
               "copy per-sample offsets");
    }
    if (!wins.empty()) {
        TDC_CK(p->wins.ensure(wins.size() * sizeof(float4)), "alloc per-sample windows");
        TDC_CK(cudaMemcpyAsync(p->wins.p, wins.data(), wins.size() * sizeof(float4), cudaMemcpyHostToDevice, st),
               "copy per-sample windows");
    }
    if (!mrecs.empty()) {
        TDC_CK(p->motion_rec.ensure(mrecs.size() * sizeof(MotionRec)), "alloc motion records");
        TDC_CK(cudaMemcpyAsync(p->motion_rec.p, mrecs.data(), mrecs.size() * sizeof(MotionRec),
                               cudaMemcpyHostToDevice, st),
               "copy motion records");
        p->stats.h2d_bytes += (int64_t)(mrecs.size() * sizeof(MotionRec));
    }
    if (!wdot.empty()) {
        TDC_CK(p->wdot.ensure(wdot.size() * sizeof(float)), "alloc per-sample window offsets");
        TDC_CK(cudaMemcpyAsync(p->wdot.p, wdot.data(), wdot.size() * sizeof(float), cudaMemcpyHostToDevice, st),
               "copy per-sample window offsets");
    }
    p->stats.h2d_bytes += (int64_t)(gres.size() + wdot.size()) * 4 +
                          (int64_t)((traj.size() + wins.size()) * sizeof(float4));
    p->stats.h2d_bytes += (int64_t)C * S * 8 + (int64_t)C * sizeof(ChirpRec) +
                          (int64_t)skip.size() * sizeof(SkipPoint) + (int64_t)S * 8 + (int64_t)C * 24;
    TDC_CK(cudaEventRecord(p->ev[1], st), "event");

    if (!p->host_reads) {
        TDC_CK(launch_range_window(p->wr.as<float>(), S, o.range_win, st), "range window kernel");
        TDC_CK(launch_prewindow(p->xw.as<float2>(), p->wr.as<float>(), C, S, s_pad, st), "prewindow kernel");
        launches += 2;
    }
    // The host vectors above are read by the async copies: wait before they go out of scope.
    TDC_CK(cudaStreamSynchronize(st), "prepare sync");

    p->opts = o;
    p->prepared = true;
    p->xs_scaled_ready = false;
    p->offsets_applied = false;
    ++p->state_epoch;
    p->plan_path = -1;  // job parameters changed
    return TDC_OK;
}

// Device grid from a host (FP32 or FP64) grid.
int upload_grid(tdc_processor *p, int &launches)
{
    NvtxRange nvtx("tdc upload grid");
    if (!p->has_grid) return fail(TDC_ERR_STATE, "setFocusGrid must be called before start()");
    const long long P = (long long)p->rows * p->cols;
    p->P = P;
    ++p->state_epoch;
    p->plan_path = -1;  // unit spans and costs follow the grid's coordinates
    cudaStream_t st = p->stream;
    const size_t elt = p->grid64 ? 8 : 4;
    TDC_CK(p->grid_hi.ensure((size_t)P * 16), "alloc grid");
    const void *src = p->grid64 ? (const void *)p->grid64 : (const void *)p->grid;
    {
        auto g = [&](long long i, int k) { return p->grid64 ? p->grid64[3 * i + k] : (double)p->grid[3 * i + k]; };
        for (int k = 0; k < 3; ++k) {
            p->axis_c[k] = p->cols > 1 ? g(1, k) - g(0, k) : 0.0;
            p->axis_r[k] = p->rows > 1 ? g(p->cols, k) - g(0, k) : 0.0;
        }
        // centre pixel of every work tile, flat and block (the planner's cost estimate under
        // a finite Doppler band)
        p->tile_centre_flat.clear();
        p->tile_centre_block.clear();
        if (P > 0) {
            const long long n_flat = (P + kFocusTile - 1) / kFocusTile;
            p->tile_centre_flat.resize((size_t)n_flat * 3);
            p->tile_radius_flat.assign((size_t)n_flat, 0.0);
            for (long long t = 0; t < n_flat; ++t) {
                const long long i = std::min(P - 1, t * kFocusTile + kFocusTile / 2);
                for (int k = 0; k < 3; ++k) p->tile_centre_flat[3 * t + k] = g(i, k);
                double r2 = 0.0;
                for (long long q = t * kFocusTile; q < std::min(P, (t + 1) * kFocusTile); ++q) {
                    const double dx = g(q, 0) - g(i, 0), dy = g(q, 1) - g(i, 1), dz = g(q, 2) - g(i, 2);
                    const double d2 = dx * dx + dy * dy + dz * dz;
                    r2 = d2 > r2 || d2 != d2 ? d2 : r2;
                }
                p->tile_radius_flat[t] = std::sqrt(r2);
            }
            // anchored ranges: distance of each pixel from its group's anchor (groups of 32
            // consecutive pixels; the anchor is the 17th pixel or the group's last)
            double span2 = 0.0;
            for (long long b = 0; b < P; b += 32) {
                const long long a = std::min(P - 1, b + 16);
                const double ax = g(a, 0), ay = g(a, 1), az = g(a, 2);
                for (long long i = b; i < std::min(P, b + 32); ++i) {
                    const double dx = g(i, 0) - ax, dy = g(i, 1) - ay, dz = g(i, 2) - az;
                    const double d2 = dx * dx + dy * dy + dz * dz;
                    span2 = d2 > span2 || d2 != d2 ? d2 : span2;
                }
            }
            p->anchor_span = std::sqrt(span2);
            const int tile_rows = kFocusTile / kBlockTileCols;
            const long long n_tr = (p->rows + tile_rows - 1) / tile_rows;
            const long long n_tc = (p->cols + kBlockTileCols - 1) / kBlockTileCols;
            p->tile_centre_block.resize((size_t)(n_tr * n_tc) * 3);
            p->tile_radius_block.assign((size_t)(n_tr * n_tc), 0.0);
            for (long long tr = 0; tr < n_tr; ++tr)
                for (long long tc = 0; tc < n_tc; ++tc) {
                    const long long r = std::min<long long>(p->rows - 1, tr * tile_rows + tile_rows / 2);
                    const long long c = std::min<long long>(p->cols - 1, tc * kBlockTileCols + kBlockTileCols / 2);
                    const long long ci = r * p->cols + c;
                    for (int k = 0; k < 3; ++k) p->tile_centre_block[3 * (tr * n_tc + tc) + k] = g(ci, k);
                    double r2 = 0.0;
                    for (long long rr = tr * tile_rows; rr < std::min<long long>(p->rows, (tr + 1) * tile_rows); ++rr)
                        for (long long cc = tc * kBlockTileCols;
                             cc < std::min<long long>(p->cols, (tc + 1) * kBlockTileCols); ++cc) {
                            const long long q = rr * p->cols + cc;
                            if (q >= P) continue;
                            const double dx = g(q, 0) - g(ci, 0), dy = g(q, 1) - g(ci, 1), dz = g(q, 2) - g(ci, 2);
                            const double d2 = dx * dx + dy * dy + dz * dz;
                            r2 = d2 > r2 || d2 != d2 ? d2 : r2;
                        }
                    p->tile_radius_block[tr * n_tc + tc] = std::sqrt(r2);
                }
        }
    }
    if (!p->host_reads) {
        for (int k = 0; k < 3; ++k) {
            p->grid_min[k] = std::numeric_limits<double>::infinity();
            p->grid_max[k] = -std::numeric_limits<double>::infinity();
        }
        for (long long i = 0; i < P; ++i)
            for (int k = 0; k < 3; ++k) {
                const double v = p->grid64 ? p->grid64[3 * i + k] : (double)p->grid[3 * i + k];
                p->grid_min[k] = std::min(p->grid_min[k], v);
                p->grid_max[k] = std::max(p->grid_max[k], v);
            }
        TDC_CK(p->grid_stage.ensure((size_t)P * 3 * elt), "alloc grid staging");
        TDC_CK(cudaMemcpyAsync(p->grid_stage.p, src, (size_t)P * 3 * elt, cudaMemcpyHostToDevice, st), "copy grid");
        src = p->grid_stage.p;
    }
    p->stats.h2d_bytes += (int64_t)P * 3 * elt;
    if (p->grid64) {
        TDC_CK(p->grid_lo.ensure((size_t)P * 16), "alloc grid");
        TDC_CK(launch_grid_from_f64(static_cast<const double *>(src), P, p->grid_hi.as<float4>(),
                                    p->grid_lo.as<float4>(), st),
               "grid kernel");
        p->grid_lo_valid = true;
    } else {
        TDC_CK(launch_grid_from_f32(static_cast<const float *>(src), P, p->grid_hi.as<float4>(), st), "grid kernel");
        p->grid_lo_valid = false;
    }
    launches += 1;
    if (p->host_reads && P > 0) {
        // bounding box of the grid on the device (order-preserving integer keys of the floats)
        const int init[6] = {0x7fffffff, 0x7fffffff, 0x7fffffff, (int)0x80000000, (int)0x80000000,
                             (int)0x80000000};
        int keys[6];
        TDC_CK(p->flag.ensure(64), "alloc flag");
        int *box = p->flag.as<int>() + 4;
        TDC_CK(cudaMemcpyAsync(box, init, sizeof(init), cudaMemcpyHostToDevice, st), "init bbox");
        TDC_CK(launch_grid_bbox(p->grid_hi.as<float4>(), P, box, st), "bbox kernel");
        TDC_CK(cudaMemcpyAsync(keys, box, sizeof(keys), cudaMemcpyDeviceToHost, st), "read bbox");
        TDC_CK(cudaStreamSynchronize(st), "grid sync");
        launches += 1;
        for (int k = 0; k < 6; ++k) {
            const int bits = keys[k] >= 0 ? keys[k] : keys[k] ^ 0x7fffffff;
            float f;
            std::memcpy(&f, &bits, 4);
            (k < 3 ? p->grid_min[k] : p->grid_max[k - 3]) = f;
        }
    }
    return TDC_OK;
}

// Smallest distance between the antenna positions' bounding box and the grid's.
double min_range(const double *amin, const double *amax, const double *gmin, const double *gmax)
{
    double r2 = 0.0;
    for (int k = 0; k < 3; ++k) {
        const double d = std::max({0.0, gmin[k] - amax[k], amin[k] - gmax[k]});
        r2 += d * d;
    }
    return std::sqrt(r2);
}

// Bound on |(R_s^2 - R0^2) / R0^2| over the acquisition (infinite when the antenna can
// reach a pixel).
double range_change_bound(const tdc_processor *p)
{
    const double rmin = min_range(p->ant_min, p->ant_max, p->grid_min, p->grid_max);
    if (!(rmin > 0.0)) return std::numeric_limits<double>::infinity();
    const double q = p->delta_max / rmin;
    return 2.0 * q + q * q;
}

int general_variant(const tdc_processor *p)
{
    const double rmax = max_range(p->ant_min, p->ant_max, p->grid_min, p->grid_max);
    const double dev = 2.0 * M_PI * 2.0 * p->resid_hz * rmax / kC0;
    bool wide = dev > kUniformPhaseTolRad;
    if (p->traj_varies) {
        // the narrow variants take the range-change series to second order and the
        // phase correction unreduced: |e| <= 0.02 and |g_s d_s| <= 4 cycles
        const double g_max = 2.0 * (std::fabs(p->F0) + std::fabs(p->F1) * std::max(0, p->S - 1)) / kC0 +
                             2.0 * p->resid_hz / kC0;
        wide = wide || range_change_bound(p) > kGeneralNarrowEps || g_max * p->delta_max > kGeneralNarrowCycles;
    }
    return (p->traj_varies ? 1 : 0) | (p->win_varies ? 2 : 0) | (wide ? 4 : 0);
}

int motion_stage_bytes_for(int s_pad, int &cb)
{
    const int row = s_pad * 8 + (int)sizeof(MotionRec);
    cb = std::max(1, kFocusStageTarget / row);
    return (int)round_up((size_t)cb * row, 128);
}

// Upper bound on |psi'| [cycles / sample] of the smooth-motion kernel (see motion_segment).
double motion_slope_bound(const tdc_processor *p)
{
    const double g0 = 2.0 * std::fabs(p->F0) / kC0, g1 = 2.0 * std::fabs(p->F1) / kC0;
    const double g_max = g0 + g1 * std::max(0, p->s_pad);
    const double dp = p->motion_v1max + 2.0 * p->motion_v2max * p->s_pad;
    return g1 * p->delta_max + g_max * dp * 1.1;
}

int motion_segment(const tdc_processor *p)
{
    if (!p->motion_fit_ok || !p->motion_enabled || !p->traj_varies || p->win_varies) return 0;
    if (general_variant(p) != 1) return 0;  // per-sample positions only, narrow, uniform sampling
    int cb = 1;
    if (focus_motion_smem_bytes(motion_stage_bytes_for(p->s_pad, cb)) > 226 * 1024) return 0;  // whole rows only
    const double rmin = min_range(p->ant_min, p->ant_max, p->grid_min, p->grid_max);
    if (!(rmin > 0.0)) return 0;
    const double g0 = 2.0 * std::fabs(p->F0) / kC0, g1 = 2.0 * std::fabs(p->F1) / kC0;
    const double g_max = g0 + g1 * std::max(0, p->s_pad);
    // psi(s) = g_s d_s: slope psi' = g1 d + g_s d', curvature c2 = psi''/2 = g1 d' + g_s d''/2, with
    // |d| <= delta_max, |d'| <= |V1| + 2 |V2| s, |d''| <= 2 |V2| + |d'|^2 / R (1 + 10%)
    const double dp = p->motion_v1max + 2.0 * p->motion_v2max * p->s_pad;
    const double slope = motion_slope_bound(p);
    const double c2 = (g1 * dp + g_max * (p->motion_v2max + dp * dp / (2.0 * rmin))) * 1.1;
    if (!std::isfinite(slope)) return 0;
    // longest segment whose chord (plus mean offset) stays within kMotionTolRad of psi
    int best = 0;
    for (int m = 8; m <= (1 << 16); m *= 2) {
        if (2.0 * M_PI * c2 * ((double)m * m - 1.0) / 6.0 > kMotionTolRad) break;
        best = m;
        if (m >= p->s_pad) break;
    }
    return best;
}

int choose_path(const tdc_processor *p)
{
    const int variant = general_variant(p);
    const bool fp64 = p->precision == TDC_PRECISION_FP64_PHASE;
    if (variant == 0) {
        // One record per chirp describes every sample (a per-sample trajectory whose
        // variation cannot change the phase or the window is focused like a per-chirp one);
        // rows too long for the stages are staged in segments.
        if (fp64) return p->per_chirp ? TDC_PATH_FP64_PHASE : TDC_PATH_GENERAL_FP64;
        return TDC_PATH_FP32_BULK;
    }
    if (fp64) return TDC_PATH_GENERAL_FP64;
    // Per-sample range change d_s = N/(2 R0) f(N/R0^2): the series of f stays accurate for
    // |N/R0^2| <= 2 dmax/Rmin + (dmax/Rmin)^2 <= 0.1.
    if ((variant & 1) && !(range_change_bound(p) <= kGeneralMaxEps)) return TDC_PATH_GENERAL_FP64;
    // positions moving smoothly within chirps: the per-sample phase linearised per segment
    if (motion_segment(p) > 0) return TDC_PATH_FP32_MOTION;
    // rows of any length fit: those too long for whole-row stages are staged in segments
    return TDC_PATH_GENERAL;
}


// With a finite Doppler band, chirps whose window (or chunk skip test) is zero for every
// pixel of a warp skip their work, but a CTA's warps wait for one another at each pipeline
// stage. The window of a pixel follows its direction from the antenna relative to the
// antenna's velocity, so warps agree on their in-band chirps when the tile is narrow along
// the velocity: flat tiles (512 consecutive pixels, at most a few grid rows) are narrow
// across the columns, block tiles (32 rows x 16 columns) along them. Block tiles are used
// when the band is finite and the velocity runs closer to the grid's column direction than
// to its row direction; the choice does not change any pixel's value.
int choose_tile_cols(const tdc_processor *p)
{
    if (!TDC_BLOCK_TILES || !std::isfinite(p->opts.bw)) return 0;
    if (p->cols < 2 * kBlockTileCols || p->rows < kFocusTile / kBlockTileCols) return 0;
    auto along = [&](const double *a) {
        const double n = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
        return n > 0.0 ? std::fabs(a[0] * p->vel_dir[0] + a[1] * p->vel_dir[1] + a[2] * p->vel_dir[2]) / n : 0.0;
    };
    return along(p->axis_c) > along(p->axis_r) ? kBlockTileCols : 0;
}

// Under a finite Doppler band a unit's cost follows its live chirps, which depend on where
// its tile lies: the units are put in order of decreasing estimated cost (the window at the
// tile's centre pixel for each chirp of the group), so the persistent CTAs take the long
// ones first and the launch does not end on a few long units. Only the order in which CTAs
// take units changes: each pixel's sums, and so the image, are the same.
// With `narrow`, each unit also gets the span of its group's chirps that any pixel of its
// tile can see in band (FocusUnit::span), from the Doppler at the tile's centre T and a bound
// on its change over the tile: with u(p) = (a - p) / |a - p| and |p - T| <= rho < |a - T| = n
// (rho the tile's radius), the directions from the antenna differ by at most asin(rho / n),
// so |u(p) - u(T)| <= 2 sin(asin(rho / n) / 2) and |fd(p) - fd(T)| <= (2 / lambda) |v| that.
// A chirp outside the span is out of band for every pixel of the tile (with a 5% margin on
// that bound and 1e-4 relative for the kernel's FP32 arithmetic), so the zero-window
// instance would skip it for every warp: skipping it in the unit changes no sum.
void plan_unit_order_and_spans(tdc_processor *p, int tile_cols, bool narrow)
{
    if (!std::isfinite(p->opts.bw) || p->rec_host.size() != (size_t)p->C || p->units_host.size() < 2) return;
    const std::vector<double> &centres = tile_cols ? p->tile_centre_block : p->tile_centre_flat;
    const std::vector<double> &radii = tile_cols ? p->tile_radius_block : p->tile_radius_flat;
    const long long n_tiles = (long long)centres.size() / 3;
    const int C = p->C, cpg = p->plan_cpg, groups = p->plan_groups;
    if ((long long)p->units_host.size() != n_tiles * groups) return;
    narrow = narrow && (long long)radii.size() == n_tiles && cpg < kUnitSpanMax;
    const double two_over_lambda = (double)(2.0f / p->lambda), half_bw = (double)(p->opts.bw / 2.0f);
    std::vector<double> cost((size_t)n_tiles * groups, 0.0);
    std::vector<int> span((size_t)n_tiles * groups, 0);
    parallel_chirps((int)n_tiles, C, [&](int, int t0, int t1) {
        for (int t = t0; t < t1; ++t) {
            const double *T = &centres[3 * (size_t)t];
            const double rho = narrow ? radii[t] : 0.0;
            for (int g = 0; g < groups; ++g) {
                const int c0 = g * cpg, c1 = std::min(C, c0 + cpg);
                long live = 0;
                int lo = c1, hi = c0;  // chirps that some pixel of the tile may see in band: [lo, hi)
                for (int c = c0; c < c1; ++c) {
                    const ChirpRec &r = p->rec_host[c];
                    const double dx = ((double)r.p_hi.x + r.p_lo.x) - T[0], dy = ((double)r.p_hi.y + r.p_lo.y) - T[1],
                                 dz = ((double)r.p_hi.z + r.p_lo.z) - T[2];
                    const double n = std::sqrt(dx * dx + dy * dy + dz * dz);
                    const double fd = -two_over_lambda * (r.vel.x * dx + r.vel.y * dy + r.vel.z * dz) / n;
                    const double off = std::fabs(fd - (double)r.p_hi.w);
                    live += off <= half_bw ? 1 : 0;
                    if (narrow) {
                        const double vn = std::sqrt((double)r.vel.x * r.vel.x + (double)r.vel.y * r.vel.y +
                                                    (double)r.vel.z * r.vel.z);
                        const double chord = rho < n ? 2.0 * std::sin(0.5 * std::asin(rho / n)) : 2.0;
                        const double bound = 1.05 * two_over_lambda * vn * chord +
                                             1e-4 * (std::fabs(fd) + std::fabs((double)r.p_hi.w) + half_bw) + 1e-6;
                        // dead for the whole tile only when provably so (NaN: kept)
                        if (!(off > half_bw + bound)) {
                            lo = std::min(lo, c);
                            hi = c + 1;
                        }
                    }
                }
                // a live chirp costs its samples' MACs and the set-up, a dead one the vote
                cost[(size_t)t * groups + g] = (double)live * (p->s_pad + 64) + (double)(c1 - c0 - live) * 24.0;
                if (narrow && !(lo == c0 && hi == c1))
                    span[(size_t)t * groups + g] = lo < hi ? unit_span(lo - c0, hi - c0) : unit_span(0, 0);
            }
        }
    });
    long long visited = 0;
    for (FocusUnit &u : p->units_host) {
        u.span = span[(size_t)u.tile * groups + u.group];
        const int c0 = u.group * cpg, n = std::min(C, c0 + cpg) - c0;
        visited += u.span ? std::max(0, unit_span_hi(u.span) - unit_span_lo(u.span)) : n;
    }
    p->span_permille = (int)std::lround(1000.0 * (double)visited / ((double)n_tiles * C));
    std::stable_sort(p->units_host.begin(), p->units_host.end(), [&](const FocusUnit &a, const FocusUnit &b) {
        return cost[(size_t)a.tile * groups + a.group] > cost[(size_t)b.tile * groups + b.group];
    });
}

// Split the chirps into groups so that tiles x groups units fill whole waves of `slots`;
// among the splits with at least min_units_per_slot units per slot when there are any.
void plan_groups(long long n_tiles, int C, int slots, int &n_groups, int &cpg, int min_units_per_slot)
{
    const long long min_units = (long long)min_units_per_slot * slots;
    const int gmax = std::max(1, std::min(C, 1024));
    n_groups = 1;
    cpg = C;
    for (int pass = 0; pass < 2; ++pass) {
        double best = std::numeric_limits<double>::infinity();
        for (int g = 1; g <= gmax; ++g) {
            const int c = (C + g - 1) / g;
            const int geff = (C + c - 1) / c;
            if (geff != g) continue;
            const long long units = n_tiles * geff;
            if (units > (1LL << 24)) break;
            if (pass == 0 && units < min_units) continue;
            const long long waves = (units + slots - 1) / slots;
            const double cost = (double)waves * (c + 0.5);
            if (cost < best - 1e-9) {
                best = cost;
                n_groups = geff;
                cpg = c;
            }
        }
        if (best < std::numeric_limits<double>::infinity()) return;
    }
}

// Scratch layout of one focus: [status words | job | units | partials].
struct ScratchLayout {
    size_t off_job, off_units, off_partial, total;
};

ScratchLayout scratch_layout(long long P, int n_units, int n_groups)
{
    ScratchLayout L;
    L.off_job = 256;
    L.off_units = round_up(L.off_job + sizeof(FocusJob), 256);
    L.off_partial = round_up(L.off_units + (size_t)n_units * sizeof(FocusUnit), 256);
    L.total = L.off_partial + (size_t)n_groups * (size_t)P * 16;
    return L;
}

int stage_bytes_for(int s_pad, int &cb)
{
    const int row = s_pad * 8 + (int)sizeof(ChirpRec);
    cb = std::max(1, kFocusStageTarget / row);
    return (int)round_up((size_t)cb * row, 128);
}

bool needs_segments(int s_pad)
{
    return focus_fp32_smem_bytes(0, false) + kFocusStages * (int)round_up((size_t)s_pad * 8 + sizeof(ChirpRec), 128) >
           226 * 1024;
}

namespace {

// Bytes the FP32 general kernel stages per (chirp, sample): the raw sample, and the
// trajectory, window and window-offset table entries where the variant reads them.
int general_row_bytes_per_sample(int variant)
{
    return 8 + ((variant & 1) ? 16 : 0) + ((variant & 2) ? 16 : 0) + ((variant & 3) == 3 ? 4 : 0);
}

// Bytes of the per-sample frequency tables staged with each row segment: the non-uniform
// sampling residual (wide variants) and 2 f_s / c0 (per-sample positions).
int general_table_bytes_per_sample(int variant)
{
    return ((variant & 4) ? 4 : 0) + ((variant & 1) ? 4 : 0);
}

}  // namespace

int general_stage_bytes_for(int s_pad, int variant, int seg, int &cb)
{
    const int row = seg * general_row_bytes_per_sample(variant) + (int)sizeof(ChirpRec);
    const int tab = seg * general_table_bytes_per_sample(variant);
    cb = seg >= s_pad ? std::max(1, (kGeneralStageTarget - tab) / row) : 1;
    return (int)round_up((size_t)cb * row + tab, 128);
}

int general_segment_samples(int s_pad, int variant)
{
    const int per = general_row_bytes_per_sample(variant) + general_table_bytes_per_sample(variant);
    const int smax = std::max(kSampleAlign, (kGeneralStageTarget - (int)sizeof(ChirpRec)) / per / kSampleAlign *
                                                kSampleAlign);
    const int nseg = (s_pad + smax - 1) / smax;
    return (int)round_up((size_t)((s_pad + nseg - 1) / nseg), kSampleAlign);
}

int general_seg_len(int s_pad, int variant)
{
    const int seg = general_segment_samples(s_pad, variant);
    if (seg >= s_pad) return s_pad;
    if (TDC_GENERAL_ALWAYS_SEGMENT) return seg;
    int cb = 1;
    const int whole = general_stage_bytes_for(s_pad, variant, s_pad, cb);
    // 227 KiB of shared memory per CTA, less the kernel's static shared memory
    if (focus_general_smem_bytes(whole) > 226 * 1024) return seg;
    const int split = general_stage_bytes_for(s_pad, variant, seg, cb);
    return focus_general_blocks_per_sm(variant, whole) < focus_general_blocks_per_sm(variant, split) ? seg : s_pad;
}

// Job record of the resident acquisition x resident grid under the current plan.
FocusJob make_job(const tdc_processor *p, float4 *partial, int cb, int path)
{
    FocusJob job;
    std::memset(&job, 0, sizeof(job));
    job.xw = p->xw.as<const float4>();
    // FP32 kernels read one record per chirp; the FP64 general kernel one per sample.
    const bool rec_per_sample = !p->per_chirp && path == TDC_PATH_GENERAL_FP64;
    job.chirps = p->per_chirp || rec_per_sample ? p->chirps.as<const ChirpRec>() : p->gen_rec.as<const ChirpRec>();
    if (path == TDC_PATH_FP32_MOTION) job.chirps = reinterpret_cast<const ChirpRec *>(p->motion_rec.p);
    job.traj = p->traj_varies ? p->traj.as<const float4>() : nullptr;
    job.wins = p->win_varies ? p->wins.as<const float4>() : nullptr;
    job.wdot = p->win_varies && p->traj_varies ? p->wdot.as<const float>() : nullptr;
    job.gres = p->gres.as<const float>();
    job.gsam = p->gres.as<const float>() + p->s_pad;
    job.grid_hi = p->grid_hi.as<const float4>();
    job.grid_lo = p->grid_lo_valid ? p->grid_lo.as<const float4>() : nullptr;
    job.skip = p->skip.as<const SkipPoint>();
    job.gs = p->gs.as<const double>();
    job.partial = partial;
    job.P = p->P;
    job.C = p->C;
    job.S = p->S;
    job.s_pad = p->s_pad;
    job.n_groups = p->plan_groups;
    job.chirps_per_group = p->plan_cpg;
    job.chunk = kChunk;
    job.stage_chirps = cb;
    job.flags = (p->opts.taper ? kFlagTaper : 0) | (p->opts.skip_test ? kFlagSkipTest : 0);
    job.n_tiles = (int)((p->P + kFocusTile - 1) / kFocusTile);
    job.per_sample = rec_per_sample ? 1 : 0;
    const double g0 = 2.0 * p->F0 / kC0, g1 = 2.0 * p->F1 / kC0;
    split_dd(g0, job.g0_hi, job.g0_lo);
    split_dd(g1, job.g1, job.g1_lo);
    job.two_over_lambda = 2.0f / p->lambda;
    job.half_bw = p->opts.bw / 2.0f;
    job.inv_bw = 1.0f / p->opts.bw;
    job.az_a = kAzimuthA;
    return job;
}

// Per-(chirp, sample) records of the FP64 general kernel, built from the caller's
// per-sample arrays the first time that kernel runs on the resident acquisition.
int sample_records(tdc_processor *p)
{
    if (p->per_chirp || p->sample_recs_ready) return TDC_OK;
    const int C = p->C, S = p->S;
    std::vector<ChirpRec> recs((size_t)C * S);
    parallel_chirps(C, S, [&](int, int cb, int ce) {
        for (int c = cb; c < ce; ++c)
            for (int s = 0; s < S; ++s)
                recs[(size_t)c * S + s] = make_record(p, c, s, p->opts.centroid != 0, p->opts.center);
    });
    TDC_CK(p->chirps.ensure(recs.size() * sizeof(ChirpRec)), "alloc per-sample records");
    TDC_CK(cudaMemcpyAsync(p->chirps.p, recs.data(), recs.size() * sizeof(ChirpRec), cudaMemcpyHostToDevice,
                           p->stream),
           "copy per-sample records");
    TDC_CK(cudaStreamSynchronize(p->stream), "per-sample records sync");
    p->stats.h2d_bytes += (int64_t)(recs.size() * sizeof(ChirpRec));
    p->sample_recs_ready = true;
    return TDC_OK;
}

// Anchored ranges for an FP32-bulk focus staged whole, cb chirps a stage: the plain kernel
// instance (unbounded band, so flat tiles; no kept per-chirp sums) with finite velocities and
// window centres (the instance then forms no Doppler window), 3 to kAnchorMaxStageChirps
// chirps a stage (with 1 or 2, i.e. rows of about 1,000 samples or more, the instance measured
// 0.4-1.8% slower than the double-float one: the Horner loop dominates there), every pixel
// within kAnchorMaxDistance of its anchor, and the block step's correction 2 pi L g1 |dR|
// within its series' range (0.25 rad: rows of 256 samples at 2 mm spacing, 128 at 1 mm).
#ifndef TDC_ANCHOR_MIN_STAGE_CHIRPS
#define TDC_ANCHOR_MIN_STAGE_CHIRPS 3
#endif
bool anchor_eligible(const tdc_processor *p, int cb)
{
    if (!p->anchor_enabled || p->keep_sums || !p->per_chirp || !p->rec_finite) return false;
    if (std::isfinite(p->opts.bw / 2.0f)) return false;
    if (cb < TDC_ANCHOR_MIN_STAGE_CHIRPS || cb > kAnchorMaxStageChirps) return false;
    if (!(p->anchor_span <= kAnchorMaxDistance)) return false;
    const double g1 = 2.0 * p->F1 / kC0;
    return 2.0 * M_PI * 8.0 * std::fabs(g1) * p->anchor_span <= 0.25;
}

int focus_plan(tdc_processor *p, FocusPlan &plan, double max_unit_work)
{
    if (!p->prepared) return fail(TDC_ERR_STATE, "acquisition not prepared");
    if (p->P <= 0) return fail(TDC_ERR_STATE, "no focus grid");
    const int path = choose_path(p);
    const long long P = p->P;
    const int C = p->C;
    if (path == TDC_PATH_GENERAL_FP64)
        if (int rc = sample_records(p)) return rc;

    int cb = 1;
    const int variant = path == TDC_PATH_GENERAL ? general_variant(p) : 0;
    // FP32-bulk rows are staged whole, or in segments when whole rows do not fit the stages
    // or leave fewer CTAs per SM than segments do (long chirps).
    const int seg_stage_bytes = (int)round_up((size_t)kSegmentSamples * 8 + sizeof(ChirpRec), 128);
    bool seg = false;
    if (path == TDC_PATH_FP32_BULK && p->s_pad > kSegmentSamples) {
        seg = needs_segments(p->s_pad);
        if (!seg) {
            int cb_whole = 1;
            seg = focus_fp32_blocks_per_sm(stage_bytes_for(p->s_pad, cb_whole)) <
                  focus_fp32_seg_blocks_per_sm(seg_stage_bytes);
        }
    }
    // FP32 general rows likewise: whole, or in segments of about kGeneralStageTarget bytes
    const int gen_seg = path == TDC_PATH_GENERAL ? general_seg_len(p->s_pad, variant) : 0;
    const int stage_bytes = path == TDC_PATH_GENERAL       ? general_stage_bytes_for(p->s_pad, variant, gen_seg, cb)
                            : path == TDC_PATH_FP32_MOTION ? motion_stage_bytes_for(p->s_pad, cb)
                            : seg                          ? seg_stage_bytes
                                                           : stage_bytes_for(p->s_pad, cb);
    const int motion_seg = path == TDC_PATH_FP32_MOTION ? motion_segment(p) : 0;
    // the segment's block step QL_m = QL e^{j 2 pi L sigma_m}: a rotation series for L |sigma| up
    // to 0.8 rad, else an accurate sincos per segment
    const bool motion_exact_ql = path == TDC_PATH_FP32_MOTION && !(2.0 * M_PI * 8.0 * motion_slope_bound(p) <= 0.8);
    int slots;
    bool anchored = false;
    if (path == TDC_PATH_FP32_MOTION) {
        const int bps = focus_motion_blocks_per_sm(stage_bytes);
        if (bps <= 0) return fail(TDC_ERR_CUDA, "smooth-motion focus kernel does not fit on the device");
        slots = p->n_sm * bps;
    } else if (path == TDC_PATH_FP32_BULK) {
        const int bps = seg ? focus_fp32_seg_blocks_per_sm(stage_bytes) : focus_fp32_blocks_per_sm(stage_bytes);
        if (bps <= 0) return fail(TDC_ERR_CUDA, "focus kernel does not fit on the device");
        slots = p->n_sm * bps;
        anchored = !seg && anchor_eligible(p, cb) && focus_fp32_anchor_blocks_per_sm(stage_bytes) >= bps;
    } else if (path == TDC_PATH_GENERAL) {
        const int bps = focus_general_blocks_per_sm(variant, stage_bytes);
        if (bps <= 0) return fail(TDC_ERR_CUDA, "general focus kernel does not fit on the device");
        slots = p->n_sm * bps;
    } else {
        slots = p->n_sm * 4;
    }

    const int tile_cols = choose_tile_cols(p);
    const long long n_tiles = tile_count(P, tile_cols, p->cols);
    // (block tiles also depend on the grid's shape, not only on its pixel count)
    const int plan_cols = tile_cols ? p->cols : 0;
    // The chirp groups (each pixel's summation order) follow the grid the job is planned for:
    // its own, or a larger one whose row block this grid is (pixel sharding across GPUs).
    const long long plan_tiles = p->plan_pixels > P ? tile_count(p->plan_pixels, tile_cols, p->cols) : n_tiles;
    if (path != p->plan_path || P != p->plan_P || C != p->plan_C || slots != p->plan_slots ||
        max_unit_work != p->plan_unit_cap || tile_cols != p->plan_tile_cols || plan_cols != p->plan_cols ||
        plan_tiles != p->plan_tiles) {
        int min_units = path == TDC_PATH_GENERAL ? kGeneralMinUnitsPerSlot : kFocusMinUnitsPerSlot;
        if (path == TDC_PATH_FP32_BULK && max_unit_work <= 0) {
            // Long launches end on their last units: units of about kUnitTargetCorr correlations
            // (up to 32 per CTA slot) shorten that tail; short launches keep fewer, larger units.
            // (Request-loop launches bound their units by max_unit_work instead: finer units there
            // delayed each request's completion.)
            const double work = (double)plan_tiles * kFocusTile * C * p->s_pad;
            const double by_work = std::floor(work / ((double)slots * kUnitTargetCorr));
            min_units = std::max(min_units, (int)std::min(32.0, by_work));
        }
        plan_groups(plan_tiles, C, slots, p->plan_groups, p->plan_cpg, min_units);
        p->plan_tiles = plan_tiles;
        if (max_unit_work > 0) {
            // bound the work of one unit (tile x chirp group): at most cap / (tile x S) chirps per group
            const int cpg_cap = std::max(1, (int)(max_unit_work / ((double)kFocusTile * p->S)));
            if (p->plan_cpg > cpg_cap) {
                p->plan_cpg = cpg_cap;
                p->plan_groups = (C + cpg_cap - 1) / cpg_cap;
            }
        }
        p->plan_unit_cap = max_unit_work;
        p->plan_tile_cols = tile_cols;
        p->plan_cols = plan_cols;
        p->units_host.clear();
        p->units_host.reserve((size_t)(n_tiles * p->plan_groups));
        for (long long t = 0; t < n_tiles; ++t)
            for (int g = 0; g < p->plan_groups; ++g) p->units_host.push_back(FocusUnit{0, (int)t, g, 0});
        // (only the whole-row FP32-bulk focus reads unit spans, and not when it keeps its
        // per-chirp sums: those would be left unwritten for the skipped chirps)
        p->span_permille = 1000;
        if (path != TDC_PATH_FP64_PHASE && path != TDC_PATH_GENERAL_FP64)
            plan_unit_order_and_spans(p, tile_cols,
                                path == TDC_PATH_FP32_BULK && !seg && !p->keep_sums && !p->offsets_applied);
        p->plan_path = path;
        p->plan_P = P;
        p->plan_C = C;
        p->plan_slots = slots;
        p->plan_uploaded = false;
    }
    const int n_units = (int)p->units_host.size();
    const ScratchLayout L = scratch_layout(P, n_units, p->plan_groups);
    if (L.total > p->scratch.cap) {
        TDC_CK(p->scratch.ensure(L.total), "alloc focus scratch");
        p->plan_uploaded = false;
    }
    unsigned char *scr = p->scratch.as<unsigned char>();
    plan.path = path;
    plan.variant = variant;
    plan.seg = seg;
    plan.cb = cb;
    plan.stage_bytes = stage_bytes;
    plan.slots = slots;
    plan.anchored = anchored;
    plan.off_job = L.off_job;
    plan.off_units = L.off_units;
    plan.job = make_job(p, reinterpret_cast<float4 *>(scr + L.off_partial), cb, path);
    plan.job.seg_len = path == TDC_PATH_GENERAL ? gen_seg : path == TDC_PATH_FP32_MOTION ? motion_seg
                                                          : seg                          ? kSegmentSamples
                                                                                         : 0;
    if (motion_exact_ql) plan.job.flags |= kFlagMotionExactQL;
    plan.job.tile_cols = tile_cols;
    plan.job.grid_cols = p->cols;
    plan.job.n_tiles = (int)n_tiles;
    // narrow variants take the phase correction in radians
    if (path == TDC_PATH_GENERAL && !(variant & 4)) plan.job.gsam = p->gres.as<const float>() + 2 * (size_t)p->s_pad;
    return TDC_OK;
}

// Focus the resident acquisition onto the resident grid: image_dev (complex float [P]).
int processor_use_slot_stream(tdc_processor *p, int priority)
{
    TDC_CK(cudaSetDevice(p->device), "cudaSetDevice");
    for (DevBuf *b : p->device_buffers()) b->release();
    TDC_CK(cudaStreamSynchronize(p->stream), "stream sync");
    cudaStream_t st = nullptr;
    TDC_CK(cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, priority), "stream creation");
    cudaStreamDestroy(p->stream);
    p->stream = st;
    for (DevBuf *b : p->device_buffers()) b->alloc_stream = st;
    return TDC_OK;
}

void processor_release_memory(tdc_processor *p)
{
    for (DevBuf *b : p->device_buffers()) b->release();
    p->prepared = false;
    p->plan_path = -1;
    p->plan_uploaded = false;
    p->grid_lo_valid = false;
}

size_t processor_device_bytes(tdc_processor *p)
{
    size_t n = 0;
    for (DevBuf *b : p->device_buffers()) n += b->cap;
    return n;
}

int focus_resident(tdc_processor *p, float2 *image_dev, cudaStream_t st, int &launches)
{
    NvtxRange nvtx("tdc focus");
    FocusPlan plan;
    if (int rc = focus_plan(p, plan)) return rc;
    const long long P = p->P;
    const int C = p->C;
    const int path = plan.path, stage_bytes = plan.stage_bytes, slots = plan.slots;
    const int n_units = (int)p->units_host.size();
    unsigned char *scr = p->scratch.as<unsigned char>();
    struct {
        size_t off_job, off_units;
    } L{plan.off_job, plan.off_units};
    // Autofocus: keep the per-(chirp, pixel) sums for the adjoint when they fit in half the
    // free device memory (whole-row FP32-bulk focus only).
    bool store = false;
    if (p->keep_sums && path == TDC_PATH_FP32_BULK && !plan.seg && p->per_chirp) {
        const size_t bytes = (size_t)C * (size_t)P * sizeof(float2);
        size_t free_b = 0, total_b = 0;
        if (bytes <= p->chirp_sums.cap ||
            (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && bytes + p->chirp_sums.cap <= free_b / 2)) {
            store = p->chirp_sums.ensure(bytes) == cudaSuccess;
            if (!store) (void)cudaGetLastError();
        }
    }
    plan.job.chirp_sums = store ? p->chirp_sums.as<float2>() : nullptr;
    const FocusJob &job = plan.job;

    TDC_CK(cudaMemcpyAsync(scr + L.off_job, &job, sizeof(job), cudaMemcpyHostToDevice, st), "copy job");
    if (!p->plan_uploaded) {
        TDC_CK(cudaMemcpyAsync(scr + L.off_units, p->units_host.data(), (size_t)n_units * sizeof(FocusUnit),
                               cudaMemcpyHostToDevice, st),
               "copy units");
        p->plan_uploaded = true;
    }
    TDC_CK(cudaMemsetAsync(scr, 0, 8, st), "reset counter");
    const FocusJob *jobs_dev = reinterpret_cast<const FocusJob *>(scr + L.off_job);
    const FocusUnit *units_dev = reinterpret_cast<const FocusUnit *>(scr + L.off_units);
    int *counter = reinterpret_cast<int *>(scr);
    int *status = counter + 1;
    if (path == TDC_PATH_FP32_BULK) {
        const int grid = std::min(n_units, slots);
        // the zero-window-skipping instances also map block tiles (which come with a finite band)
        const bool skip_zero = std::isfinite(job.half_bw) || job.tile_cols != 0;
        if (plan.seg)
            TDC_CK(launch_focus_fp32_seg(jobs_dev, units_dev, n_units, counter, status, stage_bytes, grid,
                                         skip_zero, st),
                   "focus kernel (segmented rows)");
        else
            TDC_CK(launch_focus_fp32(jobs_dev, units_dev, n_units, counter, status, stage_bytes, grid, skip_zero,
                                     store, plan.anchored && !skip_zero && !store, st),
                   "focus kernel");
    } else if (path == TDC_PATH_GENERAL) {
        const int grid = std::min(n_units, slots);
        TDC_CK(launch_focus_general(plan.variant, jobs_dev, units_dev, n_units, counter, status, stage_bytes, grid,
                                    st),
               "focus kernel (general)");
    } else if (path == TDC_PATH_FP32_MOTION) {
        const int grid = std::min(n_units, slots);
        const bool skip_zero = std::isfinite(job.half_bw) || job.tile_cols != 0;
        TDC_CK(launch_focus_motion(jobs_dev, units_dev, n_units, counter, status, stage_bytes, grid, skip_zero, st),
               "focus kernel (smooth motion)");
    } else {
        TDC_CK(launch_focus_fp64(jobs_dev, units_dev, n_units, status, job.per_sample, st), "focus kernel (fp64)");
    }
    TDC_CK(launch_focus_reduce(job.partial, p->plan_groups, P, image_dev, st), "reduce kernel");
    launches += 2;
    p->sums_epoch = store ? p->state_epoch : 0;
    p->stats.path = path;
    p->stats.correlations = (int64_t)P * C * p->S;
    const bool staged = path == TDC_PATH_FP32_BULK || path == TDC_PATH_GENERAL || path == TDC_PATH_FP32_MOTION;
    const int row = path == TDC_PATH_GENERAL ? job.seg_len : plan.seg ? kSegmentSamples : p->s_pad;
    p->stats.stage_samples = staged ? std::min(row, p->s_pad) : 0;
    p->stats.stage_chirps = staged ? (row < p->s_pad ? 1 : plan.cb) : 0;
    p->stats.general_variant = path == TDC_PATH_GENERAL ? plan.variant : 0;
    p->stats.tile_cols = job.tile_cols;
    p->stats.motion_segment = path == TDC_PATH_FP32_MOTION ? job.seg_len : 0;
    p->stats.span_permille = path == TDC_PATH_FP32_BULK && !plan.seg && !store ? p->span_permille : 1000;
    p->stats.anchor_pixels = 0;
    if (path == TDC_PATH_FP32_BULK && !plan.seg && plan.anchored && !store && !std::isfinite(job.half_bw) &&
        job.tile_cols == 0)
        p->stats.anchor_pixels = 32;
    return TDC_OK;
}

int read_status(tdc_processor *p)
{
    int status = 0;
    TDC_CK(cudaMemcpy(&status, p->scratch.as<int>() + 1, sizeof(int), cudaMemcpyDeviceToHost), "read status");
    if (status & kStatusTimeout) return fail(TDC_ERR_TIMEOUT, "focus kernel wait timed out");
    if (status & kStatusBadJob) return fail(TDC_ERR_CUDA, "focus kernel rejected its job record");
    return TDC_OK;
}

float elapsed(cudaEvent_t a, cudaEvent_t b)
{
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) return 0.f;
    return ms;
}

}  // namespace impl
}  // namespace tdc

int tdc::set_last_error(int code, const char *msg) { return fail(code, msg ? msg : ""); }

// ===========================================================================
// C ABI
// ===========================================================================

extern "C" {

const char *tdc_last_error(void) { return g_err.c_str(); }
int tdc_abi_version(void) { return TDC_GB300_ABI_VERSION; }

int tdc_processor_create(int gpu_num, tdc_processor **out)
{
    if (!out) return fail(TDC_ERR_INVALID_ARGUMENT, "null output pointer");
    *out = nullptr;
    cudaError_t e = cudaSetDevice(gpu_num);
    if (e != cudaSuccess)
        return fail(TDC_ERR_CUDA, std::string("Failed to set cuda device: ") + cudaGetErrorString(e));
    tdc_processor *p = new (std::nothrow) tdc_processor();
    if (!p) return fail(TDC_ERR_NO_MEMORY, "out of host memory");
    p->device = gpu_num;
    e = cudaDeviceGetAttribute(&p->n_sm, cudaDevAttrMultiProcessorCount, gpu_num);
    if (e == cudaSuccess) {
        // Coherent access to pageable host memory (Grace-Blackwell NVLink-C2C): the
        // kernels then read the caller's arrays in place instead of staging copies.
        int pageable = 0;
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, gpu_num);
        const char *env = std::getenv("TDC_GB300_HOST_READS");
        p->host_reads = pageable == 1 && !(env && env[0] == '0');
    }
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking);
    for (int i = 0; i < 6 && e == cudaSuccess; ++i) e = cudaEventCreate(&p->ev[i]);
    if (e != cudaSuccess) {
        tdc_processor_destroy(p);
        return cuda_fail(e, "processor init");
    }
    *out = p;
    return TDC_OK;
}

int tdc_processor_destroy(tdc_processor *p)
{
    if (!p) return TDC_OK;
    cudaSetDevice(p->device);
    // Buffers from the stream-ordered pool go back on the processor's stream before it is destroyed.
    for (DevBuf *b : p->device_buffers()) b->release();
    if (p->stream) cudaStreamSynchronize(p->stream);
    for (auto &ev : p->ev)
        if (ev) cudaEventDestroy(ev);
    if (p->stream) cudaStreamDestroy(p->stream);
    delete p;
    return TDC_OK;
}

int tdc_processor_set_raw_data(tdc_processor *p, const float *raw_iq, const float *pri_times,
                               const float *sample_times, const float *position, const float *velocity,
                               const float *attitude, int n_pri, int n_samples, float mod_rate, float start_freq,
                               const float *body_boresight)
{
    if (int rc = check_proc(p)) return rc;
    // tdcprocessor.cpp:189-195
    if (n_pri <= 0) return fail(TDC_ERR_INVALID_ARGUMENT, "nPri must be greater than 0");
    if (n_samples <= 0) return fail(TDC_ERR_INVALID_ARGUMENT, "nSamples must be greater than 0");
    if (!raw_iq || !sample_times || !position || !body_boresight)
        return fail(TDC_ERR_INVALID_ARGUMENT, "null input array");
    p->raw = raw_iq;
    p->pri_times = pri_times;
    p->sample_times = sample_times;
    p->pos = position;
    p->vel = velocity;
    p->att = attitude;
    p->C = n_pri;
    p->S = n_samples;
    p->mod_rate = mod_rate;
    p->start_freq = start_freq;
    for (int k = 0; k < 3; ++k) p->bore[k] = body_boresight[k];
    // tdcprocessor.cpp:204-208: float subtraction, then double, then cast to float.
    const float chirp_time_f = sample_times[n_samples - 1] - sample_times[0];
    const double chirp_time = chirp_time_f;
    const double end_freq = (double)start_freq + ((double)mod_rate * chirp_time);
    const double centre = ((double)start_freq + end_freq) / 2.0;
    p->lambda = (float)(kC0 / centre);
    p->pos64 = nullptr;
    p->traj_per_chirp = false;
    p->has_raw = true;
    p->prepared = false;
    return TDC_OK;
}

int tdc_processor_set_focus_grid(tdc_processor *p, const float *focus_grid, int n_rows, int n_cols)
{
    if (int rc = check_proc(p)) return rc;
    if (n_rows < 0 || n_cols < 0) return fail(TDC_ERR_INVALID_ARGUMENT, "negative grid shape");
    if (!focus_grid && (long long)n_rows * n_cols > 0) return fail(TDC_ERR_INVALID_ARGUMENT, "null focus grid");
    p->grid = focus_grid;
    p->grid64 = nullptr;
    p->rows = n_rows;
    p->cols = n_cols;
    p->has_grid = true;
    return TDC_OK;
}

int tdc_processor_set_focus_grid_f64(tdc_processor *p, const double *focus_grid, int n_rows, int n_cols)
{
    if (int rc = check_proc(p)) return rc;
    if (n_rows < 0 || n_cols < 0) return fail(TDC_ERR_INVALID_ARGUMENT, "negative grid shape");
    if (!focus_grid && (long long)n_rows * n_cols > 0) return fail(TDC_ERR_INVALID_ARGUMENT, "null focus grid");
    p->grid = nullptr;
    p->grid64 = focus_grid;
    p->rows = n_rows;
    p->cols = n_cols;
    p->has_grid = true;
    return TDC_OK;
}

int tdc_processor_set_chirp_positions_f64(tdc_processor *p, const double *position_f64, int n_pri)
{
    if (int rc = check_proc(p)) return rc;
    if (!p->has_raw) return fail(TDC_ERR_STATE, "setRawData must be called first");
    if (position_f64 && n_pri != p->C) return fail(TDC_ERR_SHAPE, "position shape is incorrect");
    p->pos64 = position_f64;
    p->prepared = false;
    return TDC_OK;
}

int tdc_processor_set_trajectory_per_chirp(tdc_processor *p, const float *position, const float *velocity,
                                           const float *attitude)
{
    if (int rc = check_proc(p)) return rc;
    if (!p->has_raw) return fail(TDC_ERR_STATE, "setRawData must be called first");
    if (!position) return fail(TDC_ERR_INVALID_ARGUMENT, "null position");
    p->pos = position;
    p->vel = velocity;
    p->att = attitude;
    p->traj_per_chirp = true;
    p->prepared = false;
    return TDC_OK;
}

int tdc_processor_set_precision(tdc_processor *p, int precision)
{
    if (int rc = check_proc(p)) return rc;
    if (precision != TDC_PRECISION_FP32_BULK && precision != TDC_PRECISION_FP64_PHASE)
        return fail(TDC_ERR_INVALID_ARGUMENT, "unknown precision");
    p->precision = precision;
    return TDC_OK;
}

int tdc_processor_set_skip_test(tdc_processor *p, int enable)
{
    if (int rc = check_proc(p)) return rc;
    p->skip_test = enable ? 1 : 0;
    p->prepared = false;
    return TDC_OK;
}

int tdc_processor_set_plan_pixels(tdc_processor *p, int64_t n_pix)
{
    if (int rc = check_proc(p)) return rc;
    if (n_pix < 0) return fail(TDC_ERR_INVALID_ARGUMENT, "n_pix must not be negative");
    p->plan_pixels = n_pix;
    return TDC_OK;
}

int tdc_processor_set_motion_path(tdc_processor *p, int enable)
{
    if (int rc = check_proc(p)) return rc;
    p->motion_enabled = enable != 0;
    return TDC_OK;
}

int tdc_processor_set_anchored_ranges(tdc_processor *p, int enable)
{
    if (int rc = check_proc(p)) return rc;
    p->anchor_enabled = enable != 0;
    p->plan_path = -1;  // the anchored instance may change the planned CTA slots
    return TDC_OK;
}

int tdc_processor_start(tdc_processor *p, float doppler_win_center, float doppler_bandwidth, int dop_centroid_win,
                        int apply_range_win, int doppler_win_taper)
{
    if (int rc = check_proc(p)) return rc;
    if (!p->has_raw) return fail(TDC_ERR_STATE, "setRawData must be called before start()");
    if (!p->has_grid) return fail(TDC_ERR_STATE, "setFocusGrid must be called before start()");
    NvtxRange nvtx("tdc start");
    const auto t0 = std::chrono::steady_clock::now();
    stats_reset(p);
    p->image_valid = false;
    int launches = 0;
    StartOpts o;
    o.center = doppler_win_center;
    o.bw = doppler_bandwidth;
    o.centroid = dop_centroid_win != 0;
    o.range_win = apply_range_win != 0;
    o.taper = doppler_win_taper != 0;
    o.skip_test = p->skip_test;
    TDC_CK(cudaSetDevice(p->device), "cudaSetDevice");
    cudaStream_t st = p->stream;
    TDC_CK(cudaEventRecord(p->ev[0], st), "event");
    if (int rc = prepare(p, o, launches)) return rc;
    if (int rc = upload_grid(p, launches)) return rc;
    TDC_CK(cudaEventRecord(p->ev[2], st), "event");
    const long long P = p->P;
    if (p->image_out && p->image_out_floats < 2 * P)
        return fail(TDC_ERR_INVALID_ARGUMENT, "image output buffer is smaller than the focus grid");
    // The reduction writes a caller-owned output in place where the device reads and
    // writes pageable host memory coherently; otherwise the image goes through device memory.
    const bool in_place = p->image_out && p->host_reads;
    if (!in_place) TDC_CK(p->image_dev.ensure((size_t)P * 8), "alloc image");
    float2 *dst = in_place ? reinterpret_cast<float2 *>(p->image_out) : p->image_dev.as<float2>();
    if (P > 0) {
        if (int rc = focus_resident(p, dst, st, launches)) return rc;
    }
    TDC_CK(cudaEventRecord(p->ev[3], st), "event");
    size_t d2h = 0;
    if (!in_place && P > 0) {
        void *host = p->image_out;
        if (!host) {
            TDC_CK(p->image_host.ensure((size_t)P * 8), "alloc host image");
            host = p->image_host.p;
        }
        TDC_CK(cudaMemcpyAsync(host, p->image_dev.p, (size_t)P * 8, cudaMemcpyDeviceToHost, st), "copy image");
        d2h = (size_t)P * 8;
    }
    TDC_CK(cudaEventRecord(p->ev[4], st), "event");
    // tdcprocessor.cpp:149-155: report any asynchronous failure of the launches.
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return fail(TDC_ERR_CUDA, std::string("Cuda runtime error occured during processing: ") +
                                      cudaGetErrorString(e));
    if (P > 0) {
        if (int rc = read_status(p)) return rc;
    }
    p->image_valid = true;
    p->stats.h2d_ms = elapsed(p->ev[0], p->ev[1]);
    p->stats.prep_ms = elapsed(p->ev[1], p->ev[2]);
    p->stats.focus_ms = elapsed(p->ev[2], p->ev[3]);
    p->stats.d2h_ms = elapsed(p->ev[3], p->ev[4]);
    p->stats.d2h_bytes = (int64_t)d2h;
    p->stats.kernel_launches = launches;
    p->stats.total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return TDC_OK;
}

const float *tdc_processor_image_buffer(const tdc_processor *p)
{
    if (!p || !p->image_valid) return nullptr;
    if (p->image_out) return p->image_out;
    return static_cast<const float *>(p->image_host.p);
}

int tdc_processor_set_image_output(tdc_processor *p, float *image_host, int64_t n_floats)
{
    if (int rc = check_proc(p)) return rc;
    if (image_host && n_floats <= 0) return fail(TDC_ERR_INVALID_ARGUMENT, "image output size must be positive");
    // The image of an earlier start() lives in the buffer it was written to.
    p->image_valid = false;
    p->image_out = image_host;
    p->image_out_floats = image_host ? n_floats : 0;
    return TDC_OK;
}

int tdc_processor_grid_shape(const tdc_processor *p, int *n_rows, int *n_cols)
{
    if (int rc = check_proc(p)) return rc;
    if (n_rows) *n_rows = p->rows;
    if (n_cols) *n_cols = p->cols;
    return TDC_OK;
}

int tdc_processor_last_stats(const tdc_processor *p, tdc_start_stats *out)
{
    if (int rc = check_proc(p)) return rc;
    if (!out) return fail(TDC_ERR_INVALID_ARGUMENT, "null output pointer");
    *out = p->stats;
    return TDC_OK;
}

// ---- device-resident entry points (for torch callers, benchmarks, autofocus) ----

int tdc_processor_prepare(tdc_processor *p, float doppler_win_center, float doppler_bandwidth,
                          int dop_centroid_win, int apply_range_win, int doppler_win_taper)
{
    if (int rc = check_proc(p)) return rc;
    StartOpts o;
    o.center = doppler_win_center;
    o.bw = doppler_bandwidth;
    o.centroid = dop_centroid_win != 0;
    o.range_win = apply_range_win != 0;
    o.taper = doppler_win_taper != 0;
    o.skip_test = p->skip_test;
    int launches = 0;
    return prepare(p, o, launches);
}

int tdc_processor_upload_grid(tdc_processor *p)
{
    if (int rc = check_proc(p)) return rc;
    int launches = 0;
    if (int rc = upload_grid(p, launches)) return rc;
    TDC_CK(cudaStreamSynchronize(p->stream), "grid sync");
    return TDC_OK;
}

int tdc_processor_focus_device(tdc_processor *p, float *image_dev, void *stream)
{
    if (int rc = check_proc(p)) return rc;
    if (!image_dev && p->P > 0) return fail(TDC_ERR_INVALID_ARGUMENT, "null image");
    TDC_CK(cudaSetDevice(p->device), "cudaSetDevice");
    int launches = 0;
    // NULL is the legacy default stream (torch's default stream), as for any CUDA API.
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    return focus_resident(p, reinterpret_cast<float2 *>(image_dev), st, launches);
}

int tdc_processor_check(tdc_processor *p, void *stream)
{
    if (int rc = check_proc(p)) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    TDC_CK(cudaStreamSynchronize(st), "focus sync");
    if (p->scratch.p) return read_status(p);
    return TDC_OK;
}

int tdc_processor_num_pixels(const tdc_processor *p, int64_t *n)
{
    if (int rc = check_proc(p)) return rc;
    if (n) *n = p->P;
    return TDC_OK;
}

int tdc_processor_reads_host_memory(const tdc_processor *p)
{
    return p && p->host_reads ? 1 : 0;
}

int tdc_processor_path(const tdc_processor *p)
{
    if (!p || !p->prepared || p->P <= 0) return -1;
    return choose_path(p);
}

int tdc_processor_set_keep_chirp_sums(tdc_processor *p, int keep)
{
    if (int rc = check_proc(p)) return rc;
    p->keep_sums = keep != 0;
    if (!p->keep_sums) {
        p->chirp_sums.release();
        p->xs_scaled.release();
        p->xs_scaled_ready = false;
        p->sums_epoch = 0;
    }
    return TDC_OK;
}

int tdc_processor_set_chirp_offsets_device(tdc_processor *p, const double *offsets_dev, void *stream)
{
    if (int rc = check_proc(p)) return rc;
    if (!p->prepared) return fail(TDC_ERR_STATE, "acquisition not prepared");
    if (!p->per_chirp) return fail(TDC_ERR_UNSUPPORTED, "chirp offsets need a per-chirp trajectory");
    TDC_CK(cudaSetDevice(p->device), "cudaSetDevice");
    TDC_CK(launch_chirp_positions(p->chirps.as<ChirpRec>(), p->pos_base.as<const double>(), offsets_dev, p->C,
                                  static_cast<cudaStream_t>(stream)),
           "chirp positions kernel");
    ++p->state_epoch;
    if (offsets_dev && !p->offsets_applied) {
        p->offsets_applied = true;
        p->plan_path = -1;  // replan without unit spans
    }
    return TDC_OK;
}

int tdc_processor_adjoint_device(tdc_processor *p, const float *grad_image_dev, double *grad_offsets_dev,
                                 void *stream)
{
    if (int rc = check_proc(p)) return rc;
    if (!p->prepared) return fail(TDC_ERR_STATE, "acquisition not prepared");
    if (p->P <= 0) return fail(TDC_ERR_STATE, "no focus grid");
    if (!grad_image_dev || !grad_offsets_dev) return fail(TDC_ERR_INVALID_ARGUMENT, "null gradient buffer");
    if (!p->per_chirp || choose_path(p) != TDC_PATH_FP32_BULK)
        return fail(TDC_ERR_UNSUPPORTED, "the adjoint needs the FP32-bulk path (per-chirp trajectory, uniform "
                                         "sample spacing)");
    if (needs_segments(p->s_pad))
        return fail(TDC_ERR_UNSUPPORTED, "the adjoint stages whole chirps: these chirps are too long");
    TDC_CK(cudaSetDevice(p->device), "cudaSetDevice");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const long long P = p->P;
    const int C = p->C;
    int cb = 1;
    const int stage_bytes = stage_bytes_for(p->s_pad, cb);
    // The forward's sums are usable when a storing focus ran on the current acquisition,
    // trajectory and grid (stream-ordered before this call).
    const bool stored = p->keep_sums && p->sums_epoch != 0 && p->sums_epoch == p->state_epoch && p->chirp_sums.p;
    if (stored && !p->xs_scaled_ready) {
        TDC_CK(p->xs_scaled.ensure((size_t)C * p->s_pad * sizeof(float2)), "alloc scaled rows");
        TDC_CK(launch_scale_rows(p->xw.as<const float2>(), C, p->s_pad, p->xs_scaled.as<float2>(), st),
               "scale rows kernel");
        p->xs_scaled_ready = true;
    }
    const int bps = adjoint_fp32_blocks_per_sm(stage_bytes, cb, stored);
    if (bps <= 0) return fail(TDC_ERR_CUDA, "adjoint kernel does not fit on the device");
    const int slots = p->n_sm * bps;
    int n_groups = 1, cpg = C;
    plan_groups((P + kFocusTile - 1) / kFocusTile, C, slots, n_groups, cpg, kFocusMinUnitsPerSlot);
    const long long n_tiles = (P + kFocusTile - 1) / kFocusTile;
    std::vector<FocusUnit> units;
    units.reserve((size_t)(n_tiles * n_groups));
    for (long long t = 0; t < n_tiles; ++t)
        for (int g = 0; g < n_groups; ++g) units.push_back(FocusUnit{0, (int)t, g, 0});
    const size_t off_job = 256;
    const size_t off_units = round_up(off_job + sizeof(FocusJob), 256);
    const size_t off_gpart = round_up(off_units + units.size() * sizeof(FocusUnit), 256);
    const size_t total = off_gpart + (size_t)n_tiles * C * 16;
    TDC_CK(p->adj_scratch.ensure(total), "alloc adjoint scratch");
    unsigned char *scr = p->adj_scratch.as<unsigned char>();
    FocusJob job = make_job(p, nullptr, cb, TDC_PATH_FP32_BULK);
    job.n_groups = n_groups;
    job.chirps_per_group = cpg;
    if (stored) {
        job.xw = p->xs_scaled.as<const float4>();
        job.chirp_sums = p->chirp_sums.as<float2>();
    }
    TDC_CK(cudaMemcpyAsync(scr + off_job, &job, sizeof(job), cudaMemcpyHostToDevice, st), "copy job");
    TDC_CK(cudaMemcpyAsync(scr + off_units, units.data(), units.size() * sizeof(FocusUnit), cudaMemcpyHostToDevice,
                           st),
           "copy units");
    TDC_CK(cudaMemsetAsync(scr, 0, 8, st), "reset counter");
    float4 *gpart = reinterpret_cast<float4 *>(scr + off_gpart);
    const int grid = (int)std::min<long long>((long long)units.size(), slots);
    TDC_CK(launch_adjoint_fp32(reinterpret_cast<const FocusJob *>(scr + off_job),
                               reinterpret_cast<const FocusUnit *>(scr + off_units), (int)units.size(),
                               reinterpret_cast<int *>(scr), reinterpret_cast<int *>(scr) + 1, stage_bytes, cb, grid,
                               reinterpret_cast<const float2 *>(grad_image_dev), gpart, stored, st),
           "adjoint kernel");
    p->stats.adjoint_stored = stored ? 1 : 0;
    TDC_CK(launch_adjoint_reduce(gpart, (int)n_tiles, C, grad_offsets_dev, st), "adjoint reduce kernel");
    // The host copies above are from stack/vector memory: finish before they go out of scope,
    // and collect the kernel's status word.
    TDC_CK(cudaStreamSynchronize(st), "adjoint sync");
    int status = 0;
    TDC_CK(cudaMemcpy(&status, scr + sizeof(int), sizeof(int), cudaMemcpyDeviceToHost), "read status");
    if (status & kStatusTimeout) return fail(TDC_ERR_TIMEOUT, "adjoint kernel wait timed out");
    return TDC_OK;
}

int tdc_range_window(float *w_dev, int n_samples, int apply_range_win, void *stream)
{
    if (n_samples <= 0) return fail(TDC_ERR_INVALID_ARGUMENT, "nSamples must be greater than 0");
    if (!w_dev) return fail(TDC_ERR_INVALID_ARGUMENT, "null window");
    TDC_CK(launch_range_window(w_dev, n_samples, apply_range_win, static_cast<cudaStream_t>(stream)),
           "range window kernel");
    return TDC_OK;
}

}  // extern "C"
