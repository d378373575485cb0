// tdc_internal.h -- structures shared by the host code and the kernels of the
// GB300 TDC engine. Not part of the public ABI (include/tdc_gb300.h is).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <string>

namespace tdc {

constexpr double kC0 = 299792458.0;  // SPEED_OF_LIGHT, tdcprocessor.cpp:37
constexpr int kChunk = 128;          // PRI_CHUNKSIZE, tuning.h:18
constexpr float kRangeA = 25.0f / 46.0f;    // RANGE_WINDOW_A_PARAMETER, tuning.h:31
constexpr float kAzimuthA = 25.0f / 46.0f;  // AZIMUTH_WINDOW_A_PARAMETER, tuning.h:38

// Focus tile geometry of the FP32-bulk kernel: 128 threads x TDC_FOCUS_PT pixels.
#ifndef TDC_FOCUS_PT
#define TDC_FOCUS_PT 4
#endif
constexpr int kFocusThreads = 128;
constexpr int kFocusPT = TDC_FOCUS_PT;
constexpr int kFocusTile = kFocusThreads * kFocusPT;
constexpr int kFocusStages = 3;
constexpr int kSampleAlign = 16;  // s_pad is a multiple of this (bulk-copy rows stay 128-byte sized)
#ifndef TDC_FOCUS_STAGE_TARGET
#define TDC_FOCUS_STAGE_TARGET 16640
#endif
constexpr int kFocusStageTarget = TDC_FOCUS_STAGE_TARGET;  // bytes of chirp rows + records per pipeline stage
// Anchored ranges of the FP32-bulk kernel (pixels of a warp share a double-float anchor
// range per chirp, each adds its FP32 range difference): at most this many chirps per stage,
// and no pixel farther than kAnchorMaxDistance from its anchor. At 5 cm the FP32 range
// difference keeps the phase within ~3e-5 rad of the double-float range's at 77 GHz (1e-5 at
// the 1.6 cm of a 1 mm grid; tests/test_anchor_error_cpu.py).
constexpr int kAnchorMaxStageChirps = 16;
constexpr double kAnchorMaxDistance = 0.05;  // metres
// Fewest work units per CTA slot the planner aims for where the grid and chirps allow
// it. CTAs that share an SM need not progress at the same rate, so with a few long
// units per slot the last units end far apart (measured on 256^2 pixels x 256 chirps
// x 1024 samples, general kernel: SMs busy 72-100% of the launch at 3 units per slot,
// +14% throughput at 4 or more).
#ifndef TDC_GENERAL_MIN_UNITS
#define TDC_GENERAL_MIN_UNITS 4
#endif
#ifndef TDC_FOCUS_MIN_UNITS
#define TDC_FOCUS_MIN_UNITS 8
#endif
constexpr int kGeneralMinUnitsPerSlot = TDC_GENERAL_MIN_UNITS;
constexpr int kFocusMinUnitsPerSlot = TDC_FOCUS_MIN_UNITS;
// Pixels per thread of the FP32 general kernel (per-sample trajectories / windows, non-uniform sampling).
#ifndef TDC_GENERAL_PT
#define TDC_GENERAL_PT 2
#endif
constexpr int kGeneralPT = TDC_GENERAL_PT;

// One chirp's trajectory record, 48 bytes (3 x float4):
//   p_hi.xyz  antenna position, high float of a double-float pair; p_hi.w = Doppler window centre [Hz]
//   p_lo.xyz  low float of the position pair; p_lo.w = 0
//   vel.xyz   velocity; vel.w = 0
struct __align__(16) ChirpRec {
    float4 p_hi;
    float4 p_lo;
    float4 vel;
};
static_assert(sizeof(ChirpRec) == 48, "ChirpRec must be 48 bytes");

// One chirp's record for the smooth-motion kernel, 80 bytes (5 x float4): positions of
// the chirp's samples as P[c, s] = P0 + V1 s + V2 s^2 (the host's fit of the per-sample
// positions).
//   p_hi.xyz, p_lo.xyz  P0 as double-float pairs; p_hi.w = Doppler window centre [Hz]; p_lo.w = 0
//   vel.xyz             velocity at sample 0 (Doppler window); vel.w = 2 V1.V2
//   v1.xyz              V1 [m / sample]; v1.w = |V1|^2
//   v2.xyz              V2 [m / sample^2]; v2.w = |V2|^2
struct __align__(16) MotionRec {
    float4 p_hi;
    float4 p_lo;
    float4 vel;
    float4 v1;
    float4 v2;
};
static_assert(sizeof(MotionRec) == 80, "MotionRec must be 80 bytes");

// One sample point of the reference's chunk skip test (tdcprocessor.cpp:355-378).
struct __align__(16) SkipPoint {
    float4 pos_fdc;  // position xyz, window centre
    float4 vel;      // velocity xyz, 0
};
static_assert(sizeof(SkipPoint) == 32, "SkipPoint must be 32 bytes");

enum FocusFlags : int {
    kFlagTaper = 1,     // dopplerWinTaper
    kFlagSkipTest = 2,  // apply the per-chunk skip test
    kFlagMotionExactQL = 4,  // smooth-motion kernel: block step per segment from an accurate sincos
};

// Everything a focus kernel needs about one job (acquisition x grid).
struct FocusJob {
    const float4 *xw;        // [C][s_pad/2]: pairs of windowed complex samples
    const ChirpRec *chirps;  // [C] (or [C][S] for per-sample trajectories)
    const float4 *grid_hi;   // [P]
    const float4 *grid_lo;   // [P] or nullptr
    const SkipPoint *skip;   // [n_chunks][9]
    const double *gs;        // [S] 2 f_s / c0 (FP64 kernels only)
    const float4 *traj;      // [C][s_pad] (P[c,s] - P[c,0], |P[c,s] - P[c,0]|^2) (FP32 general kernel, per-sample positions)
    const float4 *wins;      // [C][s_pad] (velocity x -2/(lambda B), window centre / B) per sample (FP32 general
                             // kernel, per-sample windows); the velocity term halved when positions also
                             // move within chirps
    const float *wdot;       // [C][s_pad] velocity x -2/(lambda B) . (P[c,s] - P[c,0]) (per-sample positions
                             // and windows)
    const float *gres;       // [s_pad] 2 f_s / c0 - (g0 + g1 s) (FP32 general kernel, non-uniform sampling)
    const float *gsam;       // [s_pad] 2 f_s / c0 [cycles / m] (wide variants) or 2 pi x that [rad / m]
                             // (narrow variants) (FP32 general kernel, per-sample positions)
    float4 *partial;         // [n_groups][P]: (sum.re, sum.im, comp.re, comp.im)
    float2 *chirp_sums;      // [C][P] per-(chirp, pixel) sums A = sum_s x_s z^s: written by the storing
                             // focus instance, read by the adjoint that uses them (else null)
    long long P;
    int C;
    int S;
    int s_pad;
    int n_groups;
    int chirps_per_group;
    int chunk;
    int stage_chirps;        // chirps per pipeline stage
    int flags;
    int n_tiles;
    int per_sample;          // ChirpRec per sample instead of per chirp
    float g0_hi, g0_lo;      // 2 f_0 / c0 as a double-float pair [cycles / m]
    float g1;                // 2 df / c0 per sample [cycles / m]
    float two_over_lambda;   // 2 / lambda_centre
    float half_bw;           // dopplerBandwidth / 2
    float inv_bw;            // 1 / dopplerBandwidth
    float az_a;              // azimuth window a
    float g1_lo;             // low part of g1 (double-float pair)
    int seg_len;             // samples per pipeline stage of a chirp staged in segments (FP32 bulk: 0 for
                             // whole rows; FP32 general: s_pad for whole rows)
    int tile_cols;           // 0: a tile is kFocusTile consecutive pixels; else kFocusTile / tile_cols grid
                             // rows x tile_cols columns of the grid_cols-wide row-major grid
    int grid_cols;           // columns of the focus grid (block tiles)
    int pad_;
};

// Kernels copy a FocusJob into shared memory one int per thread (128 threads); the
// no-allocation scratch reserves 256 bytes for it.
static_assert(sizeof(FocusJob) <= 256 && sizeof(FocusJob) % 8 == 0, "FocusJob layout");

// Tiles of a P-pixel grid (see FocusJob::tile_cols).
inline long long tile_count(long long P, int tile_cols, int grid_cols)
{
    if (tile_cols <= 0 || grid_cols <= 0) return (P + kFocusTile - 1) / kFocusTile;
    const long long rows = (P + grid_cols - 1) / grid_cols;
    const int tile_rows = kFocusTile / tile_cols;
    return ((rows + tile_rows - 1) / tile_rows) * ((grid_cols + tile_cols - 1) / tile_cols);
}

struct FocusUnit {
    int job;
    int tile;
    int group;
    int span;  // 0: the group's chirps; else unit_span(lo, hi): the chirps group x cpg + [lo, hi)
               // (the FP32-bulk kernels; the host sets it only for chirps the tile cannot see in band)
};
// FocusUnit::span: a marker bit and two 15-bit chirp offsets within the group (groups of
// fewer than kUnitSpanMax chirps).
constexpr int kUnitSpanMax = 1 << 15;
__host__ __device__ constexpr int unit_span(int lo, int hi) { return (1 << 30) | (lo << 15) | hi; }
__host__ __device__ constexpr int unit_span_lo(int span) { return (span >> 15) & (kUnitSpanMax - 1); }
__host__ __device__ constexpr int unit_span_hi(int span) { return span & (kUnitSpanMax - 1); }

// Kernel-side status bits (written to the status word in scratch).
enum StatusBits : int {
    kStatusTimeout = 1,
    kStatusBadJob = 2,  // a kernel found a job record outside what it takes (no work done for it)
};

// ---- launchers (defined in the .cu files) ----
cudaError_t launch_range_window(float *w, int n, int apply, cudaStream_t st);
cudaError_t launch_prewindow(float2 *xw, const float *w, int C, int S, int s_pad, cudaStream_t st);
cudaError_t launch_chirp_positions(ChirpRec *recs, const double *base, const double *off, int C, cudaStream_t st);
// Direct-read ingest (source may be pageable host memory where the device reads it coherently).
cudaError_t launch_prewindow_from(const float2 *src, const float *w, int C, int S, int s_pad, float2 *xw,
                                  cudaStream_t st);
cudaError_t launch_rows_differ(const float *a, int C, int S, int k, int *flag, cudaStream_t st);
cudaError_t launch_grid_bbox(const float4 *hi, long long P, int *out, cudaStream_t st);
cudaError_t launch_grid_from_f32(const float *grid, long long P, float4 *hi, cudaStream_t st);
cudaError_t launch_grid_from_f64(const double *grid, long long P, float4 *hi, float4 *lo, cudaStream_t st);

// FP32-bulk focus over a unit list. `jobs` and `units` are device arrays.
// Long chirps (rows longer than the stages hold): the same focus with rows staged in
// segments of job.seg_len samples; stage_bytes >= seg_len x 8 + one record.
cudaError_t launch_focus_fp32_seg(const FocusJob *jobs_dev, const FocusUnit *units_dev, int n_units,
                                  int *counter_dev, int *status_dev, int stage_bytes, int grid_ctas, bool skip_zero,
                                  cudaStream_t st);
int focus_fp32_seg_blocks_per_sm(int stage_bytes);
// skip_zero: skip chirps whose window is zero for a whole warp (any job with a finite band).
// store_sums: also write job.chirp_sums (whole-row staging only).
// anchored: anchored ranges (neither skip_zero nor store_sums; flat tiles; at most
// kAnchorMaxStageChirps chirps a stage; every pixel within kAnchorMaxDistance of its anchor).
cudaError_t launch_focus_fp32(const FocusJob *jobs_dev, const FocusUnit *units_dev, int n_units,
                              int *counter_dev, int *status_dev, int stage_bytes, int grid_ctas,
                              bool skip_zero, bool store_sums, bool anchored, cudaStream_t st);
int focus_fp32_anchor_blocks_per_sm(int stage_bytes);
// Smooth-motion focus (tdc_motion.cu): per-sample positions given by job.chirps as
// MotionRec records, rows staged whole (stage_bytes >= chirps x (s_pad x 8 + 80)),
// psi linearised over segments of job.seg_len samples (a power of two >= 8).
cudaError_t launch_focus_motion(const FocusJob *jobs_dev, const FocusUnit *units_dev, int n_units, int *counter_dev,
                                int *status_dev, int stage_bytes, int grid_ctas, bool skip_zero, cudaStream_t st);
int focus_motion_blocks_per_sm(int stage_bytes);
int focus_motion_smem_bytes(int stage_bytes);
// Plain FP64-phase focus (comparator and general fallback), one CTA per unit.
cudaError_t launch_focus_fp64(const FocusJob *jobs_dev, const FocusUnit *units_dev, int n_units,
                              int *status_dev, int per_sample, cudaStream_t st);
cudaError_t launch_focus_reduce(const float4 *partial, int n_groups, long long P, float2 *image,
                                cudaStream_t st);
// FP32 general focus (tdc_general.cu). variant bits: 1 per-sample positions, 2 per-sample
// windows, 4 wide (non-uniform sampling residual, large intra-chirp motion: reduced phase
// correction, longer range-change series); at least one set. Rows are staged job.seg_len
// samples at a time: whole rows (seg_len = s_pad, job.stage_chirps chirps a stage) or
// segments of one chirp; stage_bytes = chirps x (seg_len x row bytes per sample + one
// record) + seg_len x table bytes per sample (see general_stage_bytes_for).
cudaError_t launch_focus_general(int variant, const FocusJob *jobs_dev, const FocusUnit *units_dev, int n_units,
                                 int *counter_dev, int *status_dev, int stage_bytes, int grid_ctas, cudaStream_t st);
int focus_general_blocks_per_sm(int variant, int stage_bytes);
int focus_general_smem_bytes(int stage_bytes);

// Adjoint of the FP32-bulk focus w.r.t. per-chirp position offsets: per-(tile, chirp)
// float4 partials, then an FP64 sum over tiles into grad[C][3]. stored: job.xw holds the
// rows pre-scaled by the sample index and job.chirp_sums the forward's per-(chirp, pixel)
// sums (flat tiles).
cudaError_t launch_adjoint_fp32(const FocusJob *jobs_dev, const FocusUnit *units_dev, int n_units, int *counter_dev,
                                int *status_dev, int stage_bytes, int stage_chirps, int grid_ctas,
                                const float2 *gimg, float4 *gpart, bool stored, cudaStream_t st);
cudaError_t launch_adjoint_reduce(const float4 *gpart, int n_tiles, int C, double *grad, cudaStream_t st);
int adjoint_fp32_blocks_per_sm(int stage_bytes, int stage_chirps, bool stored);
// rows_out[c][s] = s * rows[c][s] (complex, [C][s_pad]): the adjoint's pre-scaled rows.
cudaError_t launch_scale_rows(const float2 *rows, int C, int s_pad, float2 *rows_out, cudaStream_t st);
int adjoint_fp32_smem_bytes(int stage_bytes, int stage_chirps);

// Let `fn` launch with as much dynamic shared memory as the device allows. The attribute
// is process-wide per kernel: every caller sets this same value, so threads that plan
// and launch with different sizes at the same time cannot undercut one another.
template <class F>
inline cudaError_t allow_max_dynamic_smem(F *fn)
{
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes a{};
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, reinterpret_cast<const void *>(fn));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(reinterpret_cast<const void *>(fn), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 optin - (int)a.sharedSizeBytes);
    return e;
}

// Record `msg` as the calling thread's tdc_last_error() and return `code`.
int set_last_error(int code, const char *msg);
inline int set_last_error(int code, const std::string &msg) { return set_last_error(code, msg.c_str()); }

// Occupancy of the FP32-bulk kernel at a given dynamic shared memory size.
int focus_fp32_blocks_per_sm(int stage_bytes);
int focus_fp32_smem_bytes(int stage_bytes, bool anchored = false);

}  // namespace tdc
