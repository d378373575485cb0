// tdc_processor_impl.h -- internal definition of the processor (the state behind
// the tdc_processor handle of include/tdc_gb300.h) and the host-side steps of a
// focus, shared by the C ABI (tdc_capi.cpp) and the request loop (tdc_server.cpp).
#pragma once

#include <cuda_runtime.h>

#include <cstring>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "tdc_gb300.h"
#include "tdc_internal.h"

namespace tdc {
namespace impl {

// NVTX range for profilers (no cost when no tool is attached).
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// Grow-only device buffer. With alloc_stream set, memory comes from the device's
// stream-ordered pool (cudaMallocAsync / cudaFreeAsync on that stream), so growing
// or releasing it does not synchronise the device the way cudaFree does; the owner
// then releases it before the stream is destroyed.
struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    cudaStream_t alloc_stream = nullptr;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release()
    {
        if (p) {
            if (alloc_stream) cudaFreeAsync(p, alloc_stream);
            else cudaFree(p);
        }
        p = nullptr;
        cap = 0;
    }
    cudaError_t ensure(size_t bytes)
    {
        if (bytes == 0) bytes = 16;
        if (bytes <= cap) return cudaSuccess;
        release();
        cudaError_t e = alloc_stream ? cudaMallocAsync(&p, bytes, alloc_stream) : cudaMalloc(&p, bytes);
        if (e == cudaSuccess) cap = bytes;
        else p = nullptr;
        return e;
    }
    template <class T>
    T *as() const
    {
        return static_cast<T *>(p);
    }
};

// Grow-only pinned host buffer.
struct PinnedBuf {
    void *p = nullptr;
    size_t cap = 0;
    PinnedBuf() = default;
    PinnedBuf(const PinnedBuf &) = delete;
    PinnedBuf &operator=(const PinnedBuf &) = delete;
    ~PinnedBuf() { release(); }
    void release()
    {
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
    }
    cudaError_t ensure(size_t bytes)
    {
        if (bytes == 0) bytes = 16;
        if (bytes <= cap) return cudaSuccess;
        release();
        cudaError_t e = cudaMallocHost(&p, bytes);
        if (e == cudaSuccess) cap = bytes;
        else p = nullptr;
        return e;
    }
};

inline size_t round_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

inline void split_dd(double v, float &h, float &l)
{
    h = static_cast<float>(v);
    l = static_cast<float>(v - static_cast<double>(h));
}

struct StartOpts {
    float center = 0.f;
    float bw = 0.f;
    int centroid = 0;
    int range_win = 1;
    int taper = 1;
    int skip_test = 1;
};

int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);

#define TDC_CK(call, what)                           \
    do {                                             \
        cudaError_t e_ = (call);                     \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

}  // namespace impl
}  // namespace tdc

struct tdc_processor {
    int device = 0;
    int n_sm = 0;
    bool host_reads = false;  // the device reads pageable host memory coherently (Grace-Blackwell C2C)
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[6] = {};
    // Borrowed inputs (setRawData / setFocusGrid).
    const float *raw = nullptr;
    const float *pri_times = nullptr;
    const float *sample_times = nullptr;
    const float *pos = nullptr;
    const float *vel = nullptr;
    const float *att = nullptr;
    const double *pos64 = nullptr;
    bool traj_per_chirp = false;  // pos / vel / att hold one row per chirp instead of one per sample
    int C = 0, S = 0;
    float mod_rate = 0.f, start_freq = 0.f;
    float bore[3] = {0.f, 0.f, 0.f};
    float lambda = 0.f;
    bool has_raw = false;

    const float *grid = nullptr;
    const double *grid64 = nullptr;
    int rows = 0, cols = 0;
    bool has_grid = false;

    int precision = TDC_PRECISION_FP32_BULK;
    int skip_test = 1;

    // Prepared acquisition (device resident).
    bool prepared = false;
    tdc::impl::StartOpts opts;
    bool per_chirp = true;
    bool traj_varies = false;   // positions differ within a chirp (FP32 per-sample positions)
    bool sample_recs_ready = false;  // chirps holds the per-(chirp, sample) records
    bool win_varies = false;    // the Doppler window can differ within a chirp (finite band, per-sample motion)
    double delta_max = 0.0;     // max |P[c,s] - P[c,0]| [m]
    // Smooth intra-chirp motion: every chirp's per-sample positions are P0 + V1 s + V2 s^2 to
    // within the rounding of their FP32 values (motion_rec holds the fits); the smooth-motion
    // kernel then runs instead of the FP32 general kernel, unless switched off.
    bool motion_fit_ok = false;
    bool motion_enabled = true;
    double motion_v1max = 0.0;  // max |V1| [m / sample]
    double motion_v2max = 0.0;  // max |V2| [m / sample^2]
    double F0 = 0.0, F1 = 0.0, resid_hz = 0.0;
    double ant_min[3] = {0, 0, 0}, ant_max[3] = {0, 0, 0};
    int s_pad = 0, n_chunks = 0;
    tdc::impl::DevBuf xw, chirps, skip, gs, pos_base, wr, offsets, flag;
    // FP32 general path: sample-0 records per chirp (when chirps holds one per sample),
    // per-sample offsets / windows, residual frequency table.
    tdc::impl::DevBuf gen_rec, traj, wins, wdot, gres;
    // Smooth-motion kernel: one MotionRec per chirp.
    tdc::impl::DevBuf motion_rec;
    // Autofocus: the forward's per-(chirp, pixel) sums and the rows pre-scaled by the sample
    // index, so the adjoint computes only the index-weighted sums (keep_sums on).
    tdc::impl::DevBuf chirp_sums, xs_scaled;
    bool keep_sums = false;
    bool xs_scaled_ready = false;
    uint64_t state_epoch = 1;  // bumped when the prepared acquisition, its trajectory or the grid change
    uint64_t sums_epoch = 0;   // state_epoch of the focus that wrote chirp_sums (0: none)

    // Device grid.
    long long P = 0;
    bool grid_lo_valid = false;
    double grid_min[3] = {0, 0, 0}, grid_max[3] = {0, 0, 0};
    double axis_c[3] = {0, 0, 0}, axis_r[3] = {0, 0, 0};  // grid column / row steps (first pixel's)
    // Anchored ranges of the FP32-bulk kernel: the largest distance of a pixel from the anchor
    // of its group of 32 consecutive pixels (the group's 17th pixel, or its last); the kernel
    // takes them when this is within kAnchorMaxDistance, unless switched off.
    double anchor_span = 0.0;
    bool anchor_enabled = true;
    bool rec_finite = false;  // every chirp record's velocity and window centre is finite
    double vel_dir[3] = {0, 0, 0};                         // mean antenna velocity direction (0: at rest)
    tdc::impl::DevBuf grid_stage, grid_hi, grid_lo;
    // Centre pixel (x, y, z) of each work tile, flat tiles and block tiles.
    std::vector<double> tile_centre_flat, tile_centre_block;
    // Largest distance from each tile's centre pixel to its other pixels (flat, block tiles).
    std::vector<double> tile_radius_flat, tile_radius_block;
    // Chirp offsets applied on the device since the last prepare (rec_host's positions are then
    // not the ones the kernels use: no unit spans from them).
    bool offsets_applied = false;
    int span_permille = 1000;  // chirps the planned units visit, per mille of tiles x chirps
    // Host copy of the chirp records (sample 0), for the planner's cost estimate.
    std::vector<tdc::ChirpRec> rec_host;

    // Focus plan cache + scratch.
    tdc::impl::DevBuf scratch;
    std::vector<tdc::FocusUnit> units_host;
    long long plan_P = -1;
    int plan_C = -1, plan_groups = 0, plan_cpg = 0, plan_path = -1, plan_slots = 0, plan_tile_cols = -1,
        plan_cols = -1;
    double plan_unit_cap = 0.0;
    long long plan_tiles = -1;   // tiles the chirp groups were planned for
    long long plan_pixels = 0;   // plan the chirp groups for a grid of this many pixels (0: the grid's own)
    bool plan_uploaded = false;

    // Adjoint (autofocus) scratch.
    tdc::impl::DevBuf adj_scratch;

    tdc::impl::DevBuf image_dev;
    tdc::impl::PinnedBuf image_host;
    tdc::impl::PinnedBuf table_host;  // staging of the per-acquisition tables (prepare)
    float *image_out = nullptr;  // caller-owned image output (borrowed), or null
    int64_t image_out_floats = 0;
    bool image_valid = false;

    tdc_start_stats stats{};

    // Every device buffer the processor owns.
    std::vector<tdc::impl::DevBuf *> device_buffers()
    {
        return {&xw,      &chirps,     &skip,    &gs,      &pos_base, &wr,      &offsets,     &flag,     &gen_rec,
                &traj,    &wins,       &wdot,    &gres,    &grid_stage, &grid_hi, &grid_lo, &scratch, &adj_scratch,
                &chirp_sums, &xs_scaled, &motion_rec,
                &image_dev};
    }
};

namespace tdc {
namespace impl {

// Work plan of one focus of a processor's resident acquisition onto its resident grid.
struct FocusPlan {
    int path = 0;         // tdc_path
    int variant = 0;      // FP32 general kernel variant bits (TDC_PATH_GENERAL)
    bool seg = false;     // FP32-bulk rows staged in segments (chirps longer than the stages hold)
    int cb = 1;           // chirps per pipeline stage
    int stage_bytes = 0;  // bytes per pipeline stage
    int slots = 0;        // resident CTAs of the kernel on the device
    bool anchored = false;  // FP32-bulk kernel with anchored ranges
    size_t off_job = 0;   // job record and unit table offsets in the processor's scratch
    size_t off_units = 0;
    FocusJob job{};       // partial -> the processor's scratch
};

int prepare(tdc_processor *p, const StartOpts &o, int &launches);
int upload_grid(tdc_processor *p, int &launches);
int choose_path(const tdc_processor *p);
void plan_groups(long long n_tiles, int C, int slots, int &n_groups, int &cpg, int min_units_per_slot);
// Tile shape of the resident grid: 0 (flat tiles) or the columns of a block tile.
int choose_tile_cols(const tdc_processor *p);
int stage_bytes_for(int s_pad, int &cb);
// True when a whole row of s_pad samples does not fit the FP32-bulk kernel's stages.
bool needs_segments(int s_pad);
// Stage bytes of the FP32 general kernel for a variant (bit 1 per-sample positions, 2 windows).
// FP32 general kernel stages: bytes of a stage of rows staged `seg` samples at a time
// (seg = s_pad: whole rows, cb chirps a stage; else cb = 1), the samples of a balanced
// segment, and the staging the focus uses (whole rows unless they do not fit or
// segments keep more CTAs resident).
int general_stage_bytes_for(int s_pad, int variant, int seg, int &cb);
int general_segment_samples(int s_pad, int variant);
int general_seg_len(int s_pad, int variant);
// Variant bits of the FP32 general kernel for the resident acquisition.
int general_variant(const tdc_processor *p);
// Segment length (samples, a power of two) of the smooth-motion kernel for the resident
// acquisition and grid, or 0 when that kernel does not take them.
int motion_segment(const tdc_processor *p);
int motion_stage_bytes_for(int s_pad, int &cb);
FocusJob make_job(const tdc_processor *p, float4 *partial, int cb, int path);
// Plan units (p->units_host) and make sure the processor's scratch holds them and the partials.
// max_unit_work > 0 bounds the correlations of one unit (the request loop's granularity).
int focus_plan(tdc_processor *p, FocusPlan &plan, double max_unit_work = 0.0);
// Request-loop slots: recreate the processor's stream at `priority` (cudaDeviceGetStreamPriorityRange
// order) and take its device buffers from the stream-ordered pool on that stream.
int processor_use_slot_stream(tdc_processor *p, int priority);
// Give back the processor's device memory (the resident acquisition and grid are dropped).
void processor_release_memory(tdc_processor *p);
// Device bytes the processor holds.
size_t processor_device_bytes(tdc_processor *p);

}  // namespace impl
}  // namespace tdc
