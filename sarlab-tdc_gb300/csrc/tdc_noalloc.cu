// tdc_noalloc.cu -- the focus entry point that allocates nothing.
//
// Some callers cannot allocate device memory when they focus: radar processing
// chains that provision all device memory once at start-up and must not
// allocate afterwards (real-time and certified pipelines with a fixed memory
// budget), plug-ins running inside a host framework that owns the device
// allocator, and code that must not call cudaMalloc while a stream is being
// captured. For them, tdc_focus_noalloc runs the same FP32-bulk focus kernel
// (focus_fp32_kernel) and reduce kernel as tdc_processor_focus_device, on
// device inputs and an output the caller provides, with the kernel's scratch
// (work counter, status word, job record, unit table, per-group partial sums)
// taken from a file-scope __device__ array of TDC_NOALLOC_SCRATCH_BYTES instead
// of cudaMalloc. Every GPU that loads this library holds that array until the
// process exits.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <limits>
#include <mutex>
#include <string>

#include "tdc_gb300.h"
#include "tdc_internal.h"
#include "tdc_processor_impl.h"

using namespace tdc;

namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[TDC_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
// Device address of g_noalloc_scratch per device, as last looked up with that device
// current. Calls outside stream capture look it up again (cheap), so a device reset or
// another context made current since is picked up; calls under capture use this copy.
unsigned char *g_scratch_addr[kMaxDevices] = {};

size_t round_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

constexpr size_t kOffStatus = 0;    // int counter, int status
constexpr size_t kOffJob = 256;     // FocusJob
constexpr size_t kOffUnits = 512;   // FocusUnit[n_units]

size_t layout_bytes(long long P, long long n_units, int n_groups, size_t &off_partial)
{
    off_partial = round_up(kOffUnits + (size_t)n_units * sizeof(FocusUnit), 256);
    return off_partial + (size_t)n_groups * (size_t)P * 16;
}

// Job record, unit table (tile-major, one unit per tile x chirp group) and zeroed
// counter / status written into the scratch array by the device itself.
__global__ void noalloc_setup_kernel(FocusJob job, int n_tiles, int n_groups, unsigned char *base)
{
    const long long n_units = (long long)n_tiles * n_groups;
    const long long i0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i0 == 0) {
        int *words = reinterpret_cast<int *>(base + kOffStatus);
        words[0] = 0;
        words[1] = 0;
        *reinterpret_cast<FocusJob *>(base + kOffJob) = job;
    }
    FocusUnit *units = reinterpret_cast<FocusUnit *>(base + kOffUnits);
    for (long long u = i0; u < n_units; u += (long long)gridDim.x * blockDim.x) {
        units[u] = FocusUnit{0, (int)(u / n_groups), (int)(u % n_groups), 0};
    }
}

int fail(int code, const std::string &msg) { return set_last_error(code, msg); }

void split_dd(double v, float &h, float &l)
{
    h = static_cast<float>(v);
    l = static_cast<float>(v - static_cast<double>(h));
}

// Chirp groups so that tiles x groups fill whole waves of `slots` (among the splits
// with at least kFocusMinUnitsPerSlot units per slot when there are any), limited to
// what fits in the scratch array.
bool plan(long long P, int C, int slots, int &n_groups, int &cpg, size_t &off_partial)
{
    const long long n_tiles = (P + kFocusTile - 1) / kFocusTile;
    const long long min_units = (long long)kFocusMinUnitsPerSlot * slots;
    const int gmax = std::max(1, std::min(C, 1024));
    for (int pass = 0; pass < 2; ++pass) {
        double best = std::numeric_limits<double>::infinity();
        for (int g = 1; g <= gmax; ++g) {
            const int c = (C + g - 1) / g;
            const int geff = (C + c - 1) / c;
            if (geff != g) continue;
            size_t off;
            if (layout_bytes(P, n_tiles * geff, geff, off) > TDC_NOALLOC_SCRATCH_BYTES) break;
            if (pass == 0 && n_tiles * geff < min_units) continue;
            const long long waves = (n_tiles * geff + slots - 1) / slots;
            const double cost = (double)waves * (c + 0.5);
            if (cost < best - 1e-9) {
                best = cost;
                n_groups = geff;
                cpg = c;
                off_partial = off;
            }
        }
        if (best < std::numeric_limits<double>::infinity()) return true;
    }
    return false;
}

// Checks, plans and enqueues the setup, focus and reduce kernels on `st`; nothing
// blocks. `status_word` receives the device address of the kernels' status word.
int enqueue(const tdc_noalloc_focus_args *a, float *image_dev, cudaStream_t st, int **status_word)
{
    // ---- argument and size checks first: nothing below runs for rejected sizes ----
    if (!a || !image_dev) return fail(TDC_ERR_INVALID_ARGUMENT, "null argument");
    if (a->n_pri <= 0) return fail(TDC_ERR_INVALID_ARGUMENT, "nPri must be greater than 0");
    if (a->n_samples <= 0) return fail(TDC_ERR_INVALID_ARGUMENT, "nSamples must be greater than 0");
    if (a->n_pix <= 0) return fail(TDC_ERR_INVALID_ARGUMENT, "n_pix must be greater than 0");
    if (!a->samples || !a->chirps || !a->grid_hi) return fail(TDC_ERR_INVALID_ARGUMENT, "null input array");
    if ((reinterpret_cast<uintptr_t>(a->samples) | reinterpret_cast<uintptr_t>(a->chirps) |
         reinterpret_cast<uintptr_t>(a->grid_hi) | reinterpret_cast<uintptr_t>(a->grid_lo) |
         reinterpret_cast<uintptr_t>(a->skip_points)) & 15u)
        return fail(TDC_ERR_INVALID_ARGUMENT, "input arrays must be 16-byte aligned");
    const long long P = a->n_pix;
    const int C = a->n_pri, S = a->n_samples;
    const int s_pad = (int)round_up((size_t)S, kSampleAlign);
    const long long n_tiles = (P + kFocusTile - 1) / kFocusTile;
    size_t min_off;
    const size_t min_bytes = layout_bytes(P, n_tiles, 1, min_off);
    if (min_bytes > TDC_NOALLOC_SCRATCH_BYTES || n_tiles > (1LL << 30)) {
        return fail(TDC_ERR_UNSUPPORTED, "tdc_focus_noalloc: " + std::to_string(P) + " pixels need " +
                                             std::to_string(min_bytes) + " bytes of scratch; the fixed array "
                                             "holds " + std::to_string((size_t)TDC_NOALLOC_SCRATCH_BYTES) +
                                             " (about 2M pixels)");
    }
    // Whole rows only (the processor stages longer rows in segments): the same limit as
    // the processor's choice between the two, TDC_NOALLOC_MAX_SAMPLES samples.
    if (impl::needs_segments(s_pad))
        return fail(TDC_ERR_UNSUPPORTED, "tdc_focus_noalloc: nSamples " + std::to_string(S) + " above " +
                                             std::to_string(TDC_NOALLOC_MAX_SAMPLES) +
                                             " (whole rows must fit the shared-memory stages)");
    int cb = 1;
    const int stage_bytes = impl::stage_bytes_for(s_pad, cb);

    // ---- per-device set-up: the device address of the scratch array ----
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(TDC_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(TDC_ERR_UNSUPPORTED, "device index out of range");
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(st, &cap);
    if (e != cudaSuccess) return fail(TDC_ERR_CUDA, std::string("cudaStreamIsCapturing: ") + cudaGetErrorString(e));
    unsigned char *base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        if (cap == cudaStreamCaptureStatusNone) {
            void *ptr = nullptr;
            e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
            if (e != cudaSuccess || !ptr)
                return fail(TDC_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            g_scratch_addr[dev] = static_cast<unsigned char *>(ptr);
        } else if (!g_scratch_addr[dev]) {
            return fail(TDC_ERR_UNSUPPORTED, "tdc_focus_noalloc: the first call on a device must come before "
                                             "any stream capture (it looks up the scratch array's address)");
        }
        base = g_scratch_addr[dev];
    }

    int n_sm = 0;
    e = cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return fail(TDC_ERR_CUDA, std::string("device query: ") + cudaGetErrorString(e));
    const int bps = focus_fp32_blocks_per_sm(stage_bytes);
    if (bps <= 0) return fail(TDC_ERR_CUDA, "focus kernel does not fit on the device");
    const int slots = n_sm * bps;
    int n_groups = 1, cpg = C;
    size_t off_partial = min_off;
    if (!plan(P, C, slots, n_groups, cpg, off_partial)) {
        n_groups = 1;
        cpg = C;
        off_partial = min_off;
    }

    FocusJob job{};
    job.xw = reinterpret_cast<const float4 *>(a->samples);
    job.chirps = reinterpret_cast<const ChirpRec *>(a->chirps);
    job.grid_hi = reinterpret_cast<const float4 *>(a->grid_hi);
    job.grid_lo = reinterpret_cast<const float4 *>(a->grid_lo);
    job.skip = reinterpret_cast<const SkipPoint *>(a->skip_points);
    job.gs = nullptr;
    job.partial = reinterpret_cast<float4 *>(base + off_partial);
    job.P = P;
    job.C = C;
    job.S = S;
    job.s_pad = s_pad;
    job.n_groups = n_groups;
    job.chirps_per_group = cpg;
    job.chunk = kChunk;
    job.stage_chirps = cb;
    job.flags = (a->doppler_win_taper ? kFlagTaper : 0) | (a->skip_points ? kFlagSkipTest : 0);
    job.n_tiles = (int)n_tiles;
    job.per_sample = 0;
    split_dd(a->g0, job.g0_hi, job.g0_lo);
    split_dd(a->g1, job.g1, job.g1_lo);
    job.two_over_lambda = 2.0f / a->lambda;
    job.half_bw = a->doppler_bandwidth / 2.0f;
    job.inv_bw = 1.0f / a->doppler_bandwidth;
    job.az_a = kAzimuthA;

    const long long n_units = n_tiles * n_groups;
    const int setup_blocks = (int)std::min<long long>((n_units + 255) / 256, 1024);
    noalloc_setup_kernel<<<setup_blocks, 256, 0, st>>>(job, (int)n_tiles, n_groups, base);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(TDC_ERR_CUDA, std::string("setup kernel: ") + cudaGetErrorString(e));
    const int grid = (int)std::min<long long>(n_units, slots);
    e = launch_focus_fp32(reinterpret_cast<const FocusJob *>(base + kOffJob),
                          reinterpret_cast<const FocusUnit *>(base + kOffUnits), (int)n_units,
                          reinterpret_cast<int *>(base + kOffStatus), reinterpret_cast<int *>(base + kOffStatus) + 1,
                          stage_bytes, grid, std::isfinite(job.half_bw), false, false, st);
    if (e != cudaSuccess) return fail(TDC_ERR_CUDA, std::string("focus kernel: ") + cudaGetErrorString(e));
    e = launch_focus_reduce(job.partial, n_groups, P, reinterpret_cast<float2 *>(image_dev), st);
    if (e != cudaSuccess) return fail(TDC_ERR_CUDA, std::string("reduce kernel: ") + cudaGetErrorString(e));
    *status_word = reinterpret_cast<int *>(base + kOffStatus) + 1;
    return TDC_OK;
}

}  // namespace

extern "C" int tdc_focus_noalloc(const tdc_noalloc_focus_args *a, float *image_dev, void *stream)
{
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int *status_word = nullptr;
    if (int rc = enqueue(a, image_dev, st, &status_word)) return rc;
    // Blocking: collect the kernels' status word before returning.
    int status = 0;
    cudaError_t e = cudaMemcpyAsync(&status, status_word, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(TDC_ERR_CUDA, std::string("focus: ") + cudaGetErrorString(e));
    if (status & kStatusTimeout) return fail(TDC_ERR_TIMEOUT, "focus kernel wait timed out");
    if (status & kStatusBadJob) return fail(TDC_ERR_CUDA, "focus kernel rejected its job record");
    return TDC_OK;
}

extern "C" int tdc_focus_noalloc_async(const tdc_noalloc_focus_args *a, float *image_dev, int *status_dev,
                                       void *stream)
{
    if (!status_dev) return fail(TDC_ERR_INVALID_ARGUMENT, "null status word");
    if (reinterpret_cast<uintptr_t>(status_dev) & 3u)
        return fail(TDC_ERR_INVALID_ARGUMENT, "status word must be 4-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int *status_word = nullptr;
    if (int rc = enqueue(a, image_dev, st, &status_word)) return rc;
    const cudaError_t e = cudaMemcpyAsync(status_dev, status_word, sizeof(int), cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return fail(TDC_ERR_CUDA, std::string("status copy: ") + cudaGetErrorString(e));
    return TDC_OK;
}
