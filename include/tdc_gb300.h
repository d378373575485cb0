/*
 * tdc_gb300.h -- C ABI of the GB300 time-domain-correlation (TDC) focus engine.
 *
 * Two layers:
 *
 *  1. The processor API: one function per public method of the sarlab-tdc
 *     class `TdcProcessor` (tdc-lib/include/tdcprocessor.h:42-135), which is
 *     what the reference's pybind module `_sarlabtdc`
 *     (py-sarlabtdc/src/interface.cpp:15-22) binds. Same argument meaning,
 *     same ownership rules (inputs are borrowed host pointers read during
 *     tdc_processor_start; the image buffer belongs to the processor), and the
 *     same error classes, returned as status codes instead of C++ exceptions.
 *
 *  2. The device seam: functions on device pointers that replace the kernel
 *     wrappers of tdc-lib/include/tdckernels.h:20-97 (initRangeWindow,
 *     createWindow, referenceResponse, correlateAndSum, sumScratchSize). The
 *     per-pixel, per-chunk launch sequence of the reference becomes one fused
 *     launch over all pixels and chirps.
 *
 * All functions return TDC_OK (0) or a negative tdc_status; tdc_last_error()
 * gives a message for the calling thread's most recent failure. No C++
 * exception crosses this boundary. Streams are passed as void* (a cudaStream_t;
 * NULL is the legacy default stream).
 */
#ifndef TDC_GB300_H
#define TDC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TDC_GB300_ABI_VERSION 1

typedef enum tdc_status {
    TDC_OK = 0,
    TDC_ERR_INVALID_ARGUMENT = -1, /* std::invalid_argument in the reference (tdcprocessor.cpp:189-195) */
    TDC_ERR_CUDA = -2,             /* std::runtime_error from a CUDA failure (tdcprocessor.cpp:50-53,149-154) */
    TDC_ERR_STATE = -3,            /* call order violated (start before setRawData / setFocusGrid) */
    TDC_ERR_NO_MEMORY = -4,        /* device or pinned host allocation failed */
    TDC_ERR_TIMEOUT = -5,          /* a kernel's bounded wait expired; the kernel returned early */
    TDC_ERR_UNSUPPORTED = -6,      /* input outside what this library handles (message says which) */
    TDC_ERR_SHAPE = -7             /* array shape mismatch (runtime_error in the pybind wrapper) */
} tdc_status;

/* Message for the calling thread's most recent failure ("" if none). */
const char *tdc_last_error(void);
int tdc_abi_version(void);

/* ======================================================================== */
/* 1. Processor API (replaces class TdcProcessor, tdcprocessor.h:42-135).   */
/* ======================================================================== */

typedef struct tdc_processor tdc_processor;

/* TdcProcessor(int gpuNum) -- tdcprocessor.cpp:39-55 (cudaSetDevice). */
int tdc_processor_create(int gpu_num, tdc_processor **out);
/* ~TdcProcessor() */
int tdc_processor_destroy(tdc_processor *proc);

/*
 * TdcProcessor::setRawData -- tdcprocessor.h:104-107, tdcprocessor.cpp:169-209.
 * raw_iq:       nPri x nSamples complex float (interleaved I/Q), row-major
 * pri_times:    nPri floats (stored, unused by the focus, as in the reference)
 * sample_times: nSamples floats, seconds from the PRI start
 * position:     nPri x nSamples x 3 floats (x, y, z), metres
 * velocity:     nPri x nSamples x 3 floats
 * attitude:     nPri x nSamples x 4 floats, body->local quaternion (a, b, c, d)
 * body_boresight: 3 floats
 * The pointers are borrowed: they must stay valid until the next start()
 * returns. Errors: TDC_ERR_INVALID_ARGUMENT when n_pri <= 0 or n_samples <= 0.
 */
int tdc_processor_set_raw_data(tdc_processor *proc, const float *raw_iq, const float *pri_times,
                               const float *sample_times, const float *position, const float *velocity,
                               const float *attitude, int n_pri, int n_samples, float mod_rate,
                               float start_freq, const float *body_boresight);

/* TdcProcessor::setFocusGrid -- tdcprocessor.h:121, tdcprocessor.cpp:211-217.
 * focus_grid: n_rows x n_cols x 3 floats (x, y, z), borrowed until start() returns. */
int tdc_processor_set_focus_grid(tdc_processor *proc, const float *focus_grid, int n_rows, int n_cols);

/*
 * TdcProcessor::start -- tdcprocessor.h:67-68, tdcprocessor.cpp:59-167.
 * Blocking. Windows, forms the reference response and correlates every pixel
 * against every chirp on the GPU, then copies the image to the host buffer.
 */
int tdc_processor_start(tdc_processor *proc, float doppler_win_center, float doppler_bandwidth,
                        int dop_centroid_win, int apply_range_win, int doppler_win_taper);

/* TdcProcessor::imageBuffer -- tdcprocessor.cpp:240-243. n_rows x n_cols complex
 * float (interleaved), owned by the processor, valid until the next start() or
 * destroy. NULL before the first start(). */
const float *tdc_processor_image_buffer(const tdc_processor *proc);

/* Focus-grid shape last set (getFocusedImage uses it, tdcprocessor_wrapper.cpp:155-163). */
int tdc_processor_grid_shape(const tdc_processor *proc, int *n_rows, int *n_cols);

/* ---- extensions (no reference counterpart) ---- */

/* Per-chirp antenna positions in FP64 (n_pri x 3), overriding the FP32
 * per-sample positions of setRawData for the range/phase computation. Needed
 * where FP32 rounding of metre-scale coordinates is itself above the phase
 * tolerance. Borrowed like the other inputs. NULL clears the override. */
int tdc_processor_set_chirp_positions_f64(tdc_processor *proc, const double *position_f64, int n_pri);

/* Per-chirp trajectory (ingest extension): position n_pri x 3, velocity n_pri x 3
 * or NULL (zero), attitude n_pri x 4 or NULL (identity), replacing the
 * per-sample arrays of setRawData (40 bytes per sample) for antennas that do
 * not move within a chirp. Borrowed like the other inputs. */
int tdc_processor_set_trajectory_per_chirp(tdc_processor *proc, const float *position, const float *velocity,
                                           const float *attitude);

/* FP64 focus grid (n_rows x n_cols x 3), used instead of the FP32 grid. */
int tdc_processor_set_focus_grid_f64(tdc_processor *proc, const double *focus_grid, int n_rows, int n_cols);

typedef enum tdc_precision {
    TDC_PRECISION_FP32_BULK = 0, /* double-float range/phase per (pixel, chirp), FP32 phasors + MAC */
    TDC_PRECISION_FP64_PHASE = 1 /* plain comparator: FP64 phase per sample, FP32 MAC */
} tdc_precision;

int tdc_processor_set_precision(tdc_processor *proc, int precision);

typedef struct tdc_start_stats {
    double h2d_ms;        /* host->device copies of the inputs */
    double prep_ms;       /* windowing of raw chirps + trajectory records */
    double focus_ms;      /* the fused correlate-sum launch(es) */
    double d2h_ms;        /* image copy back */
    double total_ms;      /* wall time of start() */
    int64_t h2d_bytes;
    int64_t d2h_bytes;
    int64_t correlations; /* pixels x chirps x samples */
    int path;             /* tdc_path used */
    int kernel_launches;  /* launches of this library's kernels inside start() */
    int stage_samples;    /* samples of a chirp row per pipeline stage of the FP32 kernels
                             (the whole row, or one segment of a long row; 0 on FP64 paths) */
    int stage_chirps;     /* chirp rows per pipeline stage (1 when rows are staged in segments) */
    int general_variant;  /* FP32 general kernel variant bits (1 per-sample positions, 2 per-sample
                             windows, 4 wide phase correction); 0 on the other paths */
    int tile_cols;        /* 0: work tiles of 512 consecutive pixels; else tiles of 512 / tile_cols grid
                             rows x tile_cols columns (finite Doppler band, antenna moving along the
                             grid's columns) */
    int adjoint_stored;   /* the last adjoint read the kept per-chirp sums (1) or recomputed them (0) */
    int motion_segment;   /* smooth-motion path: samples per linearised segment; 0 on the other paths */
    int anchor_pixels;    /* FP32-bulk path with anchored ranges: consecutive pixels sharing one anchor
                             (32); 0 when every pixel's range is formed in double-float */
    int span_permille;    /* chirps the work units visit, per mille of tiles x chirps: below 1000 when a
                             finite Doppler band lets units skip chirps out of band for their whole tile */
} tdc_start_stats;

typedef enum tdc_path {
    TDC_PATH_FP32_BULK = 0,    /* per-chirp trajectory, uniform sample spacing */
    TDC_PATH_FP64_PHASE = 1,   /* comparator, per-chirp trajectory */
    TDC_PATH_GENERAL = 2,      /* per-sample trajectory / window or non-uniform sample times: FP32 phasors
                                  with a double-float range at sample 0 and per-sample corrections */
    TDC_PATH_GENERAL_FP64 = 3, /* the same inputs with FP64 phase per sample (FP64 precision, or intra-chirp
                                  motion too large for the FP32 correction) */
    TDC_PATH_FP32_MOTION = 4   /* per-sample positions moving smoothly within each chirp (a quadratic in the
                                  sample index to within their FP32 rounding), uniform sample spacing, one
                                  window per chirp: the per-sample phase correction linearised per segment */
} tdc_path;

int tdc_processor_last_stats(const tdc_processor *proc, tdc_start_stats *out);

/* ======================================================================== */
/* 2. Device seam (replaces tdckernels.h:20-97).                            */
/* ======================================================================== */

/* initRangeWindow (tdckernels.h:20): w[n] = a - (1-a) cos(2 pi n / N), a = 25/46
 * (Hamming, periodic), or all ones. Device pointer, n_samples floats. */
int tdc_range_window(float *w_dev, int n_samples, int apply_range_win, void *stream);

/* Skip test of tdcprocessor.cpp:347-383 on (1, default) or off. Takes effect
 * at the next start() / prepare(). */
int tdc_processor_set_skip_test(tdc_processor *proc, int enable);

/* Plan the chirp groups of the next focuses as for a grid of n_pix pixels (0, default: the
 * resident grid's own count). A pixel's summation order depends only on the chirp groups, so
 * a processor focusing a block of rows of a larger grid gives, with the larger grid's pixel
 * count set here, bit for bit the values a focus of the whole grid gives on the same kind of
 * GPU (pixel sharding across GPUs, sarlabtdc.sharding). Extension without a reference
 * counterpart (the reference binds one GPU, tdcprocessor.cpp:39-55). */
int tdc_processor_set_plan_pixels(tdc_processor *proc, int64_t n_pix);

/* Smooth-motion path (TDC_PATH_FP32_MOTION) on (1, default) or off (0: such inputs take
 * the FP32 general kernel). Extension without a reference counterpart; takes effect at the
 * next focus. */
int tdc_processor_set_motion_path(tdc_processor *proc, int enable);

/* Anchored ranges in the FP32-bulk kernel on (1, default) or off (0). With an unbounded Doppler
 * band, finite velocities, no kept per-chirp sums and rows of 3-16 chirps per pipeline stage
 * (about 128-700 samples), groups of 32 consecutive pixels share an anchor pixel whose
 * range and phase terms are formed in double-float once per chirp; each pixel adds its range
 * difference from the anchor in FP32 (exact in form: d.(d - 2e) / (R0 + R), no cancellation).
 * Taken only when no pixel lies farther than 5 cm from its anchor (grids whose rows are a
 * multiple of 32 pixels, or narrower than 5 cm, at up to 3 mm spacing), which keeps each
 * (pixel, chirp) phase within about 3e-5 rad of the per-pixel double-float range's at 77 GHz
 * (1e-5 rad on 1 mm grids). Off: every (pixel, chirp) range in double-float. Extension without
 * a reference counterpart; takes effect at the next focus. */
int tdc_processor_set_anchored_ranges(tdc_processor *proc, int enable);

/*
 * The parts of start() before the per-pixel work, leaving the acquisition
 * resident in device memory: copy of the raw chirps, range window applied
 * once per chirp (replacing createWindow's per-pixel range window),
 * trajectory records and skip-test points (replacing the per-chunk staging
 * of tdcprocessor.cpp:310-345). Same arguments as start(). Blocking.
 */
int tdc_processor_prepare(tdc_processor *proc, float doppler_win_center, float doppler_bandwidth,
                          int dop_centroid_win, int apply_range_win, int doppler_win_taper);

/* Copy the focus grid set by setFocusGrid / setFocusGrid_f64 to the device. Blocking. */
int tdc_processor_upload_grid(tdc_processor *proc);

/*
 * The fused focus (replaces the per-pixel createWindow + referenceResponse +
 * correlateAndSum launches of tdcprocessor.cpp:82-144, and sumScratchSize):
 * image_dev[p] (complex float, interleaved) for every pixel of the resident
 * grid, from the resident acquisition. Asynchronous on `stream` (NULL = the
 * legacy default stream); the processor owns the scratch memory. Call
 * tdc_processor_check before reading results to collect device-side errors.
 */
int tdc_processor_focus_device(tdc_processor *proc, float *image_dev, void *stream);

/* Synchronise `stream` (NULL = the legacy default stream) and report a kernel-side error
 * (TDC_ERR_TIMEOUT when a bounded wait expired). */
int tdc_processor_check(tdc_processor *proc, void *stream);

/* Number of pixels of the resident grid. */
int tdc_processor_num_pixels(const tdc_processor *proc, int64_t *n_pix);

/* tdc_path the next focus will take, or -1 when nothing is resident. */
int tdc_processor_path(const tdc_processor *proc);

/* 1 when the processor's kernels read the caller's host arrays in place (the
 * device reports coherent access to pageable host memory, as over Grace-Blackwell
 * NVLink-C2C; TDC_GB300_HOST_READS=0 in the environment turns it off at
 * creation), 0 when inputs are staged by copies. */
int tdc_processor_reads_host_memory(const tdc_processor *proc);

/* Caller-owned image output (replaces the copy of tdcprocessor_wrapper.cpp:155-163):
 * later start() calls write the image, n_pix complex floats (interleaved), into
 * image_host instead of the processor's own buffer, and imageBuffer() returns
 * image_host. The buffer is borrowed until it is replaced or the processor is
 * destroyed. Where the device accesses pageable host memory coherently
 * (tdc_processor_reads_host_memory() = 1) the final reduction kernel writes it
 * in place, with no device-to-host copy (fastest for an array the host has already
 * written: a never-touched allocation takes its first-touch page faults on the GPU);
 * otherwise the image is copied into it.
 * n_floats must be >= 2 x the pixels of the grid at start(); image_host = NULL
 * returns to the processor's own buffer. */
int tdc_processor_set_image_output(tdc_processor *proc, float *image_host, int64_t n_floats);

/* ---- autofocus (no reference counterpart) ---- */

/* Antenna positions of the resident acquisition := base + offsets_dev[c] (device,
 * n_pri x 3 doubles, metres), base = the positions given to setRawData /
 * setChirpPositionsF64; NULL restores the base. Needs a per-chirp trajectory.
 * Asynchronous on `stream`. */
int tdc_processor_set_chirp_offsets_device(tdc_processor *proc, const double *offsets_dev, void *stream);

/*
 * Adjoint of tdc_processor_focus_device with respect to the per-chirp position
 * offsets: grad_offsets_dev[c] (n_pri x 3 doubles) = sum over pixels of
 * Re(conj(G_p) dI_p/dR_pc) (P_c - T_p) / R_pc, with G = grad_image_dev
 * (n_pix complex floats, dL/dRe I + j dL/dIm I, as torch stores the gradient
 * of a complex tensor). The Doppler window and skip test are held fixed. The
 * reference response is recomputed, not stored. Blocking. FP32-bulk path only.
 * After a focus that kept its per-chirp sums (tdc_processor_set_keep_chirp_sums)
 * on the same acquisition, trajectory and grid, ordered before this call on the
 * device, the adjoint reads them and recomputes only the index-weighted sums
 * (half the arithmetic); otherwise it recomputes both.
 */
int tdc_processor_adjoint_device(tdc_processor *proc, const float *grad_image_dev, double *grad_offsets_dev,
                                 void *stream);

/* keep != 0: device-resident focuses on the FP32-bulk path (whole rows) also write their
 * per-(chirp, pixel) sums A = sum_s x_s z^s, n_pri x n_pix complex floats, for the next
 * adjoint, when they fit in half the free device memory; keep = 0 frees them. Changing
 * the trajectory (tdc_processor_set_chirp_offsets_device), the grid or the prepared
 * acquisition makes kept sums stale: the adjoint then recomputes. */
int tdc_processor_set_keep_chirp_sums(tdc_processor *proc, int keep);

/* ---- request loop (no reference counterpart) ---- */

/*
 * A persistent request loop on one GPU: jobs submitted from any host thread are
 * admitted while a processor slot is free and their device footprint fits in
 * the memory budget next to the resident jobs; each focus launch carries work
 * units of the admitted jobs (continuous batching), filled in priority order:
 * least estimated remaining service time, aged by the time waited so no job
 * starves. A job's image is bitwise the same whether it ran alone or in a mix.
 */
typedef struct tdc_server tdc_server;

typedef struct tdc_job_desc {
    const float *raw_iq;         /* n_pri x n_samples complex floats */
    const float *sample_times;   /* n_samples */
    const float *position;       /* n_pri x 3 per-chirp positions, or NULL when position_f64 is set */
    const double *position_f64;  /* n_pri x 3 FP64 per-chirp positions for range and phase, or NULL */
    const float *velocity;       /* n_pri x 3, or NULL (zero) */
    const float *attitude;       /* n_pri x 4, or NULL (identity) */
    int n_pri;
    int n_samples;
    float mod_rate;
    float start_freq;
    float body_boresight[3];
    const float *grid;           /* n_pix x 3, or NULL when grid_f64 is set */
    const double *grid_f64;      /* n_pix x 3, or NULL */
    int64_t n_pix;
    float doppler_win_center;    /* start() arguments */
    float doppler_bandwidth;
    int dop_centroid_win;
    int apply_range_win;
    int doppler_win_taper;
    float *image;                /* n_pix complex floats, written before the job reports done */
} tdc_job_desc;

typedef struct tdc_job_info {
    double submit_ms;        /* times since the server started */
    double admit_ms;
    double first_launch_ms;
    double done_ms;
    int64_t correlations;
    int status;              /* tdc_status of the job */
    int path;                /* tdc_path */
} tdc_job_info;

typedef struct tdc_server_stats {
    int64_t jobs_submitted;
    int64_t jobs_done;
    int64_t jobs_failed;
    int64_t launches;
    int64_t correlations;
    int64_t device_bytes_in_use;
    int queued;
    int active;
    int64_t unbatched;    /* jobs focused alone beside the launches (the FP64 general path) */
} tdc_server_stats;

/* memory_budget_bytes = 0: half of the free device memory; max_jobs = 0: 32 (at most 64). */
int tdc_server_create(int device, size_t memory_budget_bytes, int max_jobs, tdc_server **out);
/* Inputs are borrowed until the job is done. */
int tdc_server_submit(tdc_server *srv, const tdc_job_desc *job, uint64_t *job_id);
/* Wait up to timeout_ms (< 0: forever); TDC_ERR_TIMEOUT if not finished. Returns the job's status. */
int tdc_server_wait(tdc_server *srv, uint64_t job_id, int timeout_ms, tdc_job_info *info);
int tdc_server_stats_get(tdc_server *srv, tdc_server_stats *out);
/* Finishes the submitted jobs, then releases the server. */
int tdc_server_destroy(tdc_server *srv);

/* ---- measurement helper (no reference counterpart) ---- */

/* FMA throughput probe: blocks x 256 threads x iters x 128 FMAs, FP32 (fp64 = 0)
 * or FP64. *flops receives the FLOP count (2 per FMA); the caller times the
 * launch with events on `stream`. scratch_dev: >= blocks x 8 bytes (never written
 * in practice). */
int tdc_probe_fma(int fp64, int blocks, int iters, void *scratch_dev, double *flops, void *stream);

/* Self-test of the kernels' failure detection: one CTA waits, with the same bounded
 * mbarrier wait the focus kernels use, on a barrier phase that nothing completes. After
 * limit_us (at most 2 s) the wait gives up, the CTA sets the timeout bit of a status word
 * and returns; *timed_out receives that bit (1 expected), *elapsed_ms (optional) the
 * kernel's duration. The device stays usable afterwards. */
int tdc_selftest_wait_timeout(int device, int limit_us, int *timed_out, double *elapsed_ms);

/* ---- focus without allocation (no counterpart in the reference) ---- */

/*
 * For callers that cannot allocate device memory while they focus: processing
 * chains that provision all device memory once at start-up (real-time or
 * certified radar pipelines with a fixed budget), plug-ins inside a host
 * framework that owns the device allocator, code that must not call cudaMalloc
 * during stream capture. tdc_focus_noalloc runs the FP32-bulk focus of
 * tdc_processor_focus_device, with every (pixel, chirp) range in double-float and
 * every work unit over its whole chirp group (the anchored ranges and unit spans
 * the processor plans from its host copies of the grid and trajectory are not
 * taken), on inputs and an output the caller owns; its
 * scratch memory is a fixed array inside this library (TDC_NOALLOC_SCRATCH_BYTES
 * on every GPU that loads the library, held until the process exits), so it
 * calls no cudaMalloc / cudaFree. That limits the grid to about 2M pixels, and
 * rows to TDC_NOALLOC_MAX_SAMPLES samples (whole rows are staged; the processor
 * stages longer rows in segments). Larger grids or rows return
 * TDC_ERR_UNSUPPORTED before anything runs.
 *
 * All calls on a device share the one array: calls that overlap on the GPU
 * (other streams, other host threads) race on it and must be serialised by the
 * caller. Each call outside stream capture looks up the array's device address
 * (cudaGetSymbolAddress) in the current context, so a device reset between calls
 * is harmless; a call under capture uses the address the last uncaptured call on
 * that device found, so make one call on each device before any stream capture
 * (and again after a device reset). tdc_focus_noalloc is blocking: it returns after the image
 * is written and the kernels' status word has been read (TDC_ERR_TIMEOUT when a
 * bounded wait in the focus kernel expired). tdc_focus_noalloc_async enqueues the
 * same kernels and a copy of the status word into status_dev (a device int,
 * 0 = success, 1 = a bounded wait expired) and returns without synchronising,
 * so it can be captured into a CUDA graph: the job record is a kernel argument
 * and the scratch is reset by the captured set-up kernel, so a replay focuses
 * whatever the input buffers hold at that time.
 *
 * Inputs (device pointers, 16-byte aligned):
 *   samples      n_pri rows of s_pad complex floats (interleaved): the range-
 *                windowed samples, zero from n_samples to s_pad, where s_pad is
 *                n_samples rounded up to a multiple of 16
 *   chirps       n_pri records of 12 floats: position (x, y, z) high floats,
 *                Doppler window centre [Hz], position low floats (x, y, z)
 *                (position = high + low, double-float), 0, velocity (x, y, z), 0
 *   skip_points  ceil(n_pri / 128) x 9 points x 8 floats of the reference's chunk
 *                skip test (position xyz, window centre, velocity xyz, 0), or
 *                NULL to process every chunk
 *   grid_hi      n_pix x 4 floats (x, y, z, 0); grid_lo the low floats or NULL
 *   g0, g1       2 f(s) / c = g0 + s g1 [cycles per metre], f(s) the frequency of sample s
 * Output: image_dev, n_pix complex floats (interleaved).
 */
#define TDC_NOALLOC_SCRATCH_BYTES (32u << 20)
/* Largest n_samples tdc_focus_noalloc takes: three pipeline stages of one whole row
 * (n_samples rounded up to 16, 8 bytes a sample, plus a 48-byte record) within the
 * shared memory a block may use. */
#define TDC_NOALLOC_MAX_SAMPLES 9104

typedef struct tdc_noalloc_focus_args {
    const float *samples;
    const float *chirps;
    const float *skip_points;
    const float *grid_hi;
    const float *grid_lo;
    int64_t n_pix;
    int n_pri;
    int n_samples;
    double g0;
    double g1;
    float lambda;              /* centre wavelength, used by the Doppler window */
    float doppler_bandwidth;   /* Hz; +inf for no Doppler windowing */
    int doppler_win_taper;
} tdc_noalloc_focus_args;

int tdc_focus_noalloc(const tdc_noalloc_focus_args *args, float *image_dev, void *stream);
int tdc_focus_noalloc_async(const tdc_noalloc_focus_args *args, float *image_dev, int *status_dev, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* TDC_GB300_H */
