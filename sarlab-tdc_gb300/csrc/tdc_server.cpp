// tdc_server.cpp -- persistent request loop of the GB300 TDC engine: continuous
// batching of focus jobs with memory-based admission. No reference counterpart
// (the reference processes one acquisition per blocking start() call).
//
// Jobs are submitted from any host thread and run on one GPU. Two host threads
// serve them:
//  * priority: least estimated remaining service time first, aged by the time
//    a job has waited (so short jobs finish fast and long ones are not starved);
//  * admission (admission thread): the highest-priority queued job enters when a
//    processor slot is free and its device footprint fits in the memory budget
//    next to the resident jobs; its acquisition and grid are copied and prepared
//    on the slot's own stream, created at the highest stream priority, while
//    launches run. Slot memory comes from the stream-ordered pool, so growing or
//    releasing it never synchronises the device;
//  * batching (launch thread): each launch of the focus kernel carries work units
//    (pixel tile x chirp group, bounded in size) of the active jobs in priority
//    order, later jobs backfilling what the first leave free, so a job that
//    arrives while others are on the GPU joins the next launch. Launches alternate
//    between two lowest-priority streams, one in flight on each, so a launch's
//    tail overlaps the next launch and the GPU never waits for the host;
//  * completion: after the launch holding a job's last units, its partials are
//    reduced and the image copied back on the same stream; the host collects it
//    when the job's event completes.
// Each job keeps its own decomposition (depending only on its shape) and its
// own partial buffer reduced in a fixed order, so a job's image is bitwise the
// same alone and in any mix.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <new>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "tdc_gb300.h"
#include "tdc_internal.h"
#include "tdc_processor_impl.h"

using namespace tdc;
using namespace tdc::impl;

namespace {

double now_ms()
{
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

enum JobState { kQueued = 0, kActive = 1, kCompleting = 2, kDone = 3, kFailed = 4 };

struct Job {
    uint64_t id = 0;
    tdc_job_desc d{};
    std::vector<float> pos32;  // FP32 copy of FP64-only positions (windows / skip test)
    double t_submit = 0, t_admit = 0, t_first = -1, t_done = 0;
    tdc_processor *slot = nullptr;
    FocusPlan plan;
    size_t next_unit = 0;
    size_t n_units = 0;
    double unit_work = 0;  // correlations per unit, in FP32-bulk kernel time (kind_cost)
    size_t footprint = 0;
    int state = kQueued;
    int rc = TDC_OK;
    std::string err;
    cudaEvent_t done_ev = nullptr;
};

struct Batch {
    DevBuf dev;        // [counter, status | jobs | units]
    PinnedBuf host;    // staging of jobs + units, status read-back
    cudaEvent_t ev = nullptr;
    bool in_flight = false;
    std::vector<Job *> finishing;  // jobs whose last units are in this batch
    std::vector<Job *> members;
};

constexpr size_t kBatchOffJobs = 256;
constexpr int kMaxBatchJobs = 64;

// Correlations per work unit in the request loop, and per launch: ~5e11 correlations
// (~65 ms) with at least two units per resident CTA. (On the config-4 mix, launches of 5e11
// gave p50 8.1-8.2 s against 8.5-8.8 s with 1e12, 8.7 s with 2.5e11 and 10.3 s with 2e12, at
// the same p99 and throughput.)
constexpr double kServerUnitWork = 1.0e9;
#ifndef TDC_SERVER_BATCH_WORK
#define TDC_SERVER_BATCH_WORK 5.0e11
#endif
constexpr double kServerBatchWork = TDC_SERVER_BATCH_WORK;
// Priority: shortest estimated remaining service first, aged so that waiting jobs
// are not starved (a job gains kAging seconds of priority per second it waits). On the
// config-4 mix (Poisson 20/s, 3.3x the GPU's rate): aging 0.05 gave p50 0.53 s and p99 27.9 s,
// 0.02 0.40 / 28.1 s, 0.1 1.7-2.2 / 27.8-28.1 s, 0.25 6.4 / 29.1-29.3 s, 0.5 8.5 / 29.1 s, 1.0
// 11.7 / 29.1 s, at 7,790-7,870 Gcorr/s throughout.
constexpr double kRateEstimate = 7.0e12;  // correlations per second
#ifndef TDC_SERVER_AGING
#define TDC_SERVER_AGING 0.05
#endif
constexpr double kAging = TDC_SERVER_AGING;

// The kernel a job's units run in: jobs share a launch only with jobs of the same kind (the
// same kernel instance, so a job's arithmetic does not depend on the jobs beside it). -1: not
// batched (the FP64 general path: focused alone on the side stream).
int job_kind(const FocusPlan &pl)
{
    if (pl.path == TDC_PATH_FP32_BULK) return pl.seg ? 1 : (pl.anchored ? 2 : 0);
    if (pl.path == TDC_PATH_GENERAL) return 16 + pl.variant;
    return -1;
}

// Time of a correlation on a job's kernel relative to the FP32-bulk kernel's (GB300): a
// launch's work budget and the scheduling priority count in FP32-bulk correlations.
double kind_cost(int kind)
{
    return kind >= 16 ? ((kind - 16) & 2 ? 9.0 : 5.5) : 1.0;
}

size_t device_footprint(const tdc_job_desc &d, int n_sm)
{
    const size_t C = (size_t)d.n_pri, S = (size_t)d.n_samples, P = (size_t)d.n_pix;
    const size_t s_pad = round_up(S, kSampleAlign);
    int groups = 1, cpg = d.n_pri;
    plan_groups(((long long)P + kFocusTile - 1) / kFocusTile, d.n_pri, std::max(1, n_sm * 3), groups, cpg,
                kFocusMinUnitsPerSlot);
    const int cpg_cap = std::max(1, (int)(kServerUnitWork / ((double)kFocusTile * S)));
    if (cpg > cpg_cap) groups = (d.n_pri + cpg_cap - 1) / cpg_cap;
    const size_t n_tiles = (P + kFocusTile - 1) / kFocusTile;
    size_t b = 0;
    b += C * s_pad * 8;                 // samples
    b += C * sizeof(ChirpRec);          // records
    b += ((C + kChunk - 1) / kChunk) * 9 * sizeof(SkipPoint);
    b += S * 8 + S * 4 + C * 24;        // frequency table, range window, base positions
    b += P * 3 * (d.grid_f64 ? 8 : 4);  // grid staging
    b += P * 16 * (d.grid_f64 ? 2 : 1); // grid hi / lo
    b += 1024 + n_tiles * groups * sizeof(FocusUnit) + (size_t)groups * P * 16;  // scratch
    b += P * 8;                         // image
    return b;
}

}  // namespace

struct tdc_server {
    int device = 0;
    int n_sm = 0;
    size_t budget = 0;
    int max_jobs = 0;
    double batch_work = 0;  // correlations per launch (sets the admission / fairness granularity)
    double t0 = 0;

    std::vector<tdc_processor *> slots;
    std::vector<tdc_processor *> free_slots;
    std::unordered_map<const tdc_processor *, size_t> slot_mem;  // device bytes each slot holds
    size_t mem_in_use = 0;
    std::deque<Job *> queue;
    int admitting = 0;  // jobs taken from the queue whose preparation is under way
    std::vector<Job *> active;
    std::vector<Job *> completing;
    std::unordered_map<uint64_t, std::unique_ptr<Job>> jobs;
    uint64_t next_id = 1;

    std::mutex mu;
    std::condition_variable cv_work, cv_admit, cv_done;
    bool stop = false;
    std::thread th_launch, th_admit;

    // Launches alternate between two streams, so the next launch's CTAs take the
    // SMs that the previous launch's last units leave idle.
    cudaStream_t compute[2] = {nullptr, nullptr};
    cudaStream_t side = nullptr;  // unbatched jobs (FP64 general path), launch priority
    Batch batches[2];
    int next_batch = 0;
    tdc_server_stats stats{};

    // Scheduling priority (lower first): estimated remaining service time minus
    // kAging x time waited since submission, in seconds.
    double score(const Job *j, double t_ms) const
    {
        const double rem = j->state == kQueued ? (double)j->d.n_pix * j->d.n_pri * j->d.n_samples
                                               : (double)(j->n_units - j->next_unit) * j->unit_work;
        return rem / kRateEstimate - kAging * (t_ms - j->t_submit) / 1e3;
    }

    void launch_loop();
    void admit_loop();
    int admit_one(Job *j);
    void launch_batch();
    void collect(std::vector<Job *> &finished);
    void finish_jobs(std::unique_lock<std::mutex> &lk, std::vector<Job *> &finished);
    void fail_job(Job *j, int rc, const std::string &msg);
    void note_slot_memory(tdc_processor *p);
};

void tdc_server::note_slot_memory(tdc_processor *p)
{
    const size_t now = processor_device_bytes(p);
    size_t &was = slot_mem[p];
    mem_in_use = mem_in_use - was + now;
    was = now;
}

void tdc_server::fail_job(Job *j, int rc, const std::string &msg)
{
    j->rc = rc;
    j->err = msg;
    j->state = kFailed;
    j->t_done = now_ms() - t0;
    if (j->slot) {
        free_slots.push_back(j->slot);
        j->slot = nullptr;
    }
    stats.jobs_failed++;
    cv_done.notify_all();
    cv_admit.notify_all();
}

// Copies and prepares a job's acquisition and grid on its slot (the admission
// thread, without the lock: the slot belongs to the job until it completes).
int tdc_server::admit_one(Job *j)
{
    NvtxRange nvtx("tdc server admit");
    tdc_processor *p = j->slot;
    const tdc_job_desc &d = j->d;
    int rc = tdc_processor_set_raw_data(p, d.raw_iq, nullptr, d.sample_times, j->pos32.empty() ? d.position : j->pos32.data(),
                                        d.velocity, d.attitude, d.n_pri, d.n_samples, d.mod_rate, d.start_freq,
                                        d.body_boresight);
    if (!rc) rc = tdc_processor_set_trajectory_per_chirp(p, j->pos32.empty() ? d.position : j->pos32.data(),
                                                         d.velocity, d.attitude);
    if (!rc && d.position_f64) rc = tdc_processor_set_chirp_positions_f64(p, d.position_f64, d.n_pri);
    if (!rc) {
        const int rows = 1;
        const int cols = (int)d.n_pix;
        rc = d.grid_f64 ? tdc_processor_set_focus_grid_f64(p, d.grid_f64, rows, cols)
                        : tdc_processor_set_focus_grid(p, d.grid, rows, cols);
    }
    if (!rc) rc = tdc_processor_prepare(p, d.doppler_win_center, d.doppler_bandwidth, d.dop_centroid_win,
                                        d.apply_range_win, d.doppler_win_taper);
    if (!rc) rc = tdc_processor_upload_grid(p);
    if (!rc) rc = focus_plan(p, j->plan, kServerUnitWork);
    if (rc) return rc;
    // Images go through device + pinned buffers: a kernel writing the caller's freshly
    // allocated (untouched) pages directly would take the page faults on the GPU while
    // other jobs' launches run.
    if (p->image_dev.ensure((size_t)p->P * 8) != cudaSuccess || p->image_host.ensure((size_t)p->P * 8) != cudaSuccess)
        return set_last_error(TDC_ERR_NO_MEMORY, "image buffers");
    // The slot's buffers come from the stream-ordered pool on the slot's stream:
    // settle them before the launch streams use them.
    if (cudaStreamSynchronize(p->stream) != cudaSuccess) return set_last_error(TDC_ERR_CUDA, "slot stream sync");
    j->n_units = p->units_host.size();
    j->next_unit = 0;
    j->unit_work = (double)kFocusTile * j->plan.job.chirps_per_group * d.n_samples * kind_cost(job_kind(j->plan));
    return TDC_OK;
}

// Finished launches and jobs (lock held). Jobs whose image is done move to
// `finished`; finish_jobs completes them.
void tdc_server::collect(std::vector<Job *> &finished)
{
    for (Batch &b : batches) {
        if (!b.in_flight || cudaEventQuery(b.ev) != cudaSuccess) continue;
        b.in_flight = false;
        const int status = reinterpret_cast<int *>(b.host.p)[1];
        if (status & (kStatusTimeout | kStatusBadJob)) {
            for (Job *j : b.members)
                if (j->state == kActive || j->state == kCompleting) {
                    j->rc = (status & kStatusTimeout) ? TDC_ERR_TIMEOUT : TDC_ERR_CUDA;
                    j->err = (status & kStatusTimeout) ? "focus kernel wait timed out"
                                                       : "focus kernel rejected its job record";
                }
        }
    }
    for (size_t i = 0; i < completing.size();) {
        Job *j = completing[i];
        if (cudaEventQuery(j->done_ev) != cudaSuccess) {
            ++i;
            continue;
        }
        finished.push_back(j);
        completing.erase(completing.begin() + i);
    }
}

// Copies staged images out (without the lock: the jobs' slots stay theirs until
// they are handed back here) and completes the jobs.
void tdc_server::finish_jobs(std::unique_lock<std::mutex> &lk, std::vector<Job *> &finished)
{
    if (finished.empty()) return;
    lk.unlock();
    for (Job *j : finished)
        if (j->rc == TDC_OK) std::memcpy(j->d.image, j->slot->image_host.p, (size_t)j->d.n_pix * 8);
    lk.lock();
    for (Job *j : finished) {
        if (j->rc == TDC_OK) {
            j->state = kDone;
            stats.jobs_done++;
            stats.correlations += (int64_t)j->d.n_pix * j->d.n_pri * j->d.n_samples;
        } else {
            j->state = kFailed;
            stats.jobs_failed++;
        }
        j->t_done = now_ms() - t0;
        free_slots.push_back(j->slot);
        j->slot = nullptr;
    }
    finished.clear();
    cv_done.notify_all();
    cv_admit.notify_all();
}

// Builds and enqueues the next launch into the free batch (lock held).
void tdc_server::launch_batch()
{
    NvtxRange nvtx("tdc server launch");
    const int bi = next_batch;
    Batch &b = batches[bi];
    cudaStream_t st = compute[bi];
    // Jobs of this launch in priority order (least remaining service time, aged by the
    // wait): each takes what is left of the launch's work budget and the next ones
    // backfill the rest, so a job that arrives while others run joins the next launch
    // and short jobs finish first. A launch holds at least two units per resident CTA
    // so the GPU stays full.
    std::vector<Job *> members;
    for (Job *j : active)
        if (j->next_unit < j->n_units) members.push_back(j);
    if (members.empty()) return;
    {
        const double t = now_ms() - t0;
        std::stable_sort(members.begin(), members.end(),
                         [&](Job *a, Job *b) { return score(a, t) < score(b, t); });
        // A launch takes jobs of one kind only (the first job's: job_kind), so that a job's
        // arithmetic does not depend on the jobs it shares a launch with.
        const int kind = job_kind(members[0]->plan);
        members.erase(std::remove_if(members.begin(), members.end(),
                                     [&](Job *j) { return job_kind(j->plan) != kind; }),
                      members.end());
        if ((int)members.size() > kMaxBatchJobs) members.resize(kMaxBatchJobs);
    }
    const size_t min_units = (size_t)std::max(1, 2 * n_sm * 3);
    std::vector<size_t> take(members.size(), 0);
    double left = batch_work;
    size_t taken = 0;
    for (size_t i = 0; i < members.size() && (left > 0 || taken < min_units); ++i) {
        Job *j = members[i];
        const size_t rem = j->n_units - j->next_unit;
        size_t n = (size_t)std::ceil(std::max(0.0, left) / j->unit_work);
        n = std::max(n, min_units > taken ? min_units - taken : (size_t)0);
        n = std::min(std::max<size_t>(n, 1), rem);
        take[i] = n;
        taken += n;
        left -= n * j->unit_work;
    }
    while (!members.empty() && take.back() == 0) {
        members.pop_back();
        take.pop_back();
    }
    size_t n_units = 0;
    for (size_t t : take) n_units += t;
    const size_t off_units = round_up(kBatchOffJobs + members.size() * sizeof(FocusJob), 256);
    const size_t bytes = off_units + n_units * sizeof(FocusUnit);
    if (b.dev.ensure(bytes) != cudaSuccess || b.host.ensure(bytes) != cudaSuccess) {
        for (Job *j : members) {
            j->rc = TDC_ERR_NO_MEMORY;
            j->err = "batch buffers";
        }
        return;
    }
    unsigned char *h = static_cast<unsigned char *>(b.host.p);
    std::memset(h, 0, kBatchOffJobs);
    FocusJob *hj = reinterpret_cast<FocusJob *>(h + kBatchOffJobs);
    FocusUnit *hu = reinterpret_cast<FocusUnit *>(h + off_units);
    int stage_bytes = 0;
    bool skip_zero = false;  // any job with a finite Doppler band
    bool anchored = true;    // every job planned for anchored ranges
    b.finishing.clear();
    b.members = members;
    const double t = now_ms() - t0;
    // Units go into the launch longest first, so the launch ends on short units
    // (its tail then overlaps the next launch on the other stream).
    std::vector<size_t> order(members.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](size_t a, size_t c) { return members[a]->unit_work > members[c]->unit_work; });
    size_t u = 0;
    for (size_t i : order) {
        Job *j = members[i];
        for (size_t k = 0; k < take[i]; ++k) {
            FocusUnit fu = j->slot->units_host[j->next_unit + k];
            fu.job = (int)i;
            hu[u++] = fu;
        }
    }
    for (size_t i = 0; i < members.size(); ++i) {
        Job *j = members[i];
        hj[i] = j->plan.job;
        stage_bytes = std::max(stage_bytes, j->plan.stage_bytes);
        skip_zero = skip_zero || std::isfinite(j->plan.job.half_bw);
        anchored = anchored && j->plan.anchored;
        j->next_unit += take[i];
        if (j->t_first < 0) j->t_first = t;
        if (j->next_unit == j->n_units) b.finishing.push_back(j);
    }
    int err = 0;
    err |= cudaMemcpyAsync(b.dev.p, b.host.p, bytes, cudaMemcpyHostToDevice, st) != cudaSuccess;
    anchored = anchored && !skip_zero;
    const int kind = job_kind(members[0]->plan);
    const bool seg = kind == 1;
    const bool general = kind >= 16;
    const int variant = general ? members[0]->plan.variant : 0;
    const int bps = general    ? focus_general_blocks_per_sm(variant, stage_bytes)
                    : seg      ? focus_fp32_seg_blocks_per_sm(stage_bytes)
                    : anchored ? focus_fp32_anchor_blocks_per_sm(stage_bytes)
                               : focus_fp32_blocks_per_sm(stage_bytes);
    const int grid = (int)std::min<size_t>(n_units, (size_t)std::max(1, n_sm * bps));
    unsigned char *d = static_cast<unsigned char *>(b.dev.p);
    const FocusJob *jobs_d = reinterpret_cast<const FocusJob *>(d + kBatchOffJobs);
    const FocusUnit *units_d = reinterpret_cast<const FocusUnit *>(d + off_units);
    int *counter_d = reinterpret_cast<int *>(d);
    if (general)
        err |= launch_focus_general(variant, jobs_d, units_d, (int)n_units, counter_d, counter_d + 1, stage_bytes, grid,
                                    st) != cudaSuccess;
    else if (seg)
        err |= launch_focus_fp32_seg(jobs_d, units_d, (int)n_units, counter_d, counter_d + 1, stage_bytes, grid,
                                     skip_zero, st) != cudaSuccess;
    else
        err |= launch_focus_fp32(jobs_d, units_d, (int)n_units, counter_d, counter_d + 1, stage_bytes, grid, skip_zero,
                                 false, anchored, st) != cudaSuccess;
    err |= cudaMemcpyAsync(b.host.p, b.dev.p, 8, cudaMemcpyDeviceToHost, st) != cudaSuccess;
    stats.launches++;
    if (!b.finishing.empty() && batches[bi ^ 1].in_flight) {
        // Earlier units of the finishing jobs may be in the launch on the other stream.
        err |= cudaStreamWaitEvent(st, batches[bi ^ 1].ev, 0) != cudaSuccess;
    }
    for (Job *j : b.finishing) {
        tdc_processor *p = j->slot;
        const long long P = p->P;
        err |= launch_focus_reduce(j->plan.job.partial, j->plan.job.n_groups, P, p->image_dev.as<float2>(), st) !=
               cudaSuccess;
        err |= cudaMemcpyAsync(p->image_host.p, p->image_dev.p, (size_t)P * 8, cudaMemcpyDeviceToHost, st) !=
               cudaSuccess;
        err |= cudaEventRecord(j->done_ev, st) != cudaSuccess;
        j->state = kCompleting;
        completing.push_back(j);
        active.erase(std::find(active.begin(), active.end(), j));
    }
    err |= cudaEventRecord(b.ev, st) != cudaSuccess;
    b.in_flight = true;
    next_batch ^= 1;
    if (err) {
        for (Job *j : members) {
            j->rc = TDC_ERR_CUDA;
            j->err = "batch launch failed";
        }
    }
}

// Admission thread: takes the highest-priority queued job into a free slot when
// its footprint fits the budget, and prepares it while launches run.
void tdc_server::admit_loop()
{
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
        if (stop && queue.empty()) break;
        if (queue.empty() || free_slots.empty()) {
            cv_admit.wait_for(lk, std::chrono::milliseconds(5));
            continue;
        }
        // Queued job with the least estimated remaining service time, aged by its wait.
        const double t = now_ms() - t0;
        Job *j = nullptr;
        for (Job *q : queue)
            if (!j || score(q, t) < score(j, t)) j = q;
        if (j->footprint > budget) {
            queue.erase(std::find(queue.begin(), queue.end(), j));
            fail_job(j, TDC_ERR_NO_MEMORY, "job needs more device memory than the server budget");
            continue;
        }
        // the free slot that needs the least growth
        tdc_processor *best = nullptr;
        size_t best_growth = (size_t)-1;
        for (tdc_processor *p : free_slots) {
            const size_t have = slot_mem[p];
            const size_t growth = j->footprint > have ? j->footprint - have : 0;
            if (growth < best_growth) {
                best_growth = growth;
                best = p;
            }
        }
        // Idle slots may hold memory from earlier jobs: release the largest first
        // (stream-ordered frees: no device synchronisation).
        while (mem_in_use + best_growth > budget) {
            tdc_processor *victim = nullptr;
            for (tdc_processor *p : free_slots)
                if (p != best && slot_mem[p] > 0 && (!victim || slot_mem[p] > slot_mem[victim])) victim = p;
            if (!victim) break;
            processor_release_memory(victim);
            note_slot_memory(victim);
        }
        const bool alone = active.empty() && completing.empty() && admitting == 0;
        if (mem_in_use + best_growth > budget && !alone) {
            // wait for a resident job to finish
            cv_admit.wait_for(lk, std::chrono::milliseconds(5));
            continue;
        }
        queue.erase(std::find(queue.begin(), queue.end(), j));
        free_slots.erase(std::find(free_slots.begin(), free_slots.end(), best));
        j->slot = best;
        j->t_admit = now_ms() - t0;
        ++admitting;
        // Reserve the growth now; the slot's real size is noted after preparation.
        mem_in_use += best_growth;
        slot_mem[best] += best_growth;
        lk.unlock();
        const int rc = admit_one(j);
        int rc2 = TDC_OK;
        std::string err2;
        const bool batched = job_kind(j->plan) >= 0;
        if (!rc && !batched) {
            // FP64 general path: not batched, focused on its own on the side stream (at the
            // launch streams' priority, so it shares the SMs with the batches).
            tdc_processor *p = j->slot;
            {
                std::lock_guard<std::mutex> g(mu);
                stats.unbatched++;
            }
            rc2 = tdc_processor_focus_device(p, p->image_dev.as<float>(), side);
            if (rc2) {
                err2 = tdc_last_error();
            } else if (cudaMemcpyAsync(p->image_host.p, p->image_dev.p, (size_t)p->P * 8, cudaMemcpyDeviceToHost,
                                       side) != cudaSuccess ||
                       cudaEventRecord(j->done_ev, side) != cudaSuccess) {
                rc2 = TDC_ERR_CUDA;
                err2 = "image copy";
            }
        }
        const std::string err = rc ? std::string(tdc_last_error()) : std::string();
        lk.lock();
        --admitting;
        note_slot_memory(j->slot);
        if (rc) {
            fail_job(j, rc, err);
        } else if (rc2) {
            fail_job(j, rc2, err2);
        } else if (!batched) {
            j->t_first = now_ms() - t0;
            j->state = kCompleting;
            completing.push_back(j);
        } else {
            j->state = kActive;
            active.push_back(j);
        }
        cv_work.notify_all();
    }
}

// Launch thread: keeps up to two launches in flight (one per stream) and
// collects finished jobs.
void tdc_server::launch_loop()
{
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    std::vector<Job *> finished;
    for (;;) {
        collect(finished);
        finish_jobs(lk, finished);
        const bool any_in_flight = batches[0].in_flight || batches[1].in_flight;
        if (stop && queue.empty() && admitting == 0 && active.empty() && completing.empty() && !any_in_flight)
            break;
        bool pending = false;
        for (Job *j : active)
            if (j->next_unit < j->n_units) pending = true;
        if (pending && !batches[next_batch].in_flight) {
            launch_batch();
            continue;
        }
        // Poll the launches and completions (the lock is free meanwhile).
        cv_work.wait_for(lk, std::chrono::microseconds(any_in_flight || !completing.empty() ? 200 : 2000));
    }
}

extern "C" {

int tdc_server_create(int device, size_t memory_budget_bytes, int max_jobs, tdc_server **out)
{
    if (!out) return set_last_error(TDC_ERR_INVALID_ARGUMENT, "null output pointer");
    *out = nullptr;
    if (max_jobs <= 0) max_jobs = 32;
    if (cudaSetDevice(device) != cudaSuccess) return set_last_error(TDC_ERR_CUDA, "cudaSetDevice failed");
    tdc_server *s = new (std::nothrow) tdc_server();
    if (!s) return set_last_error(TDC_ERR_NO_MEMORY, "out of host memory");
    s->device = device;
    s->max_jobs = std::min(max_jobs, kMaxBatchJobs);
    cudaDeviceGetAttribute(&s->n_sm, cudaDevAttrMultiProcessorCount, device);
    if (memory_budget_bytes == 0) {
        size_t free_b = 0, total_b = 0;
        cudaMemGetInfo(&free_b, &total_b);
        memory_budget_bytes = free_b / 2;
    }
    s->budget = memory_budget_bytes;
    s->batch_work = kServerBatchWork;
    s->t0 = now_ms();
    // Launch streams at the lowest priority, slot (preparation) streams at the
    // highest: when a launch's CTAs retire, a waiting preparation kernel gets the
    // SM before the next launch's CTAs do.
    int least = 0, greatest = 0;
    int rc = TDC_OK;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess)
        rc = set_last_error(TDC_ERR_CUDA, "stream priority range");
    for (int i = 0; i < 2 && !rc; ++i)
        if (cudaStreamCreateWithPriority(&s->compute[i], cudaStreamNonBlocking, least) != cudaSuccess ||
            cudaEventCreateWithFlags(&s->batches[i].ev, cudaEventDisableTiming) != cudaSuccess)
            rc = set_last_error(TDC_ERR_CUDA, "stream / event creation failed");
    if (!rc && cudaStreamCreateWithPriority(&s->side, cudaStreamNonBlocking, least) != cudaSuccess)
        rc = set_last_error(TDC_ERR_CUDA, "stream creation failed");
    for (int i = 0; i < s->max_jobs && !rc; ++i) {
        tdc_processor *p = nullptr;
        rc = tdc_processor_create(device, &p);
        if (!rc) {
            s->slots.push_back(p);
            s->free_slots.push_back(p);
            s->slot_mem[p] = 0;
            rc = processor_use_slot_stream(p, greatest);
        }
    }
    if (rc) {
        tdc_server_destroy(s);
        return rc;
    }
    s->th_launch = std::thread([s] { s->launch_loop(); });
    s->th_admit = std::thread([s] { s->admit_loop(); });
    *out = s;
    return TDC_OK;
}

int tdc_server_submit(tdc_server *s, const tdc_job_desc *job, uint64_t *job_id)
{
    if (!s || !job || !job_id) return set_last_error(TDC_ERR_INVALID_ARGUMENT, "null argument");
    if (job->n_pri <= 0) return set_last_error(TDC_ERR_INVALID_ARGUMENT, "nPri must be greater than 0");
    if (job->n_samples <= 0) return set_last_error(TDC_ERR_INVALID_ARGUMENT, "nSamples must be greater than 0");
    if (job->n_pix <= 0 || job->n_pix > 0x7fffffff)
        return set_last_error(TDC_ERR_INVALID_ARGUMENT, "n_pix out of range");
    if (!job->raw_iq || !job->sample_times || !job->image || !(job->position || job->position_f64) ||
        !(job->grid || job->grid_f64))
        return set_last_error(TDC_ERR_INVALID_ARGUMENT, "null input array");
    auto j = std::make_unique<Job>();
    j->d = *job;
    if (!job->position) {
        j->pos32.resize((size_t)job->n_pri * 3);
        for (size_t i = 0; i < j->pos32.size(); ++i) j->pos32[i] = (float)job->position_f64[i];
    }
    j->footprint = device_footprint(*job, s->n_sm);
    if (cudaEventCreateWithFlags(&j->done_ev, cudaEventDisableTiming) != cudaSuccess)
        return set_last_error(TDC_ERR_CUDA, "event creation failed");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return set_last_error(TDC_ERR_STATE, "server is shutting down");
    j->id = s->next_id++;
    j->t_submit = now_ms() - s->t0;
    *job_id = j->id;
    s->queue.push_back(j.get());
    s->jobs.emplace(j->id, std::move(j));
    s->stats.jobs_submitted++;
    s->cv_admit.notify_all();
    return TDC_OK;
}

int tdc_server_wait(tdc_server *s, uint64_t job_id, int timeout_ms, tdc_job_info *info)
{
    if (!s) return set_last_error(TDC_ERR_INVALID_ARGUMENT, "null server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->jobs.find(job_id);
    if (it == s->jobs.end()) return set_last_error(TDC_ERR_INVALID_ARGUMENT, "unknown job id");
    Job *j = it->second.get();
    auto done = [j] { return j->state == kDone || j->state == kFailed; };
    if (timeout_ms < 0) {
        s->cv_done.wait(lk, done);
    } else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), done)) {
        return set_last_error(TDC_ERR_TIMEOUT, "job not finished");
    }
    if (info) {
        info->submit_ms = j->t_submit;
        info->admit_ms = j->t_admit;
        info->first_launch_ms = j->t_first;
        info->done_ms = j->t_done;
        info->correlations = (int64_t)j->d.n_pix * j->d.n_pri * j->d.n_samples;
        info->status = j->rc;
        info->path = j->plan.path;
    }
    if (j->rc) return set_last_error(j->rc, j->err);
    return TDC_OK;
}

int tdc_server_stats_get(tdc_server *s, tdc_server_stats *out)
{
    if (!s || !out) return set_last_error(TDC_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    out->device_bytes_in_use = (int64_t)s->mem_in_use;
    out->queued = (int)s->queue.size() + s->admitting;
    out->active = (int)(s->active.size() + s->completing.size());
    return TDC_OK;
}

int tdc_server_destroy(tdc_server *s)
{
    if (!s) return TDC_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv_work.notify_all();
        s->cv_admit.notify_all();
    }
    if (s->th_admit.joinable()) s->th_admit.join();
    if (s->th_launch.joinable()) s->th_launch.join();
    cudaSetDevice(s->device);
    for (cudaStream_t st : {s->compute[0], s->compute[1], s->side})
        if (st) cudaStreamSynchronize(st);
    for (auto &kv : s->jobs)
        if (kv.second->done_ev) cudaEventDestroy(kv.second->done_ev);
    for (Batch &b : s->batches) {
        if (b.ev) cudaEventDestroy(b.ev);
        b.dev.release();
        b.host.release();
    }
    for (tdc_processor *p : s->slots) tdc_processor_destroy(p);
    for (cudaStream_t st : {s->compute[0], s->compute[1], s->side})
        if (st) cudaStreamDestroy(st);
    delete s;
    return TDC_OK;
}

}  // extern "C"
