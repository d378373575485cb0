// tdcprocessor.h -- C++ TdcProcessor of the GB300 TDC engine.
//
// Header-compatible with the public section of the sarlab-tdc class
// (tdc-lib/include/tdcprocessor.h:42-135): same constructor, method names,
// argument types and meaning, ownership (borrowed input pointers, processor-owned
// image buffer) and exceptions (std::invalid_argument for nPri / nSamples <= 0,
// std::runtime_error for CUDA failures). The private section is a handle to the
// C ABI of tdc_gb300.h, so C++ callers link only libtdc_gb300.so.
//
// setLoggerSinks is available when spdlog is on the include path, as in the
// reference; the engine itself logs nothing, this header logs the same
// lifecycle messages the reference's processor does (start, completion, time).
#ifndef TDCPROCESSOR_H
#define TDCPROCESSOR_H

#include <chrono>
#include <complex>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include <vector_types.h>  // float2, float3 (CUDA)

#include "tdc_gb300.h"

#if __has_include(<spdlog/logger.h>)
#include <spdlog/logger.h>
#include <spdlog/spdlog.h>
#define TDC_GB300_HAVE_SPDLOG 1
#endif

class TdcProcessor
{
public:
    explicit TdcProcessor(int gpuNum)
    {
        check(tdc_processor_create(gpuNum, &h_));
    }
    ~TdcProcessor() { tdc_processor_destroy(h_); }
    TdcProcessor(const TdcProcessor &) = delete;
    TdcProcessor &operator=(const TdcProcessor &) = delete;

    // Start the SAR processor; returns when processing is complete (tdcprocessor.h:47-68).
    void start(float dopplerWinCenter, float dopplerBandwidth, bool dopCentroidWin, bool applyRangeWin,
               bool dopplerWinTaper = true)
    {
        const auto t0 = std::chrono::steady_clock::now();
        info("Starting the TDC processor");
        check(tdc_processor_start(h_, dopplerWinCenter, dopplerBandwidth, dopCentroidWin ? 1 : 0,
                                  applyRangeWin ? 1 : 0, dopplerWinTaper ? 1 : 0));
        info("Completed SAR processing");
        const auto s = std::chrono::duration_cast<std::chrono::seconds>(std::chrono::steady_clock::now() - t0);
        info("Elapsed time: " + std::to_string(s.count()) + "s");
    }

    // Configure the raw radar data (tdcprocessor.h:70-107). Pointers are borrowed until start() returns.
    void setRawData(std::complex<float> const *rawData, float const *priTimes, float const *sampleTimes,
                    float const *position, float const *velocity, float const *attitude, int nPri, int nSamples,
                    float modRate, float startFreq, float3 bodyBoresight)
    {
        info("Setting raw data with " + std::to_string(nPri) + " PRIs and " + std::to_string(nSamples) +
             " samples/PRI");
        const float bore[3] = {bodyBoresight.x, bodyBoresight.y, bodyBoresight.z};
        check(tdc_processor_set_raw_data(h_, reinterpret_cast<const float *>(rawData), priTimes, sampleTimes,
                                         position, velocity, attitude, nPri, nSamples, modRate, startFreq, bore));
    }

    // Configure the focus grid, nRows x nCols x 3 (tdcprocessor.h:109-121).
    void setFocusGrid(float const *focusGrid, int nRows, int nCols)
    {
        info("Configure the focus grid with shape " + std::to_string(nRows) + " x " + std::to_string(nCols));
        check(tdc_processor_set_focus_grid(h_, focusGrid, nRows, nCols));
    }

#ifdef TDC_GB300_HAVE_SPDLOG
    // Log to the given sinks from now on (tdcprocessor.h:123-128).
    void setLoggerSinks(const std::vector<spdlog::sink_ptr> &sinks)
    {
        log_ = std::make_shared<spdlog::logger>("TDCPROC", sinks.begin(), sinks.end());
        log_->set_level(spdlog::level::debug);
        log_->flush_on(spdlog::level::info);
        info("Completed logging setup");
    }
#endif

    // Focused image, nRows x nCols complex float; owned by the processor (tdcprocessor.h:130-135).
    float2 const *imageBuffer() const
    {
        return reinterpret_cast<float2 const *>(tdc_processor_image_buffer(h_));
    }

    // ---- extensions (no reference counterpart) ----
    // Caller-owned image output (nFloats >= 2 x pixels); later start() calls write into it.
    void setImageOutput(float2 *image, int64_t nFloats)
    {
        check(tdc_processor_set_image_output(h_, reinterpret_cast<float *>(image), nFloats));
    }
    void setChirpPositionsF64(double const *position, int nPri)
    {
        check(tdc_processor_set_chirp_positions_f64(h_, position, nPri));
    }
    void setFocusGridF64(double const *focusGrid, int nRows, int nCols)
    {
        check(tdc_processor_set_focus_grid_f64(h_, focusGrid, nRows, nCols));
    }
    tdc_start_stats lastStats() const
    {
        tdc_start_stats s{};
        check(tdc_processor_last_stats(h_, &s));
        return s;
    }
    tdc_processor *handle() const { return h_; }

private:
    static void check(int rc)
    {
        if (rc == TDC_OK) return;
        const std::string msg = tdc_last_error();
        if (rc == TDC_ERR_INVALID_ARGUMENT) throw std::invalid_argument(msg);
        throw std::runtime_error(msg);
    }
    void info(const std::string &msg) const
    {
#ifdef TDC_GB300_HAVE_SPDLOG
        if (log_) log_->info(msg);
#else
        (void)msg;
#endif
    }

    tdc_processor *h_ = nullptr;
#ifdef TDC_GB300_HAVE_SPDLOG
    std::shared_ptr<spdlog::logger> log_;
#endif
};

#endif  // TDCPROCESSOR_H
