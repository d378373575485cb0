// C++ smoke test of include/tdcprocessor.h, shaped like the reference's
// tdctest/tdctest.cpp:21-59 (all-zero inputs, 20 x 20 grid, nPri = 750,
// nSamples = 1500, 5 Hz Doppler band, centroid windowing, range window), plus
// the invalid_argument contract of tdcprocessor.cpp:189-195.
#include <complex>
#include <cstdio>
#include <stdexcept>
#include <vector>

#include "tdcprocessor.h"

int main()
{
    TdcProcessor tdc(0);
    const int nRows = 20, nCols = 20;
    std::vector<float> grid(nRows * nCols * 3);
    tdc.setFocusGrid(grid.data(), nRows, nCols);

    const size_t nPri = 750, nSamples = 1500, n = nPri * nSamples;
    std::vector<std::complex<float>> raw(n);
    std::vector<float> priTimes(nPri), sampleTimes(nSamples), position(n * 3), velocity(n * 3), attitude(n * 4);
    const float3 bore = {0, 1, 0};
    tdc.setRawData(raw.data(), priTimes.data(), sampleTimes.data(), position.data(), velocity.data(),
                   attitude.data(), nPri, nSamples, 1.0, 1.0, bore);
    tdc.start(0.0, 5.0, true, true);
    const float2 *img = tdc.imageBuffer();
    if (img == nullptr) {
        std::puts("FAIL: null image");
        return 1;
    }
    for (int i = 0; i < nRows * nCols; ++i) {
        if (img[i].x != 0.0f || img[i].y != 0.0f) {
            std::puts("FAIL: non-zero pixel for all-zero input");
            return 1;
        }
    }
    bool threw = false;
    try {
        tdc.setRawData(raw.data(), priTimes.data(), sampleTimes.data(), position.data(), velocity.data(),
                       attitude.data(), 0, nSamples, 1.0, 1.0, bore);
    } catch (const std::invalid_argument &) {
        threw = true;
    }
    if (!threw) {
        std::puts("FAIL: nPri = 0 accepted");
        return 1;
    }
    std::puts("OK");
    return 0;
}
