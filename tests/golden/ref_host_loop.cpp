// ref_host_loop.cpp -- TEST INFRASTRUCTURE ONLY: times the reference's GPU focus path the way
// its host code drives it, for the baseline table (never part of the engine).
//
// The reference's kernels run from oracle/_ref/tdckernels.ptx, compiled from its own
// tdc-lib/src/tdckernels.cu (initRangeWindowKernel, createWindowKernel,
// referenceResponseKernel, correlateWithReference, addToImage). This program restates, in
// its own code, the host loop of TdcProcessor::start (tdc-lib/src/tdcprocessor.cpp:59-167)
// around them:
//   * once: range window kernel, sample times and a zeroed image on the device;
//   * per chunk of 128 PRIs (PRI_CHUNKSIZE, tuning.h:18): the chunk's rows staged into
//     pinned per-sample buffers (rows past the last valid one keep the previous chunk's
//     values, tdcprocessor.cpp:320-345) and copied to the device with four blocking copies
//     (:310-318);
//   * per pixel: the host skip test (:347-383, FP32 as the reference computes it), then the
//     window, reference response and correlation kernels (16 x 16 blocks, tuning.h:43-56,
//     tdckernels.cu:137-274), the NPP complex sum nppsSum_32fc_Ctx with an NppStreamContext
//     filled per call from cudaGetDevice / cudaGetDeviceProperties / cudaStreamGetFlags (as
//     tdc-lib/src/npp_utils.cpp:9-27 does on every call), and addToImage<<<1, 1>>>
//     (tdckernels.cu:285-315), all on the legacy default stream;
//   * cudaGetLastError + cudaDeviceSynchronize per chunk; the image copied back at the end.
//
// Usage: ref_host_loop <tdckernels.ptx> <input.bin> <image_out.bin>
// input.bin (little endian): int32 C, S, P; float modRate, startFreq, lambda, center, bw;
// int32 centroid, applyRangeWin, taper; float bore[3]; then raw complex64 [C][S], sample
// times float [S], position float [C][3], velocity float [C][3], attitude float [C][4]
// (w, x, y, z), grid float [P][3]. Prints one JSON line with the elapsed time.
#include <cuda.h>
#include <cuda_runtime.h>
#include <npps.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

constexpr int kChunk = 128;

void ck(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) {
        std::fprintf(stderr, "%s: %s\n", what, cudaGetErrorString(e));
        std::exit(2);
    }
}

void ckd(CUresult r, const char *what)
{
    if (r != CUDA_SUCCESS) {
        const char *msg = nullptr;
        cuGetErrorString(r, &msg);
        std::fprintf(stderr, "%s: %s\n", what, msg ? msg : "?");
        std::exit(2);
    }
}

std::vector<char> read_file(const char *path)
{
    FILE *f = std::fopen(path, "rb");
    if (!f) {
        std::fprintf(stderr, "cannot open %s\n", path);
        std::exit(2);
    }
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    std::vector<char> buf((size_t)n + 1, 0);
    if (std::fread(buf.data(), 1, (size_t)n, f) != (size_t)n) std::exit(2);
    std::fclose(f);
    buf.resize((size_t)n);
    return buf;
}

// The stream context of one NPP call, filled the way the reference fills it on every call.
NppStreamContext npp_context(cudaStream_t s)
{
    NppStreamContext c{};
    c.hStream = s;
    cudaGetDevice(&c.nCudaDeviceId);
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, c.nCudaDeviceId);
    c.nMultiProcessorCount = prop.multiProcessorCount;
    c.nMaxThreadsPerMultiProcessor = prop.maxThreadsPerMultiProcessor;
    c.nMaxThreadsPerBlock = prop.maxThreadsPerBlock;
    c.nSharedMemPerBlock = prop.sharedMemPerBlock;
    c.nCudaDevAttrComputeCapabilityMajor = prop.major;
    c.nCudaDevAttrComputeCapabilityMinor = prop.minor;
    cudaStreamGetFlags(s, &c.nStreamFlags);
    return c;
}

// Hamilton product and rotation of (w, x, y, z) quaternions, FP32.
void q_prod(const float *a, const float *b, float *o)
{
    o[0] = a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3];
    o[1] = a[0] * b[1] + a[1] * b[0] + a[2] * b[3] - a[3] * b[2];
    o[2] = a[0] * b[2] - a[1] * b[3] + a[2] * b[0] + a[3] * b[1];
    o[3] = a[0] * b[3] + a[1] * b[2] - a[2] * b[1] + a[3] * b[0];
}

void q_rot(const float *q, const float *v, float *out)
{
    const float vq[4] = {0.f, v[0], v[1], v[2]};
    const float qc[4] = {q[0], -q[1], -q[2], -q[3]};
    float t[4], r[4];
    q_prod(q, vq, t);
    q_prod(t, qc, r);
    out[0] = r[1];
    out[1] = r[2];
    out[2] = r[3];
}

// Host skip test over the 3 x 3 (PRI, sample) points of the staged chunk, FP32.
bool window_is_nonzero(const float *pos, const float *vel, const float *att, int S, const float *tgt,
                       const float *bore, float lambda, float bw, float center, bool centroid)
{
    float vals[9];
    int n = 0;
    for (int i = 0; i < 3; ++i) {
        const int r = std::max(i * (kChunk / 2) - 1, 0);
        for (int j = 0; j < 3; ++j) {
            const int s = std::max(j * (S / 2) - 1, 0);
            const size_t e = (size_t)r * S + s;
            const float *p = pos + 3 * e, *v = vel + 3 * e, *q = att + 4 * e;
            float fc = center;
            if (centroid) {
                float ant[3];
                q_rot(q, bore, ant);
                fc = 2.0f / lambda * (v[0] * ant[0] + v[1] * ant[1] + v[2] * ant[2]);
            }
            const float d[3] = {tgt[0] - p[0], tgt[1] - p[1], tgt[2] - p[2]};
            const float nrm = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            const float fd = 2.0f / lambda * (v[0] * d[0] + v[1] * d[1] + v[2] * d[2]) / nrm;
            vals[n++] = std::fabs(fd - fc);
        }
    }
    float m = vals[0];
    for (int k = 1; k < 9; ++k)
        if (vals[k] < m) m = vals[k];
    return m <= bw / 2.0f;
}

struct F3 {
    float x, y, z;
};

}  // namespace

int main(int argc, char **argv)
{
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s <tdckernels.ptx> <input.bin> <image_out.bin>\n", argv[0]);
        return 2;
    }
    std::vector<char> ptx = read_file(argv[1]);
    ptx.push_back('\0');
    const std::vector<char> in = read_file(argv[2]);
    const char *q = in.data();
    auto take = [&](void *dst, size_t n) {
        std::memcpy(dst, q, n);
        q += n;
    };
    int C, S, P, centroid_i, range_win_i, taper_i;
    float mod_rate, start_freq, lambda, center, bw, bore[3];
    take(&C, 4);
    take(&S, 4);
    take(&P, 4);
    take(&mod_rate, 4);
    take(&start_freq, 4);
    take(&lambda, 4);
    take(&center, 4);
    take(&bw, 4);
    take(&centroid_i, 4);
    take(&range_win_i, 4);
    take(&taper_i, 4);
    take(bore, 12);
    std::vector<float> raw((size_t)C * S * 2), st(S), pos((size_t)C * 3), vel((size_t)C * 3), att((size_t)C * 4),
        grid((size_t)P * 3);
    take(raw.data(), raw.size() * 4);
    take(st.data(), st.size() * 4);
    take(pos.data(), pos.size() * 4);
    take(vel.data(), vel.size() * 4);
    take(att.data(), att.size() * 4);
    take(grid.data(), grid.size() * 4);
    bool centroid = centroid_i != 0, range_win = range_win_i != 0, taper = taper_i != 0;

    ck(cudaSetDevice(0), "cudaSetDevice");
    ck(cudaFree(nullptr), "context");
    CUmodule mod;
    ckd(cuModuleLoadData(&mod, ptx.data()), "cuModuleLoadData");
    CUfunction k_range, k_window, k_ref, k_corr, k_add;
    ckd(cuModuleGetFunction(&k_range, mod, "_Z21initRangeWindowKernelPfib"), "initRangeWindowKernel");
    ckd(cuModuleGetFunction(&k_window, mod, "_Z18createWindowKernelPfPKfPK6float3S4_PK6float4S2_S2_fffbbiii"),
        "createWindowKernel");
    ckd(cuModuleGetFunction(&k_ref, mod, "_Z23referenceResponseKernelP6float2PKfPK6float3S2_S3_ffiii"),
        "referenceResponseKernel");
    ckd(cuModuleGetFunction(&k_corr, mod, "_Z22correlateWithReferencePK6float2PS_iii"), "correlateWithReference");
    ckd(cuModuleGetFunction(&k_add, mod, "_Z10addToImageP6float2S0_"), "addToImage");

    const size_t n = (size_t)kChunk * S;
    float *d_rw, *d_st, *d_win, *d_pos, *d_vel, *d_att;
    float2 *d_raw, *d_ref, *d_img, *d_sum;
    ck(cudaMalloc(&d_rw, S * 4), "alloc");
    ck(cudaMalloc(&d_st, S * 4), "alloc");
    ck(cudaMalloc(&d_win, n * 4), "alloc");
    ck(cudaMalloc(&d_pos, n * 12), "alloc");
    ck(cudaMalloc(&d_vel, n * 12), "alloc");
    ck(cudaMalloc(&d_att, n * 16), "alloc");
    ck(cudaMalloc(&d_raw, n * 8), "alloc");
    ck(cudaMalloc(&d_ref, n * 8), "alloc");
    ck(cudaMalloc(&d_img, (size_t)std::max(P, 1) * 8), "alloc");
    ck(cudaMalloc(&d_sum, 8), "alloc");
    size_t scratch_bytes = 0;
    if (nppsSumGetBufferSize_32fc_Ctx((size_t)kChunk * S, &scratch_bytes, npp_context(nullptr)) != NPP_SUCCESS) {
        std::fprintf(stderr, "nppsSumGetBufferSize_32fc_Ctx failed\n");
        return 2;
    }
    Npp8u *d_scratch;
    ck(cudaMalloc(&d_scratch, std::max<size_t>(scratch_bytes, 16)), "alloc");
    float *h_raw, *h_pos, *h_vel, *h_att;
    ck(cudaMallocHost(&h_raw, n * 8), "pinned");
    ck(cudaMallocHost(&h_pos, n * 12), "pinned");
    ck(cudaMallocHost(&h_vel, n * 12), "pinned");
    ck(cudaMallocHost(&h_att, n * 16), "pinned");
    std::memset(h_raw, 0, n * 8);
    std::memset(h_pos, 0, n * 12);
    std::memset(h_vel, 0, n * 12);
    std::memset(h_att, 0, n * 16);

    ck(cudaDeviceSynchronize(), "sync");
    const auto t0 = std::chrono::steady_clock::now();
    {
        void *args[] = {&d_rw, &S, &range_win};
        ckd(cuLaunchKernel(k_range, (S + 31) / 32, 1, 1, 32, 1, 1, 0, nullptr, args, nullptr), "range window");
    }
    ck(cudaMemcpy(d_st, st.data(), S * 4, cudaMemcpyHostToDevice), "copy sample times");
    ck(cudaMemset(d_img, 0, (size_t)std::max(P, 1) * 8), "zero image");
    const int n_chunks = (C + kChunk - 1) / kChunk;
    long processed = 0, skipped = 0;
    const unsigned gx = (S + 15) / 16, gy = kChunk / 16;
    F3 bore3{bore[0], bore[1], bore[2]};
    for (int k = 0; k < n_chunks; ++k) {
        const int valid = std::min(kChunk, C - k * kChunk);
        std::memcpy(h_raw, raw.data() + (size_t)k * kChunk * S * 2, (size_t)valid * S * 8);
        for (int r = 0; r < valid; ++r) {
            const int c = k * kChunk + r;
            for (int s = 0; s < S; ++s) {
                const size_t e = (size_t)r * S + s;
                std::memcpy(h_pos + 3 * e, pos.data() + 3 * (size_t)c, 12);
                std::memcpy(h_vel + 3 * e, vel.data() + 3 * (size_t)c, 12);
                std::memcpy(h_att + 4 * e, att.data() + 4 * (size_t)c, 16);
            }
        }
        ck(cudaMemcpy(d_raw, h_raw, n * 8, cudaMemcpyHostToDevice), "copy raw");
        ck(cudaMemcpy(d_pos, h_pos, n * 12, cudaMemcpyHostToDevice), "copy position");
        ck(cudaMemcpy(d_vel, h_vel, n * 12, cudaMemcpyHostToDevice), "copy velocity");
        ck(cudaMemcpy(d_att, h_att, n * 16, cudaMemcpyHostToDevice), "copy attitude");
        for (int p = 0; p < P; ++p) {
            const float *t = grid.data() + 3 * (size_t)p;
            if (!window_is_nonzero(h_pos, h_vel, h_att, S, t, bore, lambda, bw, center, centroid)) {
                ++skipped;
                continue;
            }
            ++processed;
            F3 tgt{t[0], t[1], t[2]};
            int ki = k;
            {
                void *args[] = {&d_win, &d_rw, &d_pos, &d_vel, &d_att, &tgt, &bore3, &lambda, &bw, &center,
                                &centroid, &taper, &ki, &C, &S};
                ckd(cuLaunchKernel(k_window, gx, gy, 1, 16, 16, 1, 0, nullptr, args, nullptr), "window");
            }
            {
                void *args[] = {&d_ref, &d_win, &d_pos, &d_st, &tgt, &start_freq, &mod_rate, &ki, &C, &S};
                ckd(cuLaunchKernel(k_ref, gx, gy, 1, 16, 16, 1, 0, nullptr, args, nullptr), "reference response");
            }
            {
                void *args[] = {&d_raw, &d_ref, &ki, &C, &S};
                ckd(cuLaunchKernel(k_corr, gx, gy, 1, 16, 16, 1, 0, nullptr, args, nullptr), "correlation");
            }
            if (nppsSum_32fc_Ctx(reinterpret_cast<const Npp32fc *>(d_ref), (size_t)valid * S,
                                 reinterpret_cast<Npp32fc *>(d_sum), d_scratch, npp_context(nullptr)) != NPP_SUCCESS) {
                std::fprintf(stderr, "nppsSum_32fc_Ctx failed\n");
                return 2;
            }
            float2 *pix = d_img + p;
            {
                void *args[] = {&pix, &d_sum};
                ckd(cuLaunchKernel(k_add, 1, 1, 1, 1, 1, 1, 0, nullptr, args, nullptr), "addToImage");
            }
        }
        ck(cudaGetLastError(), "chunk");
        ck(cudaDeviceSynchronize(), "chunk sync");
    }
    std::vector<float> img((size_t)P * 2);
    if (P > 0) ck(cudaMemcpy(img.data(), d_img, (size_t)P * 8, cudaMemcpyDeviceToHost), "copy image");
    const auto t1 = std::chrono::steady_clock::now();
    const double ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    FILE *f = std::fopen(argv[3], "wb");
    if (!f || std::fwrite(img.data(), 4, img.size(), f) != img.size()) return 2;
    std::fclose(f);
    std::printf("{\"ms\": %.3f, \"pixels\": %d, \"chirps\": %d, \"samples\": %d, \"chunks\": %d, "
                "\"processed\": %ld, \"skipped\": %ld, \"npp_scratch_bytes\": %zu}\n",
                ms, P, C, S, n_chunks, processed, skipped, scratch_bytes);
    return 0;
}
