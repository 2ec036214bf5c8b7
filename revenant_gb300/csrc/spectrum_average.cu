// Averaged power spectrum: lw-radio-dsp's Spectrum::compute on the GPU.
//
// third_party/lw-radio-dsp/src/spectrum.cpp:32-44 and src/fft.cpp:31-50: an
// N-point windowed FFT of a frame, |X|^2 scaled by 1 / (sum of the window)^2,
// fftshifted (bin k reads transform bin (k + N - N/2) mod N), averaged, then
// 10 log10(max(p, 1e-30)) (include/lwdsp/types.h:38). Two averages:
//   RV_AVERAGE_MEAN        the mean of `average` consecutive frames (the
//                          "averaged over 16 frames" of the single-receiver
//                          configuration);
//   RV_AVERAGE_EXPONENTIAL lwdsp's avg = a * avg + (1 - a) * p, frame by frame,
//                          the first frame seeding avg.
// The transform is this library's radix-2 DIT, not pocketfft, so results
// agree with an FP64 restatement to a stated tolerance rather than bit for bit.
//
// lwdsp keeps the exponential average between calls (Spectrum::Impl::avg);
// here the caller may pass `avg_dev` (N floats of linear power): it receives
// the final average and, with `resume` set, seeds the next call.
//
// One CTA per output spectrum: it transforms its frames one after another in
// shared memory and keeps the running power per bin in shared memory, so no
// scratch buffer is needed.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "common.cuh"
#include "revenant_gb300.h"

namespace rv {
namespace {

constexpr uint32_t kMaxSize = 8192;  // 96 KiB of shared memory per CTA

__global__ void k_spectrum_average(const rv_cf32* __restrict__ iq, const float* __restrict__ window,
                                   const rv_cf32* __restrict__ tw, float* __restrict__ out,
                                   float* __restrict__ avg, rv_spectrum_average_params p, uint32_t stages) {
    extern __shared__ float2 x[];  // [N] transform, then [N] float running power
    float* acc = reinterpret_cast<float*>(x + p.size);
    const uint32_t N = p.size, half = N / 2;
    const uint32_t spectrum = blockIdx.x;
    const uint32_t per = (p.mode == RV_AVERAGE_MEAN) ? p.average : p.frames;
    for (uint32_t f = 0; f < per; ++f) {
        const uint64_t frame = (uint64_t)spectrum * per + f;
        const rv_cf32* src = iq + frame * N;
        for (uint32_t n = threadIdx.x; n < N; n += blockDim.x) {
            const float2 v = ld_cf32(&src[n]);
            const float w = window[n];
            x[brev(n, stages)] = make_float2(v.x * w, v.y * w);
        }
        __syncthreads();
        for (uint32_t st = 0; st < stages; ++st) {
            const uint32_t hs = 1u << st, step = N >> (st + 1u);
            for (uint32_t b = threadIdx.x; b < half; b += blockDim.x) {
                const uint32_t j = b & (hs - 1u);
                const uint32_t ia = ((b >> st) << (st + 1u)) + j;
                butterfly(x[ia], x[ia + hs], ld_cf32(&tw[j * step]));
            }
            __syncthreads();
        }
        for (uint32_t k = threadIdx.x; k < N; k += blockDim.x) {
            const float2 v = x[(k + N - half) & (N - 1u)];
            const float pw = (v.x * v.x + v.y * v.y) * p.norm;
            if (p.mode == RV_AVERAGE_MEAN) {
                acc[k] = (f == 0) ? pw : acc[k] + pw;
            } else {
                // the first frame of a fresh average blends with itself, as
                // lwdsp's avg = power; avg = a*avg + (1-a)*power does
                const float prev = (f > 0) ? acc[k] : (p.resume ? avg[k] : pw);
                acc[k] = p.alpha * prev + (1.0F - p.alpha) * pw;
            }
        }
        __syncthreads();
    }
    for (uint32_t k = threadIdx.x; k < N; k += blockDim.x) {
        float pw = acc[k];
        if (p.mode == RV_AVERAGE_MEAN) pw = pw / (float)p.average;
        if (avg != nullptr) avg[(uint64_t)spectrum * N + k] = pw;
        out[(uint64_t)spectrum * N + k] = 10.0F * log10f(fmaxf(pw, 1e-30F));
    }
}

}  // namespace
}  // namespace rv

extern "C" int32_t rv_spectrum_average(void* stream, const rv_spectrum_average_params* p, const rv_cf32* iq_dev,
                                       uint64_t iq_len, const float* window_dev, uint64_t window_len,
                                       const rv_cf32* twiddles_dev, uint64_t twiddles_len, float* out_dev,
                                       uint64_t out_len, float* avg_dev, uint64_t avg_len) {
    using rv::set_error_fmt;
    if (p == nullptr || iq_dev == nullptr || window_dev == nullptr || twiddles_dev == nullptr || out_dev == nullptr)
        return set_error_fmt(RV_ERR_INVALID, "rv_spectrum_average: NULL argument");
    const uint32_t N = p->size;
    if (!rv::is_pow2(N) || N < 16 || N > rv::kMaxSize)
        return set_error_fmt(RV_ERR_INVALID, "spectrum average: size %u must be a power of two in [16, %u]", N,
                             rv::kMaxSize);
    if (p->mode != RV_AVERAGE_MEAN && p->mode != RV_AVERAGE_EXPONENTIAL)
        return set_error_fmt(RV_ERR_INVALID, "spectrum average: mode %u", p->mode);
    if (p->frames == 0) return set_error_fmt(RV_ERR_INVALID, "spectrum average: no frames");
    uint32_t spectra;
    if (p->mode == RV_AVERAGE_MEAN) {
        if (p->average == 0 || p->frames % p->average != 0)
            return set_error_fmt(RV_ERR_INVALID, "spectrum average: %u frames are not a multiple of the %u averaged",
                                 p->frames, p->average);
        spectra = p->frames / p->average;
    } else {
        if (!(p->alpha >= 0.0F && p->alpha <= 0.999F))
            return set_error_fmt(RV_ERR_INVALID, "spectrum average: exponential weight %g outside [0, 0.999]",
                                 (double)p->alpha);
        spectra = 1;
        if (p->resume && avg_dev == nullptr)
            return set_error_fmt(RV_ERR_INVALID, "spectrum average: resume needs the previous average");
    }
    if (p->mode == RV_AVERAGE_MEAN && p->resume)
        return set_error_fmt(RV_ERR_INVALID, "spectrum average: only the exponential average resumes");
    if (iq_len < (uint64_t)p->frames * N) return set_error_fmt(RV_ERR_INVALID, "spectrum average: input too short");
    if (window_len != N || twiddles_len != N)
        return set_error_fmt(RV_ERR_INVALID, "spectrum average: window and twiddles must hold %u entries", N);
    if (out_len < (uint64_t)spectra * N) return set_error_fmt(RV_ERR_INVALID, "spectrum average: output too short");
    if (avg_dev != nullptr && avg_len < (uint64_t)spectra * N)
        return set_error_fmt(RV_ERR_INVALID, "spectrum average: average buffer too short");
    const size_t shared = (size_t)N * (sizeof(float2) + sizeof(float));
    if (shared > 48 * 1024) {
        if (int32_t st = rv::cuda_status(cudaFuncSetAttribute(rv::k_spectrum_average,
                                                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shared),
                                         "spectrum average: shared memory"))
            return st;
    }
    rv::k_spectrum_average<<<spectra, 256, shared, reinterpret_cast<cudaStream_t>(stream)>>>(
        iq_dev, window_dev, twiddles_dev, out_dev, avg_dev, *p, rv::ilog2(N));
    if (int32_t st = rv::cuda_status(cudaGetLastError(), "spectrum average")) return st;
    return rv::clear_error();
}

// make_window (third_party/lw-radio-dsp/src/primitives.cpp:124-148): the
// symmetric Hann / Blackman-Harris over n points, evaluated in double.
extern "C" int32_t rv_build_lwdsp_window(uint32_t kind, uint32_t n, float* window, double* norm) {
    if (window == nullptr || n < 2) return rv::set_error_fmt(RV_ERR_INVALID, "rv_build_lwdsp_window: bad arguments");
    const double pi = 3.141592653589793238462643383279502884;
    const double m = (double)(n - 1);
    double sum = 0.0;
    for (uint32_t i = 0; i < n; ++i) {
        const double x = (double)i / m;
        double v;
        if (kind == RV_WINDOW_HANN) {
            v = 0.5 - 0.5 * cos(2.0 * pi * x);
        } else if (kind == RV_WINDOW_BLACKMAN_HARRIS) {
            v = 0.35875 - 0.48829 * cos(2.0 * pi * x) + 0.14128 * cos(4.0 * pi * x) - 0.01168 * cos(6.0 * pi * x);
        } else if (kind == RV_WINDOW_RECTANGULAR) {
            v = 1.0;
        } else {
            return rv::set_error_fmt(RV_ERR_INVALID, "rv_build_lwdsp_window: window kind %u", kind);
        }
        window[i] = (float)v;
        sum += (double)window[i];
    }
    // power_spectrum's 1 / wsum^2, with wsum summed in double over the floats
    if (norm) *norm = 1.0 / (sum * sum);
    return rv::clear_error();
}
