// The scene synthesiser's noise field on the GPU (siggen::Scene::fill_noise,
// core/dsp/synth/wideband.cpp:535-580).
//
// The reference cuts the stream into 4096-sample noise blocks; block b draws
// from its own std::mt19937_64 seeded with derive_stream_seed(seed ^ b,
// noise domain) (wideband.cpp:46-53, a splitmix64-style finaliser), two draws
// per complex sample, and turns each pair into Gaussian I/Q by Box-Muller in
// FP64:  radial = ((d0 >> 11) + 1) 2^-53,  angular = (d1 >> 11) 2^-53,
// magnitude = sigma sqrt(-2 ln radial),  sample = (float)(magnitude cos 2 pi
// angular), (float)(magnitude sin 2 pi angular).
//
// Here one warp owns one noise block. The generator is the published
// MT19937-64 (Matsumoto and Nishimura; the C++ standard's mt19937_64
// parameters), its 312-word state in shared memory twisted cooperatively: the
// first 156 words depend only on the old state, the next 155 on the old
// state and the first 156 new words, the last on new words 0 and 155, so the
// twist runs as three passes over a double-buffered state. The 312 tempered
// outputs of each twist are 156 samples. The draws are integers and match the
// reference bit for bit; the FP64 logarithm, sine and cosine are CUDA's, so a
// sample can differ from the reference's in its last FP32 bit where the FP64
// value sits within an FP64 ulp of an FP32 rounding boundary.
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace rv {
namespace {

constexpr uint32_t kNoiseBlock = 4096;   // samples per noise block (wideband.cpp:36)
constexpr uint64_t kNoiseDomain = 0x1a59017e55ce0d02ull;  // wideband.cpp:41
constexpr uint32_t kN = 312, kHalf = 156;
constexpr uint64_t kMatrixA = 0xB5026F5AA96619E9ull;
constexpr uint64_t kUpper = 0xFFFFFFFF80000000ull, kLower = 0x7FFFFFFFull;
constexpr uint32_t kWarps = 8;           // noise blocks per CTA
constexpr double kMantissaStep = 1.0 / 9007199254740992.0;
constexpr double kTwoPi = 6.283185307179586476925286766559;

__host__ __device__ inline uint64_t derive_stream_seed(uint64_t master, uint64_t domain) {
    uint64_t z = master + domain * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ uint64_t twist_word(uint64_t lo_word, uint64_t hi_word, uint64_t far) {
    const uint64_t y = (lo_word & kUpper) | (hi_word & kLower);
    return far ^ (y >> 1) ^ ((y & 1ull) ? kMatrixA : 0ull);
}

__device__ __forceinline__ uint64_t temper(uint64_t y) {
    y ^= (y >> 29) & 0x5555555555555555ull;
    y ^= (y << 17) & 0x71D67FFFEDA60000ull;
    y ^= (y << 37) & 0xFFF7EEE000000000ull;
    return y ^ (y >> 43);
}

// One warp: noise block `block`, samples of [lo, hi) within it written to
// out[s - start] (as cf32) or their raw draw pairs to draws[2 (s - start)].
template <bool kDraws>
__device__ void noise_block(uint64_t* st, uint64_t* nx, uint64_t seed, uint64_t block, uint64_t lo, uint64_t hi,
                            uint64_t start, double sigma, float2* out, uint64_t* draws) {
    const uint32_t lane = threadIdx.x & 31u;
    if (lane == 0) {  // std::mt19937_64's seeding recurrence
        uint64_t x = derive_stream_seed(seed ^ block, kNoiseDomain);
        st[0] = x;
        for (uint32_t i = 1; i < kN; ++i) {
            x = 6364136223846793005ull * (x ^ (x >> 62)) + i;
            st[i] = x;
        }
    }
    __syncwarp();
    const uint64_t block_start = block * kNoiseBlock;
    // twists until the block's last needed sample: sample s uses draws 2s, 2s+1
    const uint32_t last = (uint32_t)(hi - block_start);  // exclusive, <= 4096
    for (uint32_t base = 0; base < last; base += kHalf) {
        for (uint32_t i = lane; i < kHalf; i += 32) nx[i] = twist_word(st[i], st[i + 1], st[i + kHalf]);
        __syncwarp();
        for (uint32_t i = kHalf + lane; i < kN - 1; i += 32) nx[i] = twist_word(st[i], st[i + 1], nx[i - kHalf]);
        __syncwarp();
        if (lane == 0) nx[kN - 1] = twist_word(st[kN - 1], nx[0], nx[kHalf - 1]);
        __syncwarp();
        for (uint32_t j = lane; j < kHalf; j += 32) {
            const uint64_t s = block_start + base + j;
            if (s >= lo && s < hi) {
                const uint64_t d0 = temper(nx[2 * j]), d1 = temper(nx[2 * j + 1]);
                if (kDraws) {
                    draws[2 * (s - start)] = d0;
                    draws[2 * (s - start) + 1] = d1;
                } else {
                    const double radial = (double)((d0 >> 11) + 1ull) * kMantissaStep;
                    const double angular = (double)(d1 >> 11) * kMantissaStep;
                    const double magnitude = sigma * sqrt(-2.0 * log(radial));
                    const double angle = kTwoPi * angular;
                    out[s - start] = make_float2((float)(magnitude * cos(angle)), (float)(magnitude * sin(angle)));
                }
            }
        }
        __syncwarp();
        uint64_t* t = st;  // the new state is the old state of the next twist
        st = nx;
        nx = t;
    }
}

template <bool kDraws>
__global__ void __launch_bounds__(kWarps * 32)
k_scene_noise(uint64_t seed, double sigma, uint64_t start, uint64_t count, uint64_t first_block, uint64_t nblocks,
              float2* out, uint64_t* draws) {
    __shared__ uint64_t state[kWarps][2][kN];
    const uint32_t w = threadIdx.x >> 5;
    const uint64_t end = start + count;
    for (uint64_t k = (uint64_t)blockIdx.x * kWarps + w; k < nblocks; k += (uint64_t)gridDim.x * kWarps) {
        const uint64_t block = first_block + k;
        const uint64_t bs = block * kNoiseBlock;
        const uint64_t lo = bs > start ? bs : start, hi = bs + kNoiseBlock < end ? bs + kNoiseBlock : end;
        noise_block<kDraws>(state[w][0], state[w][1], seed, block, lo, hi, start, sigma, out, draws);
    }
}

int32_t launch(cudaStream_t s, uint64_t seed, double sigma, uint64_t start, uint64_t count, float2* out,
               uint64_t* draws) {
    if (count == 0) return RV_OK;
    const uint64_t first = start / kNoiseBlock, last = (start + count - 1) / kNoiseBlock;
    const uint64_t nblocks = last - first + 1;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint64_t want = (nblocks + kWarps - 1) / kWarps, cap = (uint64_t)sms * 8u;
    const unsigned grid = (unsigned)(want < cap ? want : cap);
    if (draws)
        k_scene_noise<true><<<grid, kWarps * 32, 0, s>>>(seed, sigma, start, count, first, nblocks, out, draws);
    else
        k_scene_noise<false><<<grid, kWarps * 32, 0, s>>>(seed, sigma, start, count, first, nblocks, out, draws);
    return cuda_status(cudaGetLastError(), "scene noise");
}

}  // namespace
}  // namespace rv

using namespace rv;

extern "C" double rv_scene_noise_sigma(double noise_power_full_band_dbfs) {
    // wideband.cpp:108-111 db_to_power and :200-203: the power split evenly
    // between I and Q
    const double power = pow(10.0, noise_power_full_band_dbfs * 0.1);
    return sqrt(power * 0.5);
}

extern "C" int32_t rv_scene_noise(void* stream, uint64_t seed, double sigma, uint64_t start, uint64_t count,
                                  rv_cf32* out, uint64_t out_len) {
    if (out == nullptr && count > 0) return set_error_fmt(RV_ERR_INVALID, "scene noise: NULL output");
    if (out_len < count) return set_error_fmt(RV_ERR_INVALID, "scene noise: output of %llu for %llu samples",
                                              (unsigned long long)out_len, (unsigned long long)count);
    if (!(sigma >= 0.0)) return set_error_fmt(RV_ERR_INVALID, "scene noise: sigma must be >= 0");
    if (start + count < start) return set_error_fmt(RV_ERR_INVALID, "scene noise: range wraps");
    if (int32_t st = launch(reinterpret_cast<cudaStream_t>(stream), seed, sigma, start, count,
                            reinterpret_cast<float2*>(out), nullptr))
        return st;
    return clear_error();
}

extern "C" int32_t rv_scene_noise_draws(void* stream, uint64_t seed, uint64_t start, uint64_t count, uint64_t* draws,
                                        uint64_t draws_len) {
    if (draws == nullptr && count > 0) return set_error_fmt(RV_ERR_INVALID, "scene noise draws: NULL output");
    if (draws_len < 2 * count) return set_error_fmt(RV_ERR_INVALID, "scene noise draws: needs 2 per sample");
    if (start + count < start) return set_error_fmt(RV_ERR_INVALID, "scene noise draws: range wraps");
    if (int32_t st = launch(reinterpret_cast<cudaStream_t>(stream), seed, 0.0, start, count, nullptr, draws))
        return st;
    return clear_error();
}
