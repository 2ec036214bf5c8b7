// extern "C" access to the reference's scene synthesiser
// (core/dsp/synth/wideband.cpp siggen::Scene), compiled from the reference
// sources into oracle/_ref/libsynref.so. Test infrastructure only: the noise
// tests render noise-only scenes with it and compare the library's GPU noise
// field against them. Only wideband.cpp is compiled; the modulators it can
// call for emitters are left unresolved and the library is loaded lazily, so
// a scene here must have no emitters.
#include <complex>
#include <cstdint>
#include <random>
#include <span>
#include <vector>

#include "core/dsp/synth/wideband.h"

using namespace revenant;

extern "C" {

// Scene::render of a noise-only scene: `count` samples from `start`.
int refsyn_noise(std::uint64_t seed, std::int64_t rate, double noise_dbfs, std::uint64_t start, std::uint64_t count,
                 float* out) {
    siggen::SceneSpec spec;
    spec.rate = rate;
    spec.seed = seed;
    spec.add_noise = true;
    spec.noise_power_full_band_dbfs = noise_dbfs;
    spec.duration_samples = start + count;
    spec.worker_threads = 1;
    auto scene = siggen::Scene::create(spec);
    if (!scene) return -1;
    std::vector<std::complex<float>> buf(count);
    scene->render(start, std::span<std::complex<float>>(buf));
    for (std::uint64_t i = 0; i < count; ++i) {
        out[2 * i] = buf[i].real();
        out[2 * i + 1] = buf[i].imag();
    }
    return 0;
}

// The libstdc++ std::mt19937_64 stream of one noise block, for pinning the
// GPU generator's draws: the block's seed is given (the reference derives it
// with derive_stream_seed, which the tests restate).
void refsyn_mt64(std::uint64_t seed, std::uint64_t n, std::uint64_t* out) {
    std::mt19937_64 engine(seed);
    for (std::uint64_t i = 0; i < n; ++i) out[i] = engine();
}

}  // extern "C"
