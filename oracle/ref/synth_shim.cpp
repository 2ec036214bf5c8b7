// extern "C" access to the reference's scene synthesiser
// (core/dsp/synth/wideband.cpp siggen::Scene), compiled from the reference
// sources into oracle/_ref/libsynref.so. Test infrastructure only: the
// scene tests render noise-only scenes, tone AM and NFM emitters, and scenes
// of noise plus such emitters with it, and compare the library's GPU noise
// field and emitters against them. wideband.cpp and modulators.cpp are
// compiled; what the other modes and the FM stations would call is left
// unresolved and the library is loaded lazily, so only those emitters may be
// used here.
#include <complex>
#include <cstdio>
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

static std::int64_t g_tone2 = 0, g_low = 300, g_high = 3000;

static double g_wpm = 20.0, g_rise = 5.0, g_gap = 7.0;
static char g_text[64] = "CQ DE REVENANT";

static std::uint64_t g_seed = 0;
static double g_baud = 1200.0;
static std::uint64_t g_symbols = 256;

// The FSK fields of the next spec (payload seed, baud, payload length).
void refsyn_set_fsk(std::uint64_t seed, double baud, std::uint64_t symbols) {
    g_seed = seed;
    g_baud = baud;
    g_symbols = symbols;
}

static double g_rolloff = 0.35;
static std::uint64_t g_span = 8;

// The PSK fields of the next spec (rolloff, pulse span; baud, count and seed
// are the FSK setter's).
void refsyn_set_psk(double rolloff, std::uint64_t span) {
    g_rolloff = rolloff;
    g_span = span;
}

// The CW fields of the next spec.
void refsyn_set_cw(double wpm, double rise_ms, double gap_dots, const char* text) {
    g_wpm = wpm;
    g_rise = rise_ms;
    g_gap = gap_dots;
    std::snprintf(g_text, sizeof g_text, "%s", text);
}

// The SSB fields of the next tone spec (second tone, audio passband).
void refsyn_set_ssb(std::int64_t tone2, std::int64_t low, std::int64_t high) {
    g_tone2 = tone2;
    g_low = low;
    g_high = high;
}

static siggen::ModulatorSpec tone_spec(int kind, std::int64_t rate, std::int64_t carrier, std::int64_t tone,
                                      std::int64_t deviation, double amplitude, double phase, double index) {
    siggen::ModulatorSpec spec;
    spec.kind = static_cast<siggen::Modulation>(kind);
    spec.ssb.tone_hz = tone;
    spec.ssb.tone2_hz = g_tone2;
    spec.ssb.audio_low_hz = g_low;
    spec.ssb.audio_high_hz = g_high;
    spec.psk.symbol_rate = g_baud;
    spec.psk.symbol_count = g_symbols;
    spec.psk.rolloff = g_rolloff;
    spec.psk.span_symbols = g_span;
    spec.fsk.symbol_rate = g_baud;
    spec.fsk.symbol_count = g_symbols;
    spec.fsk.deviation = deviation;
    spec.common.seed = g_seed;
    spec.cw.words_per_minute = g_wpm;
    spec.cw.rise_fall_ms = g_rise;
    spec.cw.message_gap_dots = g_gap;
    spec.cw.text = g_text;
    spec.common.rate = rate;
    spec.common.carrier_offset = carrier;
    spec.common.amplitude = amplitude;
    spec.common.initial_phase = phase;
    spec.am.modulation_index = index;
    spec.am.tone_hz = tone;
    spec.nfm.tone_hz = tone;
    spec.nfm.deviation = deviation;
    return spec;
}

// Modulator::accumulate of a tone AM (kind 1) or NFM (kind 2) emitter into
// `io` (count cf32, added to), emitter indices [first, first + count).
int refsyn_tone(int kind, std::int64_t rate, std::int64_t carrier, std::int64_t tone, std::int64_t deviation,
                double amplitude, double phase, double index, std::uint64_t first, std::uint64_t count, double gain,
                float* io) {
    auto m = siggen::Modulator::create(tone_spec(kind, rate, carrier, tone, deviation, amplitude, phase, index));
    if (!m) return -1;
    std::vector<std::complex<float>> buf(count);
    for (std::uint64_t i = 0; i < count; ++i) buf[i] = {io[2 * i], io[2 * i + 1]};
    m->accumulate(first, std::span<std::complex<float>>(buf), gain);
    for (std::uint64_t i = 0; i < count; ++i) {
        io[2 * i] = buf[i].real();
        io[2 * i + 1] = buf[i].imag();
    }
    return 0;
}

// Scene::render of noise plus one tone emitter placed by amplitude (gain 1)
// over emitter window [on, off).
int refsyn_scene_tone(std::uint64_t seed, std::int64_t rate, double noise_dbfs, int kind, std::int64_t carrier,
                      std::int64_t tone, std::int64_t deviation, double amplitude, double phase, double index,
                      std::uint64_t on, std::uint64_t off, std::uint64_t start, std::uint64_t count, float* out) {
    siggen::SceneSpec spec;
    spec.rate = rate;
    spec.seed = seed;
    spec.add_noise = true;
    spec.noise_power_full_band_dbfs = noise_dbfs;
    spec.duration_samples = start + count;
    spec.worker_threads = 1;
    siggen::EmitterPlacement e;
    e.modulator = tone_spec(kind, rate, carrier, tone, deviation, amplitude, phase, index);
    e.use_snr = false;
    e.start_sample = on;
    e.end_sample = off;
    spec.emitters.push_back(e);
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

// Scene::create of a random population over `palette` (siggen::Modulation
// values) and Scene::render of [start, start + count) into out (may be
// NULL); the truth rows as 8 doubles each: start, end (-1 = always on),
// carrier, modulation, mean power, SNR in the occupied band, extent low, high.
int refsyn_random_scene(std::uint64_t seed, std::int64_t rate, std::int64_t duration, double noise_dbfs,
                        std::uint32_t emitters, std::uint32_t bursts, std::int64_t span_lo, std::int64_t span_hi,
                        double snr_min, double snr_max, double min_s, double max_s, std::uint32_t npalette,
                        const int* palette, std::uint64_t start, std::uint64_t count, float* out, double* truth,
                        std::uint32_t truth_cap, std::uint32_t* truth_count) {
    siggen::SceneSpec spec;
    spec.rate = rate;
    spec.seed = seed;
    spec.duration_samples = duration;
    spec.add_noise = true;
    spec.noise_power_full_band_dbfs = noise_dbfs;
    spec.worker_threads = 1;
    spec.random.emitter_count = emitters;
    spec.random.bursts_per_emitter = bursts;
    spec.random.span_low_hz = span_lo;
    spec.random.span_high_hz = span_hi;
    spec.random.snr_in_occupied_bandwidth_db_min = snr_min;
    spec.random.snr_in_occupied_bandwidth_db_max = snr_max;
    spec.random.min_burst_seconds = min_s;
    spec.random.max_burst_seconds = max_s;
    for (std::uint32_t i = 0; i < npalette; ++i) spec.random.palette.push_back(static_cast<siggen::Modulation>(palette[i]));
    auto scene = siggen::Scene::create(spec);
    if (!scene) return -1;
    const auto& t = scene->truth();
    *truth_count = static_cast<std::uint32_t>(t.size());
    for (std::uint32_t i = 0; i < t.size() && i < truth_cap; ++i) {
        double* r = truth + 8 * i;
        r[0] = static_cast<double>(t[i].start_sample);
        r[1] = t[i].end_sample == siggen::kAlwaysOn ? -1.0 : static_cast<double>(t[i].end_sample);
        r[2] = static_cast<double>(t[i].carrier_offset_hz);
        r[3] = static_cast<double>(t[i].modulation);
        r[4] = t[i].mean_power;
        r[5] = t[i].snr_in_occupied_bandwidth_db;
        r[6] = static_cast<double>(t[i].extent.low_hz);
        r[7] = static_cast<double>(t[i].extent.high_hz);
    }
    if (out != nullptr && count > 0) {
        std::vector<std::complex<float>> buf(count);
        scene->render(start, std::span<std::complex<float>>(buf));
        for (std::uint64_t i = 0; i < count; ++i) {
            out[2 * i] = buf[i].real();
            out[2 * i + 1] = buf[i].imag();
        }
    }
    return 0;
}

// Modulator::accumulate of an AM, NFM, USB or LSB emitter modulated by
// supplied audio (ModulatorSpec::audio), SSB through a `taps`-tap Hilbert
// network over the [low, high] Hz audio passband.
int refsyn_audio_emitter(int kind, std::int64_t rate, std::int64_t carrier, std::int64_t deviation, double amplitude,
                         double phase, double index, const float* audio, std::uint64_t len, std::uint32_t taps,
                         std::int64_t low, std::int64_t high, std::uint64_t first, std::uint64_t count, double gain,
                         float* io) {
    siggen::ModulatorSpec spec = tone_spec(kind, rate, carrier, 1000, deviation, amplitude, phase, index);
    spec.audio.assign(audio, audio + len);
    spec.ssb.hilbert_taps = taps;
    spec.ssb.audio_low_hz = low;
    spec.ssb.audio_high_hz = high;
    auto m = siggen::Modulator::create(spec);
    if (!m) return -1;
    std::vector<std::complex<float>> buf(count);
    for (std::uint64_t i = 0; i < count; ++i) buf[i] = {io[2 * i], io[2 * i + 1]};
    m->accumulate(first, std::span<std::complex<float>>(buf), gain);
    for (std::uint64_t i = 0; i < count; ++i) {
        io[2 * i] = buf[i].real();
        io[2 * i + 1] = buf[i].imag();
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
