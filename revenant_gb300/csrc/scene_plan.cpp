// The scene synthesiser's random population (siggen::Scene::create,
// core/dsp/synth/wideband.cpp:375-482, with randomise_mode :124-177, the
// uniform helpers :62-104, level_for :206-235 and add_bursts :243-266) for
// every palette (all eight modulations are rendered). Every draw comes from
// std::mt19937_64 in the reference's order, so the layout (modes, carriers,
// levels, burst windows) is the reference's exactly; the bursts come back
// sorted by start, the order the scene adds them in.
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <limits>
#include <random>
#include <vector>

#include "revenant_gb300.h"
#include "scene.h"

namespace rv {
int32_t set_error_fmt(int32_t code, const char* fmt, ...);
int32_t clear_error();
}  // namespace rv

namespace {

using rv::set_error_fmt;

constexpr double kTwoPi = 6.283185307179586476925286766559;
constexpr double kMantissaStep = 1.0 / 9007199254740992.0;
constexpr uint64_t kLayoutDomain = 0x1a59017e55ce0d01ull;  // wideband.cpp:40

uint64_t derive_stream_seed(uint64_t master, uint64_t domain) {
    uint64_t z = master + domain * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

double uniform_unit(std::mt19937_64& g) { return (double)(g() >> 11) * kMantissaStep; }
double uniform_range(std::mt19937_64& g, double lo, double hi) { return lo + (hi - lo) * uniform_unit(g); }

// [0, bound) by rejection
uint64_t uniform_below(std::mt19937_64& g, uint64_t bound) {
    if (bound <= 1) return 0;
    const uint64_t buckets = std::numeric_limits<uint64_t>::max() / bound, ceiling = buckets * bound;
    uint64_t draw = g();
    while (draw >= ceiling) draw = g();
    return draw / buckets;
}

int64_t uniform_between(std::mt19937_64& g, int64_t lo, int64_t hi) {
    if (hi <= lo) return lo;
    return lo + (int64_t)uniform_below(g, (uint64_t)(hi - lo) + 1u);
}

template <class T, size_t N>
T pick(std::mt19937_64& g, const T (&choices)[N]) {
    return choices[uniform_below(g, N)];
}

double db_to_power(double db) { return std::pow(10.0, db * 0.1); }
double power_to_db(double p) { return 10.0 * std::log10(p); }

// modulators.cpp:261-310 extent_for, for the built modes; `baud` is FSK's
// symbol rate (the nominal one when placing, the realised one for the truth)
void extent(const rv_tone_emitter& e, int64_t& lo, int64_t& hi, double baud = 0.0) {
    int64_t half = 0;
    switch (e.modulation) {
        case RV_EMITTER_FSK2: half = e.deviation + (int64_t)std::llround(baud * 0.5); break;
        case RV_EMITTER_BPSK:
        case RV_EMITTER_QPSK: half = (int64_t)std::llround((1.0 + e.rolloff) * baud * 0.5); break;
        case RV_EMITTER_CW: half = (int64_t)std::llround(1.5 * (e.words_per_minute / 1.2)); break;
        case RV_EMITTER_AM: half = e.tone_hz; break;
        case RV_EMITTER_NFM: half = e.deviation + e.tone_hz; break;
        case RV_EMITTER_USB:
            lo = e.carrier_offset + e.audio_low_hz, hi = e.carrier_offset + e.audio_high_hz;
            return;
        default:  // LSB
            lo = e.carrier_offset - e.audio_high_hz, hi = e.carrier_offset - e.audio_low_hz;
            return;
    }
    lo = e.carrier_offset - half, hi = e.carrier_offset + half;
}

// Modulator::create's nominal_mean_power (modulators.cpp:675-803) for the
// built modes, amplitude 1
double nominal_power(const rv_tone_emitter& e) {
    const double power = e.amplitude * e.amplitude;
    switch (e.modulation) {
        case RV_EMITTER_CW: {
            const double rate = (double)e.rate;
            const std::vector<rv::CwElement> el =
                rv::cw_elements(e.text, 1.2 * rate / e.words_per_minute, e.message_gap_dots);
            const double ramp_samples = e.rise_fall_ms * 0.001 * rate;
            double keyed = 0.0;
            for (const rv::CwElement& x : el) {
                if (!x.keyed) continue;
                const double length = (double)(x.stop - x.start);
                const double ramp = std::min(ramp_samples, length * 0.5);
                keyed += length - 1.25 * ramp;
            }
            return power * keyed / (double)el.back().stop;
        }
        case RV_EMITTER_AM: return power * (1.0 + e.modulation_index * e.modulation_index * 0.5);
        case RV_EMITTER_NFM:
        case RV_EMITTER_FSK2:
        case RV_EMITTER_BPSK:
        case RV_EMITTER_QPSK: return power;
        default: return e.tone2_hz != 0 ? 0.5 * power : power;
    }
}

}  // namespace

extern "C" int32_t rv_scene_plan(const rv_scene_population* p, rv_scene_burst* out, uint32_t capacity,
                                 uint32_t* count) {
    if (p == nullptr || count == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_scene_plan: NULL argument");
    *count = 0;
    if (p->rate <= 0 || p->rate > 1000000000) return set_error_fmt(RV_ERR_INVALID, "rv_scene_plan: rate");
    if (!std::isfinite(p->noise_dbfs)) return set_error_fmt(RV_ERR_INVALID, "rv_scene_plan: noise floor must be finite");
    if (p->emitter_count == 0) return rv::clear_error();
    // wideband.cpp:379-393
    if (p->span_high_hz <= p->span_low_hz)
        return set_error_fmt(RV_ERR_INVALID, "rv_scene_plan: random population needs an increasing placement span");
    if (p->bursts_per_emitter == 0) return set_error_fmt(RV_ERR_INVALID, "rv_scene_plan: at least one burst per emitter");
    if (p->bursts_per_emitter > 1 && p->duration_samples == 0)
        return set_error_fmt(RV_ERR_INVALID, "rv_scene_plan: bursty emitters need a bounded scene");
    if (p->snr_max_db < p->snr_min_db) return set_error_fmt(RV_ERR_INVALID, "rv_scene_plan: SNR range is inverted");
    if (p->palette_count > 8) return set_error_fmt(RV_ERR_INVALID, "rv_scene_plan: palette of more than 8");
    std::vector<int32_t> palette(p->palette, p->palette + p->palette_count);
    if (palette.empty()) palette = {0, 1, 2, 3, 4, 5, 6, 7};  // all_modulations()
    for (int32_t m : palette)
        if (m < RV_EMITTER_CW || m > RV_EMITTER_QPSK)
            return set_error_fmt(RV_ERR_INVALID, "rv_scene_plan: modulation %d is not a siggen::Modulation", m);
    const int64_t window = p->duration_samples / (int64_t)p->bursts_per_emitter;
    if (p->bursts_per_emitter > 1 && window < 2)
        return set_error_fmt(RV_ERR_INVALID, "rv_scene_plan: the bursts do not fit in the scene");
    const double noise_power = db_to_power(p->noise_dbfs);
    std::mt19937_64 g(derive_stream_seed(p->seed, kLayoutDomain));
    std::vector<rv_scene_burst> bursts;
    for (uint32_t slot = 0; slot < p->emitter_count; ++slot) {
        rv_tone_emitter e;
        memset(&e, 0, sizeof e);
        e.modulation = palette[uniform_below(g, palette.size())];
        e.rate = p->rate;
        e.amplitude = 1.0;
        e.initial_phase = uniform_range(g, 0.0, kTwoPi);
        const uint64_t payload_seed = g();
        // ModulatorSpec defaults (modulators.h), then randomise_mode
        e.modulation_index = 0.8, e.tone_hz = 1000, e.deviation = 5000;
        e.audio_low_hz = 300, e.audio_high_hz = 3000;
        e.words_per_minute = 20.0, e.rise_fall_ms = 5.0, e.message_gap_dots = 7.0;
        e.symbol_rate = 1200.0, e.symbol_count = 256, e.rolloff = 0.35, e.span_symbols = 8;
        e.seed = payload_seed;
        strcpy(e.text, "CQ DE REVENANT");
        switch (e.modulation) {
            case RV_EMITTER_CW: {
                static const int kWpm[] = {12, 18, 20, 25, 30};
                e.words_per_minute = (double)pick(g, kWpm);
                e.rise_fall_ms = 5.0;
                break;
            }
            case RV_EMITTER_AM: {
                e.modulation_index = uniform_range(g, 0.3, 0.9);
                static const int64_t kTone[] = {400, 1000, 1500, 2500};
                e.tone_hz = pick(g, kTone);
                break;
            }
            case RV_EMITTER_NFM: {
                static const int64_t kDev[] = {2500, 5000}, kTone[] = {400, 1000, 1500};
                e.deviation = pick(g, kDev);
                e.tone_hz = pick(g, kTone);
                break;
            }
            case RV_EMITTER_FSK2: {
                static const int64_t kBaud[] = {1200, 2400, 4800, 9600};
                static const double kIndex[] = {0.5, 1.0, 2.0};
                const int64_t baud = pick(g, kBaud);
                e.symbol_rate = (double)baud;
                const double index = pick(g, kIndex);
                e.deviation = (int64_t)std::llround(0.5 * index * (double)baud);
                e.symbol_count = 256;
                break;
            }
            case RV_EMITTER_BPSK:
            case RV_EMITTER_QPSK: {
                static const int64_t kBaud[] = {1200, 2400, 4800, 9600, 19200};
                static const double kRolloff[] = {0.2, 0.35, 0.5};
                e.symbol_rate = (double)pick(g, kBaud);
                e.rolloff = pick(g, kRolloff);
                e.symbol_count = 256;
                break;
            }
            default: {
                static const int64_t kTone[] = {700, 1000, 1500, 2200};
                e.tone_hz = pick(g, kTone);
                e.tone2_hz = uniform_unit(g) < 0.25 ? 1900 : 0;
                if (e.tone2_hz == e.tone_hz) e.tone2_hz = 0;
                break;
            }
        }
        // placed by the occupied band measured with the carrier at zero
        int64_t rlo, rhi;
        extent(e, rlo, rhi, e.symbol_rate);
        const int64_t nyquist = p->rate / 2;
        const int64_t lowest = std::max(p->span_low_hz, -nyquist) - rlo;
        const int64_t highest = std::min(p->span_high_hz, nyquist) - rhi;
        if (lowest > highest)
            return set_error_fmt(RV_ERR_INVALID, "rv_scene_plan: an emitter %lld Hz wide does not fit the span",
                                 (long long)(rhi - rlo));
        e.carrier_offset = uniform_between(g, lowest, highest);
        std::vector<std::pair<int64_t, int64_t>> windows;
        const double snr = uniform_range(g, p->snr_min_db, p->snr_max_db);
        if (p->bursts_per_emitter == 1) {
            windows.emplace_back(0, p->duration_samples == 0 ? std::numeric_limits<int64_t>::max() : p->duration_samples);
        } else {
            for (uint32_t b = 0; b < p->bursts_per_emitter; ++b) {
                const double seconds = uniform_range(g, p->min_burst_seconds, p->max_burst_seconds);
                int64_t length = std::max<int64_t>(1, (int64_t)std::llround(seconds * (double)p->rate));
                length = std::min(length, std::max<int64_t>(1, window * 9 / 10));
                const int64_t jitter = (int64_t)uniform_below(g, (uint64_t)(window - length) + 1u);
                const int64_t start = window * (int64_t)b + jitter;
                windows.emplace_back(start, start + length);
            }
        }
        // level_for with use_snr (wideband.cpp:206-235)
        int64_t lo, hi;
        double realised = 0.0;
        if (e.modulation == RV_EMITTER_FSK2 || e.modulation == RV_EMITTER_BPSK ||
            e.modulation == RV_EMITTER_QPSK) {  // the modulator's extent uses the symbol clock's rate
            rv::SymbolClock clock;
            if (!rv::build_symbol_clock(e.symbol_count, e.rate, e.symbol_rate, clock))
                return set_error_fmt(RV_ERR_INVALID, "rv_scene_plan: FSK symbol clock unusable");
            realised = clock.effective_rate(e.rate);
        }
        extent(e, lo, hi, realised);
        const double bandwidth = std::max(1.0, (double)(hi - lo));
        const double in_band = noise_power * bandwidth / (double)p->rate;
        if (noise_power <= 0.0) return set_error_fmt(RV_ERR_INVALID, "rv_scene_plan: SNR placement needs a noise floor");
        const double nominal = nominal_power(e);
        const double power = nominal > 0.0 ? in_band * db_to_power(snr) : 0.0;
        const double gain = nominal > 0.0 ? std::sqrt(in_band * db_to_power(snr) / nominal) : 0.0;
        for (const auto& w : windows) {  // add_bursts: clamped to the scene
            int64_t start = w.first, end = w.second;
            if (p->duration_samples > 0) {
                if (start >= p->duration_samples) continue;
                end = std::min(end, p->duration_samples);
            }
            if (end <= start) continue;
            rv_scene_burst b;
            memset(&b, 0, sizeof b);
            b.emitter = e;
            b.start = (uint64_t)start;
            b.end = end == std::numeric_limits<int64_t>::max() ? UINT64_MAX : (uint64_t)end;
            b.gain = gain;
            b.mean_power = power;
            b.snr_in_occupied_bandwidth_db = in_band > 0.0 ? power_to_db(power / in_band) : 0.0;
            b.extent_low_hz = lo;
            b.extent_high_hz = hi;
            b.payload_seed = payload_seed;
            bursts.push_back(b);
        }
    }
    std::stable_sort(bursts.begin(), bursts.end(),
                     [](const rv_scene_burst& a, const rv_scene_burst& b) { return a.start < b.start; });
    *count = (uint32_t)bursts.size();
    if (out)
        for (uint32_t i = 0; i < *count && i < capacity; ++i) out[i] = bursts[i];
    return rv::clear_error();
}
