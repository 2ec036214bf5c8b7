// Host planning for the receive chain, restated in this project's C++.
//
// Tables the kernels read are designed on the host in double and rounded to
// float once, as the reference does (core/dsp/pfb.h:113-162): the prototype
// (core/dsp/pfb_design.cpp:381-513), the twiddle circle (:515-590), the NCO
// circle (core/dsp/vrx_reference.cpp:364), the spectrum window and channel
// correction (core/dsp/spectrum_reference.cpp:195-280) and every per-receiver
// table of plan_vrx (core/dsp/vrx_reference.cpp:1808-2662). The formulas are
// the published ones (Kaiser-windowed sinc, four-term Blackman-Harris, one-pole
// de-emphasis) evaluated with the same association order as the reference, so
// the float tables come out identical bit for bit; tests/test_planner.py
// checks that against the reference's own planner.
//
// Receiver placement and rate planning is integer arithmetic on exact
// rationals (core/engine/vrx_place.cpp:199-330, vrx_reference.cpp:1201-1700).
#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <complex>
#include <limits>
#include <numeric>
#include <string>
#include <vector>

#include "revenant_gb300.h"

namespace rv {
int32_t set_error_fmt(int32_t code, const char* fmt, ...);
int32_t clear_error();
int32_t validate_grid(const rv_grid_params* g);
int32_t validate_grid_upto(const rv_grid_params* g, uint32_t max_channels);
int32_t validate_fine(const rv_vrx_fine_config* c, const rv_vrx_fine_params* p);
int32_t validate_demod(const rv_vrx_demod_config* c, const rv_vrx_demod_params* p);
int32_t validate_carrier(const rv_vrx_carrier_config* c, const rv_vrx_carrier_params* p);
uint32_t demod_fine_history(const rv_vrx_demod_config* c);
bool is_complex_mode(uint32_t m);
}  // namespace rv

namespace {

using rv::set_error_fmt;

constexpr double kPi = 3.14159265358979323846264338327950288;
constexpr double kTwoPi = 2.0 * kPi;

// ---- shared design primitives ------------------------------------------

// Modified Bessel function I0 by its power series, stopped at 1e-18 relative.
double bessel_i0(double x) {
    const double quarter_square = 0.25 * x * x;
    double term = 1.0, sum = 1.0;
    for (int k = 1; k < 256; ++k) {
        term *= quarter_square / (static_cast<double>(k) * static_cast<double>(k));
        sum += term;
        if (term < 1e-18 * sum) break;
    }
    return sum;
}

// Kaiser's empirical beta for a stopband attenuation in dB.
double kaiser_beta(double attenuation_db) {
    if (attenuation_db > 50.0) return 0.1102 * (attenuation_db - 8.7);
    if (attenuation_db >= 21.0) {
        const double excess = attenuation_db - 21.0;
        return 0.5842 * pow(excess, 0.4) + 0.07886 * excess;
    }
    return 0.0;
}

// Kaiser's length estimate N-1 = (A - 8) / (2.285 * dw), plus one.
uint32_t kaiser_taps_for(double attenuation_db, double transition_fraction) {
    if (!(transition_fraction > 0.0)) return 0;
    const double transition_radians = kTwoPi * transition_fraction;
    const double order = (attenuation_db - 8.0) / (2.285 * transition_radians);
    if (!(order > 0.0)) return 2;
    return static_cast<uint32_t>(ceil(order)) + 1u;
}

double attenuation_reachable(uint32_t taps, double transition_fraction) {
    if (taps < 2 || !(transition_fraction > 0.0)) return 0.0;
    const double transition_radians = kTwoPi * transition_fraction;
    return 2.285 * transition_radians * static_cast<double>(taps - 1u) + 8.0;
}

double sinc_pi(double z) {
    if (z == 0.0) return 1.0;
    const double scaled = kPi * z;
    return sin(scaled) / scaled;
}

double kaiser_window(size_t index, size_t length, double beta, double i0_beta) {
    if (length < 2) return 1.0;
    const double position = 2.0 * static_cast<double>(index) / static_cast<double>(length - 1) - 1.0;
    const double inner = std::max(0.0, 1.0 - position * position);
    return bessel_i0(beta * sqrt(inner)) / i0_beta;
}

int64_t iabs(int64_t v) { return v < 0 ? -v : v; }

void reduce_rational(int64_t& num, int64_t& den) {
    if (den < 0) {
        num = -num;
        den = -den;
    }
    const int64_t g = std::gcd(num, den);
    if (g > 1) {
        num /= g;
        den /= g;
    }
}

float to_float_unsigned_zero(double v) {
    const float f = static_cast<float>(v);
    return f == 0.0f ? 0.0f : f;
}

// In-place radix-2 FFT in double, for measuring a designed prototype's
// stopband (a diagnostic, not a kernel table).
void fft_double(std::vector<std::complex<double>>& data) {
    const size_t n = data.size();
    if (n < 2) return;
    for (size_t i = 1, j = 0; i < n; ++i) {
        size_t bit = n >> 1;
        for (; (j & bit) != 0; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) std::swap(data[i], data[j]);
    }
    std::vector<std::complex<double>> w(n / 2);
    for (size_t k = 0; k < w.size(); ++k) {
        const double angle = -2.0 * kPi * static_cast<double>(k) / static_cast<double>(n);
        w[k] = std::complex<double>(cos(angle), sin(angle));
    }
    for (size_t span = 2; span <= n; span <<= 1) {
        const size_t half = span / 2, stride = n / span;
        for (size_t base = 0; base < n; base += span) {
            for (size_t k = 0; k < half; ++k) {
                const std::complex<double> upper = data[base + k + half] * w[k * stride];
                const std::complex<double> lower = data[base + k];
                data[base + k] = lower + upper;
                data[base + k + half] = lower - upper;
            }
        }
    }
}

double measure_stopband_db(const std::vector<float>& taps, uint32_t channels) {
    if (taps.empty() || channels == 0) return 0.0;
    const size_t kMaxPoints = size_t{1} << 21;
    size_t points = 1;
    while (points < taps.size()) points <<= 1;
    for (int d = 0; d < 4 && points < kMaxPoints; ++d) points <<= 1;
    std::vector<std::complex<double>> spectrum(points, std::complex<double>(0.0, 0.0));
    for (size_t n = 0; n < taps.size(); ++n) spectrum[n] = std::complex<double>(static_cast<double>(taps[n]), 0.0);
    fft_double(spectrum);
    const double dc = std::abs(spectrum[0]);
    if (!(dc > 0.0)) return 0.0;
    const double stop_edge = 0.75 / static_cast<double>(channels);
    const size_t first = static_cast<size_t>(ceil(stop_edge * static_cast<double>(points)));
    const size_t last = points / 2;
    if (first > last) return 0.0;
    double peak = 0.0;
    for (size_t i = first; i <= last; ++i) peak = std::max(peak, std::abs(spectrum[i]));
    if (!(peak > 0.0)) return -600.0;
    return std::max(-600.0, 20.0 * log10(peak / dc));
}

// ---- prototype, twiddles, NCO, spectrum window ---------------------------

int32_t design_prototype(const rv_grid_params& g, double attenuation_db, std::vector<float>& taps,
                         double* stopband, uint64_t* group_delay, uint32_t max_channels = 2048) {
    if (int32_t st = rv::validate_grid_upto(&g, max_channels)) return st;
    if (!isfinite(attenuation_db) || attenuation_db < 0.0 || attenuation_db > 300.0)
        return set_error_fmt(RV_ERR_INVALID, "design_prototype: stopband target %g dB is outside [0, 300]", attenuation_db);
    const uint32_t M = g.channels;
    const uint32_t L = g.taps_per_branch - 1u;
    const size_t design_length = static_cast<size_t>(M) * L;
    const size_t used = design_length + 1;
    const double reachable = 2.285 * kPi * static_cast<double>(L) + 8.0;
    const double design_db = std::min(attenuation_db, reachable);
    const double beta = kaiser_beta(design_db);
    const double i0_beta = bessel_i0(beta);
    if (!(i0_beta > 0.0) || !isfinite(i0_beta))
        return set_error_fmt(RV_ERR_INVALID, "design_prototype: non-finite Kaiser normalisation");
    const double centre = 0.5 * static_cast<double>(design_length);
    const double inverse_channels = 1.0 / static_cast<double>(M);
    std::vector<double> work(used, 0.0);
    double sum = 0.0;
    for (size_t n = 0; n < used; ++n) {
        const double offset = static_cast<double>(n) - centre;
        const double position = (centre > 0.0) ? offset / centre : 0.0;
        const double radicand = std::max(0.0, 1.0 - position * position);
        const double window = bessel_i0(beta * sqrt(radicand)) / i0_beta;
        const double angle = kPi * offset * inverse_channels;
        const double sinc = (offset == 0.0) ? 1.0 : sin(angle) / angle;
        work[n] = inverse_channels * sinc * window;
        sum += work[n];
    }
    if (!(sum > 0.0) || !isfinite(sum))
        return set_error_fmt(RV_ERR_INVALID, "design_prototype: taps sum to %g", sum);
    taps.assign(static_cast<size_t>(M) * g.taps_per_branch, 0.0f);
    for (size_t n = 0; n < used; ++n) taps[n] = static_cast<float>(work[n] / sum);
    if (group_delay) *group_delay = design_length / 2;
    if (stopband) *stopband = measure_stopband_db(taps, M);
    return RV_OK;
}

int32_t build_twiddles(uint32_t M, std::vector<rv_cf32>& out, uint32_t cap = 2048) {
    if (M == 0 || (M & (M - 1)) != 0) return set_error_fmt(RV_ERR_INVALID, "build_twiddles: %u is not a power of two", M);
    if (M > cap) return set_error_fmt(RV_ERR_INVALID, "build_twiddles: %u exceeds %u", M, cap);
    const uint32_t half = M / 2, quarter = M / 4, octant = M / 8;
    std::vector<double> oc(octant + 1, 0.0), os(octant + 1, 0.0);
    for (uint32_t i = 0; i <= octant; ++i) {
        const double a = 2.0 * kPi * static_cast<double>(i) / static_cast<double>(M);
        oc[i] = cos(a);
        os[i] = sin(a);
    }
    std::vector<double> re(M, 0.0), im(M, 0.0);
    for (uint32_t j = 0; j <= quarter && j < M; ++j) {
        if (j <= octant) {
            re[j] = oc[j];
            im[j] = -os[j];
        } else {
            re[j] = os[quarter - j];
            im[j] = -oc[quarter - j];
        }
    }
    for (uint32_t j = quarter + 1; j <= half; ++j) {
        re[j] = -re[half - j];
        im[j] = im[half - j];
    }
    for (uint32_t j = half + 1; j < M; ++j) {
        re[j] = re[M - j];
        im[j] = -im[M - j];
    }
    out.resize(M);
    for (uint32_t j = 0; j < M; ++j) out[j] = rv_cf32{to_float_unsigned_zero(re[j]), to_float_unsigned_zero(im[j])};
    return RV_OK;
}

int32_t build_nco_table(uint32_t log2, std::vector<rv_cf32>& out) {
    if (log2 > 24) return set_error_fmt(RV_ERR_INVALID, "build_nco_table: log2 size %u exceeds 24", log2);
    const uint32_t size = 1u << log2;
    out.assign(size, rv_cf32{0.0f, 0.0f});
    if (size == 1) {
        out[0] = rv_cf32{1.0f, 0.0f};
        return RV_OK;
    }
    const uint32_t quarter = size / 4u, octant = size / 8u;
    std::vector<double> c(size, 0.0), s(size, 0.0);
    for (uint32_t i = 0; i <= octant; ++i) {
        const double a = kTwoPi * static_cast<double>(i) / static_cast<double>(size);
        c[i] = cos(a);
        s[i] = sin(a);
    }
    for (uint32_t i = octant + 1u; i <= quarter; ++i) {
        c[i] = s[quarter - i];
        s[i] = c[quarter - i];
    }
    for (uint32_t i = quarter + 1u; i < size; ++i) {
        c[i] = -s[i - quarter];
        s[i] = c[i - quarter];
    }
    for (uint32_t i = 0; i < size; ++i)
        out[i] = rv_cf32{(c[i] == 0.0) ? 0.0f : static_cast<float>(c[i]), (s[i] == 0.0) ? 0.0f : static_cast<float>(-s[i])};
    return RV_OK;
}

// |H(x)|/|H(0)| of a prototype at x = numerator/denominator channel spacings,
// the phase reduced in integers before the transcendental.
double prototype_magnitude(const std::vector<float>& taps, uint32_t channels, int64_t num, int64_t den) {
    double re = 0.0, im = 0.0, direct = 0.0;
    const double scale = static_cast<double>(den) * static_cast<double>(channels);
    for (size_t n = 0; n < taps.size(); ++n) {
        const double tap = static_cast<double>(taps[n]);
        direct += tap;
        if (tap == 0.0) continue;
        const int64_t span = den * static_cast<int64_t>(channels);
        int64_t reduced = (num * static_cast<int64_t>(n)) % span;
        if (reduced < 0) reduced += span;
        const double angle = -kTwoPi * static_cast<double>(reduced) / scale;
        re += tap * cos(angle);
        im += tap * sin(angle);
    }
    const double magnitude = sqrt(re * re + im * im);
    const double reference = fabs(direct);
    return (reference > 0.0) ? magnitude / reference : 0.0;
}

int32_t build_spectrum_window(uint32_t size, uint32_t taps_per_branch, double attenuation_db,
                              std::vector<float>& out) {
    if (size < 4 || (size & (size - 1)) != 0)
        return set_error_fmt(RV_ERR_INVALID, "build_spectrum_window: %u is not a power of two of at least 4", size);
    const double count = static_cast<double>(size);
    std::vector<double> w(size, 0.0);
    double sum = 0.0;
    for (uint32_t n = 0; n < size; ++n) {
        const double phase = kTwoPi * static_cast<double>(n) / count;
        const double value = 0.35875 - 0.48829 * cos(phase) + 0.14128 * cos(2.0 * phase) - 0.01168 * cos(3.0 * phase);
        w[n] = value;
        sum += value;
    }
    if (!(sum > 0.0)) return set_error_fmt(RV_ERR_INVALID, "build_spectrum_window: window sums to %g", sum);
    out.assign(size + size / 2, 0.0f);
    for (uint32_t n = 0; n < size; ++n) out[n] = static_cast<float>(w[n] / sum);
    // The channel-shape correction is designed against the 64-channel
    // prototype at the same taps per branch (the shipped grid).
    rv_grid_params cg{64u, taps_per_branch, 32u};
    std::vector<float> proto;
    if (int32_t st = design_prototype(cg, attenuation_db, proto, nullptr, nullptr)) return st;
    const double ceiling = pow(10.0, static_cast<double>(12.0f) / 10.0);
    for (uint32_t bin = 0; bin < size / 2; ++bin) {
        const int64_t num = 2 * static_cast<int64_t>(bin) - static_cast<int64_t>(size) / 2;
        const double response = prototype_magnitude(proto, 64u, num, static_cast<int64_t>(size));
        const double gain = 1.0 / (response * response);
        const double limited = (gain > ceiling || !isfinite(gain)) ? ceiling : gain;
        out[size + bin] = static_cast<float>(limited);
    }
    return RV_OK;
}

// ---- exact NCO phase (core/dsp/vrx_reference.cpp:308-362) -----------------

uint64_t turn_fixed64(int64_t numerator, int64_t denominator) {
    if (denominator <= 0 || numerator < 0 || numerator >= denominator) return 0;
    int64_t rem = numerator;
    uint64_t q = 0;
    for (int step = 0; step < 4; ++step) {
        rem <<= 16;
        q = (q << 16) | static_cast<uint64_t>(rem / denominator);
        rem %= denominator;
    }
    if (2 * rem >= denominator) ++q;
    return q;
}

int32_t nco_delta(int64_t hz_num, int64_t hz_den, int64_t rate, uint64_t* out) {
    if (hz_den == 0) return set_error_fmt(RV_ERR_INVALID, "nco_delta: frequency denominator is zero");
    if (rate <= 0) return set_error_fmt(RV_ERR_INVALID, "nco_delta: rate must be positive");
    int64_t num = hz_num, den = hz_den;
    reduce_rational(num, den);
    const int64_t period = den * rate;
    if (period <= 0 || period > (int64_t{1} << 31))
        return set_error_fmt(RV_ERR_INVALID, "nco_delta: reduced period %lld exceeds 2^31", (long long)period);
    int64_t reduced = num % period;
    if (reduced < 0) reduced += period;
    *out = turn_fixed64(reduced, period);
    return RV_OK;
}

// ---- passbands and rates (core/dsp/vrx_reference.cpp:1201-1760) ----------

struct Band {
    int64_t low = 0, high = 0;
    int64_t width() const { return high - low; }
    int64_t reach_from(int64_t o) const {
        const int64_t below = o - low, above = high - o;
        return below > above ? below : above;
    }
    bool operator!=(const Band& b) const { return low != b.low || high != b.high; }
};

Band default_passband(uint32_t mode) {
    switch (mode) {
        case RV_DEMOD_RAW: return {-6000, 6000};
        case RV_DEMOD_AM:
        case RV_DEMOD_SAM: return {-5000, 5000};
        case RV_DEMOD_NFM: return {-8000, 8000};
        case RV_DEMOD_WFM: return {-100000, 100000};
        case RV_DEMOD_USB: return {300, 2700};
        case RV_DEMOD_LSB: return {-2700, -300};
        case RV_DEMOD_DSB: return {-3000, 3000};
        case RV_DEMOD_CW: return {-600, 600};
        case RV_DEMOD_P25P1: return {-6250, 6250};
        case RV_DEMOD_DSTAR: return {-3000, 3000};
        case RV_DEMOD_TETRA: return {-12500, 12500};
        case RV_DEMOD_DMR: return {-6250, 6250};
    }
    return {};
}

int32_t resolve_passband(const rv_vrx_request& r, Band* out) {
    if (r.passband_low != 0 || r.passband_high != 0) {
        if (r.passband_low >= r.passband_high)
            return set_error_fmt(RV_ERR_INVALID, "resolve_passband: the passband runs from %lld Hz to %lld Hz, which is empty or inverted",
                                 (long long)r.passband_low, (long long)r.passband_high);
        *out = {r.passband_low, r.passband_high};
        return RV_OK;
    }
    if (r.bandwidth < 0) return set_error_fmt(RV_ERR_INVALID, "resolve_passband: bandwidth cannot be negative");
    if (r.bandwidth == 0) {
        const Band fallback = default_passband(r.demod);
        if (fallback.width() <= 0) return set_error_fmt(RV_ERR_INVALID, "resolve_passband: no default passband for mode %u", r.demod);
        *out = fallback;
        return RV_OK;
    }
    if (r.demod > 12) return set_error_fmt(RV_ERR_INVALID, "resolve_passband: mode %u is not a demodulator", r.demod);
    const int64_t half = r.bandwidth / 2;
    if (r.demod == RV_DEMOD_USB) *out = {0, r.bandwidth};
    else if (r.demod == RV_DEMOD_LSB) *out = {-r.bandwidth, 0};
    else *out = {-half, half};
    return RV_OK;
}

int64_t max_channel_bandwidth(const rv_vrx_placement& p) {
    if (p.channel_rate <= 0 || p.residual_denominator <= 0) return 0;
    const int64_t scaled = p.channel_rate * p.residual_denominator - 2 * iabs(p.residual_numerator);
    if (scaled <= 0) return 0;
    return scaled / p.residual_denominator;
}

Band clamp_to_channel(const rv_vrx_placement& p, Band b) {
    const int64_t widest = max_channel_bandwidth(p);
    if (widest <= 0) return {};
    const int64_t limit = widest / 2;
    return {std::clamp(b.low, -limit, limit), std::clamp(b.high, -limit, limit)};
}

int32_t channel_carries(const rv_vrx_placement& p, Band b) {
    const int64_t widest = max_channel_bandwidth(p);
    if (widest <= 0)
        return set_error_fmt(RV_ERR_INVALID, "one grid channel can carry nothing for a receiver placed here: the receiver is at least half a channel from the channel's centre");
    if (clamp_to_channel(p, b).width() > 0) return RV_OK;
    return set_error_fmt(RV_ERR_INVALID, "a passband of %lld to %lld Hz has nothing inside the +/-%lld Hz one grid channel can carry here",
                         (long long)b.low, (long long)b.high, (long long)(widest / 2));
}

Band mix_frame(Band b, uint32_t mode, int64_t pitch) {
    if (mode != RV_DEMOD_CW) return b;
    return {b.low + pitch, b.high + pitch};
}

int64_t minimum_demod_rate(uint32_t mode, Band b) {
    const int64_t width = b.width();
    if (width <= 0) return 0;
    const int64_t shape_floor = (3 * width + 1) / 2;
    const int64_t floor_rate = std::max(shape_floor, 2 * b.reach_from(0));
    switch (mode) {
        case RV_DEMOD_AM: return std::max(floor_rate, 2 * width);
        case RV_DEMOD_P25P1:
        case RV_DEMOD_DSTAR:
        case RV_DEMOD_DMR: return std::max<int64_t>(floor_rate, 9600);
        case RV_DEMOD_TETRA: return std::max<int64_t>(floor_rate, 36000);
        default: return floor_rate;
    }
}

int64_t complex_tap_rate_step(uint32_t mode) {
    switch (mode) {
        case RV_DEMOD_P25P1:
        case RV_DEMOD_DSTAR:
        case RV_DEMOD_DMR: return 48000;
        case RV_DEMOD_TETRA: return 72000;
        default: return 0;
    }
}

int64_t fm_deviation(uint32_t mode, int64_t bandwidth) {
    if (bandwidth <= 0) return 0;
    if (mode == RV_DEMOD_NFM) return std::max<int64_t>(1, bandwidth / 5);
    if (mode == RV_DEMOD_WFM) return std::max<int64_t>(1, (3 * bandwidth) / 8);
    return 0;
}

float vrx_demod_gain(uint32_t mode, int64_t demod_rate, int64_t deviation) {
    if (mode != RV_DEMOD_NFM && mode != RV_DEMOD_WFM) return 1.0f;
    if (deviation <= 0 || demod_rate <= 0) return 1.0f;
    return static_cast<float>(static_cast<double>(demod_rate) / (kTwoPi * static_cast<double>(deviation)));
}

uint32_t carrier_power(uint32_t mode) {
    if (mode == RV_DEMOD_SAM) return 1u;
    if (mode == RV_DEMOD_DSB) return 2u;
    return 0u;
}

// ---- per-receiver tables (core/dsp/vrx_reference.cpp:1808-2242) ----------

int32_t design_fine_taps(const rv_vrx_fine_config& c, int64_t channel_rate, int64_t half_width,
                         int64_t centre_num, int64_t centre_den, double attenuation_db,
                         std::vector<rv_cf32>& table) {
    if (c.taps < 2 || c.taps > 256) return set_error_fmt(RV_ERR_INVALID, "design_fine_taps: %u taps is outside [2, 256]", c.taps);
    if (c.phases < 1 || c.phases > 4096) return set_error_fmt(RV_ERR_INVALID, "design_fine_taps: %u phases", c.phases);
    if (channel_rate <= 0) return set_error_fmt(RV_ERR_INVALID, "design_fine_taps: channel rate must be positive");
    if (half_width <= 0 || 2 * half_width >= channel_rate)
        return set_error_fmt(RV_ERR_INVALID, "design_fine_taps: half-width %lld Hz is outside (0, %lld)", (long long)half_width, (long long)(channel_rate / 2));
    if (centre_den == 0) return set_error_fmt(RV_ERR_INVALID, "design_fine_taps: filter centre denominator is zero");
    if (!isfinite(attenuation_db) || attenuation_db < 0.0 || attenuation_db > 300.0)
        return set_error_fmt(RV_ERR_INVALID, "design_fine_taps: stopband target outside [0, 300]");
    const size_t phases = c.phases, taps = c.taps, length = phases * taps;
    const double centre = (static_cast<double>(length) - 1.0) / 2.0;
    const double cutoff = static_cast<double>(half_width) / static_cast<double>(channel_rate);
    const double beta = kaiser_beta(attenuation_db);
    const double i0_beta = bessel_i0(beta);
    std::vector<double> proto(length, 0.0);
    for (size_t i = 0; i < length; ++i) {
        const double position = (static_cast<double>(i) - centre) / static_cast<double>(phases);
        const double window = kaiser_window(i, length, beta, i0_beta);
        proto[i] = 2.0 * cutoff * sinc_pi(2.0 * cutoff * position) * window;
    }
    for (size_t p = 0; p < phases; ++p) {
        double sum = 0.0;
        for (size_t k = 0; k < taps; ++k) sum += proto[p + k * phases];
        if (fabs(sum) < 1e-12) continue;
        for (size_t k = 0; k < taps; ++k) proto[p + k * phases] /= sum;
    }
    table.assign(length + 1, rv_cf32{0.0f, 0.0f});
    const int64_t period = 2 * iabs(centre_den) * static_cast<int64_t>(phases) * channel_rate;
    const int64_t numerator = (centre_den < 0) ? -centre_num : centre_num;
    for (size_t i = 0; i < length; ++i) {
        const int64_t twice_offset = 2 * static_cast<int64_t>(i) - (static_cast<int64_t>(length) - 1);
        int64_t turns = (numerator * twice_offset) % period;
        if (turns < 0) turns += period;
        const double angle = kTwoPi * static_cast<double>(turns) / static_cast<double>(period);
        table[i] = rv_cf32{static_cast<float>(proto[i] * cos(angle)), static_cast<float>(proto[i] * sin(angle))};
    }
    return RV_OK;
}

int32_t design_audio_taps(uint32_t taps, int64_t demod_rate, int64_t audio_rate, double attenuation_db,
                          double cutoff_hz, std::vector<float>& out) {
    if (taps == 0 || taps > 4096) return set_error_fmt(RV_ERR_INVALID, "design_audio_taps: %u taps", taps);
    if (demod_rate <= 0 || audio_rate <= 0) return set_error_fmt(RV_ERR_INVALID, "design_audio_taps: rates must be positive");
    if (audio_rate > demod_rate) return set_error_fmt(RV_ERR_INVALID, "design_audio_taps: audio rate above the demodulation rate");
    if ((cutoff_hz < 0.0 || cutoff_hz >= 0.5 * static_cast<double>(audio_rate)) && cutoff_hz != 0.0)
        return set_error_fmt(RV_ERR_INVALID, "design_audio_taps: cutoff %g Hz outside (0, %g)", cutoff_hz, 0.5 * static_cast<double>(audio_rate));
    const double cutoff = (cutoff_hz > 0.0) ? cutoff_hz / static_cast<double>(demod_rate)
                                            : 0.45 * static_cast<double>(audio_rate) / static_cast<double>(demod_rate);
    const double centre = (static_cast<double>(taps) - 1.0) / 2.0;
    const double beta = kaiser_beta(attenuation_db);
    const double i0_beta = bessel_i0(beta);
    std::vector<double> d(taps, 0.0);
    double sum = 0.0;
    for (uint32_t i = 0; i < taps; ++i) {
        const double position = static_cast<double>(i) - centre;
        const double window = kaiser_window(i, taps, beta, i0_beta);
        d[i] = 2.0 * cutoff * sinc_pi(2.0 * cutoff * position) * window;
        sum += d[i];
    }
    const double scale = (fabs(sum) < 1e-12) ? 1.0 : 1.0 / sum;
    out.assign(taps, 0.0f);
    for (uint32_t i = 0; i < taps; ++i) out[i] = static_cast<float>(d[i] * scale);
    return RV_OK;
}

std::vector<float> design_dc_weights(uint32_t taps) {
    if (taps <= 1) return std::vector<float>{1.0f};
    std::vector<double> w(taps, 0.0);
    double sum = 0.0;
    for (uint32_t i = 0; i < taps; ++i) {
        const double phase = kTwoPi * static_cast<double>(i + 1u) / static_cast<double>(taps + 1u);
        w[i] = 0.5 - 0.5 * cos(phase);
        sum += w[i];
    }
    const double scale = (sum < 1e-12) ? 1.0 : 1.0 / sum;
    std::vector<float> out(taps, 0.0f);
    for (uint32_t i = 0; i < taps; ++i) out[i] = static_cast<float>(w[i] * scale);
    return out;
}

// De-emphasis curves (engine::Deemphasis): 0 default, 1 none, 2 75us, 3 50us.
double deemphasis_seconds(uint32_t curve) {
    if (curve == 2) return 75.0e-6;
    if (curve == 3) return 50.0e-6;
    return 0.0;
}

constexpr int64_t kCompositeAudioRateHz = 114000;

uint32_t resolve_deemphasis(uint32_t mode, uint32_t requested, int64_t audio_rate) {
    if (requested != 0) return rv::is_complex_mode(mode) ? 1u : requested;
    if (mode == RV_DEMOD_WFM) return (audio_rate >= kCompositeAudioRateHz) ? 1u : 2u;
    return 1u;
}

bool resolve_stereo(uint32_t mode, bool requested, int64_t audio_rate) {
    if (!requested) return false;
    return mode == RV_DEMOD_WFM && audio_rate < kCompositeAudioRateHz;
}

struct Deemphasis {
    std::vector<float> taps;
    double group_delay = 0.0;
    bool truncated = false;
};

int32_t design_deemphasis_taps(uint32_t curve, int64_t audio_rate, Deemphasis& out) {
    const double tau = deemphasis_seconds(curve);
    if (tau <= 0.0) {
        out.taps = std::vector<float>{1.0f};
        return RV_OK;
    }
    if (audio_rate <= 0) return set_error_fmt(RV_ERR_INVALID, "design_deemphasis_taps: audio rate must be positive");
    const double period = 1.0 / static_cast<double>(audio_rate);
    const double pole = exp(-period / tau);
    const double kFloatFloor = 1.0 / 16777216.0;
    const double exact_length = log(kFloatFloor * (1.0 - pole)) / log(pole);
    uint32_t length = static_cast<uint32_t>(ceil(std::max(1.0, exact_length))) + 1u;
    if (length > 1024u) {
        length = 1024u;
        out.truncated = true;
    }
    std::vector<double> response(length, 0.0);
    double sum = 0.0, weighted = 0.0, term = 1.0;
    for (uint32_t k = 0; k < length; ++k) {
        response[k] = term;
        sum += term;
        weighted += static_cast<double>(k) * term;
        term *= pole;
    }
    const double scale = 1.0 / sum;
    out.taps.resize(length);
    for (uint32_t k = 0; k < length; ++k) out.taps[k] = static_cast<float>(response[k] * scale);
    out.group_delay = weighted / sum;
    return RV_OK;
}

int32_t fold_deemphasis(const std::vector<float>& dec, const std::vector<float>& de, uint32_t decimation,
                        std::vector<float>& out) {
    if (dec.empty() || de.empty()) return set_error_fmt(RV_ERR_INVALID, "fold_deemphasis: both filters need at least one tap");
    if (decimation == 0) return set_error_fmt(RV_ERR_INVALID, "fold_deemphasis: decimation is zero");
    if (de.size() == 1 && de[0] == 1.0f) {
        out = dec;
        return RV_OK;
    }
    const size_t stride = decimation;
    const size_t length = dec.size() + (de.size() - 1u) * stride;
    if (length > 4096) return set_error_fmt(RV_ERR_INVALID, "fold_deemphasis: folds to %zu taps, the audio filter holds 4096", length);
    std::vector<double> folded(length, 0.0);
    for (size_t k = 0; k < de.size(); ++k) {
        const double weight = static_cast<double>(de[k]);
        const size_t offset = k * stride;
        for (size_t j = 0; j < dec.size(); ++j) folded[offset + j] += weight * static_cast<double>(dec[j]);
    }
    out.assign(length, 0.0f);
    for (size_t i = 0; i < length; ++i) out[i] = static_cast<float>(folded[i]);
    return RV_OK;
}

uint32_t stereo_pilot_taps(int64_t demod_rate) {
    if (demod_rate <= 0) return 0;
    const double transition = 3000.0 / static_cast<double>(demod_rate);
    uint32_t taps = std::clamp(kaiser_taps_for(70.0, transition), 16u, 2048u);
    if ((taps % 2u) == 0u) ++taps;
    return std::min(taps, 2048u);
}

int32_t design_stereo_tables(int64_t demod_rate, uint32_t audio_taps, uint32_t pilot_taps,
                             std::vector<float>& pilot, std::vector<float>& rotation) {
    if (demod_rate <= 0) return set_error_fmt(RV_ERR_INVALID, "design_stereo_tables: rate must be positive");
    if (pilot_taps == 0 || pilot_taps > 2048) return set_error_fmt(RV_ERR_INVALID, "design_stereo_tables: %u pilot taps", pilot_taps);
    if (audio_taps == 0 || audio_taps > 4096) return set_error_fmt(RV_ERR_INVALID, "design_stereo_tables: %u audio taps", audio_taps);
    if (2 * 19000 >= demod_rate) return set_error_fmt(RV_ERR_INVALID, "design_stereo_tables: %lld S/s cannot carry the 38 kHz subcarrier", (long long)demod_rate);
    const double rate = static_cast<double>(demod_rate);
    const double cutoff = 1000.0 / rate;
    const double centre = (static_cast<double>(pilot_taps) - 1.0) / 2.0;
    const double beta = kaiser_beta(70.0);
    const double i0_beta = bessel_i0(beta);
    std::vector<double> proto(pilot_taps, 0.0);
    double sum = 0.0;
    for (uint32_t k = 0; k < pilot_taps; ++k) {
        const double position = static_cast<double>(k) - centre;
        const double window = kaiser_window(k, pilot_taps, beta, i0_beta);
        proto[k] = 2.0 * cutoff * sinc_pi(2.0 * cutoff * position) * window;
        sum += proto[k];
    }
    const double scale = (fabs(sum) < 1e-12) ? 1.0 : 1.0 / sum;
    const double pilot_turns = 19000.0 / rate;
    pilot.resize(2u * static_cast<size_t>(pilot_taps));
    for (uint32_t k = 0; k < pilot_taps; ++k) {
        const double turns = fmod(pilot_turns * static_cast<double>(k), 1.0);
        const double angle = kTwoPi * turns;
        const double weight = proto[k] * scale;
        pilot[2u * k] = static_cast<float>(weight * cos(angle));
        pilot[2u * k + 1u] = static_cast<float>(weight * sin(angle));
    }
    const double sub_turns = 2.0 * pilot_turns;
    const int64_t pivot = static_cast<int64_t>(audio_taps / 2u);
    rotation.resize(2u * static_cast<size_t>(audio_taps));
    for (uint32_t t = 0; t < audio_taps; ++t) {
        const double offset = static_cast<double>(static_cast<int64_t>(t) - pivot);
        const double turns = fmod(sub_turns * offset, 1.0);
        const double angle = kTwoPi * turns;
        rotation[2u * t] = static_cast<float>(2.0 * cos(angle));
        rotation[2u * t + 1u] = static_cast<float>(2.0 * sin(angle));
    }
    return RV_OK;
}

void carrier_gains(double bn, double zeta, int64_t rate, double* k1, double* k2) {
    *k1 = *k2 = 0.0;
    if (!(bn > 0.0) || !(zeta > 0.0) || rate <= 0) return;
    const double period = 1.0 / static_cast<double>(rate);
    const double theta = bn * period / (zeta + 1.0 / (4.0 * zeta));
    const double d = 1.0 + 2.0 * zeta * theta + theta * theta;
    *k1 = 4.0 * zeta * theta / d;
    *k2 = 4.0 * theta * theta / d;
}

int32_t design_carrier_loop(int64_t demod_rate, int64_t reach_hz, rv_vrx_carrier_params& out) {
    if (demod_rate <= 0) return set_error_fmt(RV_ERR_INVALID, "design_carrier_loop: rate must be positive");
    if (reach_hz <= 0) return set_error_fmt(RV_ERR_INVALID, "design_carrier_loop: passband reaching %lld Hz holds no carrier", (long long)reach_hz);
    const double fs = static_cast<double>(demod_rate);
    const double zeta = 0.70710678118654752440;
    double k1a, k2a, k1t, k2t;
    carrier_gains(400.0, zeta, demod_rate, &k1a, &k2a);
    carrier_gains(30.0, zeta, demod_rate, &k1t, &k2t);
    auto one_pole = [fs](double seconds) { return static_cast<float>(1.0 - exp(-1.0 / (seconds * fs))); };
    auto samples = [fs](double seconds) { return static_cast<uint32_t>(std::max(1.0, round(seconds * fs))); };
    memset(&out, 0, sizeof out);
    out.k1_acquire = static_cast<float>(k1a);
    out.k2_acquire = static_cast<float>(k2a);
    out.k1_track = static_cast<float>(k1t);
    out.k2_track = static_cast<float>(k2t);
    out.level_alpha = one_pole(0.005);
    out.lock_alpha = one_pole(0.020);
    out.clamp_radians = static_cast<float>(std::min(kTwoPi * static_cast<double>(reach_hz) / fs, 0.5 * kPi));
    out.hold_in = samples(0.010);
    out.hold_out = samples(0.200);
    return RV_OK;
}

// ---- placement (core/engine/vrx_place.cpp) -------------------------------

int64_t divide_nearest(int64_t num, int64_t den) {
    const int64_t q = num / den, r = num % den;
    const int64_t twice = 2 * (r < 0 ? -r : r);
    if (twice < (den < 0 ? -den : den)) return q;
    return (r < 0) ? q - 1 : q + 1;
}

bool clamp_breaks_demodulator(uint32_t mode) {
    return mode == RV_DEMOD_NFM || mode == RV_DEMOD_WFM || mode == RV_DEMOD_P25P1 || mode == RV_DEMOD_DSTAR ||
           mode == RV_DEMOD_TETRA || mode == RV_DEMOD_DMR;
}

uint32_t channel_count_for(int64_t rate, int64_t widest) {
    if (rate <= 0 || widest <= 0) return 2;
    const uint64_t at_one = static_cast<uint64_t>(rate) / static_cast<uint64_t>(widest);
    if (at_one < 2) return 2;
    uint64_t f = 1;
    while ((f << 1) <= at_one) f <<= 1;
    return static_cast<uint32_t>(f);
}

int32_t place(const rv_grid_params& g, int64_t rate, const rv_vrx_request& r, rv_vrx_placement& out) {
    if (int32_t st = rv::validate_grid(&g)) return st;
    if (rate <= 0) return set_error_fmt(RV_ERR_INVALID, "place: sample rate must be positive");
    if (rate % static_cast<int64_t>(g.decimation) != 0)
        return set_error_fmt(RV_ERR_INVALID, "place: source rate %lld is not divisible by the decimation %u", (long long)rate, g.decimation);
    const int64_t channel_rate = rate / static_cast<int64_t>(g.decimation);
    const int64_t nyquist = rate / 2;
    if (r.center > nyquist || r.center < -nyquist)
        return set_error_fmt(RV_ERR_INVALID, "place: centre %lld Hz is outside the source's +/-%lld Hz", (long long)r.center, (long long)nyquist);
    if (r.demod > 12) return set_error_fmt(RV_ERR_INVALID, "place: mode %u is not a demodulator", r.demod);
    Band requested;
    if (int32_t st = resolve_passband(r, &requested)) return st;
    const int64_t M = g.channels;
    const int64_t signed_index = divide_nearest(r.center * M, rate);
    int64_t wrapped = signed_index % M;
    if (wrapped < 0) wrapped += M;
    memset(&out, 0, sizeof out);
    out.channel = static_cast<uint32_t>(wrapped);
    // channel_centre (core/dsp/pfb_design.cpp:327-350): exact rational
    const int64_t sidx = (out.channel < g.channels / 2) ? static_cast<int64_t>(out.channel)
                                                        : static_cast<int64_t>(out.channel) - M;
    int64_t cn = sidx * rate, cd = M;
    const int64_t cg = std::gcd(cn, cd);
    if (cg > 1) {
        cn /= cg;
        cd /= cg;
    }
    out.centre_numerator = cn;
    out.centre_denominator = cd;
    out.channel_rate = channel_rate;
    out.residual_numerator = r.center * cd - cn;
    out.residual_denominator = cd;
    const int64_t span = rate * out.residual_denominator;
    while (2 * out.residual_numerator > span) out.residual_numerator -= span;
    while (2 * out.residual_numerator <= -span) out.residual_numerator += span;
    const int64_t dg = std::gcd(out.residual_numerator, out.residual_denominator);
    if (dg > 1) {
        out.residual_numerator /= dg;
        out.residual_denominator /= dg;
    }
    const Band granted = clamp_to_channel(out, requested);
    out.granted_low = granted.low;
    out.granted_high = granted.high;
    out.bandwidth_clamped = (granted != requested) ? 1u : 0u;
    if (out.bandwidth_clamped && clamp_breaks_demodulator(r.demod)) {
        const Band plan = default_passband(r.demod);
        const int64_t got = granted.high - granted.low;
        if (plan.width() > 0 && got < plan.width()) {
            const uint32_t would = channel_count_for(rate, plan.width());
            return set_error_fmt(RV_ERR_INVALID,
                                 "place: this receiver needs %lld Hz of passband and one channel of this %u "
                                 "channel grid could carry %lld Hz of it; refused rather than narrowed, "
                                 "because a truncated passband demodulates wrongly. %u channels would carry it",
                                 (long long)plan.width(), g.channels, (long long)got, would);
        }
    }
    return RV_OK;
}

// ---- plan_vrx (core/dsp/vrx_reference.cpp:2243-2662) ---------------------

struct Plan {
    rv_vrx_plan_info info{};
    std::vector<rv_cf32> fine_taps;
    std::vector<float> weights;
};

constexpr double kFineAttenuationDb = 80.0;
constexpr double kAudioAttenuationDb = 80.0;

int32_t plan_vrx(const rv_grid_params& g, int64_t rate, const rv_vrx_request& r, const rv_vrx_placement& pl,
                 Plan& plan) {
    if (int32_t st = rv::validate_grid(&g)) return st;
    if (rate <= 0) return set_error_fmt(RV_ERR_INVALID, "plan_vrx: sample rate must be positive");
    if (pl.channel_rate <= 0) return set_error_fmt(RV_ERR_INVALID, "plan_vrx: placement carries no channel rate; call place first");
    if (pl.residual_denominator <= 0) return set_error_fmt(RV_ERR_INVALID, "plan_vrx: non-positive residual denominator");
    rv_vrx_plan_info& p = plan.info;
    memset(&p, 0, sizeof p);
    p.placement = pl;
    p.mode = r.demod;
    p.channel_rate = pl.channel_rate;
    p.audio_rate = (r.audio_rate > 0) ? r.audio_rate : 48000;
    if (p.mode > 12) return set_error_fmt(RV_ERR_INVALID, "plan_vrx: demodulator %u is unknown", p.mode);
    const bool complex_output = rv::is_complex_mode(p.mode);
    Band requested;
    if (int32_t st = resolve_passband(r, &requested)) return st;
    if (int32_t st = channel_carries(pl, requested)) return st;
    const Band band = clamp_to_channel(pl, requested);
    p.passband_low = band.low;
    p.passband_high = band.high;
    p.bandwidth = band.width();
    p.bandwidth_clamped = (band != requested) ? 1u : 0u;
    const int64_t cw_pitch = std::max<int64_t>(0, r.cw_pitch);
    const Band mixed = mix_frame(band, p.mode, cw_pitch);
    // demod_rate_for: round the minimum rate up to a multiple of the audio
    // rate (or of the decoder's symbol-friendly step for complex taps)
    {
        const int64_t required = minimum_demod_rate(p.mode, mix_frame(band, p.mode, cw_pitch));
        const int64_t tap_step = complex_tap_rate_step(p.mode);
        const int64_t step = (tap_step > 0) ? tap_step : p.audio_rate;
        const int64_t multiple = std::max<int64_t>(1, (required + step - 1) / step);
        p.demod_rate = multiple * step;
    }
    const uint32_t decimation = static_cast<uint32_t>(p.demod_rate / p.audio_rate);
    const double stop_edge = 0.5 * static_cast<double>(std::min(p.demod_rate, p.channel_rate));
    const double transition_limit = 2.0 * std::min(stop_edge - static_cast<double>(mixed.high),
                                                   stop_edge + static_cast<double>(mixed.low));
    const double transition_wanted = 0.5 * static_cast<double>(p.bandwidth);
    const double transition = std::min(transition_limit, transition_wanted);
    if (!(transition > 0.0))
        return set_error_fmt(RV_ERR_INVALID, "plan_vrx: a passband of %lld to %lld Hz leaves no transition band",
                             (long long)band.low, (long long)band.high);
    p.fine.phases = 256;
    p.fine.nco_log2 = 16;
    p.fine.taps = std::clamp(kaiser_taps_for(kFineAttenuationDb, transition / static_cast<double>(p.channel_rate)), 8u, 256u);
    int64_t fnum = 2 * pl.residual_numerator + pl.residual_denominator * (band.low + band.high);
    int64_t fden = 2 * pl.residual_denominator;
    int64_t mnum = pl.residual_numerator, mden = pl.residual_denominator;
    if (p.mode == RV_DEMOD_CW) mnum = pl.residual_numerator - pl.residual_denominator * cw_pitch;
    reduce_rational(fnum, fden);
    reduce_rational(mnum, mden);
    p.filter_numerator = fnum;
    p.filter_denominator = fden;
    p.mix_numerator = mnum;
    p.mix_denominator = mden;
    p.demod.mode = p.mode;
    p.demod.decimation = complex_output ? 1u : decimation;
    p.output_rate = complex_output ? p.demod_rate : p.audio_rate;
    const bool programme_audio = (p.mode == RV_DEMOD_WFM) && p.audio_rate < kCompositeAudioRateHz;
    const double audio_nyquist = 0.5 * static_cast<double>(p.audio_rate);
    const double audio_pass = programme_audio ? std::min(15000.0, 0.8 * audio_nyquist) : 0.8 * audio_nyquist;
    const double audio_stop = programme_audio ? std::min(19000.0, audio_nyquist) : audio_nyquist;
    p.deemphasis = resolve_deemphasis(p.mode, r.deemphasis, p.audio_rate);
    Deemphasis curve;
    if (int32_t st = design_deemphasis_taps(p.deemphasis, p.audio_rate, curve)) return st;
    p.deemphasis_taps = static_cast<uint32_t>(curve.taps.size());
    double pass_hz = 0.0, stop_hz = 0.0;
    if (p.demod.decimation == 1u) {
        p.audio_decimation_taps = 1u;
    } else {
        const double fraction = (audio_stop - audio_pass) / static_cast<double>(p.demod_rate);
        pass_hz = audio_pass;
        stop_hz = audio_stop;
        uint32_t taps = std::clamp(kaiser_taps_for(kAudioAttenuationDb, fraction), 3u, 1024u);
        if ((taps % 2u) == 0u) ++taps;
        p.audio_decimation_taps = std::min(taps, 1024u);
    }
    p.stereo = resolve_stereo(p.mode, r.stereo != 0, p.audio_rate) ? 1u : 0u;
    if (complex_output) {
        p.demod.channels = 2u;
        p.demod.pilot_taps = 0u;
    } else if (p.stereo) {
        p.demod.channels = 2u;
        p.demod.pilot_taps = stereo_pilot_taps(p.demod_rate);
        if (p.demod.pilot_taps == 0) return set_error_fmt(RV_ERR_INVALID, "plan_vrx: no pilot filter at %lld S/s", (long long)p.demod_rate);
    } else {
        p.demod.channels = 1u;
        p.demod.pilot_taps = 0u;
    }
    if (p.mode == RV_DEMOD_AM || p.mode == RV_DEMOD_SAM)
        p.demod.dc_taps = static_cast<uint32_t>(std::clamp<int64_t>(p.demod_rate / 200, 16, 4096));
    else
        p.demod.dc_taps = 1u;
    p.deviation = fm_deviation(p.mode, p.bandwidth);
    p.demod_gain = vrx_demod_gain(p.mode, p.demod_rate, p.deviation);
    p.carrier.power = carrier_power(p.mode);
    p.carrier.nco_log2 = p.fine.nco_log2;
    if (p.carrier.power != 0) {
        if (int32_t st = design_carrier_loop(p.demod_rate, Band{band.low, band.high}.reach_from(0), p.carrier_loop))
            return st;
    }
    // tables (plan_vrx proper)
    if (int32_t st = design_fine_taps(p.fine, p.channel_rate, p.bandwidth / 2, p.filter_numerator,
                                      p.filter_denominator, kFineAttenuationDb, plan.fine_taps))
        return st;
    if (int32_t st = nco_delta(p.mix_numerator, p.mix_denominator, p.demod_rate, &p.fine_nco_delta)) return st;
    const double audio_cutoff = (stop_hz > 0.0) ? 0.5 * (pass_hz + stop_hz) : 0.0;
    std::vector<float> dec, folded;
    if (int32_t st = design_audio_taps(p.audio_decimation_taps, p.demod_rate, p.output_rate, kAudioAttenuationDb,
                                       audio_cutoff, dec))
        return st;
    if (int32_t st = fold_deemphasis(dec, curve.taps, p.demod.decimation, folded)) return st;
    p.demod.audio_taps = static_cast<uint32_t>(folded.size());
    const std::vector<float> dc = design_dc_weights(p.demod.dc_taps);
    std::vector<float> pilot, rotation;
    if (p.demod.pilot_taps != 0) {
        if (int32_t st = design_stereo_tables(p.demod_rate, p.demod.audio_taps, p.demod.pilot_taps, pilot, rotation))
            return st;
    }
    plan.weights.clear();
    plan.weights.insert(plan.weights.end(), folded.begin(), folded.end());
    plan.weights.insert(plan.weights.end(), dc.begin(), dc.end());
    plan.weights.insert(plan.weights.end(), pilot.begin(), pilot.end());
    plan.weights.insert(plan.weights.end(), rotation.begin(), rotation.end());
    p.fine_tap_count = plan.fine_taps.size();
    p.demod_weight_count = plan.weights.size();
    return RV_OK;
}

}  // namespace

namespace rv {

// Shared with the chain runner.
int32_t plan_receiver(const rv_grid_params& g, int64_t rate, const rv_vrx_request& r, rv_vrx_plan_info& info,
                      std::vector<rv_cf32>& taps, std::vector<float>& weights) {
    rv_vrx_placement pl;
    if (int32_t st = place(g, rate, r, pl)) return st;
    Plan plan;
    if (int32_t st = plan_vrx(g, rate, r, pl, plan)) return st;
    info = plan.info;
    taps.swap(plan.fine_taps);
    weights.swap(plan.weights);
    return RV_OK;
}

int32_t design_prototype_table(const rv_grid_params& g, double atten, std::vector<float>& taps) {
    return design_prototype(g, atten, taps, nullptr, nullptr);
}
int32_t build_twiddle_table(uint32_t M, std::vector<rv_cf32>& out) { return build_twiddles(M, out); }
int32_t build_nco(uint32_t log2, std::vector<rv_cf32>& out) { return build_nco_table(log2, out); }
int32_t build_window(uint32_t n, uint32_t t, double a, std::vector<float>& out) {
    return build_spectrum_window(n, t, a, out);
}

}  // namespace rv

extern "C" {

int32_t rv_design_prototype(const rv_grid_params* grid, double atten, float* taps, uint64_t taps_len,
                            double* stopband_db, uint64_t* group_delay) {
    if (grid == nullptr || taps == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_design_prototype: NULL");
    std::vector<float> t;
    if (int32_t st = design_prototype(*grid, atten, t, stopband_db, group_delay)) return st;
    if (taps_len != t.size()) return set_error_fmt(RV_ERR_INVALID, "rv_design_prototype: wants %zu taps, buffer holds %llu", t.size(), (unsigned long long)taps_len);
    memcpy(taps, t.data(), t.size() * sizeof(float));
    return rv::clear_error();
}

// design_prototype for grids past the reference's 2048 channels (C4's
// M = 4096): the same Kaiser-windowed sinc and normalisation.
int32_t rv_design_prototype_wide(const rv_grid_params* grid, double atten, float* taps, uint64_t taps_len,
                                 double* stopband_db, uint64_t* group_delay) {
    if (grid == nullptr || taps == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_design_prototype_wide: NULL");
    std::vector<float> t;
    if (int32_t st = design_prototype(*grid, atten, t, stopband_db, group_delay, 16384)) return st;
    if (taps_len != t.size())
        return set_error_fmt(RV_ERR_INVALID, "rv_design_prototype_wide: wants %zu taps, buffer holds %llu", t.size(),
                             (unsigned long long)taps_len);
    memcpy(taps, t.data(), t.size() * sizeof(float));
    return rv::clear_error();
}

int32_t rv_build_twiddles(uint32_t channels, rv_cf32* table, uint64_t len) {
    if (table == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_build_twiddles: NULL");
    std::vector<rv_cf32> t;
    if (int32_t st = build_twiddles(channels, t)) return st;
    if (len != t.size()) return set_error_fmt(RV_ERR_INVALID, "rv_build_twiddles: wants %zu entries", t.size());
    memcpy(table, t.data(), t.size() * sizeof(rv_cf32));
    return rv::clear_error();
}

// The same first-octant construction for transforms beyond the channel
// grid's 2048 (the averaged spectrum, up to 8192 points, and wider DFTs).
int32_t rv_build_fft_twiddles(uint32_t n, rv_cf32* table, uint64_t len) {
    if (table == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_build_fft_twiddles: NULL");
    std::vector<rv_cf32> t;
    if (int32_t st = build_twiddles(n, t, 1u << 16)) return st;
    if (len != t.size()) return set_error_fmt(RV_ERR_INVALID, "rv_build_fft_twiddles: wants %zu entries", t.size());
    memcpy(table, t.data(), t.size() * sizeof(rv_cf32));
    return rv::clear_error();
}

int32_t rv_build_nco_table(uint32_t log2_size, rv_cf32* table, uint64_t len) {
    if (table == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_build_nco_table: NULL");
    std::vector<rv_cf32> t;
    if (int32_t st = build_nco_table(log2_size, t)) return st;
    if (len != t.size()) return set_error_fmt(RV_ERR_INVALID, "rv_build_nco_table: wants %zu entries", t.size());
    memcpy(table, t.data(), t.size() * sizeof(rv_cf32));
    return rv::clear_error();
}

int32_t rv_build_spectrum_window(uint32_t transform, uint32_t taps_per_branch, double atten, float* window,
                                 uint64_t len) {
    if (window == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_build_spectrum_window: NULL");
    std::vector<float> t;
    if (int32_t st = build_spectrum_window(transform, taps_per_branch, atten, t)) return st;
    if (len != t.size()) return set_error_fmt(RV_ERR_INVALID, "rv_build_spectrum_window: wants %zu floats", t.size());
    memcpy(window, t.data(), t.size() * sizeof(float));
    return rv::clear_error();
}

int32_t rv_place(const rv_grid_params* grid, int64_t rate, const rv_vrx_request* request, rv_vrx_placement* out) {
    if (grid == nullptr || request == nullptr || out == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_place: NULL");
    if (int32_t st = place(*grid, rate, *request, *out)) return st;
    return rv::clear_error();
}

uint32_t rv_channel_count_for(int64_t rate, int64_t widest) { return channel_count_for(rate, widest); }

int32_t rv_plan_vrx(const rv_grid_params* grid, int64_t rate, const rv_vrx_request* request,
                    const rv_vrx_placement* placement, rv_vrx_plan_info* info, rv_cf32* fine_taps,
                    uint64_t fine_taps_len, float* weights, uint64_t weights_len) {
    if (grid == nullptr || request == nullptr || placement == nullptr || info == nullptr)
        return set_error_fmt(RV_ERR_INVALID, "rv_plan_vrx: NULL");
    Plan plan;
    if (int32_t st = plan_vrx(*grid, rate, *request, *placement, plan)) return st;
    *info = plan.info;
    if (fine_taps != nullptr) {
        if (fine_taps_len != plan.fine_taps.size()) return set_error_fmt(RV_ERR_INVALID, "rv_plan_vrx: fine tap buffer holds %llu, plan has %zu", (unsigned long long)fine_taps_len, plan.fine_taps.size());
        memcpy(fine_taps, plan.fine_taps.data(), plan.fine_taps.size() * sizeof(rv_cf32));
    }
    if (weights != nullptr) {
        if (weights_len != plan.weights.size()) return set_error_fmt(RV_ERR_INVALID, "rv_plan_vrx: weight buffer holds %llu, plan has %zu", (unsigned long long)weights_len, plan.weights.size());
        memcpy(weights, plan.weights.data(), plan.weights.size() * sizeof(float));
    }
    return rv::clear_error();
}

// resample_block (core/dsp/vrx_reference.cpp:2786-2850): block parameters
// from the absolute output index, re-deriving the first input exactly.
static int32_t resample_block(const rv_vrx_fine_config& fine, int64_t channel_rate, int64_t out_rate, uint64_t nco,
                              uint32_t channel_base, uint32_t channel_mask, uint32_t fine_mask, uint64_t first_output,
                              uint32_t count, rv_vrx_fine_block* block);

int32_t rv_fine_block(const rv_vrx_plan_info* plan, uint32_t channel_base, uint32_t channel_mask, uint32_t fine_mask,
                      uint64_t first_output, uint32_t count, rv_vrx_fine_block* block) {
    if (plan == nullptr || block == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_fine_block: NULL");
    if (plan->channel_rate <= 0 || plan->demod_rate <= 0) return set_error_fmt(RV_ERR_INVALID, "fine_block: the plan carries no rates");
    if (count == 0) return set_error_fmt(RV_ERR_INVALID, "fine_block: a dispatch of zero outputs has nothing to do");
    return resample_block(plan->fine, plan->channel_rate, plan->demod_rate, plan->fine_nco_delta, channel_base,
                          channel_mask, fine_mask, first_output, count, block);
}

// ---- the display tap (core/dsp/vrx_reference.cpp:2938-3080) --------------

// The largest R at which 256 taps still reach 80 dB across Fdisp/2.
uint32_t rv_display_max_decimation(void) {
    uint32_t best = 1;
    for (uint32_t r = 1; r <= 4096u; ++r) {
        if (attenuation_reachable(RV_DISPLAY_TAPS, 1.0 / (2.0 * static_cast<double>(r))) < 80.0) break;
        best = r;
    }
    return best;
}

static std::vector<uint32_t> display_ladder(int64_t channel_rate) {
    std::vector<uint32_t> rungs{1u};
    if (channel_rate <= 0) return rungs;
    const uint32_t cap = rv_display_max_decimation();
    for (;;) {
        uint32_t next = 0;
        for (uint32_t d = 2u * rungs.back(); d <= cap; ++d)
            if (channel_rate % static_cast<int64_t>(d) == 0) {
                next = d;
                break;
            }
        if (next == 0) return rungs;
        rungs.push_back(next);
    }
}

int32_t rv_display_ladder(int64_t channel_rate, uint32_t* rungs, uint32_t capacity, uint32_t* count) {
    if (count == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_display_ladder: NULL");
    const std::vector<uint32_t> v = display_ladder(channel_rate);
    *count = static_cast<uint32_t>(v.size());
    if (rungs)
        for (uint32_t i = 0; i < *count && i < capacity; ++i) rungs[i] = v[i];
    return rv::clear_error();
}

uint32_t rv_display_decimation(int64_t channel_rate, int64_t reach_hz) {
    if (channel_rate <= 0 || reach_hz <= 0) return 1u;
    // Fdisp/4 >= 2 reach: the pane is at least four reaches across
    const int64_t wanted = channel_rate / (8 * reach_hz);
    uint32_t chosen = 1u;
    for (uint32_t rung : display_ladder(channel_rate))
        if (static_cast<int64_t>(rung) <= wanted) chosen = rung;
    return chosen;
}

int32_t rv_plan_vrx_display(const rv_vrx_plan_info* plan, rv_vrx_display_plan* out, rv_cf32* taps, uint64_t taps_len) {
    if (plan == nullptr || out == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_plan_vrx_display: NULL");
    if (plan->channel_rate <= 0) return set_error_fmt(RV_ERR_INVALID, "plan_vrx_display: the plan carries no channel rate");
    if (plan->mix_denominator == 0 || plan->placement.residual_denominator == 0)
        return set_error_fmt(RV_ERR_INVALID, "plan_vrx_display: the plan carries no mix frequency");
    // the passband in the frame the fine stage mixes to DC
    const double shift = static_cast<double>(plan->placement.residual_numerator) /
                             static_cast<double>(plan->placement.residual_denominator) -
                         static_cast<double>(plan->mix_numerator) / static_cast<double>(plan->mix_denominator);
    const double reach = std::max(std::fabs(static_cast<double>(plan->passband_low) + shift),
                                  std::fabs(static_cast<double>(plan->passband_high) + shift));
    rv_vrx_display_plan d;
    memset(&d, 0, sizeof d);
    d.channel_rate = plan->channel_rate;
    d.reach_hz = std::max<int64_t>(1, static_cast<int64_t>(std::ceil(reach)));
    d.decimation = rv_display_decimation(plan->channel_rate, d.reach_hz);
    d.display_rate = plan->channel_rate / static_cast<int64_t>(d.decimation);
    d.fine.taps = RV_DISPLAY_TAPS;
    d.fine.phases = 1u;
    d.fine.nco_log2 = plan->fine.nco_log2;
    d.group_delay_channel_samples = (static_cast<double>(RV_DISPLAY_TAPS) - 1.0) / 2.0;
    // flat to the pane's edge Fdisp/4, in stopband by 3 Fdisp/4 (or Fc/2)
    const double fc = static_cast<double>(plan->channel_rate), fdisp = static_cast<double>(d.display_rate);
    d.pass_hz = 0.25 * fdisp;
    d.stop_hz = std::min(0.75 * fdisp, 0.5 * fc);
    const double reachable = attenuation_reachable(RV_DISPLAY_TAPS, (d.stop_hz - d.pass_hz) / fc);
    if (reachable < 80.0)
        return set_error_fmt(RV_ERR_INVALID, "plan_vrx_display: %u taps reach %.1f dB across %.0f to %.0f Hz at %lld S/s",
                             RV_DISPLAY_TAPS, reachable, d.pass_hz, d.stop_hz, (long long)plan->channel_rate);
    d.attenuation_db = std::min(100.0, reachable);
    // the cutoff midway between the edges
    const int64_t half_width = static_cast<int64_t>(0.5 * (d.pass_hz + d.stop_hz));
    std::vector<rv_cf32> table;
    if (int32_t st = design_fine_taps(d.fine, plan->channel_rate, half_width, plan->mix_numerator, plan->mix_denominator,
                                      d.attenuation_db, table))
        return st;
    if (int32_t st = nco_delta(plan->mix_numerator, plan->mix_denominator, d.display_rate, &d.nco_delta)) return st;
    d.tap_count = table.size();
    *out = d;
    if (taps != nullptr) {
        if (taps_len != table.size())
            return set_error_fmt(RV_ERR_INVALID, "rv_plan_vrx_display: tap buffer holds %llu, plan has %zu",
                                 (unsigned long long)taps_len, table.size());
        memcpy(taps, table.data(), table.size() * sizeof(rv_cf32));
    }
    return rv::clear_error();
}

int32_t rv_display_block(const rv_vrx_display_plan* plan, uint32_t channel_base, uint32_t channel_mask,
                         uint32_t display_mask, uint64_t first_output, uint32_t count, rv_vrx_fine_block* block) {
    if (plan == nullptr || block == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_display_block: NULL");
    if (plan->channel_rate <= 0 || plan->display_rate <= 0)
        return set_error_fmt(RV_ERR_INVALID, "display_block: the plan carries no rates");
    if (count == 0) return set_error_fmt(RV_ERR_INVALID, "display_block: a dispatch of zero outputs has nothing to do");
    return resample_block(plan->fine, plan->channel_rate, plan->display_rate, plan->nco_delta, channel_base,
                          channel_mask, display_mask, first_output, count, block);
}

static int32_t resample_block(const rv_vrx_fine_config& fine, int64_t channel_rate, int64_t out_rate, uint64_t nco,
                              uint32_t channel_base, uint32_t channel_mask, uint32_t fine_mask, uint64_t first_output,
                              uint32_t count, rv_vrx_fine_block* block) {
    const uint64_t fc = static_cast<uint64_t>(channel_rate), fd = static_cast<uint64_t>(out_rate);
    const uint64_t step_whole = fc / fd, step_rem = fc % fd;
    const uint64_t whole = first_output / fd, part = first_output % fd;
    const uint64_t carry_product = part * step_rem;
    const uint64_t first_input = first_output * step_whole + whole * step_rem + carry_product / fd;
    const uint64_t frac0 = carry_product % fd;
    memset(block, 0, sizeof *block);
    rv_vrx_fine_params& o = block->params;
    o.chan_base = channel_base;
    o.chan_mask = channel_mask;
    o.in_offset = static_cast<uint32_t>(first_input & channel_mask);
    o.out_offset = static_cast<uint32_t>(first_output & fine_mask);
    o.out_mask = fine_mask;
    o.count = count;
    o.step_whole = static_cast<uint32_t>(step_whole);
    o.step_rem = static_cast<uint32_t>(step_rem);
    o.out_rate = static_cast<uint32_t>(fd);
    o.frac0 = static_cast<uint32_t>(frac0);
    o.inv_out_rate = 1.0f / static_cast<float>(fd);
    const uint64_t phase = nco * first_output;
    o.nco_phase_high = static_cast<uint32_t>(phase >> 32);
    o.nco_phase_low = static_cast<uint32_t>(phase);
    o.nco_delta_high = static_cast<uint32_t>(nco >> 32);
    o.nco_delta_low = static_cast<uint32_t>(nco);
    if (int32_t st = rv::validate_fine(&fine, &o)) return st;
    const uint64_t last_acc = frac0 + static_cast<uint64_t>(count - 1u) * step_rem;
    block->first_input = first_input;
    block->newest_input = first_input + static_cast<uint64_t>(count - 1u) * step_whole + last_acc / fd;
    block->oldest_input = first_input - static_cast<uint64_t>(fine.taps - 1u);
    return rv::clear_error();
}

int32_t rv_demod_block(const rv_vrx_plan_info* plan, uint32_t fine_mask, uint64_t first_audio, uint32_t count,
                       rv_vrx_demod_block* block) {
    if (plan == nullptr || block == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_demod_block: NULL");
    if (count == 0) return set_error_fmt(RV_ERR_INVALID, "demod_block: a dispatch of zero outputs has nothing to do");
    const uint64_t first_fine = first_audio * static_cast<uint64_t>(plan->demod.decimation);
    memset(block, 0, sizeof *block);
    block->first_fine = first_fine;
    block->params.in_mask = fine_mask;
    block->params.in_offset = static_cast<uint32_t>(first_fine & fine_mask);
    block->params.count = count;
    block->params.gain = plan->demod_gain;
    if (int32_t st = rv::validate_demod(&plan->demod, &block->params)) return st;
    block->oldest_fine = first_fine - rv::demod_fine_history(&plan->demod);
    return rv::clear_error();
}

int32_t rv_carrier_block(const rv_vrx_plan_info* plan, uint32_t fine_mask, uint64_t first_fine, uint32_t count,
                         int32_t reset, float shift, rv_vrx_carrier_params* out) {
    if (plan == nullptr || out == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_carrier_block: NULL");
    if (plan->carrier.power == 0) return set_error_fmt(RV_ERR_INVALID, "carrier_block: this receiver runs no carrier loop");
    *out = plan->carrier_loop;
    out->in_mask = fine_mask;
    out->in_offset = static_cast<uint32_t>(first_fine & fine_mask);
    out->count = count;
    out->flags = reset ? 1u : 0u;
    out->shift = reset ? 0.0f : shift;
    if (int32_t st = rv::validate_carrier(&plan->carrier, out)) return st;
    return rv::clear_error();
}

}  // extern "C"
