// Host-side pieces of the scene synthesiser shared by the emitter dispatch
// (scene_noise.cu) and the scene planner (scene_plan.cpp): the Morse code
// and the keyed elements of a CW message cycle.
#pragma once

#include <math.h>

#include <cmath>
#include <stdint.h>

#include <random>
#include <utility>
#include <vector>

namespace rv {

// International Morse code (ITU-R M.1677): the letters, digits and the
// punctuation the reference keys (modulators.cpp:124-145), upper case.
struct MorseCode {
    char character;
    const char* code;
};
inline constexpr MorseCode kMorse[] = {
    {'A', ".-"},    {'B', "-..."},  {'C', "-.-."},  {'D', "-.."},   {'E', "."},      {'F', "..-."},
    {'G', "--."},   {'H', "...."},  {'I', ".."},    {'J', ".---"},  {'K', "-.-"},    {'L', ".-.."},
    {'M', "--"},    {'N', "-."},    {'O', "---"},   {'P', ".--."},  {'Q', "--.-"},   {'R', ".-."},
    {'S', "..."},   {'T', "-"},     {'U', "..-"},   {'V', "...-"},  {'W', ".--"},    {'X', "-..-"},
    {'Y', "-.--"},  {'Z', "--.."},  {'0', "-----"}, {'1', ".----"}, {'2', "..---"},  {'3', "...--"},
    {'4', "....-"}, {'5', "....."}, {'6', "-...."}, {'7', "--..."}, {'8', "---.."},  {'9', "----."},
    {'.', ".-.-.-"}, {',', "--..--"}, {'?', "..--.."}, {'/', "-..-."}, {'=', "-...-"}, {'+', ".-.-."},
    {'-', "-....-"}, {':', "---..."},
};

inline const char* morse(char c) {
    const char upper = (c >= 'a' && c <= 'z') ? (char)(c - 'a' + 'A') : c;  // no locale
    for (const MorseCode& m : kMorse)
        if (m.character == upper) return m.code;
    return nullptr;
}

struct CwElement {
    int64_t start, stop;
    int32_t keyed, pad;
};

// The keyed message as elements of [start, stop) samples within one cycle
// (modulators.cpp:675-741): runs in dot units (a dot on, a dash three; one dot
// between elements, three between characters, seven between words, then the
// message gap), their cumulative edges rounded to samples, each edge at least
// one sample past the last.
inline std::vector<CwElement> cw_elements(const char* text, double dot_samples, double gap_dots) {
    std::vector<std::pair<bool, double>> runs;
    auto add_off = [&runs](double dots) {
        if (dots <= 0.0) return;
        if (!runs.empty() && !runs.back().first) runs.back().second += dots;
        else runs.emplace_back(false, dots);
    };
    for (const char* c = text; *c != '\0'; ++c) {
        if (*c == ' ') {
            add_off(4.0);
            continue;
        }
        for (const char* e = morse(*c); *e != '\0'; ++e) {
            runs.emplace_back(true, *e == '.' ? 1.0 : 3.0);
            add_off(1.0);
        }
        add_off(2.0);
    }
    add_off(gap_dots - 3.0 > 0.0 ? gap_dots - 3.0 : 0.0);
    std::vector<CwElement> out;
    double cumulative = 0.0;
    int64_t previous = 0;
    for (const auto& run : runs) {
        cumulative += run.second;
        int64_t edge = (int64_t)llround(cumulative * dot_samples);
        if (edge <= previous) edge = previous + 1;
        out.push_back(CwElement{previous, edge, run.first ? 1 : 0, 0});
        previous = edge;
    }
    return out;
}

// modulators.cpp:454-472 random_bits: LSB first from std::mt19937_64(seed)
inline std::vector<uint8_t> random_bits(size_t count, uint64_t seed) {
    std::vector<uint8_t> bits(count, 0);
    std::mt19937_64 engine(seed);
    uint64_t word = 0;
    unsigned remaining = 0;
    for (size_t i = 0; i < count; ++i) {
        if (remaining == 0) word = engine(), remaining = 64;
        bits[i] = (uint8_t)(word & 1u);
        word >>= 1;
        --remaining;
    }
    return bits;
}

// modulators.cpp:216-257 build_symbol_clock: symbol k spans
// [floor(k cycle / symbols), floor((k + 1) cycle / symbols)) of a cycle of
// llround(symbols rate / baud) samples. False when the grid is unusable.
struct SymbolClock {
    uint64_t symbols = 0;
    int64_t cycle = 0;
    std::vector<int64_t> boundary;
    // :402-423 index_at
    uint64_t index_at(int64_t position) const {
        uint64_t e = (uint64_t)((position * (int64_t)symbols) / cycle);
        if (e >= symbols) e = symbols - 1;
        while (e + 1 < symbols && boundary[e + 1] <= position) ++e;
        while (e > 0 && boundary[e] > position) --e;
        return e;
    }
    double effective_rate(int64_t rate) const { return (double)symbols * (double)rate / (double)cycle; }
};

inline bool build_symbol_clock(uint64_t symbols, int64_t rate, double baud, SymbolClock& c) {
    if (symbols == 0 || symbols > 1000000) return false;
    const double per = (double)rate / baud, real = (double)symbols * per;
    if (!std::isfinite(real) || real >= 9.0e15) return false;
    const int64_t cycle = (int64_t)llround(real);
    if (cycle < (int64_t)symbols * 2) return false;
    if ((double)symbols * (double)cycle >= 1.8e19) return false;
    c.symbols = symbols;
    c.cycle = cycle;
    c.boundary.resize(symbols + 1);
    for (uint64_t k = 0; k <= symbols; ++k) c.boundary[k] = ((int64_t)k * cycle) / (int64_t)symbols;
    return true;
}

// A PSK emitter's tables (Modulator::create, modulators.cpp:885-1016): the
// symbol constellation (BPSK bit 1 -> +1, QPSK first bit the in-phase sign,
// second the quadrature, 1/sqrt 2 each), the root-raised-cosine table at 512
// steps a symbol with its ends pinned to zero, the table scale and base, the
// energy-normalising gain and the envelope's evaluation stride.
struct PskPlan {
    SymbolClock clock;
    std::vector<float> sym_re, sym_im, rrc;
    std::vector<double> boundary_d;
    double scale = 0, base = 0, limit = 0, cycle_span = 0, gain = 1;
    int64_t stride = 1;
    uint64_t span = 0;
};

// modulators.cpp:172-196 root_raised_cosine
inline double root_raised_cosine(double t, double beta) {
    const double pi = 3.141592653589793238462643383279502884;
    if (std::fabs(t) < 1e-9) return 1.0 + beta * (4.0 / pi - 1.0);
    if (beta <= 0.0) return std::sin(pi * t) / (pi * t);
    const double quarter = 1.0 / (4.0 * beta);
    if (std::fabs(std::fabs(t) - quarter) < 1e-9) {
        const double leading = (1.0 + 2.0 / pi) * std::sin(pi / (4.0 * beta));
        const double trailing = (1.0 - 2.0 / pi) * std::cos(pi / (4.0 * beta));
        return (beta / std::sqrt(2.0)) * (leading + trailing);
    }
    const double four_beta_t = 4.0 * beta * t;
    const double numerator = std::sin(pi * t * (1.0 - beta)) + four_beta_t * std::cos(pi * t * (1.0 + beta));
    const double denominator = pi * t * (1.0 - four_beta_t * four_beta_t);
    return numerator / denominator;
}

// modulators.cpp:1092-1101 rrc_tap_at
inline double rrc_tap_at(const float* rrc, double limit, double position) {
    if (position <= 0.0 || position >= limit) return 0.0;
    const size_t lower = (size_t)position;
    const double fraction = position - (double)lower;
    const double a = (double)rrc[lower], b = (double)rrc[lower + 1];
    return a + fraction * (b - a);
}

inline bool psk_plan(bool quadrature, uint64_t symbol_count, uint64_t seed, int64_t rate, double baud, double rolloff,
                     uint64_t span, PskPlan& p) {
    const uint64_t bps = quadrature ? 2u : 1u;
    const std::vector<uint8_t> bits = random_bits(symbol_count * bps, seed);
    const uint64_t symbols = bits.size() / bps;
    if (span >= symbols) return false;
    if (!build_symbol_clock(symbols, rate, baud, p.clock)) return false;
    const double unit = 1.0 / std::sqrt(2.0);
    p.sym_re.resize(symbols);
    p.sym_im.resize(symbols);
    for (uint64_t k = 0; k < symbols; ++k) {
        if (quadrature) {
            p.sym_re[k] = (float)(bits[2 * k] != 0 ? -unit : unit);
            p.sym_im[k] = (float)(bits[2 * k + 1] != 0 ? -unit : unit);
        } else {
            p.sym_re[k] = bits[k] != 0 ? 1.0f : -1.0f;
            p.sym_im[k] = 0.0f;
        }
    }
    const size_t steps = 512, table = 2 * span * steps + 1;
    p.rrc.resize(table);
    for (size_t i = 0; i < table; ++i) {
        const double t = (double)i / (double)steps - (double)span;
        p.rrc[i] = (float)root_raised_cosine(t, rolloff);
    }
    p.rrc.front() = 0.0f;
    p.rrc.back() = 0.0f;
    const double sps = (double)p.clock.cycle / (double)p.clock.symbols;
    p.scale = (double)steps / sps;
    p.base = (double)span * (double)steps;
    p.limit = (double)(table - 1);
    p.cycle_span = (double)p.clock.cycle;
    p.boundary_d.resize(symbols);
    for (uint64_t k = 0; k < symbols; ++k) p.boundary_d[k] = (double)p.clock.boundary[k];
    const int64_t reach = (int64_t)std::ceil((double)span * sps);
    double energy = 0.0;
    for (int64_t offset = -reach; offset <= reach; ++offset) {
        const double tap = rrc_tap_at(p.rrc.data(), p.limit, ((double)offset / sps) * (double)steps + p.base);
        energy += tap * tap;
    }
    p.gain = energy > 0.0 ? std::sqrt(sps / energy) : 1.0;
    p.stride = 1;
    const double budget = sps / 1024.0;
    while (p.stride * 2 <= 1024 && (double)(p.stride * 2) <= budget) p.stride *= 2;
    p.span = span;
    return true;
}

}  // namespace rv
