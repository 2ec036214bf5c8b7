// Host-side pieces of the scene synthesiser shared by the emitter dispatch
// (scene_noise.cu) and the scene planner (scene_plan.cpp): the Morse code
// and the keyed elements of a CW message cycle.
#pragma once

#include <math.h>
#include <stdint.h>

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

}  // namespace rv
