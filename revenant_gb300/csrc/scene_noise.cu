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
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <vector>

#include "common.cuh"
#include "scene.h"

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

// ---- tone-modulated emitters: siggen::Modulator::accumulate_am / _nfm /
// _ssb (core/dsp/synth/modulators.cpp:1244-1392). The carrier and tone are unit
// phasors advanced by complex multiply and re-anchored every 1024 emitter
// samples from the exact phase of the anchor index (walk_anchored,
// modulators.cpp:99-122, so a sample's value does not depend on where a render
// starts). One thread walks one anchored segment. The anchors' cos/sin and the
// steps' are computed on the host with the C library, as the reference does,
// so the recurrence and every sample of AM and SSB are the reference's bit for
// bit; NFM's per-sample cos/sin of the phase deviation are CUDA's. A tone SSB
// emitter is one rotation per tone at carrier +/- tone (the analytic signal of
// a cosine, modulators.cpp:789-803); its two phasors take the carrier's and
// the tone's places here.

constexpr uint32_t kAnchorInterval = 1024;  // kPhaseAnchorInterval, modulators.cpp:34

struct Anchor {
    double cr, ci, tr, ti;  // carrier and tone phasors at an anchor index
};

struct ToneRun {
    double level, index, beta;                           // gain x amplitude (SSB: its scale); AM index; NFM beta
    bool two_tone;
    double c_step_re, c_step_im, t_step_re, t_step_im;   // per-sample rotations
    uint64_t first, count, first_anchor;                 // emitter indices; anchor of segment 0
    int32_t kind;
};

__global__ void k_tone_emitter(ToneRun r, const Anchor* __restrict__ anchors, uint32_t segments,
                               float2* __restrict__ out) {
    const uint32_t seg = blockIdx.x * blockDim.x + threadIdx.x;
    if (seg >= segments) return;
    const uint64_t anchor = r.first_anchor + (uint64_t)seg * kAnchorInterval;
    const uint64_t end = r.first + r.count;
    const uint64_t stop = anchor + kAnchorInterval < end ? anchor + kAnchorInterval : end;
    const Anchor a = anchors[seg];
    double cr = a.cr, ci = a.ci, tr = a.tr, ti = a.ti;
    for (uint64_t index = anchor; index < stop; ++index) {
        if (index >= r.first) {
            float2 add;
            if (r.kind == RV_EMITTER_AM) {
                const double envelope = r.level * (1.0 + r.index * tr);
                add = make_float2((float)(envelope * cr), (float)(envelope * ci));
            } else if (r.kind == RV_EMITTER_USB || r.kind == RV_EMITTER_LSB) {
                double re = cr, im = ci;
                if (r.two_tone) {
                    re += tr;
                    im += ti;
                }
                add = make_float2((float)(r.level * re), (float)(r.level * im));
            } else {
                const double deviation = r.beta * ti;
                const double cosine = cos(deviation), sine = sin(deviation);
                const double re = cr * cosine - ci * sine;
                const double im = cr * sine + ci * cosine;
                add = make_float2((float)(r.level * re), (float)(r.level * im));
            }
            float2& o = out[index - r.first];
            o = make_float2(o.x + add.x, o.y + add.y);
        }
        const double ncr = cr * r.c_step_re - ci * r.c_step_im, nci = cr * r.c_step_im + ci * r.c_step_re;
        const double ntr = tr * r.t_step_re - ti * r.t_step_im, nti = tr * r.t_step_im + ti * r.t_step_re;
        cr = ncr, ci = nci, tr = ntr, ti = nti;
    }
}

// modulators.cpp:439-449 exact_phase: the phase of `frequency` at `index`,
// reduced in integers so it stays exact at any index.
double exact_phase(int64_t frequency, int64_t rate, uint64_t index) {
    int64_t reduced = frequency % rate;
    if (reduced < 0) reduced += rate;
    const int64_t position = (int64_t)(index % (uint64_t)rate);
    const int64_t turns = (reduced * position) % rate;
    return kTwoPi * (double)turns / (double)rate;
}

// One anchored segment of a CW emitter: the carrier phasor as for the other
// modes, keyed by the element holding index % cycle, with raised-cosine edges
// of `ramp` samples (modulators.cpp:1055-1090, cos(pi t / ramp) on the device).
__global__ void k_cw_emitter(ToneRun r, const Anchor* __restrict__ anchors, uint32_t segments,
                             const CwElement* __restrict__ el, uint32_t nel, double ramp_samples,
                             float2* __restrict__ out) {
    const uint32_t seg = blockIdx.x * blockDim.x + threadIdx.x;
    if (seg >= segments) return;
    const uint64_t anchor = r.first_anchor + (uint64_t)seg * kAnchorInterval;
    const uint64_t end = r.first + r.count;
    const uint64_t stop = anchor + kAnchorInterval < end ? anchor + kAnchorInterval : end;
    const Anchor a = anchors[seg];
    double cr = a.cr, ci = a.ci;
    const int64_t cycle = el[nel - 1].stop;
    const double pi = 3.141592653589793238462643383279502884;
    for (uint64_t index = anchor; index < stop; ++index) {
        if (index >= r.first) {
            const int64_t position = (int64_t)(index % (uint64_t)cycle);
            uint32_t lo = 0, hi = nel - 1;  // the element with start <= position < stop
            while (lo < hi) {
                const uint32_t mid = (lo + hi) >> 1;
                if (el[mid].stop <= position) lo = mid + 1;
                else hi = mid;
            }
            double envelope = 0.0;
            const CwElement e = el[lo];
            if (e.keyed) {
                const double length = (double)(e.stop - e.start);
                const double ramp = ramp_samples < length * 0.5 ? ramp_samples : length * 0.5;
                if (ramp <= 0.0) {
                    envelope = 1.0;
                } else {
                    const double from_start = (double)(position - e.start), to_end = (double)(e.stop - position);
                    envelope = 1.0;
                    if (from_start < ramp) envelope *= 0.5 - 0.5 * cos(pi * from_start / ramp);
                    if (to_end <= ramp) envelope *= 0.5 - 0.5 * cos(pi * to_end / ramp);
                }
            }
            const double level = r.level * envelope;
            float2& o = out[index - r.first];
            o = make_float2(o.x + (float)(level * cr), o.y + (float)(level * ci));
        }
        const double ncr = cr * r.c_step_re - ci * r.c_step_im, nci = cr * r.c_step_im + ci * r.c_step_re;
        cr = ncr, ci = nci;
    }
}

// One FSK segment (modulators.cpp:1393-1441): a unit phasor anchored at
// `anchor` and advanced by one rotation per sample, written over
// [begin, stop). Segments end at symbol boundaries and at the 1024-sample
// anchor grid; their anchors' and rotations' cos/sin come from the host.
struct FskSegment {
    uint64_t anchor, begin, stop;
    double re, im, step_re, step_im;
};

__global__ void k_fsk_emitter(const FskSegment* __restrict__ seg, uint32_t n, double level, uint64_t first,
                              float2* __restrict__ out) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const FskSegment g = seg[k];
    double re = g.re, im = g.im;
    for (uint64_t index = g.anchor; index < g.stop; ++index) {
        if (index >= g.begin) {
            float2& o = out[index - first];
            o = make_float2(o.x + (float)(level * re), o.y + (float)(level * im));
        }
        const double nre = re * g.step_re - im * g.step_im, nim = re * g.step_im + im * g.step_re;
        re = nre, im = nim;
    }
}

// The FSK segments of emitter indices [first, end): the reference's walk
// (modulators.cpp:1393-1441) with the bits, symbol clock and per-symbol
// phase prefix of Modulator::create (:850-882).
bool fsk_segments(const rv_tone_emitter* e, uint64_t first, uint64_t end, std::vector<FskSegment>& out) {
    SymbolClock clock;
    const std::vector<uint8_t> bits = random_bits(e->symbol_count, e->seed);
    if (!build_symbol_clock(bits.size(), e->rate, e->symbol_rate, clock)) return false;
    const double rate = (double)e->rate;
    const double upper = kTwoPi * (double)e->deviation / rate, lower = -upper;
    std::vector<double> prefix(clock.symbols + 1, 0.0);
    double accumulated = 0.0;
    for (uint64_t k = 0; k < clock.symbols; ++k) {
        prefix[k] = accumulated;
        accumulated += (bits[k] != 0 ? upper : lower) * (double)(clock.boundary[k + 1] - clock.boundary[k]);
        accumulated = fmod(accumulated, kTwoPi);
    }
    const double cycle_phase = accumulated;
    const double carrier_step = kTwoPi * (double)e->carrier_offset / rate;
    const int64_t cycle = clock.cycle;
    uint64_t index = first;
    while (index < end) {
        const int64_t repeat = (int64_t)index / cycle;
        const int64_t position = (int64_t)index - repeat * cycle;
        const uint64_t symbol = clock.index_at(position);
        const int64_t base = repeat * cycle;
        const uint64_t symbol_start = (uint64_t)(base + clock.boundary[symbol]);
        const uint64_t symbol_stop = (uint64_t)(base + clock.boundary[symbol + 1]);
        const uint64_t grid = index - index % kAnchorInterval;
        const uint64_t anchor = grid > symbol_start ? grid : symbol_start;
        uint64_t stop = end < symbol_stop ? end : symbol_stop;
        if (grid + kAnchorInterval < stop) stop = grid + kAnchorInterval;
        const double sense = bits[symbol] != 0 ? 1.0 : -1.0;
        const double phase = e->initial_phase + exact_phase(e->carrier_offset, e->rate, anchor) +
                             fmod((double)repeat * cycle_phase, kTwoPi) + prefix[symbol] +
                             sense * upper * (double)(anchor - symbol_start);
        const double step = carrier_step + sense * upper;
        out.push_back(FskSegment{anchor, index, stop, cos(phase), sin(phase), cos(step), sin(step)});
        index = stop;
    }
    return true;
}

// ---- PSK (Modulator::accumulate_psk, modulators.cpp:1443-1527) ----------
struct PskDev {
    const float* sym_re;
    const float* sym_im;
    const float* rrc;
    const double* boundary_d;
    const int64_t* boundary;
    double scale, base, limit, cycle_span, gain, level, c_step_re, c_step_im;
    int64_t cycle, stride;
    uint64_t symbols, span, first, count, first_anchor;
};

__device__ double d_rrc_tap(const PskDev& p, double position) {
    if (position <= 0.0 || position >= p.limit) return 0.0;
    const uint64_t lower = (uint64_t)position;
    const double fraction = position - (double)lower;
    const double a = (double)p.rrc[lower], b = (double)p.rrc[lower + 1];
    return a + fraction * (b - a);
}

__device__ uint64_t d_index_at(const PskDev& p, int64_t position) {
    uint64_t e = (uint64_t)((position * (int64_t)p.symbols) / p.cycle);
    if (e >= p.symbols) e = p.symbols - 1;
    while (e + 1 < p.symbols && p.boundary[e + 1] <= position) ++e;
    while (e > 0 && p.boundary[e] > position) --e;
    return e;
}

// modulators.cpp:1104-1151 psk_envelope: the pulses of the 2 span + 1 nearest
// symbols, wrapped around the repeating payload, in offset order
__device__ float2 d_psk_envelope(const PskDev& p, int64_t position_in_cycle, uint64_t symbol) {
    const int64_t symbols = (int64_t)p.symbols, span = (int64_t)p.span;
    const double position = (double)position_in_cycle;
    double in_phase = 0.0, quadrature = 0.0;
    for (int64_t offset = -span; offset <= span; ++offset) {
        int64_t wrapped = (int64_t)symbol + offset;
        double shift = 0.0;
        if (wrapped < 0) {
            wrapped += symbols;
            shift = -p.cycle_span;
        } else if (wrapped >= symbols) {
            wrapped -= symbols;
            shift = p.cycle_span;
        }
        const double centre = p.boundary_d[wrapped] + shift;
        const double tap = d_rrc_tap(p, (position - centre) * p.scale + p.base);
        if (tap == 0.0) continue;
        in_phase += (double)p.sym_re[wrapped] * tap;
        quadrature += (double)p.sym_im[wrapped] * tap;
    }
    return make_float2((float)(in_phase * p.gain), (float)(quadrature * p.gain));
}

__device__ float2 d_psk_envelope_at(const PskDev& p, uint64_t index) {
    const int64_t position = (int64_t)(index % (uint64_t)p.cycle);
    return d_psk_envelope(p, position, d_index_at(p, position));
}

__global__ void k_psk_emitter(PskDev p, const Anchor* __restrict__ anchors, uint32_t segments,
                              float2* __restrict__ out) {
    const uint32_t seg = blockIdx.x * blockDim.x + threadIdx.x;
    if (seg >= segments) return;
    const uint64_t anchor = p.first_anchor + (uint64_t)seg * kAnchorInterval;
    const uint64_t end = p.first + p.count;
    const uint64_t stop = anchor + kAnchorInterval < end ? anchor + kAnchorInterval : end;
    uint64_t index = anchor > p.first ? anchor : p.first;
    double cr = anchors[seg].cr, ci = anchors[seg].ci;
    for (uint64_t k = anchor; k < index; ++k) {
        const double ncr = cr * p.c_step_re - ci * p.c_step_im, nci = cr * p.c_step_im + ci * p.c_step_re;
        cr = ncr, ci = nci;
    }
    if (p.stride == 1) {
        int64_t position = (int64_t)(index % (uint64_t)p.cycle);
        uint64_t symbol = d_index_at(p, position);
        for (; index < stop; ++index) {
            const float2 env = d_psk_envelope(p, position, symbol);
            const double ip = (double)env.x, qd = (double)env.y;
            const double re = ip * cr - qd * ci, im = ip * ci + qd * cr;
            float2& o = out[index - p.first];
            o = make_float2(o.x + (float)(p.level * re), o.y + (float)(p.level * im));
            const double ncr = cr * p.c_step_re - ci * p.c_step_im, nci = cr * p.c_step_im + ci * p.c_step_re;
            cr = ncr, ci = nci;
            ++position;
            if (position >= p.cycle) {
                position = 0;
                symbol = 0;
            } else if (position >= p.boundary[symbol + 1]) {
                ++symbol;
            }
        }
        return;
    }
    // the envelope interpolated between evaluations at absolute multiples of the stride
    const double inverse_stride = 1.0 / (double)p.stride;
    uint64_t node = index - index % (uint64_t)p.stride;
    float2 near_point = d_psk_envelope_at(p, node), far_point = d_psk_envelope_at(p, node + (uint64_t)p.stride);
    for (; index < stop; ++index) {
        if (index >= node + (uint64_t)p.stride) {
            node += (uint64_t)p.stride;
            near_point = far_point;
            far_point = d_psk_envelope_at(p, node + (uint64_t)p.stride);
        }
        const double weight = (double)(index - node) * inverse_stride;
        const double lr = (double)near_point.x, li = (double)near_point.y;
        const double ip = lr + weight * ((double)far_point.x - lr);
        const double qd = li + weight * ((double)far_point.y - li);
        const double re = ip * cr - qd * ci, im = ip * ci + qd * cr;
        float2& o = out[index - p.first];
        o = make_float2(o.x + (float)(p.level * re), o.y + (float)(p.level * im));
        const double ncr = cr * p.c_step_re - ci * p.c_step_im, nci = cr * p.c_step_im + ci * p.c_step_re;
        cr = ncr, ci = nci;
    }
}

// ---- supplied audio (modulators.cpp:1244-1392 with spec.audio) -----------
struct AudioRun {
    const float* audio;      // AM and SSB: the audio; NFM: unused
    const double* phase;     // NFM: the FM phase integral, audio_len + 1 values
    const double* hilbert;   // SSB: the transformer's taps
    uint64_t audio_len, taps, first, count, first_anchor;
    double level, index, sense, c_step_re, c_step_im;
    int32_t kind;
};

__device__ __forceinline__ double audio_at(const AudioRun& r, uint64_t i) {
    return i < r.audio_len ? (double)r.audio[i] : 0.0;
}

__global__ void k_audio_emitter(AudioRun r, const Anchor* __restrict__ anchors, uint32_t segments,
                                float2* __restrict__ out) {
    const uint32_t seg = blockIdx.x * blockDim.x + threadIdx.x;
    if (seg >= segments) return;
    const uint64_t anchor = r.first_anchor + (uint64_t)seg * kAnchorInterval;
    const uint64_t end = r.first + r.count;
    const uint64_t stop = anchor + kAnchorInterval < end ? anchor + kAnchorInterval : end;
    double cr = anchors[seg].cr, ci = anchors[seg].ci;
    for (uint64_t index = anchor; index < stop; ++index) {
        if (index >= r.first) {
            float2 add;
            if (r.kind == RV_EMITTER_AM) {
                const double envelope = r.level * (1.0 + r.index * audio_at(r, index));
                add = make_float2((float)(envelope * cr), (float)(envelope * ci));
            } else if (r.kind == RV_EMITTER_NFM) {
                const uint64_t last = r.audio_len;  // phase has audio_len + 1 values
                const double deviation = r.phase[index < last ? index : last];
                const double cosine = cos(deviation), sine = sin(deviation);
                const double re = cr * cosine - ci * sine, im = cr * sine + ci * cosine;
                add = make_float2((float)(r.level * re), (float)(r.level * im));
            } else {
                // hilbert_at: odd lags only, ascending tap index
                const int64_t half = (int64_t)(r.taps / 2), centre = (int64_t)index;
                double total = 0.0;
                for (uint64_t i = (half % 2) == 0 ? 1u : 0u; i < r.taps; i += 2) {
                    const int64_t source = centre + half - (int64_t)i;
                    if (source < 0) continue;
                    total += r.hilbert[i] * audio_at(r, (uint64_t)source);
                }
                const double in_phase = audio_at(r, index), quadrature = r.sense * total;
                const double re = in_phase * cr - quadrature * ci, im = in_phase * ci + quadrature * cr;
                add = make_float2((float)(r.level * re), (float)(r.level * im));
            }
            float2& o = out[index - r.first];
            o = make_float2(o.x + add.x, o.y + add.y);
        }
        const double ncr = cr * r.c_step_re - ci * r.c_step_im, nci = cr * r.c_step_im + ci * r.c_step_re;
        cr = ncr, ci = nci;
    }
}

}  // namespace
}  // namespace rv

using namespace rv;

extern "C" int32_t rv_emitter_accumulate(void* stream, const rv_tone_emitter* e, uint64_t first, uint64_t count,
                                         double gain, rv_cf32* out, uint64_t out_len) {
    if (e == nullptr || (out == nullptr && count > 0)) return set_error_fmt(RV_ERR_INVALID, "emitter: NULL argument");
    if (e->modulation < RV_EMITTER_CW || e->modulation > RV_EMITTER_QPSK)
        return set_error_fmt(RV_ERR_UNSUPPORTED, "emitter: modulation %d (a siggen::Modulation)", e->modulation);
    const bool fsk = e->modulation == RV_EMITTER_FSK2;
    const bool psk = e->modulation == RV_EMITTER_BPSK || e->modulation == RV_EMITTER_QPSK;
    const bool ssb = e->modulation == RV_EMITTER_USB || e->modulation == RV_EMITTER_LSB;
    // modulators.cpp:310-332 validate_common, :334-343 the tone, :517-546 the mode
    if (e->rate <= 0 || e->rate > 1000000000) return set_error_fmt(RV_ERR_INVALID, "emitter: rate %lld", (long long)e->rate);
    if (!isfinite(e->amplitude) || e->amplitude < 0.0 || !isfinite(e->initial_phase))
        return set_error_fmt(RV_ERR_INVALID, "emitter: amplitude and initial phase must be finite (amplitude >= 0)");
    if (llabs(e->carrier_offset) * 2 > e->rate) return set_error_fmt(RV_ERR_INVALID, "emitter: carrier past Nyquist");
    const bool cw = e->modulation == RV_EMITTER_CW;
    if (fsk) {  // modulators.cpp:593-609
        if (!isfinite(e->symbol_rate) || e->symbol_rate <= 0.0 || e->deviation <= 0 || e->symbol_count == 0)
            return set_error_fmt(RV_ERR_INVALID, "emitter: FSK needs a positive symbol rate, deviation and count");
        if ((llabs(e->carrier_offset) + e->deviation) * 2 > e->rate)
            return set_error_fmt(RV_ERR_INVALID, "emitter: FSK tones past Nyquist");
    }
    if (psk) {  // modulators.cpp:612-631
        if (!isfinite(e->symbol_rate) || e->symbol_rate <= 0.0 || !isfinite(e->rolloff) || e->rolloff < 0.0 ||
            e->rolloff > 1.0 || e->span_symbols == 0 || e->symbol_count == 0)
            return set_error_fmt(RV_ERR_INVALID, "emitter: PSK needs a positive baud, rolloff in [0, 1], span and count");
    }
    if (!cw && !fsk && !psk && (e->tone_hz <= 0 || e->tone_hz * 2 >= e->rate))
        return set_error_fmt(RV_ERR_INVALID, "emitter: tone past Nyquist");
    if (cw) {  // modulators.cpp:485-515
        if (!isfinite(e->words_per_minute) || e->words_per_minute <= 0.0 || !isfinite(e->rise_fall_ms) ||
            e->rise_fall_ms < 0.0 || !isfinite(e->message_gap_dots) || e->message_gap_dots < 0.0)
            return set_error_fmt(RV_ERR_INVALID, "emitter: CW timing must be positive (rise/fall and gap >= 0)");
        if (1.2 * (double)e->rate / e->words_per_minute < 2.0)
            return set_error_fmt(RV_ERR_INVALID, "emitter: CW dot shorter than two samples");
        if (memchr(e->text, 0, sizeof e->text) == nullptr)
            return set_error_fmt(RV_ERR_INVALID, "emitter: CW text is not NUL-terminated");
        bool keyed = false;
        for (const char* c = e->text; *c != '\0'; ++c) {
            if (*c == ' ') continue;
            if (morse(*c) == nullptr) return set_error_fmt(RV_ERR_INVALID, "emitter: no Morse code for '%c'", *c);
            keyed = true;
        }
        if (!keyed) return set_error_fmt(RV_ERR_INVALID, "emitter: CW text has nothing to key");
    }
    if (e->modulation == RV_EMITTER_AM && (!isfinite(e->modulation_index) || e->modulation_index < 0.0))
        return set_error_fmt(RV_ERR_INVALID, "emitter: AM modulation index must be finite and >= 0");
    if (e->modulation == RV_EMITTER_NFM && e->deviation <= 0)
        return set_error_fmt(RV_ERR_INVALID, "emitter: NFM deviation must be positive");
    if (ssb) {  // modulators.cpp:547-569
        if (e->audio_low_hz <= 0 || e->audio_high_hz <= e->audio_low_hz)
            return set_error_fmt(RV_ERR_INVALID, "emitter: SSB audio passband must be a positive increasing range");
        if (e->tone_hz < e->audio_low_hz || e->tone_hz > e->audio_high_hz)
            return set_error_fmt(RV_ERR_INVALID, "emitter: SSB tone outside the audio passband");
        if (e->tone2_hz != 0 && (e->tone2_hz <= 0 || e->tone2_hz * 2 >= e->rate || e->tone2_hz < e->audio_low_hz ||
                                 e->tone2_hz > e->audio_high_hz))
            return set_error_fmt(RV_ERR_INVALID, "emitter: SSB second tone outside the audio passband");
    }
    if (out_len < count) return set_error_fmt(RV_ERR_INVALID, "emitter: output too short");
    if (count == 0) return clear_error();
    if (first + count < first) return set_error_fmt(RV_ERR_INVALID, "emitter: range wraps");
    ToneRun r{};
    r.kind = e->modulation;
    r.level = gain * e->amplitude;
    r.index = e->modulation_index;
    r.beta = (double)e->deviation / (double)e->tone_hz;
    // the two phasors: carrier and tone, or (SSB) carrier +/- tone 1 and tone 2
    const int64_t sense = e->modulation == RV_EMITTER_LSB ? -1 : 1;
    const int64_t f1 = ssb ? e->carrier_offset + sense * e->tone_hz : e->carrier_offset;
    const int64_t f2 = ssb ? e->carrier_offset + sense * e->tone2_hz : e->tone_hz;
    const double p2 = ssb ? e->initial_phase : 0.0;
    r.two_tone = ssb && e->tone2_hz != 0;
    if (ssb) r.level = r.two_tone ? 0.5 * r.level : r.level;
    const double c_step = kTwoPi * (double)f1 / (double)e->rate;
    const double t_step = kTwoPi * (double)f2 / (double)e->rate;
    r.c_step_re = cos(c_step), r.c_step_im = sin(c_step);
    r.t_step_re = cos(t_step), r.t_step_im = sin(t_step);
    r.first = first, r.count = count;
    if (fsk) {
        std::vector<FskSegment> segs;
        if (!fsk_segments(e, first, first + count, segs))
            return set_error_fmt(RV_ERR_INVALID, "emitter: FSK symbol clock unusable at this rate and baud");
        cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
        FskSegment* d = nullptr;
        if (int32_t st = cuda_status(cudaMallocAsync(&d, segs.size() * sizeof(FskSegment), s), "fsk segments"))
            return st;
        int32_t st = cuda_status(cudaMemcpyAsync(d, segs.data(), segs.size() * sizeof(FskSegment),
                                                 cudaMemcpyHostToDevice, s),
                                 "fsk segments");
        if (st == RV_OK) {
            k_fsk_emitter<<<(unsigned)((segs.size() + 127) / 128), 128, 0, s>>>(d, (uint32_t)segs.size(), r.level, first,
                                                                             reinterpret_cast<float2*>(out));
            st = cuda_status(cudaGetLastError(), "fsk emitter");
        }
        cudaFreeAsync(d, s);
        if (st == RV_OK) st = cuda_status(cudaStreamSynchronize(s), "fsk emitter");
        return st ? st : clear_error();
    }
    r.first_anchor = first - first % kAnchorInterval;
    const uint64_t segs = (first + count - r.first_anchor + kAnchorInterval - 1) / kAnchorInterval;
    PskPlan plan;
    if (psk && !psk_plan(e->modulation == RV_EMITTER_QPSK, e->symbol_count, e->seed, e->rate, e->symbol_rate,
                         e->rolloff, e->span_symbols, plan))
        return set_error_fmt(RV_ERR_INVALID, "emitter: PSK payload shorter than its pulse, or symbol clock unusable");
    if (segs > (1u << 30)) return set_error_fmt(RV_ERR_INVALID, "emitter: range too long");
    std::vector<Anchor> anchors(segs);
    for (uint64_t k = 0; k < segs; ++k) {
        const uint64_t a = r.first_anchor + k * kAnchorInterval;
        const double cp = e->initial_phase + exact_phase(f1, e->rate, a);
        const double tp = p2 + exact_phase(f2, e->rate, a);
        anchors[k] = Anchor{cos(cp), sin(cp), cos(tp), sin(tp)};
    }
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    Anchor* d_anchors = nullptr;
    if (int32_t st = cuda_status(cudaMallocAsync(&d_anchors, segs * sizeof(Anchor), s), "emitter anchors")) return st;
    int32_t st = cuda_status(cudaMemcpyAsync(d_anchors, anchors.data(), segs * sizeof(Anchor), cudaMemcpyHostToDevice, s),
                             "emitter anchors");
    // PSK tables in one device allocation: symbols (re, im), pulse, boundaries
    void* d_psk = nullptr;
    PskDev pd{};
    if (st == RV_OK && psk) {
        const size_t n = plan.clock.symbols, t = plan.rrc.size();
        const size_t bytes = n * 4 * 2 + t * 4 + 64 + n * 8 + (n + 1) * 8 + 64;
        st = cuda_status(cudaMallocAsync(&d_psk, bytes, s), "psk tables");
        if (st == RV_OK) {
            std::vector<uint8_t> blob(bytes, 0);
            size_t at = 0;
            auto put = [&](const void* src, size_t len) {
                const size_t o = (at + 15) & ~size_t(15);
                memcpy(blob.data() + o, src, len);
                at = o + len;
                return o;
            };
            const size_t o_re = put(plan.sym_re.data(), n * 4), o_im = put(plan.sym_im.data(), n * 4);
            const size_t o_rrc = put(plan.rrc.data(), t * 4), o_bd = put(plan.boundary_d.data(), n * 8);
            const size_t o_b = put(plan.clock.boundary.data(), (n + 1) * 8);
            st = cuda_status(cudaMemcpyAsync(d_psk, blob.data(), at, cudaMemcpyHostToDevice, s), "psk tables");
            cudaStreamSynchronize(s);  // the host blob goes out of scope
            uint8_t* b = static_cast<uint8_t*>(d_psk);
            pd.sym_re = reinterpret_cast<const float*>(b + o_re);
            pd.sym_im = reinterpret_cast<const float*>(b + o_im);
            pd.rrc = reinterpret_cast<const float*>(b + o_rrc);
            pd.boundary_d = reinterpret_cast<const double*>(b + o_bd);
            pd.boundary = reinterpret_cast<const int64_t*>(b + o_b);
        }
        pd.scale = plan.scale, pd.base = plan.base, pd.limit = plan.limit, pd.cycle_span = plan.cycle_span;
        pd.gain = plan.gain, pd.level = r.level, pd.c_step_re = r.c_step_re, pd.c_step_im = r.c_step_im;
        pd.cycle = plan.clock.cycle, pd.stride = plan.stride, pd.symbols = plan.clock.symbols, pd.span = plan.span;
        pd.first = first, pd.count = count, pd.first_anchor = r.first_anchor;
    }
    std::vector<CwElement> elements;
    CwElement* d_elements = nullptr;
    if (st == RV_OK && cw) {
        elements = cw_elements(e->text, 1.2 * (double)e->rate / e->words_per_minute, e->message_gap_dots);
        st = cuda_status(cudaMallocAsync(&d_elements, elements.size() * sizeof(CwElement), s), "emitter elements");
        if (st == RV_OK)
            st = cuda_status(cudaMemcpyAsync(d_elements, elements.data(), elements.size() * sizeof(CwElement),
                                             cudaMemcpyHostToDevice, s),
                             "emitter elements");
    }
    if (st == RV_OK) {
        const unsigned grid = (unsigned)((segs + 127) / 128);
        if (psk)
            k_psk_emitter<<<grid, 128, 0, s>>>(pd, d_anchors, (uint32_t)segs, reinterpret_cast<float2*>(out));
        else if (cw)
            k_cw_emitter<<<grid, 128, 0, s>>>(r, d_anchors, (uint32_t)segs, d_elements, (uint32_t)elements.size(),
                                              e->rise_fall_ms * 0.001 * (double)e->rate,
                                              reinterpret_cast<float2*>(out));
        else
            k_tone_emitter<<<grid, 128, 0, s>>>(r, d_anchors, (uint32_t)segs, reinterpret_cast<float2*>(out));
        st = cuda_status(cudaGetLastError(), "emitter");
    }
    if (d_elements) cudaFreeAsync(d_elements, s);
    if (d_psk) cudaFreeAsync(d_psk, s);
    cudaFreeAsync(d_anchors, s);
    // the host table must outlive the copy
    if (st == RV_OK) st = cuda_status(cudaStreamSynchronize(s), "emitter");
    return st ? st : clear_error();
}

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

extern "C" int32_t rv_emitter_accumulate_audio(void* stream, const rv_tone_emitter* e, const float* audio,
                                               uint64_t audio_len, uint32_t hilbert_taps, uint64_t first,
                                               uint64_t count, double gain, rv_cf32* out, uint64_t out_len) {
    if (e == nullptr || (audio == nullptr && audio_len > 0) || (out == nullptr && count > 0))
        return set_error_fmt(RV_ERR_INVALID, "emitter audio: NULL argument");
    const int32_t m = e->modulation;
    if (m != RV_EMITTER_AM && m != RV_EMITTER_NFM && m != RV_EMITTER_USB && m != RV_EMITTER_LSB)
        return set_error_fmt(RV_ERR_UNSUPPORTED, "emitter audio: AM, NFM, USB or LSB");
    if (e->rate <= 0 || e->rate > 1000000000 || !isfinite(e->amplitude) || e->amplitude < 0.0 ||
        !isfinite(e->initial_phase) || llabs(e->carrier_offset) * 2 > e->rate)
        return set_error_fmt(RV_ERR_INVALID, "emitter audio: rate, amplitude, phase or carrier");
    if (m == RV_EMITTER_AM && (!isfinite(e->modulation_index) || e->modulation_index < 0.0))
        return set_error_fmt(RV_ERR_INVALID, "emitter audio: AM modulation index");
    if (m == RV_EMITTER_NFM && e->deviation <= 0) return set_error_fmt(RV_ERR_INVALID, "emitter audio: NFM deviation");
    const bool ssb = m == RV_EMITTER_USB || m == RV_EMITTER_LSB;
    if (ssb) {  // modulators.cpp:550-552, :570-587
        if (e->audio_low_hz <= 0 || e->audio_high_hz <= e->audio_low_hz)
            return set_error_fmt(RV_ERR_INVALID, "emitter audio: SSB audio passband must be a positive increasing range");
        if (hilbert_taps < 3 || hilbert_taps % 2 == 0)
            return set_error_fmt(RV_ERR_INVALID, "emitter audio: Hilbert transformer length must be odd and >= 3");
        if ((double)e->audio_low_hz < (double)e->rate / (double)hilbert_taps)
            return set_error_fmt(RV_ERR_INVALID, "emitter audio: the Hilbert transformer does not reach the passband");
    }
    if (out_len < count) return set_error_fmt(RV_ERR_INVALID, "emitter audio: output too short");
    if (count == 0) return clear_error();
    const double rate = (double)e->rate;
    AudioRun r{};
    r.kind = m, r.level = gain * e->amplitude, r.index = e->modulation_index;
    r.sense = m == RV_EMITTER_LSB ? -1.0 : 1.0;
    r.audio_len = audio_len, r.taps = hilbert_taps, r.first = first, r.count = count;
    r.first_anchor = first - first % kAnchorInterval;
    const double step = kTwoPi * (double)e->carrier_offset / rate;
    r.c_step_re = cos(step), r.c_step_im = sin(step);
    std::vector<double> phase, hilbert;
    if (m == RV_EMITTER_NFM) {  // modulators.cpp:769-780
        phase.assign(audio_len + 1, 0.0);
        const double scale = kTwoPi * (double)e->deviation / rate;
        double accumulated = 0.0;
        for (uint64_t i = 0; i < audio_len; ++i) {
            accumulated += scale * (double)audio[i];
            accumulated = fmod(accumulated, kTwoPi);
            phase[i + 1] = accumulated;
        }
    }
    if (ssb) {  // modulators.cpp:807-823: 2 / (pi lag) under a Blackman window, odd lags
        const double pi = 3.141592653589793238462643383279502884;
        hilbert.assign(hilbert_taps, 0.0);
        const int64_t half = (int64_t)(hilbert_taps / 2);
        for (uint32_t i = 0; i < hilbert_taps; ++i) {
            const int64_t lag = (int64_t)i - half;
            if (lag == 0 || lag % 2 == 0) continue;
            const double ideal = 2.0 / (pi * (double)lag);
            const double position = (double)i / (double)(hilbert_taps - 1);
            const double window = 0.42 - 0.5 * cos(kTwoPi * position) + 0.08 * cos(2.0 * kTwoPi * position);
            hilbert[i] = ideal * window;
        }
    }
    const uint64_t segs = (first + count - r.first_anchor + kAnchorInterval - 1) / kAnchorInterval;
    std::vector<Anchor> anchors(segs);
    for (uint64_t k = 0; k < segs; ++k) {
        const double cp = e->initial_phase + exact_phase(e->carrier_offset, e->rate, r.first_anchor + k * kAnchorInterval);
        anchors[k] = Anchor{cos(cp), sin(cp), 0.0, 0.0};
    }
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const size_t a_bytes = segs * sizeof(Anchor), au_bytes = audio_len * sizeof(float);
    const size_t p_bytes = phase.size() * sizeof(double), h_bytes = hilbert.size() * sizeof(double);
    uint8_t* d = nullptr;
    const size_t total = a_bytes + au_bytes + p_bytes + h_bytes + 64;
    if (int32_t st = cuda_status(cudaMallocAsync(reinterpret_cast<void**>(&d), total, s), "emitter audio")) return st;
    size_t at = 0;
    auto put = [&](const void* src, size_t len) -> uint8_t* {
        at = (at + 15) & ~size_t(15);
        uint8_t* where = d + at;
        if (len) cudaMemcpyAsync(where, src, len, cudaMemcpyHostToDevice, s);
        at += len;
        return where;
    };
    const Anchor* d_anchors = reinterpret_cast<const Anchor*>(put(anchors.data(), a_bytes));
    r.audio = reinterpret_cast<const float*>(put(audio, au_bytes));
    r.phase = reinterpret_cast<const double*>(put(phase.data(), p_bytes));
    r.hilbert = reinterpret_cast<const double*>(put(hilbert.data(), h_bytes));
    k_audio_emitter<<<(unsigned)((segs + 127) / 128), 128, 0, s>>>(r, d_anchors, (uint32_t)segs,
                                                                  reinterpret_cast<float2*>(out));
    int32_t st = cuda_status(cudaGetLastError(), "emitter audio");
    cudaFreeAsync(d, s);
    if (st == RV_OK) st = cuda_status(cudaStreamSynchronize(s), "emitter audio");
    return st ? st : clear_error();
}
