// Per-receiver noise stages (core/dsp/noise_reference.cpp; the shaders
// core/shaders/noise_blank.comp, noise_line.comp, noise_spectral.comp).
//
//   blank detect  flag[j] = sum > 0 and |x[j]|^2 W > T sum, the sum over the
//                 W channel samples ending `guard` before j, oldest first.
//                 A block stages the powers of its samples and of the window
//                 behind them in shared memory once; each thread then sums its
//                 own W in order.
//   blank apply   blanked[i] = 0 where a flag lies in [i - hang, i + lead].
//   line          a cascade of up to four notch sections, then a normalised
//                 leaky LMS predictor (adaptive line enhancer) whose error is
//                 the output. The predictor's taps are split over `lanes`
//                 threads, lane l owning taps l, l + lanes, ...; each lane sums
//                 its products in tap order and the partial sums are added in
//                 lane order, the twin's order. One block per call, the state
//                 held in shared memory for the call.
//   spectral      50 % overlap-add with square-root Hann windows, a direct DFT
//                 per bin (one thread per bin, terms in index order), power
//                 smoothing, minimum tracking and over-subtraction with a gain
//                 floor, the inverse per sample (one thread per sample). One
//                 block per call; frames are sequential through the state.
// Every product and sum is a rounded fp32 operation in the twin's order.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <cmath>

#include "common.cuh"

namespace {

using rv::cuda_status;
using rv::set_error_fmt;

constexpr double kPi = 3.14159265358979323846;
constexpr double kBlankWindowSeconds = 0.5e-3;
constexpr uint32_t kBlankHang = 2;
constexpr uint32_t kBlankThreads = 256;

bool is_mask(uint32_t m) { return rv::is_pow2((uint64_t)m + 1u); }
__host__ __device__ inline uint32_t line_sections(uint32_t flags) {
    return (flags & RV_LINE_NOTCH) == 0u ? 0u : 1u + ((flags >> RV_LINE_NOTCH_COUNT_SHIFT) & 3u);
}

// ---- validation (noise_reference.cpp:127-156, 231-263, 556-566) ----------

int32_t validate_blanker(const rv_blanker_config& c, const rv_blanker_params& p, const char* who) {
    if (c.pass != RV_BLANK_DETECT && c.pass != RV_BLANK_APPLY)
        return set_error_fmt(RV_ERR_INVALID, "%s: pass %u is neither detect nor apply", who, c.pass);
    if (c.window < RV_BLANK_MIN_WINDOW || c.window > RV_BLANK_MAX_WINDOW)
        return set_error_fmt(RV_ERR_INVALID, "%s: a %u sample window is outside [%u, %u]", who, c.window,
                             RV_BLANK_MIN_WINDOW, RV_BLANK_MAX_WINDOW);
    if (!is_mask(p.chan_mask) || !is_mask(p.out_mask))
        return set_error_fmt(RV_ERR_INVALID, "%s: masks %#x and %#x must each be a power of two minus one", who,
                             p.chan_mask, p.out_mask);
    const uint64_t reach = (uint64_t)c.hang + c.guard + c.window + c.lead + p.count;
    const uint64_t smaller = (uint64_t)std::min(p.chan_mask, p.out_mask) + 1u;
    if (reach >= smaller)
        return set_error_fmt(RV_ERR_INVALID, "%s: %u samples plus their reach do not fit a %llu sample ring", who,
                             p.count, (unsigned long long)smaller);
    if (!(p.threshold > 0.0F)) return set_error_fmt(RV_ERR_INVALID, "%s: the threshold must be a positive power ratio", who);
    return RV_OK;
}

int32_t validate_line(const rv_line_config& c, const rv_line_params& p) {
    if (c.lanes == 0 || c.taps == 0 || c.taps % c.lanes != 0)
        return set_error_fmt(RV_ERR_INVALID, "noise line: %u taps do not divide over %u lanes", c.taps, c.lanes);
    if (!rv::is_pow2(c.history))
        return set_error_fmt(RV_ERR_INVALID, "noise line: a history of %u is not a power of two", c.history);
    if (p.stride == 0 || p.stride > RV_LINE_MAX_STRIDE)
        return set_error_fmt(RV_ERR_INVALID, "noise line: stride %u is outside [1, %u]", p.stride, RV_LINE_MAX_STRIDE);
    if (p.delay == 0) return set_error_fmt(RV_ERR_INVALID, "noise line: the predictor's delay must be at least one sample");
    const uint64_t reach = (uint64_t)p.delay + (uint64_t)(c.taps - 1u) * p.stride;
    if (reach >= c.history)
        return set_error_fmt(RV_ERR_INVALID, "noise line: a predictor reaching %llu samples back does not fit a %u sample history",
                             (unsigned long long)reach, c.history);
    if (!(p.eps > 0.0F)) return set_error_fmt(RV_ERR_INVALID, "noise line: the normalisation's eps must be positive");
    if ((p.flags & ~(uint32_t)(RV_LINE_NOTCH | RV_LINE_ALE | RV_LINE_GUARD | (3u << RV_LINE_NOTCH_COUNT_SHIFT))) != 0u)
        return set_error_fmt(RV_ERR_INVALID, "noise line: flags %#x set a bit the kernel does not read", p.flags);
    return RV_OK;
}

int32_t validate_spectral(const rv_spectral_config& c, const rv_spectral_params& p) {
    if (!rv::is_pow2(c.frame) || c.frame < RV_SPECTRAL_MIN_FRAME || c.frame > RV_SPECTRAL_MAX_FRAME)
        return set_error_fmt(RV_ERR_INVALID, "noise reduction: a frame of %u is not a power of two in [%u, %u]", c.frame,
                             RV_SPECTRAL_MIN_FRAME, RV_SPECTRAL_MAX_FRAME);
    if (!(p.eps > 0.0F)) return set_error_fmt(RV_ERR_INVALID, "noise reduction: eps must be positive");
    return RV_OK;
}

// ---- blanker -------------------------------------------------------------

__device__ __forceinline__ float power_of(float2 s) { return s.x * s.x + s.y * s.y; }

// Dynamic shared memory: the powers of samples [i0 - guard - window, i0 + blockDim).
__global__ void k_blank_detect(rv_blanker_config c, rv_blanker_params p, const float2* __restrict__ chan,
                               float* __restrict__ flags) {
    extern __shared__ float pw[];
    const uint32_t i0 = blockIdx.x * blockDim.x;
    const uint32_t behind = c.guard + c.window;
    const uint32_t staged = behind + blockDim.x;
    for (uint32_t u = threadIdx.x; u < staged; u += blockDim.x) {
        const uint32_t at = (p.chan_first + i0 - behind + u) & p.chan_mask;
        pw[u] = power_of(__ldg(chan + p.chan_base + at));
    }
    __syncthreads();
    const uint32_t i = i0 + threadIdx.x;
    if (i >= p.count) return;
    const float pj = pw[behind + threadIdx.x];
    float sum = 0.0F;
    for (uint32_t m = 0; m < c.window; ++m) sum = sum + pw[threadIdx.x + m];  // oldest first
    const float lhs = pj * (float)c.window;
    const float rhs = p.threshold * sum;
    flags[(p.out_first + i) & p.out_mask] = (sum > 0.0F && lhs > rhs) ? 1.0F : 0.0F;
}

__global__ void k_blank_apply(rv_blanker_config c, rv_blanker_params p, const float2* __restrict__ chan,
                              const float* __restrict__ flags, float2* __restrict__ blanked) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.count) return;
    const uint32_t ch = (p.chan_first + i) & p.chan_mask;
    const uint32_t o = (p.out_first + i) & p.out_mask;
    bool hit = false;
    for (uint32_t m = 0; m <= c.hang + c.lead; ++m) hit = hit || flags[(o - c.hang + m) & p.out_mask] != 0.0F;
    blanked[o] = hit ? make_float2(0.0F, 0.0F) : __ldg(chan + p.chan_base + ch);
}

// ---- line ----------------------------------------------------------------

struct Biquad {
    float x1, x2, y1, y2;
};

// y = b0 x + b1 x1 + b2 x2 - a1 y1 - a2 y2, the twin's operation order.
__device__ __forceinline__ float biquad(Biquad& s, float b0, float b1, float b2, float a1, float a2, float x) {
    const float t0 = b0 * x;
    const float t1 = b1 * s.x1;
    const float t2 = b2 * s.x2;
    const float t3 = a1 * s.y1;
    const float t4 = a2 * s.y2;
    float acc = t0 + t1;
    acc = acc + t2;
    acc = acc - t3;
    acc = acc - t4;
    s.x2 = s.x1;
    s.x1 = x;
    s.y2 = s.y1;
    s.y1 = acc;
    return acc;
}

// One block of `lanes` threads. Dynamic shared memory: weights[taps],
// reference[taps], history[history], part_y[lanes], part_p[lanes].
__global__ void k_noise_line(rv_line_config c, rv_line_params p, float* __restrict__ audio, float* __restrict__ state) {
    extern __shared__ float sm[];
    float* w = sm;
    float* ref = w + c.taps;
    float* hist = ref + c.taps;
    float* part_y = hist + c.history;
    float* part_p = part_y + c.lanes;
    __shared__ float s_v, s_out;
    const uint32_t lane = threadIdx.x;
    for (uint32_t k = lane; k < c.taps + c.history; k += blockDim.x) {
        const float v = state[RV_LINE_STATE_WEIGHTS + k];
        if (k < c.taps)
            w[k] = v;
        else
            hist[k - c.taps] = v;
    }
    const bool notch = (p.flags & RV_LINE_NOTCH) != 0u;
    const bool ale = (p.flags & RV_LINE_ALE) != 0u;
    const bool guard = ale && (p.flags & RV_LINE_GUARD) != 0u;
    const uint32_t sections = line_sections(p.flags);
    const uint32_t per_lane = c.taps / c.lanes;
    const uint32_t hmask = c.history - 1u;
    // the scalar recursions run on thread 0
    Biquad n0{state[0], state[1], state[2], state[3]};
    Biquad more[3];
    for (uint32_t s = 0; s < 3; ++s) {
        more[s] = Biquad{0, 0, 0, 0};
        if (s + 1u < sections)
            more[s] = Biquad{state[RV_LINE_STATE_MORE + 4 * s], state[RV_LINE_STATE_MORE + 4 * s + 1],
                             state[RV_LINE_STATE_MORE + 4 * s + 2], state[RV_LINE_STATE_MORE + 4 * s + 3]};
    }
    Biquad g{state[RV_LINE_STATE_GUARD], state[RV_LINE_STATE_GUARD + 1], state[RV_LINE_STATE_GUARD + 2],
             state[RV_LINE_STATE_GUARD + 3]};
    uint32_t position = (uint32_t)state[RV_LINE_STATE_POSITION];
    __syncthreads();
    for (uint32_t n = 0; n < p.count; ++n) {
        if (lane == 0) {
            const float x = audio[n];
            float v = x;
            if (notch) {
                v = biquad(n0, p.b0, p.b1, p.b2, p.a1, p.a2, x);
                for (uint32_t s = 0; s + 1u < sections; ++s)
                    v = biquad(more[s], p.more[s].b0, p.more[s].b1, p.more[s].b2, p.more[s].a1, p.more[s].a2, v);
            }
            s_v = v;
            s_out = v;
        }
        if (ale) {
            __syncthreads();
            float py = 0.0F, pp = 0.0F;
            for (uint32_t j = 0; j < per_lane; ++j) {
                const uint32_t k = lane + j * c.lanes;
                const float r = hist[(position - p.delay - k * p.stride) & hmask];
                ref[k] = r;
                const float wy = w[k] * r;
                py = py + wy;
                const float rr = r * r;
                pp = pp + rr;
            }
            part_y[lane] = py;
            part_p[lane] = pp;
            __syncthreads();
            float y = 0.0F, pwr = 0.0F;
            for (uint32_t l = 0; l < c.lanes; ++l) {
                y = y + part_y[l];
                pwr = pwr + part_p[l];
            }
            const float v = s_v;
            const float e = v - y;
            const float gain = p.mu * rv::det_recip(pwr + p.eps);
            const float ge = gain * e;
            for (uint32_t j = 0; j < per_lane; ++j) {
                const uint32_t k = lane + j * c.lanes;
                const float kept = p.leak * w[k];
                const float step = ge * ref[k];
                w[k] = kept + step;
            }
            __syncthreads();  // every lane has read the history before it moves
            if (lane == 0) {
                hist[position & hmask] = v;
                float out = e;
                if (guard) out = v - biquad(g, p.gb0, p.gb1, p.gb2, p.ga1, p.ga2, y);
                s_out = out;
            }
        }
        if (lane == 0) audio[n] = s_out;
        position = position + 1u;
    }
    __syncthreads();
    for (uint32_t k = lane; k < c.taps + c.history; k += blockDim.x)
        state[RV_LINE_STATE_WEIGHTS + k] = k < c.taps ? w[k] : hist[k - c.taps];
    if (lane == 0) {
        state[0] = n0.x1;
        state[1] = n0.x2;
        state[2] = n0.y1;
        state[3] = n0.y2;
        for (uint32_t s = 0; s + 1u < sections; ++s) {
            state[RV_LINE_STATE_MORE + 4 * s] = more[s].x1;
            state[RV_LINE_STATE_MORE + 4 * s + 1] = more[s].x2;
            state[RV_LINE_STATE_MORE + 4 * s + 2] = more[s].y1;
            state[RV_LINE_STATE_MORE + 4 * s + 3] = more[s].y2;
        }
        state[RV_LINE_STATE_POSITION] = (float)(position & hmask);
        state[RV_LINE_STATE_GUARD] = g.x1;
        state[RV_LINE_STATE_GUARD + 1] = g.x2;
        state[RV_LINE_STATE_GUARD + 2] = g.y1;
        state[RV_LINE_STATE_GUARD + 3] = g.y2;
    }
}

// ---- spectral ------------------------------------------------------------

// One block of N threads. Dynamic shared memory: cos, sin, analysis,
// synthesis [N each], hist [N], tail [H], queue [H], smoothed [K], minimum
// [K], work [N], y_re [K], y_im [K].
__global__ void k_noise_spectral(uint32_t n, rv_spectral_params p, const float* __restrict__ tables,
                                 float* __restrict__ audio, float* __restrict__ state) {
    extern __shared__ float sm[];
    const uint32_t h = n / 2u, bins = h + 1u, mask = n - 1u;
    float* cosine = sm;
    float* sine = cosine + n;
    float* analysis = sine + n;
    float* synthesis = analysis + n;
    float* hist = synthesis + n;
    float* tail = hist + n;
    float* queue = tail + h;
    float* smoothed = queue + h;
    float* minimum = smoothed + bins;
    float* work = minimum + bins;
    float* y_re = work + n;
    float* y_im = y_re + bins;
    const uint32_t t = threadIdx.x;
    for (uint32_t i = t; i < 4u * n; i += blockDim.x) cosine[i] = tables[i];
    // state: [0] phase, [1] frames seen, then hist, tail, queue, smoothed, minimum (contiguous, as here)
    const uint32_t body = n + h + h + 2u * bins;
    for (uint32_t i = t; i < body; i += blockDim.x) hist[i] = state[2 + i];
    uint32_t phase = (uint32_t)state[0];
    float seen = state[1];
    __syncthreads();
    uint32_t s = 0;
    while (s < p.count) {
        const uint32_t length = min(h - phase, p.count - s);
        for (uint32_t i = t; i < length; i += blockDim.x) {
            const float x = audio[s + i];
            hist[h + phase + i] = x;
            audio[s + i] = queue[phase + i];
        }
        phase += length;
        s += length;
        if (phase != h) break;  // the call ends inside a hop
        __syncthreads();
        work[t] = hist[t] * analysis[t];
        __syncthreads();
        if (t < bins) {
            const uint32_t k = t;
            float re = 0.0F, im = 0.0F;
            for (uint32_t u = 0; u < n; ++u) {
                const uint32_t at = (k * u) & mask;
                const float xc = work[u] * cosine[at];
                re = re + xc;
                const float xs = work[u] * sine[at];
                im = im - xs;
            }
            const float rr = re * re;
            const float ii = im * im;
            const float power = rr + ii;
            float level = power, floor_power = power;
            if (seen != 0.0F) {
                const float previous = smoothed[k];
                const float kept = p.smoothing * previous;
                const float fresh = p.smoothing_complement * power;
                level = kept + fresh;
                const float held = minimum[k];
                if (held < level) {
                    const float decayed = p.gamma * held;
                    const float lagged = p.beta * previous;
                    const float lift = level - lagged;
                    const float risen = p.rise * lift;
                    floor_power = decayed + risen;
                } else {
                    floor_power = level;
                }
            }
            smoothed[k] = level;
            minimum[k] = floor_power;
            const float noise = p.bias * floor_power;
            const float ratio = noise * rv::det_recip(level + p.eps);
            const float cut = p.alpha * ratio;
            float gain = 1.0F - cut;
            gain = fmaxf(gain, p.floor_gain);
            y_re[k] = gain * re;
            y_im[k] = gain * im;
        }
        __syncthreads();
        {
            float acc = 0.0F;
            for (uint32_t k = 1; k < h; ++k) {
                const uint32_t at = (k * t) & mask;
                const float a = y_re[k] * cosine[at];
                const float b = y_im[k] * sine[at];
                const float term = a - b;
                acc = acc + term;
            }
            const float nyquist = (t & 1u) != 0u ? -y_re[h] : y_re[h];
            const float doubled = 2.0F * acc;
            float sum = y_re[0] + nyquist;
            sum = sum + doubled;
            work[t] = sum * synthesis[t];
        }
        __syncthreads();
        if (t < h) {
            queue[t] = tail[t] + work[t];
            tail[t] = work[h + t];
            hist[t] = hist[h + t];
        }
        __syncthreads();
        phase = 0;
        seen = fminf(seen + 1.0F, 2.0F);
    }
    __syncthreads();
    for (uint32_t i = t; i < body; i += blockDim.x) state[2 + i] = hist[i];
    if (t == 0) {
        state[0] = (float)phase;
        state[1] = seen;
    }
}

}  // namespace

extern "C" {

// ---- host designers --------------------------------------------------------

int32_t rv_design_blanker(int64_t channel_rate, rv_blanker_config* out) {
    if (out == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_design_blanker: NULL");
    memset(out, 0, sizeof *out);
    const double window = std::round(kBlankWindowSeconds * (double)channel_rate);
    out->window = (uint32_t)std::clamp(window, (double)RV_BLANK_MIN_WINDOW, (double)RV_BLANK_MAX_WINDOW);
    out->hang = kBlankHang;
    out->lead = kBlankHang;
    out->guard = out->lead + 2u;
    return rv::clear_error();
}

float rv_blanker_threshold(double threshold_db) { return (float)std::pow(10.0, threshold_db / 10.0); }

int32_t rv_design_notch(double audio_hz, double depth_db, double width_hz, int64_t audio_rate, rv_notch_design* out) {
    if (out == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_design_notch: NULL");
    if (audio_rate <= 0) return set_error_fmt(RV_ERR_INVALID, "notch: no audio rate to design at");
    const double fa = (double)audio_rate;
    if (!(audio_hz > 0.0) || !(audio_hz < 0.5 * fa))
        return set_error_fmt(RV_ERR_INVALID, "notch: %g Hz is not inside the audio band of a %lld S/s stream", audio_hz,
                             (long long)audio_rate);
    if (!(width_hz > 0.0) || !(width_hz < 0.25 * fa))
        return set_error_fmt(RV_ERR_INVALID, "notch: a %g Hz width does not fit a %lld S/s stream", width_hz,
                             (long long)audio_rate);
    // poles at rp = 1 - pi w / Fa on the notch's angle, zeros at
    // rz = 1 - (1 - rp) 10^(-depth/20), unit gain at the far band edge
    const double omega = 2.0 * kPi * audio_hz / fa;
    const double rp = 1.0 - kPi * width_hz / fa;
    const double rz = 1.0 - (1.0 - rp) * std::pow(10.0, -depth_db / 20.0);
    const double c = std::cos(omega);
    rv_notch_design d;
    d.b0 = 1.0;
    d.b1 = -2.0 * rz * c;
    d.b2 = rz * rz;
    d.a1 = -2.0 * rp * c;
    d.a2 = rp * rp;
    const double z = (omega < 0.5 * kPi) ? -1.0 : 1.0;
    const double numerator = d.b0 + d.b1 * z + d.b2;
    const double denominator = 1.0 + d.a1 * z + d.a2;
    const double scale = denominator / numerator;
    d.b0 *= scale;
    d.b1 *= scale;
    d.b2 *= scale;
    *out = d;
    return rv::clear_error();
}

uint64_t rv_line_state_size(const rv_line_config* c) {
    return c == nullptr ? 0u : (uint64_t)RV_LINE_STATE_WEIGHTS + c->taps + c->history;
}

int32_t rv_spectral_config_for(int64_t audio_rate, rv_spectral_config* out) {
    if (out == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_spectral_config_for: NULL");
    const uint64_t wanted = audio_rate > 0 ? (uint64_t)audio_rate / 90u : (uint64_t)RV_SPECTRAL_MIN_FRAME;
    uint64_t floor = 1;
    while (floor * 2u <= std::max<uint64_t>(wanted, 1u)) floor *= 2u;
    out->frame = (uint32_t)std::clamp<uint64_t>(floor, RV_SPECTRAL_MIN_FRAME, RV_SPECTRAL_MAX_FRAME);
    return rv::clear_error();
}

int32_t rv_design_spectral_tables(const rv_spectral_config* c, float* tables, uint64_t len) {
    if (c == nullptr || tables == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_design_spectral_tables: NULL");
    const uint32_t n = c->frame;
    if (!rv::is_pow2(n) || n < RV_SPECTRAL_MIN_FRAME || n > RV_SPECTRAL_MAX_FRAME)
        return set_error_fmt(RV_ERR_INVALID, "rv_design_spectral_tables: frame %u", n);
    if (len < 4ull * n) return set_error_fmt(RV_ERR_INVALID, "rv_design_spectral_tables: %llu floats, 4N wanted",
                                             (unsigned long long)len);
    const double step = 2.0 * kPi / (double)n;
    for (uint32_t k = 0; k < n; ++k) {
        double cs = std::cos(step * (double)k), sn = std::sin(step * (double)k);
        // the quarter and half points exactly, so the table is exactly odd
        if (k == 0) {
            cs = 1.0;
            sn = 0.0;
        } else if (4u * k == n) {
            cs = 0.0;
            sn = 1.0;
        } else if (2u * k == n) {
            cs = -1.0;
            sn = 0.0;
        } else if (4u * k == 3u * n) {
            cs = 0.0;
            sn = -1.0;
        }
        tables[k] = (float)cs;
        tables[n + k] = (float)sn;
        // square-root Hann offset half a sample; the synthesis one carries 1/N
        const double window = std::sin(kPi * ((double)k + 0.5) / (double)n);
        tables[2u * n + k] = (float)window;
        tables[3u * n + k] = (float)(window / (double)n);
    }
    return rv::clear_error();
}

int32_t rv_design_spectral_params(double strength, rv_spectral_params* out) {
    if (out == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_design_spectral_params: NULL");
    const double s = std::clamp(strength, 0.0, 1.0);
    memset(out, 0, sizeof *out);
    out->smoothing = (float)0.7;
    out->smoothing_complement = (float)(1.0 - 0.7);
    out->gamma = (float)0.998;
    out->beta = (float)0.96;
    out->rise = (float)((1.0 - 0.998) / (1.0 - 0.96));
    out->bias = (float)2.4;
    out->alpha = (float)(1.0 + s);
    out->floor_gain = (float)std::pow(10.0, -(6.0 + 12.0 * s) / 20.0);
    out->eps = (float)1.0e-12;
    return rv::clear_error();
}

uint64_t rv_spectral_state_size(const rv_spectral_config* c) {
    if (c == nullptr) return 0u;
    const uint64_t n = c->frame;
    return 2u + n + n / 2u + n / 2u + 2u * (n / 2u + 1u);
}

// ---- launches --------------------------------------------------------------

int32_t rv_blank_detect(void* stream, const rv_blanker_config* config, const rv_blanker_params* params,
                        const rv_cf32* chan, uint64_t chan_len, float* flags, uint64_t flags_len) {
    if (config == nullptr || params == nullptr || chan == nullptr || flags == nullptr)
        return set_error_fmt(RV_ERR_INVALID, "rv_blank_detect: NULL argument");
    rv_blanker_config c = *config;
    c.pass = RV_BLANK_DETECT;
    if (int32_t st = validate_blanker(c, *params, "rv_blank_detect")) return st;
    if (flags_len < (uint64_t)params->out_mask + 1u)
        return set_error_fmt(RV_ERR_INVALID, "rv_blank_detect: %llu flags for a %llu sample ring",
                             (unsigned long long)flags_len, (unsigned long long)params->out_mask + 1u);
    if (chan_len < (uint64_t)params->chan_base + params->chan_mask + 1u)
        return set_error_fmt(RV_ERR_INVALID, "rv_blank_detect: the channel ring is shorter than its base and mask");
    if (params->count == 0) return rv::clear_error();
    const uint32_t smem = (c.guard + c.window + kBlankThreads) * sizeof(float);
    k_blank_detect<<<(params->count + kBlankThreads - 1u) / kBlankThreads, kBlankThreads, smem, (cudaStream_t)stream>>>(
        c, *params, reinterpret_cast<const float2*>(chan), flags);
    if (int32_t st = cuda_status(cudaGetLastError(), "rv_blank_detect")) return st;
    return rv::clear_error();
}

int32_t rv_blank_apply(void* stream, const rv_blanker_config* config, const rv_blanker_params* params,
                       const rv_cf32* chan, uint64_t chan_len, const float* flags, uint64_t flags_len, rv_cf32* blanked,
                       uint64_t blanked_len) {
    if (config == nullptr || params == nullptr || chan == nullptr || flags == nullptr || blanked == nullptr)
        return set_error_fmt(RV_ERR_INVALID, "rv_blank_apply: NULL argument");
    rv_blanker_config c = *config;
    c.pass = RV_BLANK_APPLY;
    if (int32_t st = validate_blanker(c, *params, "rv_blank_apply")) return st;
    if (flags_len < (uint64_t)params->out_mask + 1u || blanked_len < (uint64_t)params->out_mask + 1u)
        return set_error_fmt(RV_ERR_INVALID, "rv_blank_apply: the flag and blanked rings must each hold out_mask + 1 values");
    if (chan_len < (uint64_t)params->chan_base + params->chan_mask + 1u)
        return set_error_fmt(RV_ERR_INVALID, "rv_blank_apply: the channel ring is shorter than its base and mask");
    if (params->count == 0) return rv::clear_error();
    k_blank_apply<<<(params->count + 255u) / 256u, 256, 0, (cudaStream_t)stream>>>(
        c, *params, reinterpret_cast<const float2*>(chan), flags, reinterpret_cast<float2*>(blanked));
    if (int32_t st = cuda_status(cudaGetLastError(), "rv_blank_apply")) return st;
    return rv::clear_error();
}

int32_t rv_noise_line(void* stream, const rv_line_config* config, const rv_line_params* params, float* audio,
                      uint64_t audio_len, float* state, uint64_t state_len) {
    if (config == nullptr || params == nullptr || audio == nullptr || state == nullptr)
        return set_error_fmt(RV_ERR_INVALID, "rv_noise_line: NULL argument");
    if (int32_t st = validate_line(*config, *params)) return st;
    if (audio_len < params->count)
        return set_error_fmt(RV_ERR_INVALID, "rv_noise_line: %u samples asked of a %llu sample buffer", params->count,
                             (unsigned long long)audio_len);
    if (state_len < rv_line_state_size(config))
        return set_error_fmt(RV_ERR_INVALID, "rv_noise_line: a %llu float state where %llu are needed",
                             (unsigned long long)state_len, (unsigned long long)rv_line_state_size(config));
    if (config->lanes > 1024u) return set_error_fmt(RV_ERR_UNSUPPORTED, "rv_noise_line: %u lanes", config->lanes);
    const size_t smem = ((size_t)2u * config->taps + config->history + 2u * config->lanes) * sizeof(float);
    if (smem > 200u * 1024u)
        return set_error_fmt(RV_ERR_UNSUPPORTED, "rv_noise_line: %zu bytes of state exceed shared memory", smem);
    if (smem > 48u * 1024u)
        if (int32_t st = cuda_status(cudaFuncSetAttribute(k_noise_line, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                                     "rv_noise_line"))
            return st;
    k_noise_line<<<1, config->lanes, smem, (cudaStream_t)stream>>>(*config, *params, audio, state);
    if (int32_t st = cuda_status(cudaGetLastError(), "rv_noise_line")) return st;
    return rv::clear_error();
}

int32_t rv_noise_spectral(void* stream, const rv_spectral_config* config, const rv_spectral_params* params,
                          const float* tables, uint64_t tables_len, float* audio, uint64_t audio_len, float* state,
                          uint64_t state_len) {
    if (config == nullptr || params == nullptr || tables == nullptr || audio == nullptr || state == nullptr)
        return set_error_fmt(RV_ERR_INVALID, "rv_noise_spectral: NULL argument");
    if (int32_t st = validate_spectral(*config, *params)) return st;
    const uint32_t n = config->frame;
    if (tables_len < 4ull * n)
        return set_error_fmt(RV_ERR_INVALID, "rv_noise_spectral: %llu table entries where %u are needed",
                             (unsigned long long)tables_len, 4u * n);
    if (audio_len < params->count)
        return set_error_fmt(RV_ERR_INVALID, "rv_noise_spectral: %u samples asked of a %llu sample buffer", params->count,
                             (unsigned long long)audio_len);
    if (state_len < rv_spectral_state_size(config))
        return set_error_fmt(RV_ERR_INVALID, "rv_noise_spectral: a %llu float state where %llu are needed",
                             (unsigned long long)state_len, (unsigned long long)rv_spectral_state_size(config));
    const uint32_t bins = n / 2u + 1u;
    const size_t smem = ((size_t)4u * n + n + n / 2u + n / 2u + 2u * bins + n + 2u * bins) * sizeof(float);
    k_noise_spectral<<<1, n, smem, (cudaStream_t)stream>>>(n, *params, tables, audio, state);
    if (int32_t st = cuda_status(cudaGetLastError(), "rv_noise_spectral")) return st;
    return rv::clear_error();
}

}  // extern "C"
