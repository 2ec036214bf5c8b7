/*
 * planner.c — CPU restatement of the reference's receive-chain planner.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT. It lets the oracle chain (and bench.py's
 * reference arm) build every table and block parameter itself, without the
 * GPU library: the prototype (core/dsp/pfb_design.cpp:381-513), the twiddle
 * circle (:515-590), the NCO circle (core/dsp/vrx_reference.cpp:364), receiver
 * placement (core/engine/vrx_place.cpp:199-330), plan_vrx and its tables
 * (core/dsp/vrx_reference.cpp:1201-2662) and the block parameters
 * (resample_block :2786-2850, demod_block :2873, carrier_block :2911).
 *
 * Tables are designed in double and rounded to float once, with the
 * reference's formulas in its association order, so they equal the
 * reference's bit for bit; tests/test_oracle_planner.py checks that against
 * the reference's own planner compiled from source (oracle/ref) and against
 * the GPU library's planner. Integer placement and rate planning is exact
 * rational arithmetic.
 */
#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

#define PI 3.14159265358979323846264338327950288
#define TWO_PI (2.0 * PI)
#define FINE_ATTENUATION_DB 80.0
#define AUDIO_ATTENUATION_DB 80.0
#define COMPOSITE_AUDIO_RATE 114000

int32_t or_fail(const char* fmt, ...);

static int64_t iabs64(int64_t v) { return v < 0 ? -v : v; }
static int64_t imin64(int64_t a, int64_t b) { return a < b ? a : b; }
static int64_t imax64(int64_t a, int64_t b) { return a > b ? a : b; }
static int64_t iclamp64(int64_t v, int64_t lo, int64_t hi) { return v < lo ? lo : (v > hi ? hi : v); }
static uint32_t uclamp(uint32_t v, uint32_t lo, uint32_t hi) { return v < lo ? lo : (v > hi ? hi : v); }

static int64_t gcd64(int64_t a, int64_t b) {
    a = iabs64(a);
    b = iabs64(b);
    while (b != 0) {
        const int64_t t = a % b;
        a = b;
        b = t;
    }
    return a;
}

static void reduce_rational(int64_t* num, int64_t* den) {
    if (*den < 0) {
        *num = -*num;
        *den = -*den;
    }
    const int64_t g = gcd64(*num, *den);
    if (g > 1) {
        *num /= g;
        *den /= g;
    }
}

/* ---- Kaiser design primitives (the published formulas) ---------------- */

static double bessel_i0(double x) {
    const double quarter_square = 0.25 * x * x;
    double term = 1.0, sum = 1.0;
    for (int k = 1; k < 256; ++k) {
        term *= quarter_square / ((double)k * (double)k);
        sum += term;
        if (term < 1e-18 * sum) break;
    }
    return sum;
}

static double kaiser_beta(double attenuation_db) {
    if (attenuation_db > 50.0) return 0.1102 * (attenuation_db - 8.7);
    if (attenuation_db >= 21.0) {
        const double excess = attenuation_db - 21.0;
        return 0.5842 * pow(excess, 0.4) + 0.07886 * excess;
    }
    return 0.0;
}

static uint32_t kaiser_taps_for(double attenuation_db, double transition_fraction) {
    if (!(transition_fraction > 0.0)) return 0;
    const double transition_radians = TWO_PI * transition_fraction;
    const double order = (attenuation_db - 8.0) / (2.285 * transition_radians);
    if (!(order > 0.0)) return 2;
    return (uint32_t)ceil(order) + 1u;
}

static double sinc_pi(double z) {
    if (z == 0.0) return 1.0;
    const double scaled = PI * z;
    return sin(scaled) / scaled;
}

static double kaiser_window(size_t index, size_t length, double beta, double i0_beta) {
    if (length < 2) return 1.0;
    const double position = 2.0 * (double)index / (double)(length - 1) - 1.0;
    const double inner = fmax(0.0, 1.0 - position * position);
    return bessel_i0(beta * sqrt(inner)) / i0_beta;
}

/* ---- prototype, twiddles, NCO ------------------------------------------ */

int32_t or_design_prototype(const rv_grid_params* g, double attenuation_db, float* taps, uint64_t taps_len) {
    if (g == NULL || taps == NULL) return or_fail("design_prototype: NULL");
    const uint32_t M = g->channels;
    if (M < 2 || M > 2048 || (M & (M - 1)) != 0 || g->taps_per_branch < 1 || g->decimation == 0 ||
        M % g->decimation != 0)
        return or_fail("design_prototype: grid M=%u T=%u D=%u", M, g->taps_per_branch, g->decimation);
    if (taps_len != (uint64_t)M * g->taps_per_branch) return or_fail("design_prototype: %llu taps", (unsigned long long)taps_len);
    const uint32_t L = g->taps_per_branch - 1u;
    const size_t design_length = (size_t)M * L, used = design_length + 1;
    const double reachable = 2.285 * PI * (double)L + 8.0;
    const double design_db = attenuation_db < reachable ? attenuation_db : reachable;
    const double beta = kaiser_beta(design_db);
    const double i0_beta = bessel_i0(beta);
    const double centre = 0.5 * (double)design_length;
    const double inverse_channels = 1.0 / (double)M;
    double* work = (double*)calloc(used, sizeof(double));
    if (work == NULL) return or_fail("design_prototype: out of memory");
    double sum = 0.0;
    for (size_t n = 0; n < used; ++n) {
        const double offset = (double)n - centre;
        const double position = (centre > 0.0) ? offset / centre : 0.0;
        const double radicand = fmax(0.0, 1.0 - position * position);
        const double window = bessel_i0(beta * sqrt(radicand)) / i0_beta;
        const double angle = PI * offset * inverse_channels;
        const double sinc = (offset == 0.0) ? 1.0 : sin(angle) / angle;
        work[n] = inverse_channels * sinc * window;
        sum += work[n];
    }
    memset(taps, 0, taps_len * sizeof(float));
    for (size_t n = 0; n < used; ++n) taps[n] = (float)(work[n] / sum);
    free(work);
    return 0;
}

static float unsigned_zero(double v) {
    const float f = (float)v;
    return f == 0.0f ? 0.0f : f;
}

int32_t or_build_twiddles(uint32_t M, rv_cf32* out, uint64_t len) {
    if (out == NULL || M == 0 || (M & (M - 1)) != 0 || M > 2048 || len != M) return or_fail("build_twiddles: %u", M);
    const uint32_t half = M / 2, quarter = M / 4, octant = M / 8;
    double* oc = (double*)calloc(octant + 1, sizeof(double));
    double* os = (double*)calloc(octant + 1, sizeof(double));
    double* re = (double*)calloc(M, sizeof(double));
    double* im = (double*)calloc(M, sizeof(double));
    for (uint32_t i = 0; i <= octant; ++i) {
        const double a = 2.0 * PI * (double)i / (double)M;
        oc[i] = cos(a);
        os[i] = sin(a);
    }
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
    for (uint32_t j = 0; j < M; ++j) {
        out[j].re = unsigned_zero(re[j]);
        out[j].im = unsigned_zero(im[j]);
    }
    free(oc);
    free(os);
    free(re);
    free(im);
    return 0;
}

int32_t or_build_nco_table(uint32_t log2, rv_cf32* out, uint64_t len) {
    if (out == NULL || log2 > 24 || len != (1ull << log2)) return or_fail("build_nco_table: log2 %u", log2);
    const uint32_t size = 1u << log2;
    if (size == 1) {
        out[0].re = 1.0f;
        out[0].im = 0.0f;
        return 0;
    }
    const uint32_t quarter = size / 4u, octant = size / 8u;
    double* c = (double*)calloc(size, sizeof(double));
    double* s = (double*)calloc(size, sizeof(double));
    for (uint32_t i = 0; i <= octant; ++i) {
        const double a = TWO_PI * (double)i / (double)size;
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
    for (uint32_t i = 0; i < size; ++i) {
        out[i].re = (c[i] == 0.0) ? 0.0f : (float)c[i];
        out[i].im = (s[i] == 0.0) ? 0.0f : (float)(-s[i]);
    }
    free(c);
    free(s);
    return 0;
}

/* ---- exact NCO phase (vrx_reference.cpp:308-362) ----------------------- */

static uint64_t turn_fixed64(int64_t numerator, int64_t denominator) {
    if (denominator <= 0 || numerator < 0 || numerator >= denominator) return 0;
    int64_t rem = numerator;
    uint64_t q = 0;
    for (int step = 0; step < 4; ++step) {
        rem <<= 16;
        q = (q << 16) | (uint64_t)(rem / denominator);
        rem %= denominator;
    }
    if (2 * rem >= denominator) ++q;
    return q;
}

static int32_t nco_delta(int64_t hz_num, int64_t hz_den, int64_t rate, uint64_t* out) {
    if (hz_den == 0 || rate <= 0) return or_fail("nco_delta: bad rational");
    int64_t num = hz_num, den = hz_den;
    reduce_rational(&num, &den);
    const int64_t period = den * rate;
    if (period <= 0 || period > ((int64_t)1 << 31)) return or_fail("nco_delta: period %lld", (long long)period);
    int64_t reduced = num % period;
    if (reduced < 0) reduced += period;
    *out = turn_fixed64(reduced, period);
    return 0;
}

/* ---- passbands and rates (vrx_reference.cpp:1201-1760) ---------------- */

typedef struct Band {
    int64_t low, high;
} Band;

static int64_t band_width(Band b) { return b.high - b.low; }
static int64_t band_reach(Band b, int64_t o) {
    const int64_t below = o - b.low, above = b.high - o;
    return below > above ? below : above;
}

static int is_complex_mode(uint32_t m) {
    return m == RV_DEMOD_RAW || m == RV_DEMOD_P25P1 || m == RV_DEMOD_DSTAR || m == RV_DEMOD_TETRA || m == RV_DEMOD_DMR;
}

static Band default_passband(uint32_t mode) {
    Band b = {0, 0};
    switch (mode) {
        case RV_DEMOD_RAW: b.low = -6000, b.high = 6000; break;
        case RV_DEMOD_AM:
        case RV_DEMOD_SAM: b.low = -5000, b.high = 5000; break;
        case RV_DEMOD_NFM: b.low = -8000, b.high = 8000; break;
        case RV_DEMOD_WFM: b.low = -100000, b.high = 100000; break;
        case RV_DEMOD_USB: b.low = 300, b.high = 2700; break;
        case RV_DEMOD_LSB: b.low = -2700, b.high = -300; break;
        case RV_DEMOD_DSB: b.low = -3000, b.high = 3000; break;
        case RV_DEMOD_CW: b.low = -600, b.high = 600; break;
        case RV_DEMOD_P25P1: b.low = -6250, b.high = 6250; break;
        case RV_DEMOD_DSTAR: b.low = -3000, b.high = 3000; break;
        case RV_DEMOD_TETRA: b.low = -12500, b.high = 12500; break;
        case RV_DEMOD_DMR: b.low = -6250, b.high = 6250; break;
        default: break;
    }
    return b;
}

static int32_t resolve_passband(const rv_vrx_request* r, Band* out) {
    if (r->passband_low != 0 || r->passband_high != 0) {
        if (r->passband_low >= r->passband_high) return or_fail("resolve_passband: empty or inverted passband");
        out->low = r->passband_low;
        out->high = r->passband_high;
        return 0;
    }
    if (r->bandwidth < 0) return or_fail("resolve_passband: negative bandwidth");
    if (r->bandwidth == 0) {
        *out = default_passband(r->demod);
        if (band_width(*out) <= 0) return or_fail("resolve_passband: no default passband for mode %u", r->demod);
        return 0;
    }
    if (r->demod > 12) return or_fail("resolve_passband: mode %u", r->demod);
    const int64_t half = r->bandwidth / 2;
    if (r->demod == RV_DEMOD_USB) {
        out->low = 0;
        out->high = r->bandwidth;
    } else if (r->demod == RV_DEMOD_LSB) {
        out->low = -r->bandwidth;
        out->high = 0;
    } else {
        out->low = -half;
        out->high = half;
    }
    return 0;
}

static int64_t max_channel_bandwidth(const rv_vrx_placement* p) {
    if (p->channel_rate <= 0 || p->residual_denominator <= 0) return 0;
    const int64_t scaled = p->channel_rate * p->residual_denominator - 2 * iabs64(p->residual_numerator);
    if (scaled <= 0) return 0;
    return scaled / p->residual_denominator;
}

static Band clamp_to_channel(const rv_vrx_placement* p, Band b) {
    const int64_t widest = max_channel_bandwidth(p);
    Band out = {0, 0};
    if (widest <= 0) return out;
    const int64_t limit = widest / 2;
    out.low = iclamp64(b.low, -limit, limit);
    out.high = iclamp64(b.high, -limit, limit);
    return out;
}

static Band mix_frame(Band b, uint32_t mode, int64_t pitch) {
    if (mode == RV_DEMOD_CW) {
        b.low += pitch;
        b.high += pitch;
    }
    return b;
}

static int64_t minimum_demod_rate(uint32_t mode, Band b) {
    const int64_t width = band_width(b);
    if (width <= 0) return 0;
    const int64_t shape_floor = (3 * width + 1) / 2;
    const int64_t floor_rate = imax64(shape_floor, 2 * band_reach(b, 0));
    switch (mode) {
        case RV_DEMOD_AM: return imax64(floor_rate, 2 * width);
        case RV_DEMOD_P25P1:
        case RV_DEMOD_DSTAR:
        case RV_DEMOD_DMR: return imax64(floor_rate, 9600);
        case RV_DEMOD_TETRA: return imax64(floor_rate, 36000);
        default: return floor_rate;
    }
}

static int64_t complex_tap_rate_step(uint32_t mode) {
    switch (mode) {
        case RV_DEMOD_P25P1:
        case RV_DEMOD_DSTAR:
        case RV_DEMOD_DMR: return 48000;
        case RV_DEMOD_TETRA: return 72000;
        default: return 0;
    }
}

static int64_t fm_deviation(uint32_t mode, int64_t bandwidth) {
    if (bandwidth <= 0) return 0;
    if (mode == RV_DEMOD_NFM) return imax64(1, bandwidth / 5);
    if (mode == RV_DEMOD_WFM) return imax64(1, (3 * bandwidth) / 8);
    return 0;
}

static float demod_gain(uint32_t mode, int64_t demod_rate, int64_t deviation) {
    if (mode != RV_DEMOD_NFM && mode != RV_DEMOD_WFM) return 1.0f;
    if (deviation <= 0 || demod_rate <= 0) return 1.0f;
    return (float)((double)demod_rate / (TWO_PI * (double)deviation));
}

/* ---- per-receiver tables (vrx_reference.cpp:1808-2242) ----------------- */

static int32_t design_fine_taps(const rv_vrx_fine_config* c, int64_t channel_rate, int64_t half_width, int64_t centre_num,
                                int64_t centre_den, double attenuation_db, rv_cf32* table) {
    if (c->taps < 2 || c->taps > 256 || c->phases < 1 || c->phases > 4096 || channel_rate <= 0 || half_width <= 0 ||
        2 * half_width >= channel_rate || centre_den == 0)
        return or_fail("design_fine_taps: bad parameters");
    const size_t phases = c->phases, taps = c->taps, length = phases * taps;
    const double centre = ((double)length - 1.0) / 2.0;
    const double cutoff = (double)half_width / (double)channel_rate;
    const double beta = kaiser_beta(attenuation_db);
    const double i0_beta = bessel_i0(beta);
    double* proto = (double*)calloc(length, sizeof(double));
    if (proto == NULL) return or_fail("design_fine_taps: out of memory");
    for (size_t i = 0; i < length; ++i) {
        const double position = ((double)i - centre) / (double)phases;
        const double window = kaiser_window(i, length, beta, i0_beta);
        proto[i] = 2.0 * cutoff * sinc_pi(2.0 * cutoff * position) * window;
    }
    for (size_t p = 0; p < phases; ++p) {
        double sum = 0.0;
        for (size_t k = 0; k < taps; ++k) sum += proto[p + k * phases];
        if (fabs(sum) < 1e-12) continue;
        for (size_t k = 0; k < taps; ++k) proto[p + k * phases] /= sum;
    }
    const int64_t period = 2 * iabs64(centre_den) * (int64_t)phases * channel_rate;
    const int64_t numerator = (centre_den < 0) ? -centre_num : centre_num;
    for (size_t i = 0; i < length; ++i) {
        const int64_t twice_offset = 2 * (int64_t)i - ((int64_t)length - 1);
        int64_t turns = (numerator * twice_offset) % period;
        if (turns < 0) turns += period;
        const double angle = TWO_PI * (double)turns / (double)period;
        table[i].re = (float)(proto[i] * cos(angle));
        table[i].im = (float)(proto[i] * sin(angle));
    }
    table[length].re = table[length].im = 0.0f;
    free(proto);
    return 0;
}

static int32_t design_audio_taps(uint32_t taps, int64_t demod_rate, int64_t audio_rate, double attenuation_db,
                                 double cutoff_hz, float* out) {
    if (taps == 0 || taps > 4096 || demod_rate <= 0 || audio_rate <= 0 || audio_rate > demod_rate)
        return or_fail("design_audio_taps: bad parameters");
    const double cutoff = (cutoff_hz > 0.0) ? cutoff_hz / (double)demod_rate : 0.45 * (double)audio_rate / (double)demod_rate;
    const double centre = ((double)taps - 1.0) / 2.0;
    const double beta = kaiser_beta(attenuation_db);
    const double i0_beta = bessel_i0(beta);
    double* d = (double*)calloc(taps, sizeof(double));
    double sum = 0.0;
    for (uint32_t i = 0; i < taps; ++i) {
        const double position = (double)i - centre;
        const double window = kaiser_window(i, taps, beta, i0_beta);
        d[i] = 2.0 * cutoff * sinc_pi(2.0 * cutoff * position) * window;
        sum += d[i];
    }
    const double scale = (fabs(sum) < 1e-12) ? 1.0 : 1.0 / sum;
    for (uint32_t i = 0; i < taps; ++i) out[i] = (float)(d[i] * scale);
    free(d);
    return 0;
}

static void design_dc_weights(uint32_t taps, float* out) {
    if (taps <= 1) {
        out[0] = 1.0f;
        return;
    }
    double* w = (double*)calloc(taps, sizeof(double));
    double sum = 0.0;
    for (uint32_t i = 0; i < taps; ++i) {
        const double phase = TWO_PI * (double)(i + 1u) / (double)(taps + 1u);
        w[i] = 0.5 - 0.5 * cos(phase);
        sum += w[i];
    }
    const double scale = (sum < 1e-12) ? 1.0 : 1.0 / sum;
    for (uint32_t i = 0; i < taps; ++i) out[i] = (float)(w[i] * scale);
    free(w);
}

static double deemphasis_seconds(uint32_t curve) {
    if (curve == 2) return 75.0e-6;
    if (curve == 3) return 50.0e-6;
    return 0.0;
}

static uint32_t resolve_deemphasis(uint32_t mode, uint32_t requested, int64_t audio_rate) {
    if (requested != 0) return is_complex_mode(mode) ? 1u : requested;
    if (mode == RV_DEMOD_WFM) return (audio_rate >= COMPOSITE_AUDIO_RATE) ? 1u : 2u;
    return 1u;
}

/* The one-pole de-emphasis response truncated where it falls below FP32's
 * resolution (at most 1024 taps); *count taps into out (room for 1024). */
static int32_t design_deemphasis_taps(uint32_t curve, int64_t audio_rate, float* out, uint32_t* count) {
    const double tau = deemphasis_seconds(curve);
    if (tau <= 0.0) {
        out[0] = 1.0f;
        *count = 1;
        return 0;
    }
    if (audio_rate <= 0) return or_fail("design_deemphasis_taps: audio rate");
    const double period = 1.0 / (double)audio_rate;
    const double pole = exp(-period / tau);
    const double float_floor = 1.0 / 16777216.0;
    const double exact_length = log(float_floor * (1.0 - pole)) / log(pole);
    uint32_t length = (uint32_t)ceil(fmax(1.0, exact_length)) + 1u;
    if (length > 1024u) length = 1024u;
    double response[1024];
    double sum = 0.0, term = 1.0;
    for (uint32_t k = 0; k < length; ++k) {
        response[k] = term;
        sum += term;
        term *= pole;
    }
    const double scale = 1.0 / sum;
    for (uint32_t k = 0; k < length; ++k) out[k] = (float)(response[k] * scale);
    *count = length;
    return 0;
}

/* The decimation filter with the de-emphasis folded in at the audio rate;
 * *count taps into out (room for 4096). */
static int32_t fold_deemphasis(const float* dec, uint32_t ndec, const float* de, uint32_t nde, uint32_t decimation,
                               float* out, uint32_t* count) {
    if (ndec == 0 || nde == 0 || decimation == 0) return or_fail("fold_deemphasis: bad parameters");
    if (nde == 1 && de[0] == 1.0f) {
        memcpy(out, dec, ndec * sizeof(float));
        *count = ndec;
        return 0;
    }
    const size_t stride = decimation;
    const size_t length = ndec + (nde - 1u) * stride;
    if (length > 4096) return or_fail("fold_deemphasis: %zu taps", length);
    double* folded = (double*)calloc(length, sizeof(double));
    for (size_t k = 0; k < nde; ++k) {
        const double weight = (double)de[k];
        const size_t offset = k * stride;
        for (size_t j = 0; j < ndec; ++j) folded[offset + j] += weight * (double)dec[j];
    }
    for (size_t i = 0; i < length; ++i) out[i] = (float)folded[i];
    free(folded);
    *count = (uint32_t)length;
    return 0;
}

static uint32_t stereo_pilot_taps(int64_t demod_rate) {
    if (demod_rate <= 0) return 0;
    const double transition = 3000.0 / (double)demod_rate;
    uint32_t taps = uclamp(kaiser_taps_for(70.0, transition), 16u, 2048u);
    if ((taps % 2u) == 0u) ++taps;
    return taps < 2048u ? taps : 2048u;
}

static int32_t design_stereo_tables(int64_t demod_rate, uint32_t audio_taps, uint32_t pilot_taps, float* pilot,
                                    float* rotation) {
    if (demod_rate <= 0 || pilot_taps == 0 || pilot_taps > 2048 || audio_taps == 0 || audio_taps > 4096 ||
        2 * 19000 >= demod_rate)
        return or_fail("design_stereo_tables: bad parameters");
    const double rate = (double)demod_rate;
    const double cutoff = 1000.0 / rate;
    const double centre = ((double)pilot_taps - 1.0) / 2.0;
    const double beta = kaiser_beta(70.0);
    const double i0_beta = bessel_i0(beta);
    double* proto = (double*)calloc(pilot_taps, sizeof(double));
    double sum = 0.0;
    for (uint32_t k = 0; k < pilot_taps; ++k) {
        const double position = (double)k - centre;
        const double window = kaiser_window(k, pilot_taps, beta, i0_beta);
        proto[k] = 2.0 * cutoff * sinc_pi(2.0 * cutoff * position) * window;
        sum += proto[k];
    }
    const double scale = (fabs(sum) < 1e-12) ? 1.0 : 1.0 / sum;
    const double pilot_turns = 19000.0 / rate;
    for (uint32_t k = 0; k < pilot_taps; ++k) {
        const double turns = fmod(pilot_turns * (double)k, 1.0);
        const double angle = TWO_PI * turns;
        const double weight = proto[k] * scale;
        pilot[2u * k] = (float)(weight * cos(angle));
        pilot[2u * k + 1u] = (float)(weight * sin(angle));
    }
    free(proto);
    const double sub_turns = 2.0 * pilot_turns;
    const int64_t pivot = (int64_t)(audio_taps / 2u);
    for (uint32_t t = 0; t < audio_taps; ++t) {
        const double offset = (double)((int64_t)t - pivot);
        const double turns = fmod(sub_turns * offset, 1.0);
        const double angle = TWO_PI * turns;
        rotation[2u * t] = (float)(2.0 * cos(angle));
        rotation[2u * t + 1u] = (float)(2.0 * sin(angle));
    }
    return 0;
}

static void carrier_gains(double bn, double zeta, int64_t rate, double* k1, double* k2) {
    *k1 = *k2 = 0.0;
    if (!(bn > 0.0) || !(zeta > 0.0) || rate <= 0) return;
    const double period = 1.0 / (double)rate;
    const double theta = bn * period / (zeta + 1.0 / (4.0 * zeta));
    const double d = 1.0 + 2.0 * zeta * theta + theta * theta;
    *k1 = 4.0 * zeta * theta / d;
    *k2 = 4.0 * theta * theta / d;
}

static int32_t design_carrier_loop(int64_t demod_rate, int64_t reach_hz, rv_vrx_carrier_params* out) {
    if (demod_rate <= 0 || reach_hz <= 0) return or_fail("design_carrier_loop: bad parameters");
    const double fs = (double)demod_rate;
    const double zeta = 0.70710678118654752440;
    double k1a, k2a, k1t, k2t;
    carrier_gains(400.0, zeta, demod_rate, &k1a, &k2a);
    carrier_gains(30.0, zeta, demod_rate, &k1t, &k2t);
    memset(out, 0, sizeof *out);
    out->k1_acquire = (float)k1a;
    out->k2_acquire = (float)k2a;
    out->k1_track = (float)k1t;
    out->k2_track = (float)k2t;
    out->level_alpha = (float)(1.0 - exp(-1.0 / (0.005 * fs)));
    out->lock_alpha = (float)(1.0 - exp(-1.0 / (0.020 * fs)));
    const double clamp = TWO_PI * (double)reach_hz / fs;
    out->clamp_radians = (float)(clamp < 0.5 * PI ? clamp : 0.5 * PI);
    out->hold_in = (uint32_t)fmax(1.0, round(0.010 * fs));
    out->hold_out = (uint32_t)fmax(1.0, round(0.200 * fs));
    return 0;
}

/* ---- placement (core/engine/vrx_place.cpp) ----------------------------- */

static int64_t divide_nearest(int64_t num, int64_t den) {
    const int64_t q = num / den, r = num % den;
    const int64_t twice = 2 * (r < 0 ? -r : r);
    if (twice < (den < 0 ? -den : den)) return q;
    return (r < 0) ? q - 1 : q + 1;
}

static int clamp_breaks_demodulator(uint32_t mode) {
    return mode == RV_DEMOD_NFM || mode == RV_DEMOD_WFM || mode == RV_DEMOD_P25P1 || mode == RV_DEMOD_DSTAR ||
           mode == RV_DEMOD_TETRA || mode == RV_DEMOD_DMR;
}

int32_t or_place(const rv_grid_params* g, int64_t rate, const rv_vrx_request* r, rv_vrx_placement* out) {
    if (g == NULL || r == NULL || out == NULL) return or_fail("place: NULL");
    if (g->channels < 2 || (g->channels & (g->channels - 1)) != 0 || g->decimation == 0 || g->channels % g->decimation != 0)
        return or_fail("place: grid");
    if (rate <= 0 || rate % (int64_t)g->decimation != 0) return or_fail("place: rate %lld", (long long)rate);
    const int64_t channel_rate = rate / (int64_t)g->decimation;
    const int64_t nyquist = rate / 2;
    if (r->center > nyquist || r->center < -nyquist) return or_fail("place: centre outside the source");
    if (r->demod > 12) return or_fail("place: mode %u", r->demod);
    Band requested;
    if (resolve_passband(r, &requested)) return -1;
    const int64_t M = g->channels;
    const int64_t signed_index = divide_nearest(r->center * M, rate);
    int64_t wrapped = signed_index % M;
    if (wrapped < 0) wrapped += M;
    memset(out, 0, sizeof *out);
    out->channel = (uint32_t)wrapped;
    const int64_t sidx = (out->channel < g->channels / 2) ? (int64_t)out->channel : (int64_t)out->channel - M;
    int64_t cn = sidx * rate, cd = M;
    const int64_t cg = gcd64(cn, cd);
    if (cg > 1) {
        cn /= cg;
        cd /= cg;
    }
    out->centre_numerator = cn;
    out->centre_denominator = cd;
    out->channel_rate = channel_rate;
    out->residual_numerator = r->center * cd - cn;
    out->residual_denominator = cd;
    const int64_t span = rate * out->residual_denominator;
    while (2 * out->residual_numerator > span) out->residual_numerator -= span;
    while (2 * out->residual_numerator <= -span) out->residual_numerator += span;
    const int64_t dg = gcd64(out->residual_numerator, out->residual_denominator);
    if (dg > 1) {
        out->residual_numerator /= dg;
        out->residual_denominator /= dg;
    }
    const Band granted = clamp_to_channel(out, requested);
    out->granted_low = granted.low;
    out->granted_high = granted.high;
    out->bandwidth_clamped = (granted.low != requested.low || granted.high != requested.high) ? 1u : 0u;
    if (out->bandwidth_clamped && clamp_breaks_demodulator(r->demod)) {
        const Band plan = default_passband(r->demod);
        if (band_width(plan) > 0 && granted.high - granted.low < band_width(plan))
            return or_fail("place: refused rather than narrowed");
    }
    return 0;
}

/* ---- plan_vrx (vrx_reference.cpp:2243-2662) ---------------------------- */

/* The plan's scalars into *p and, when taps / weights are not NULL, its
 * tables (exactly fine_tap_count / demod_weight_count long). */
int32_t or_plan_vrx(const rv_grid_params* g, int64_t rate, const rv_vrx_request* r, const rv_vrx_placement* pl,
                    rv_vrx_plan_info* p, rv_cf32* taps, uint64_t taps_len, float* weights, uint64_t weights_len) {
    if (g == NULL || r == NULL || pl == NULL || p == NULL) return or_fail("plan_vrx: NULL");
    if (rate <= 0 || pl->channel_rate <= 0 || pl->residual_denominator <= 0) return or_fail("plan_vrx: placement");
    memset(p, 0, sizeof *p);
    p->placement = *pl;
    p->mode = r->demod;
    p->channel_rate = pl->channel_rate;
    p->audio_rate = (r->audio_rate > 0) ? r->audio_rate : 48000;
    if (p->mode > 12) return or_fail("plan_vrx: mode %u", p->mode);
    const int complex_output = is_complex_mode(p->mode);
    Band requested;
    if (resolve_passband(r, &requested)) return -1;
    if (max_channel_bandwidth(pl) <= 0 || band_width(clamp_to_channel(pl, requested)) <= 0)
        return or_fail("plan_vrx: the channel carries nothing of the passband");
    const Band band = clamp_to_channel(pl, requested);
    p->passband_low = band.low;
    p->passband_high = band.high;
    p->bandwidth = band_width(band);
    p->bandwidth_clamped = (band.low != requested.low || band.high != requested.high) ? 1u : 0u;
    const int64_t cw_pitch = imax64(0, r->cw_pitch);
    const Band mixed = mix_frame(band, p->mode, cw_pitch);
    {
        const int64_t required = minimum_demod_rate(p->mode, mixed);
        const int64_t tap_step = complex_tap_rate_step(p->mode);
        const int64_t step = (tap_step > 0) ? tap_step : p->audio_rate;
        const int64_t multiple = imax64(1, (required + step - 1) / step);
        p->demod_rate = multiple * step;
    }
    const uint32_t decimation = (uint32_t)(p->demod_rate / p->audio_rate);
    const double stop_edge = 0.5 * (double)imin64(p->demod_rate, p->channel_rate);
    const double limit_a = stop_edge - (double)mixed.high, limit_b = stop_edge + (double)mixed.low;
    const double transition_limit = 2.0 * (limit_a < limit_b ? limit_a : limit_b);
    const double transition_wanted = 0.5 * (double)p->bandwidth;
    const double transition = transition_limit < transition_wanted ? transition_limit : transition_wanted;
    if (!(transition > 0.0)) return or_fail("plan_vrx: no transition band");
    p->fine.phases = 256;
    p->fine.nco_log2 = 16;
    p->fine.taps = uclamp(kaiser_taps_for(FINE_ATTENUATION_DB, transition / (double)p->channel_rate), 8u, 256u);
    int64_t fnum = 2 * pl->residual_numerator + pl->residual_denominator * (band.low + band.high);
    int64_t fden = 2 * pl->residual_denominator;
    int64_t mnum = pl->residual_numerator, mden = pl->residual_denominator;
    if (p->mode == RV_DEMOD_CW) mnum = pl->residual_numerator - pl->residual_denominator * cw_pitch;
    reduce_rational(&fnum, &fden);
    reduce_rational(&mnum, &mden);
    p->filter_numerator = fnum;
    p->filter_denominator = fden;
    p->mix_numerator = mnum;
    p->mix_denominator = mden;
    p->demod.mode = p->mode;
    p->demod.decimation = complex_output ? 1u : decimation;
    p->output_rate = complex_output ? p->demod_rate : p->audio_rate;
    const int programme_audio = (p->mode == RV_DEMOD_WFM) && p->audio_rate < COMPOSITE_AUDIO_RATE;
    const double audio_nyquist = 0.5 * (double)p->audio_rate;
    const double audio_pass = programme_audio ? fmin(15000.0, 0.8 * audio_nyquist) : 0.8 * audio_nyquist;
    const double audio_stop = programme_audio ? fmin(19000.0, audio_nyquist) : audio_nyquist;
    p->deemphasis = resolve_deemphasis(p->mode, r->deemphasis, p->audio_rate);
    float de[1024];
    uint32_t nde = 0;
    if (design_deemphasis_taps(p->deemphasis, p->audio_rate, de, &nde)) return -1;
    p->deemphasis_taps = nde;
    double pass_hz = 0.0, stop_hz = 0.0;
    if (p->demod.decimation == 1u) {
        p->audio_decimation_taps = 1u;
    } else {
        const double fraction = (audio_stop - audio_pass) / (double)p->demod_rate;
        pass_hz = audio_pass;
        stop_hz = audio_stop;
        uint32_t t = uclamp(kaiser_taps_for(AUDIO_ATTENUATION_DB, fraction), 3u, 1024u);
        if ((t % 2u) == 0u) ++t;
        p->audio_decimation_taps = t < 1024u ? t : 1024u;
    }
    p->stereo = (r->stereo != 0 && p->mode == RV_DEMOD_WFM && p->audio_rate < COMPOSITE_AUDIO_RATE) ? 1u : 0u;
    if (complex_output) {
        p->demod.channels = 2u;
        p->demod.pilot_taps = 0u;
    } else if (p->stereo) {
        p->demod.channels = 2u;
        p->demod.pilot_taps = stereo_pilot_taps(p->demod_rate);
        if (p->demod.pilot_taps == 0) return or_fail("plan_vrx: no pilot filter");
    } else {
        p->demod.channels = 1u;
        p->demod.pilot_taps = 0u;
    }
    if (p->mode == RV_DEMOD_AM || p->mode == RV_DEMOD_SAM)
        p->demod.dc_taps = (uint32_t)iclamp64(p->demod_rate / 200, 16, 4096);
    else
        p->demod.dc_taps = 1u;
    p->deviation = fm_deviation(p->mode, p->bandwidth);
    p->demod_gain = demod_gain(p->mode, p->demod_rate, p->deviation);
    p->carrier.power = p->mode == RV_DEMOD_SAM ? 1u : (p->mode == RV_DEMOD_DSB ? 2u : 0u);
    p->carrier.nco_log2 = p->fine.nco_log2;
    if (p->carrier.power != 0)
        if (design_carrier_loop(p->demod_rate, band_reach(band, 0), &p->carrier_loop)) return -1;
    if (nco_delta(p->mix_numerator, p->mix_denominator, p->demod_rate, &p->fine_nco_delta)) return -1;
    /* the tables */
    const size_t fine_count = (size_t)p->fine.phases * p->fine.taps + 1u;
    float* dec = (float*)calloc(p->audio_decimation_taps, sizeof(float));
    float* folded = (float*)calloc(4096, sizeof(float));
    const double audio_cutoff = (stop_hz > 0.0) ? 0.5 * (pass_hz + stop_hz) : 0.0;
    uint32_t audio_taps = 0;
    int32_t st = design_audio_taps(p->audio_decimation_taps, p->demod_rate, p->output_rate, AUDIO_ATTENUATION_DB,
                                   audio_cutoff, dec);
    if (!st) st = fold_deemphasis(dec, p->audio_decimation_taps, de, nde, p->demod.decimation, folded, &audio_taps);
    p->demod.audio_taps = audio_taps;
    const size_t pilot_count = 2u * (size_t)p->demod.pilot_taps, rotation_count = p->demod.pilot_taps ? 2u * (size_t)audio_taps : 0u;
    p->fine_tap_count = fine_count;
    p->demod_weight_count = audio_taps + p->demod.dc_taps + pilot_count + rotation_count;
    if (!st && taps != NULL) {
        if (taps_len != fine_count) st = or_fail("plan_vrx: fine tap buffer of %llu for %zu", (unsigned long long)taps_len, fine_count);
        if (!st)
            st = design_fine_taps(&p->fine, p->channel_rate, p->bandwidth / 2, p->filter_numerator, p->filter_denominator,
                                  FINE_ATTENUATION_DB, taps);
    }
    if (!st && weights != NULL) {
        if (weights_len != p->demod_weight_count) {
            st = or_fail("plan_vrx: weight buffer of %llu for %llu", (unsigned long long)weights_len,
                         (unsigned long long)p->demod_weight_count);
        } else {
            memcpy(weights, folded, audio_taps * sizeof(float));
            design_dc_weights(p->demod.dc_taps, weights + audio_taps);
            if (p->demod.pilot_taps)
                st = design_stereo_tables(p->demod_rate, audio_taps, p->demod.pilot_taps,
                                          weights + audio_taps + p->demod.dc_taps,
                                          weights + audio_taps + p->demod.dc_taps + pilot_count);
        }
    }
    free(dec);
    free(folded);
    return st;
}

/* ---- block parameters ---------------------------------------------------- */

/* resample_block (vrx_reference.cpp:2786-2850): the fine dispatch's
 * parameters from its absolute first output, the first input re-derived
 * exactly. */
int32_t or_fine_block(const rv_vrx_plan_info* plan, uint32_t channel_base, uint32_t channel_mask, uint32_t fine_mask,
                      uint64_t first_output, uint32_t count, rv_vrx_fine_block* block) {
    if (plan == NULL || block == NULL || plan->channel_rate <= 0 || plan->demod_rate <= 0 || count == 0)
        return or_fail("fine_block: bad parameters");
    const uint64_t fc = (uint64_t)plan->channel_rate, fd = (uint64_t)plan->demod_rate, nco = plan->fine_nco_delta;
    const uint64_t step_whole = fc / fd, step_rem = fc % fd;
    const uint64_t whole = first_output / fd, part = first_output % fd;
    const uint64_t carry_product = part * step_rem;
    const uint64_t first_input = first_output * step_whole + whole * step_rem + carry_product / fd;
    const uint64_t frac0 = carry_product % fd;
    memset(block, 0, sizeof *block);
    rv_vrx_fine_params* o = &block->params;
    o->chan_base = channel_base;
    o->chan_mask = channel_mask;
    o->in_offset = (uint32_t)(first_input & channel_mask);
    o->out_offset = (uint32_t)(first_output & fine_mask);
    o->out_mask = fine_mask;
    o->count = count;
    o->step_whole = (uint32_t)step_whole;
    o->step_rem = (uint32_t)step_rem;
    o->out_rate = (uint32_t)fd;
    o->frac0 = (uint32_t)frac0;
    o->inv_out_rate = 1.0f / (float)fd;
    const uint64_t phase = nco * first_output;
    o->nco_phase_high = (uint32_t)(phase >> 32);
    o->nco_phase_low = (uint32_t)phase;
    o->nco_delta_high = (uint32_t)(nco >> 32);
    o->nco_delta_low = (uint32_t)nco;
    const uint64_t last_acc = frac0 + (uint64_t)(count - 1u) * step_rem;
    block->first_input = first_input;
    block->newest_input = first_input + (uint64_t)(count - 1u) * step_whole + last_acc / fd;
    block->oldest_input = first_input - (uint64_t)(plan->fine.taps - 1u);
    return 0;
}

uint32_t or_demod_fine_history(const rv_vrx_demod_config* c) {
    const uint32_t det = (c->mode == RV_DEMOD_AM || c->mode == RV_DEMOD_SAM) ? c->dc_taps - 1u
                         : (c->mode == RV_DEMOD_NFM || c->mode == RV_DEMOD_WFM) ? 1u
                                                                                 : 0u;
    const uint32_t audio = c->audio_taps - 1u;
    const uint32_t pilot = c->pilot_taps == 0 ? 0u : c->audio_taps / 2u + c->pilot_taps - 1u;
    return (audio > pilot ? audio : pilot) + det;
}

/* demod_block (vrx_reference.cpp:2873). */
int32_t or_demod_block(const rv_vrx_plan_info* plan, uint32_t fine_mask, uint64_t first_audio, uint32_t count,
                       rv_vrx_demod_block* block) {
    if (plan == NULL || block == NULL || count == 0) return or_fail("demod_block: bad parameters");
    const uint64_t first_fine = first_audio * (uint64_t)plan->demod.decimation;
    memset(block, 0, sizeof *block);
    block->first_fine = first_fine;
    block->params.in_mask = fine_mask;
    block->params.in_offset = (uint32_t)(first_fine & fine_mask);
    block->params.count = count;
    block->params.gain = plan->demod_gain;
    block->oldest_fine = first_fine - or_demod_fine_history(&plan->demod);
    return 0;
}

/* carrier_block (vrx_reference.cpp:2911). */
int32_t or_carrier_block(const rv_vrx_plan_info* plan, uint32_t fine_mask, uint64_t first_fine, uint32_t count,
                         int32_t reset, float shift, rv_vrx_carrier_params* out) {
    if (plan == NULL || out == NULL || plan->carrier.power == 0) return or_fail("carrier_block: no carrier loop");
    *out = plan->carrier_loop;
    out->in_mask = fine_mask;
    out->in_offset = (uint32_t)(first_fine & fine_mask);
    out->count = count;
    out->flags = reset ? 1u : 0u;
    out->shift = reset ? 0.0f : shift;
    return 0;
}
