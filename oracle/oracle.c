/*
 * oracle.c — CPU restatement of the reference's receive-chain twins.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT: loaded only by tests/, by
 * __graft_entry__.smoke() as the checker, and by bench.py's CPU arm. See
 * oracle.h. Compiled with -ffp-contract=off -fno-fast-math so that every
 * float expression below rounds once per operation, as the reference's
 * core/dsp/reference_fp.h pledge requires, and run under a scoped hardware
 * denormal flush (the reference's ScopedDenormalFlush,
 * core/dsp/denormal_mode.h), because the device flushes fp32 denormals.
 */
#define _GNU_SOURCE
#include "oracle.h"

#include <fenv.h>
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

/* ------------------------------------------------------------------ */
/* errors                                                             */

static __thread char g_error[512];

const char* or_last_error(void) { return g_error; }

static int32_t fail(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_error, sizeof g_error, fmt, ap);
    va_end(ap);
    return -1;
}

static int32_t ok(void) {
    g_error[0] = 0;
    return 0;
}

/* The same message slot for the planner restatement (planner.c). */
int32_t or_fail(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_error, sizeof g_error, fmt, ap);
    va_end(ap);
    return -1;
}

/* ------------------------------------------------------------------ */
/* scoped denormal flush (core/dsp/denormal_mode.h ScopedDenormalFlush) */
/* Sets the floating-point environment's flush-to-zero bits through   */
/* <fenv.h> and restores the caller's environment afterwards.          */

typedef struct {
    fenv_t saved;
} flush_scope;

static void flush_begin(flush_scope* s) {
    fegetenv(&s->saved);
    fenv_t env = s->saved;
#if defined(__x86_64__)
    env.__mxcsr |= (1u << 15) | (1u << 6); /* FTZ | DAZ */
#elif defined(__aarch64__)
    env.__fpcr |= (1u << 24); /* FZ */
#else
#error "oracle: no denormal-flush control for this architecture"
#endif
    fesetenv(&env);
}

static void flush_end(flush_scope* s) { fesetenv(&s->saved); }

static int is_pow2_u64(uint64_t v) { return v != 0 && (v & (v - 1)) == 0; }

static uint32_t bits_of(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}
static float float_of(uint32_t u) {
    float f;
    memcpy(&f, &u, 4);
    return f;
}

/* ------------------------------------------------------------------ */
/* deterministic transcendentals                                      */
/* core/dsp/vrx_reference.cpp:227-306 (rsqrt, sqrt, recip, atan),      */
/* core/dsp/spectrum_reference.cpp det_log2. Newton iterations from a  */
/* bit-trick seed and a fixed odd polynomial, all correctly-rounded    */
/* + - * so every IEEE implementation agrees.                          */

static const float kHalfPiF = (float)1.57079632679489661923;
static const float kPiF = (float)3.14159265358979323846;
static const float kAtanC[10] = {
    (float)0.9999999998,  (float)-0.3333331929, (float)0.1999923872, (float)-0.1427217912,
    (float)0.1099615976,  (float)-0.0853800324, (float)0.0603537785, (float)-0.0336503503,
    (float)0.0122847765,  (float)-0.0021090222};

static float det_rsqrt(float value) {
    const float seed = float_of(0x5F375A86u - (bits_of(value) >> 1));
    const float half_value = 0.5F * value;
    float r = seed;
    for (int i = 0; i < 4; ++i) r = r * (1.5F - half_value * (r * r));
    return r;
}

static float det_sqrt(float value) {
    if (!(value > 0.0F)) return 0.0F;
    return value * det_rsqrt(value);
}

static float det_recip(float value) {
    const float seed = float_of(0x7EF311C3u - bits_of(value));
    float r = seed;
    for (int i = 0; i < 4; ++i) r = r * (2.0F - value * r);
    return r;
}

static float det_atan_unit(float t) {
    const float u = t * t;
    float p = kAtanC[9];
    for (int i = 8; i >= 0; --i) p = p * u + kAtanC[i];
    return t * p;
}

static float det_atan2(float y, float x) {
    const float ay = fabsf(y);
    const float ax = fabsf(x);
    if (ay == 0.0F && ax == 0.0F) return 0.0F;
    const float numerator = (ax < ay) ? ax : ay;
    const float denominator = (ay < ax) ? ax : ay;
    const float ratio = numerator * det_recip(denominator);
    float angle = det_atan_unit(ratio);
    if (ay > ax) angle = kHalfPiF - angle;
    if (x < 0.0F) angle = kPiF - angle;
    return (y < 0.0F) ? -angle : angle;
}

static const float kLogC[5] = {2.88539008177792681F, 0.96179669392597560F, 0.57707801635558536F,
                               0.41219858311113240F, 0.32059889797532520F};
static const float kSqrt2F = 1.41421356237309505F;
static const float kDecibelsPerOctave = 3.01029995663981195F;

static float det_log2(float value) {
    const uint32_t bits = bits_of(value);
    int exponent = (int)((bits >> 23) & 0xFFu) - 127;
    float mantissa = float_of((bits & 0x007FFFFFu) | 0x3F800000u);
    if (mantissa > kSqrt2F) {
        mantissa = mantissa * 0.5F;
        exponent = exponent + 1;
    }
    const float t = (mantissa - 1.0F) * det_recip(mantissa + 1.0F);
    const float u = t * t;
    float p = kLogC[4];
    for (int i = 3; i >= 0; --i) p = p * u + kLogC[i];
    const float fraction = t * p;
    return (float)exponent + fraction;
}

#define WRAP_DET1(name)                \
    float or_##name(float v) {          \
        flush_scope s;                 \
        flush_begin(&s);               \
        const float r = name(v);       \
        flush_end(&s);                 \
        return r;                      \
    }
WRAP_DET1(det_rsqrt)
WRAP_DET1(det_sqrt)
WRAP_DET1(det_recip)
WRAP_DET1(det_log2)

float or_det_atan2(float y, float x) {
    flush_scope s;
    flush_begin(&s);
    const float r = det_atan2(y, x);
    flush_end(&s);
    return r;
}

/* ------------------------------------------------------------------ */
/* convert (core/dsp/convert.cpp reference_convert_*; constants        */
/* core/dsp/convert.h:43-106)                                          */

static const float kCu8Bias = 127.5F;
static const float kCu8Scale = 0.00784313772F;      /* 0x3C008081 */
static const float kCs8Scale = 0.0078125F;          /* 2^-7  */
static const float kCs16Scale = 0.000030517578125F; /* 2^-15 */
static const float kCs24Scale = 0.00000011920928955078125F; /* 2^-23 */

static uint32_t load_word(const uint8_t* b, uint64_t word) {
    const uint8_t* p = b + word * 4;
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) |
           ((uint32_t)p[3] << 24);
}

static int32_t sign_extend(uint32_t raw, int bits) {
    const uint32_t shifted = raw << (32 - bits);
    int32_t s;
    memcpy(&s, &shifted, 4);
    return s >> (32 - bits);
}

int32_t or_convert(int32_t format, const rv_convert_params* p, const void* packed,
                   uint64_t packed_bytes, rv_cf32* ring, uint64_t ring_len) {
    uint64_t bytes_per_sample;
    switch (format) {
        case RV_FORMAT_CU8:
        case RV_FORMAT_CS8: bytes_per_sample = 2; break;
        case RV_FORMAT_CS16: bytes_per_sample = 4; break;
        case RV_FORMAT_CS24: bytes_per_sample = 6; break;
        default: return fail("convert: unknown format %d", format);
    }
    /* core/dsp/convert.cpp check_request */
    const uint64_t capacity = (uint64_t)p->ring_mask + 1u;
    if ((capacity & (uint64_t)p->ring_mask) != 0)
        return fail("convert: ring_mask %u is not a power of two minus one", p->ring_mask);
    if (ring_len < capacity)
        return fail("convert: ring holds %llu samples, mask %u implies %llu",
                    (unsigned long long)ring_len, p->ring_mask, (unsigned long long)capacity);
    if (p->count > capacity)
        return fail("convert: %u samples into a ring of %llu would alias", p->count,
                    (unsigned long long)capacity);
    const uint64_t last_sample = (uint64_t)p->src_offset + p->count;
    if (last_sample > 0xFFFFFFFFull)
        return fail("convert: src_offset %u plus count %u overflows 32 bits", p->src_offset,
                    p->count);
    const uint64_t words_needed = (last_sample * bytes_per_sample + 3u) / 4u;
    if (words_needed > 0x100000000ull)
        return fail("convert: request reaches past the 32-bit word index");
    if (packed_bytes < words_needed * 4u)
        return fail("convert: reads %llu whole words, source holds %llu bytes",
                    (unsigned long long)words_needed, (unsigned long long)packed_bytes);
    if (p->count == 0) return ok();

    const uint8_t* b = (const uint8_t*)packed;
    flush_scope s;
    flush_begin(&s);
    for (uint32_t index = 0; index < p->count; ++index) {
        const uint32_t src = p->src_offset + index;
        float iv, qv;
        if (format == RV_FORMAT_CU8 || format == RV_FORMAT_CS8) {
            const uint32_t word = load_word(b, src >> 1);
            const int shift = (int)((src & 1u) << 4);
            const uint32_t i_raw = (word >> shift) & 0xFFu;
            const uint32_t q_raw = (word >> (shift + 8)) & 0xFFu;
            if (format == RV_FORMAT_CU8) {
                iv = ((float)i_raw - kCu8Bias) * kCu8Scale;
                qv = ((float)q_raw - kCu8Bias) * kCu8Scale;
            } else {
                iv = (float)sign_extend(i_raw, 8) * kCs8Scale;
                qv = (float)sign_extend(q_raw, 8) * kCs8Scale;
            }
        } else if (format == RV_FORMAT_CS16) {
            const uint32_t word = load_word(b, src);
            iv = (float)sign_extend(word & 0xFFFFu, 16) * kCs16Scale;
            qv = (float)sign_extend(word >> 16, 16) * kCs16Scale;
        } else {
            /* six bytes a sample, little-endian, I in bytes 0-2, Q in 3-5 */
            const uint8_t* q = b + (uint64_t)src * 6u;
            const uint32_t i_raw = (uint32_t)q[0] | ((uint32_t)q[1] << 8) | ((uint32_t)q[2] << 16);
            const uint32_t q_raw = (uint32_t)q[3] | ((uint32_t)q[4] << 8) | ((uint32_t)q[5] << 16);
            iv = (float)sign_extend(i_raw, 24) * kCs24Scale;
            qv = (float)sign_extend(q_raw, 24) * kCs24Scale;
        }
        rv_cf32* out = &ring[(p->dst_offset + index) & p->ring_mask];
        out->re = iv;
        out->im = qv;
    }
    flush_end(&s);
    return ok();
}

/* ------------------------------------------------------------------ */
/* grid validation (core/dsp/pfb_design.cpp validate(GridParams))      */

static int32_t validate_grid(const rv_grid_params* g) {
    if (g->channels < 2) return fail("grid: channel count %u is below 2", g->channels);
    if (!is_pow2_u64(g->channels)) return fail("grid: channel count %u is not a power of two", g->channels);
    if (g->channels > 2048) return fail("grid: channel count %u exceeds 2048", g->channels);
    if (g->taps_per_branch == 0) return fail("grid: zero taps per branch");
    if (g->decimation == 0) return fail("grid: zero decimation");
    if (g->channels % g->decimation != 0)
        return fail("grid: decimation %u does not divide %u", g->decimation, g->channels);
    if ((uint64_t)g->channels * g->taps_per_branch > (1u << 20))
        return fail("grid: prototype exceeds 2^20 taps");
    return 0;
}

/* ------------------------------------------------------------------ */
/* branch FIR (core/dsp/pfb_branch_reference.cpp:22-145)               */
/* y[b][(M-r)&(M-1)] = sum_{q ascending} x[(base - (qM+r)) & mask] * h[qM+r] */

static void branch_block(uint32_t M, uint32_t T, uint32_t base, uint32_t mask, const float* taps,
                         const rv_cf32* ring, rv_cf32* out_block) {
    for (uint32_t r = 0; r < M; ++r) {
        float acc_re = 0.0F, acc_im = 0.0F;
        for (uint32_t q = 0; q < T; ++q) {
            const uint32_t n = q * M + r;
            const rv_cf32 s = ring[(base - n) & mask];
            const float c = taps[n];
            acc_re = acc_re + s.re * c;
            acc_im = acc_im + s.im * c;
        }
        rv_cf32* o = &out_block[(M - r) & (M - 1u)];
        o->re = acc_re;
        o->im = acc_im;
    }
}

static int32_t pfb_branch_any(const rv_grid_params* g, const rv_pfb_branch_params* p, const float* taps,
                              uint64_t taps_len, const rv_cf32* ring, uint64_t ring_len, rv_cf32* out,
                              uint64_t out_len);

int32_t or_pfb_branch(const rv_grid_params* g, const rv_pfb_branch_params* p, const float* taps,
                      uint64_t taps_len, const rv_cf32* ring, uint64_t ring_len, rv_cf32* out,
                      uint64_t out_len) {
    if (validate_grid(g) != 0) return -1;
    return pfb_branch_any(g, p, taps, taps_len, ring, ring_len, out, out_len);
}

/* the same branch FIR for grids past 2048 channels (C4) */
int32_t or_pfb_branch_wide(const rv_grid_params* g, const rv_pfb_branch_params* p, const float* taps,
                           uint64_t taps_len, const rv_cf32* ring, uint64_t ring_len, rv_cf32* out,
                           uint64_t out_len) {
    if (g->channels > 16384) return fail("grid: channel count %u exceeds 16384", g->channels);
    if (g->channels <= 2048 && validate_grid(g) != 0) return -1;
    if (g->channels < 2 || !is_pow2_u64(g->channels) || g->taps_per_branch == 0 || g->decimation == 0 ||
        g->channels % g->decimation != 0)
        return fail("grid: invalid");
    return pfb_branch_any(g, p, taps, taps_len, ring, ring_len, out, out_len);
}

static int32_t pfb_branch_any(const rv_grid_params* g, const rv_pfb_branch_params* p, const float* taps,
                              uint64_t taps_len, const rv_cf32* ring, uint64_t ring_len, rv_cf32* out,
                              uint64_t out_len) {
    const uint32_t M = g->channels, T = g->taps_per_branch, D = g->decimation;
    if (taps_len != (uint64_t)M * T) return fail("pfb_branch: wants %u taps", M * T);
    if (out_len != (uint64_t)p->block_count * M) return fail("pfb_branch: output length");
    if (p->block_count == 0) return ok();
    const uint64_t capacity = (uint64_t)p->ring_mask + 1u;
    if ((capacity & (uint64_t)p->ring_mask) != 0) return fail("pfb_branch: ring_mask");
    if (ring_len < capacity) return fail("pfb_branch: ring shorter than mask implies");
    const uint64_t span = (uint64_t)M * T + (uint64_t)(p->block_count - 1u) * D;
    if (span > capacity) return fail("pfb_branch: needs %llu samples of history, ring %llu",
                                     (unsigned long long)span, (unsigned long long)capacity);
    flush_scope s;
    flush_begin(&s);
    for (uint32_t b = 0; b < p->block_count; ++b)
        branch_block(M, T, p->base_offset + b * D, p->ring_mask, taps, ring, out + (uint64_t)b * M);
    flush_end(&s);
    return ok();
}

/* ------------------------------------------------------------------ */
/* radix-2 DIT FFT (core/dsp/pfb_fft_reference.cpp:54-102)             */
/* bit-reversed load, stage s: half span h=2^s, twiddle W[j*(M>>(s+1))],*/
/* ia = ((b>>s)<<(s+1)) + j, value = b*w, a+value / a-value            */

static uint32_t reverse_bits(uint32_t v, uint32_t stages) {
    uint32_t r = 0;
    for (uint32_t bit = 0; bit < stages; ++bit) r |= ((v >> bit) & 1u) << (stages - 1u - bit);
    return r;
}

static void fft_block(const rv_cf32* in, const rv_cf32* tw, rv_cf32* x, uint32_t n,
                      uint32_t stages) {
    for (uint32_t i = 0; i < n; ++i) x[i] = in[reverse_bits(i, stages)];
    const uint32_t butterflies = n >> 1;
    for (uint32_t st = 0; st < stages; ++st) {
        const uint32_t half = 1u << st;
        const uint32_t step = n >> (st + 1u);
        for (uint32_t b = 0; b < butterflies; ++b) {
            const uint32_t j = b & (half - 1u);
            const uint32_t ia = ((b >> st) << (st + 1u)) + j;
            const uint32_t ib = ia + half;
            const float ar = x[ia].re, ai = x[ia].im, br = x[ib].re, bi = x[ib].im;
            const float wr = tw[j * step].re, wi = tw[j * step].im;
            const float vr = br * wr - bi * wi;
            const float vi = br * wi + bi * wr;
            x[ia].re = ar + vr;
            x[ia].im = ai + vi;
            x[ib].re = ar - vr;
            x[ib].im = ai - vi;
        }
    }
}

static uint32_t log2_u32(uint32_t v) {
    uint32_t s = 0;
    while (s < 31 && (1u << s) < v) ++s;
    return s;
}

int32_t or_fft_radix2(const rv_cf32* tw, const rv_cf32* in, rv_cf32* out, uint32_t size,
                      uint32_t batch) {
    if (!is_pow2_u64(size) || size < 2) return fail("fft_radix2: size %u", size);
    const uint32_t stages = log2_u32(size);
    flush_scope s;
    flush_begin(&s);
    for (uint32_t b = 0; b < batch; ++b)
        fft_block(in + (uint64_t)b * size, tw, out + (uint64_t)b * size, size, stages);
    flush_end(&s);
    return ok();
}

/* core/dsp/pfb_fft_reference.cpp validate(PfbFftParams) */
static int32_t validate_fft(const rv_pfb_fft_params* p) {
    if (!is_pow2_u64(p->channels) || p->channels < 2) return fail("pfb_fft: channels %u", p->channels);
    if (p->stages >= 32 || (1u << p->stages) != p->channels) return fail("pfb_fft: stages");
    if (p->decimation == 0 || p->decimation > p->channels || p->channels % p->decimation != 0)
        return fail("pfb_fft: decimation must divide channels");
    if (!is_pow2_u64(p->out_ring_blocks)) return fail("pfb_fft: out_ring_blocks");
    if (p->out_ring_mask != p->out_ring_blocks - 1u) return fail("pfb_fft: out_ring_mask");
    if (p->block_count > p->out_ring_blocks) return fail("pfb_fft: dispatch overruns the ring");
    return 0;
}

/* Phase correction exp(-j 2 pi k m D / M) from the twiddle circle and the
 * channel-major scatter (core/dsp/pfb_fft_reference.cpp:185-228). */
static void fft_finish(const rv_pfb_fft_params* p, const rv_cf32* x, const rv_cf32* tw,
                       uint32_t m_abs, rv_cf32* ring) {
    const uint32_t M = p->channels;
    const uint32_t slot = m_abs & p->out_ring_mask;
    const uint32_t dm = ((m_abs & (M - 1u)) * p->decimation) & (M - 1u);
    for (uint32_t k = 0; k < M; ++k) {
        float vr = x[k].re, vi = x[k].im;
        if (p->decimation != M) {
            const rv_cf32 c = tw[(k * dm) & (M - 1u)];
            const float pr = vr * c.re - vi * c.im;
            const float pi = vr * c.im + vi * c.re;
            vr = pr;
            vi = pi;
        }
        rv_cf32* o = &ring[(uint64_t)k * p->out_ring_blocks + slot];
        o->re = vr;
        o->im = vi;
    }
}

int32_t or_pfb_fft(const rv_pfb_fft_params* p, const rv_cf32* branch, uint64_t branch_len,
                   const rv_cf32* tw, uint64_t tw_len, rv_cf32* ring, uint64_t ring_len) {
    if (validate_fft(p) != 0) return -1;
    const uint32_t M = p->channels;
    if (tw_len != M) return fail("pfb_fft: needs %u twiddles", M);
    if (branch_len < (uint64_t)p->block_count * M) return fail("pfb_fft: branch values");
    if (ring_len < (uint64_t)M * p->out_ring_blocks) return fail("pfb_fft: channel ring");
    rv_cf32* x = (rv_cf32*)malloc(sizeof(rv_cf32) * M);
    flush_scope s;
    flush_begin(&s);
    for (uint32_t b = 0; b < p->block_count; ++b) {
        fft_block(branch + (uint64_t)b * M, tw, x, M, p->stages);
        fft_finish(p, x, tw, p->block_base + b, ring);
    }
    flush_end(&s);
    free(x);
    return ok();
}

/* ------------------------------------------------------------------ */
/* coarse chain over host threads (convert -> branch -> FFT)           */

typedef struct {
    const rv_grid_params* g;
    const float* taps;
    const rv_cf32* tw;
    const uint8_t* packed;
    uint64_t samples;
    uint64_t first_block;
    uint32_t b0, b1;
    uint32_t out_ring_blocks;
    rv_cf32* ring;
} coarse_job;

static void* coarse_worker(void* arg) {
    const coarse_job* j = (const coarse_job*)arg;
    const uint32_t M = j->g->channels, T = j->g->taps_per_branch, D = j->g->decimation;
    const uint32_t stages = log2_u32(M);
    const uint32_t support = M * T;
    if (j->b1 <= j->b0) return NULL;
    /* Block b is centred on absolute input n0 = (first_block + b) * D and
     * reads x[n0 - (M*T - 1) .. n0]; samples before the capture read as zero.
     * The worker converts its whole input span once, then filters from it. */
    const int64_t first = (int64_t)((j->first_block + j->b0) * (uint64_t)D) - (int64_t)(support - 1u);
    const uint64_t span = (uint64_t)(j->b1 - j->b0 - 1u) * D + support;
    rv_cf32* x_lin = (rv_cf32*)malloc(sizeof(rv_cf32) * span);
    rv_cf32* br = (rv_cf32*)malloc(sizeof(rv_cf32) * M);
    rv_cf32* x = (rv_cf32*)malloc(sizeof(rv_cf32) * M);
    rv_pfb_fft_params fp = {M, D, stages, 0, 1, j->out_ring_blocks, j->out_ring_blocks - 1u};
    flush_scope s;
    flush_begin(&s);
    for (uint64_t w = 0; w < span; ++w) {
        const int64_t n = first + (int64_t)w;
        rv_cf32 v = {0.0F, 0.0F};
        if (n >= 0 && (uint64_t)n < j->samples) {
            const uint32_t word = load_word(j->packed, (uint64_t)n);
            v.re = (float)sign_extend(word & 0xFFFFu, 16) * kCs16Scale;
            v.im = (float)sign_extend(word >> 16, 16) * kCs16Scale;
        }
        x_lin[w] = v;
    }
    for (uint32_t b = j->b0; b < j->b1; ++b) {
        /* x_lin[(b - b0) * D + support - 1] is x[n0]; index it as a ring with
         * an all-ones mask so (base - n) & mask is the linear offset. */
        const uint32_t base = (b - j->b0) * D + support - 1u;
        branch_block(M, T, base, 0xFFFFFFFFu, j->taps, x_lin, br);
        fft_block(br, j->tw, x, M, stages);
        fft_finish(&fp, x, j->tw, (uint32_t)(j->first_block + b), j->ring);
    }
    flush_end(&s);
    free(x_lin);
    free(br);
    free(x);
    return NULL;
}

int32_t or_coarse_cs16(const rv_grid_params* g, const float* taps, const rv_cf32* tw,
                       const void* packed, uint64_t samples, uint64_t first_block,
                       uint32_t block_count, uint32_t out_ring_blocks, rv_cf32* ring,
                       int32_t threads) {
    if (validate_grid(g) != 0) return -1;
    if (!is_pow2_u64(out_ring_blocks) || block_count > out_ring_blocks)
        return fail("coarse: out_ring_blocks must be a power of two >= block_count");
    int n = threads > 0 ? threads : (int)sysconf(_SC_NPROCESSORS_ONLN);
    if (n < 1) n = 1;
    if ((uint32_t)n > block_count) n = block_count ? (int)block_count : 1;
    pthread_t* tid = (pthread_t*)calloc((size_t)n, sizeof(pthread_t));
    coarse_job* jobs = (coarse_job*)calloc((size_t)n, sizeof(coarse_job));
    for (int t = 0; t < n; ++t) {
        coarse_job* j = &jobs[t];
        j->g = g;
        j->taps = taps;
        j->tw = tw;
        j->packed = (const uint8_t*)packed;
        j->samples = samples;
        j->first_block = first_block;
        j->b0 = (uint32_t)(((uint64_t)block_count * t) / n);
        j->b1 = (uint32_t)(((uint64_t)block_count * (t + 1)) / n);
        j->out_ring_blocks = out_ring_blocks;
        j->ring = ring;
        if (n == 1) coarse_worker(j);
        else pthread_create(&tid[t], NULL, coarse_worker, j);
    }
    if (n > 1)
        for (int t = 0; t < n; ++t) pthread_join(tid[t], NULL);
    free(tid);
    free(jobs);
    return ok();
}

/* ------------------------------------------------------------------ */
/* FP64 channelizer yardstick                                          */

int32_t or_pfb_f64(const rv_grid_params* g, const float* taps, const rv_cf32* ring,
                   uint32_t ring_mask, uint32_t base_offset, uint32_t block_count,
                   uint32_t block_base, double* out_re, double* out_im) {
    if (validate_grid(g) != 0 && g->channels <= 2048) return -1;
    const uint32_t M = g->channels, T = g->taps_per_branch, D = g->decimation;
    double* br = (double*)malloc(sizeof(double) * 2 * M);
    double* cs = (double*)malloc(sizeof(double) * 2 * M);
    const double two_pi = 6.283185307179586476925286766559;
    for (uint32_t j = 0; j < M; ++j) {
        cs[2 * j] = cos(two_pi * j / M);
        cs[2 * j + 1] = -sin(two_pi * j / M);
    }
    for (uint32_t b = 0; b < block_count; ++b) {
        const uint32_t base = base_offset + b * D;
        for (uint32_t r = 0; r < M; ++r) {
            double ar = 0, ai = 0;
            for (uint32_t q = 0; q < T; ++q) {
                const uint32_t n = q * M + r;
                const rv_cf32 s = ring[(base - n) & ring_mask];
                ar += (double)s.re * taps[n];
                ai += (double)s.im * taps[n];
            }
            const uint32_t slot = (M - r) & (M - 1u);
            br[2 * slot] = ar;
            br[2 * slot + 1] = ai;
        }
        const uint32_t m_abs = block_base + b;
        const uint32_t dm = ((m_abs & (M - 1u)) * D) & (M - 1u);
        for (uint32_t k = 0; k < M; ++k) {
            double yr = 0, yi = 0;
            for (uint32_t n = 0; n < M; ++n) {
                const uint32_t e = (uint32_t)(((uint64_t)k * n) & (M - 1u));
                yr += br[2 * n] * cs[2 * e] - br[2 * n + 1] * cs[2 * e + 1];
                yi += br[2 * n] * cs[2 * e + 1] + br[2 * n + 1] * cs[2 * e];
            }
            const uint32_t e = (k * dm) & (M - 1u);
            const double zr = yr * cs[2 * e] - yi * cs[2 * e + 1];
            const double zi = yr * cs[2 * e + 1] + yi * cs[2 * e];
            out_re[(uint64_t)k * block_count + b] = zr;
            out_im[(uint64_t)k * block_count + b] = zi;
        }
    }
    free(br);
    free(cs);
    return ok();
}

/* ------------------------------------------------------------------ */
/* spectrum (core/dsp/spectrum_reference.cpp:286-390)                  */

int32_t or_spectrum(const rv_spectrum_params* p, const rv_cf32* ring, uint64_t ring_len,
                    const rv_cf32* tw, uint64_t tw_len, const float* window, uint64_t window_len,
                    float* frame, uint64_t frame_len) {
    if (!is_pow2_u64(p->channels) || p->channels < 2) return fail("spectrum: channels");
    if (!is_pow2_u64(p->transform) || p->transform < 4) return fail("spectrum: transform");
    if (p->transform > 2048) return fail("spectrum: transform above 2048");
    if (p->stages >= 32 || (1u << p->stages) != p->transform) return fail("spectrum: stages");
    if (!is_pow2_u64(p->chan_blocks)) return fail("spectrum: chan_blocks");
    if (p->chan_mask != p->chan_blocks - 1u) return fail("spectrum: chan_mask");
    if (p->transform > p->chan_blocks) return fail("spectrum: window longer than the ring");
    const uint32_t N = p->transform, M = p->channels, half = N / 2;
    if (tw_len != N) return fail("spectrum: twiddles");
    if (window_len != (uint64_t)N + half) return fail("spectrum: window length");
    if (ring_len < (uint64_t)M * p->chan_blocks) return fail("spectrum: ring");
    if (frame_len < (uint64_t)M * half) return fail("spectrum: frame");
    rv_cf32* w = (rv_cf32*)malloc(sizeof(rv_cf32) * N);
    rv_cf32* x = (rv_cf32*)malloc(sizeof(rv_cf32) * N);
    flush_scope s;
    flush_begin(&s);
    for (uint32_t ch = 0; ch < M; ++ch) {
        const uint64_t origin = (uint64_t)ch * p->chan_blocks;
        for (uint32_t n = 0; n < N; ++n) {
            const rv_cf32 v = ring[origin + ((p->in_offset + n) & p->chan_mask)];
            const float gain = window[n];
            w[n].re = v.re * gain;
            w[n].im = v.im * gain;
        }
        fft_block(w, tw, x, N, p->stages);
        const uint64_t out_origin = (uint64_t)((ch + M / 2) & (M - 1u)) * half;
        for (uint32_t bin = 0; bin < half; ++bin) {
            const rv_cf32 v = x[(bin + N - N / 4) & (N - 1u)];
            const float power = v.re * v.re + v.im * v.im;
            const float flattened = power * window[N + bin];
            const float floored = (flattened < 1.0e-20F) ? 1.0e-20F : flattened;
            frame[out_origin + bin] = det_log2(floored) * kDecibelsPerOctave;
        }
    }
    flush_end(&s);
    free(w);
    free(x);
    return ok();
}

/* ------------------------------------------------------------------ */
/* spectrum levels (core/dsp/spectrum_levels_reference.cpp:75-135)     */

static uint32_t rank_of(uint32_t count, uint32_t permille) {
    return (count / 1000u) * permille + ((count % 1000u) * permille) / 1000u;
}

int32_t or_spectrum_levels(const rv_spectrum_levels_params* p, const float* frame,
                           uint64_t frame_len, float* levels) {
    if (p->bins == 0) return fail("levels: no bins");
    if (p->low_permille > 1000 || p->high_permille > 1000) return fail("levels: permille");
    if (p->low_permille >= p->high_permille) return fail("levels: low must sit below high");
    if (frame_len < p->bins) return fail("levels: frame shorter than bins");
    static __thread uint32_t histogram[1024];
    memset(histogram, 0, sizeof histogram);
    flush_scope s;
    flush_begin(&s);
    for (uint32_t i = 0; i < p->bins; ++i) {
        float t = (frame[i] - (-200.0F)) * 4.26666666666666666F;
        t = (t < 0.0F) ? 0.0F : t;
        t = (t > 1023.0F) ? 1023.0F : t;
        ++histogram[(uint32_t)t];
    }
    uint32_t lo = rank_of(p->bins, p->low_permille), hi = rank_of(p->bins, p->high_permille);
    if (lo > p->bins - 1u) lo = p->bins - 1u;
    if (hi > p->bins - 1u) hi = p->bins - 1u;
    uint32_t lb = 0, hb = 0, cum = 0;
    int lf = 0, hf = 0;
    for (uint32_t b = 0; b < 1024; ++b) {
        cum += histogram[b];
        if (!lf && cum > lo) { lb = b; lf = 1; }
        if (!hf && cum > hi) { hb = b; hf = 1; }
    }
    levels[0] = -200.0F + ((float)lb + 0.5F) * 0.234375F;
    levels[1] = -200.0F + ((float)hb + 0.5F) * 0.234375F;
    flush_end(&s);
    return ok();
}

/* ------------------------------------------------------------------ */
/* fine stage (core/dsp/vrx_reference.cpp:489-620)                     */

static int32_t validate_fine(const rv_vrx_fine_config* c, const rv_vrx_fine_params* p) {
    if (c->taps < 2 || c->taps > 256) return fail("vrx fine: %u taps outside [2, 256]", c->taps);
    if (c->phases < 1 || c->phases > 4096) return fail("vrx fine: phases");
    if (c->nco_log2 > 24) return fail("vrx fine: nco_log2");
    if (p->out_rate == 0) return fail("vrx fine: output rate is zero");
    if (p->frac0 >= p->out_rate) return fail("vrx fine: frac0 must be below the output rate");
    const uint64_t cap = (uint64_t)p->chan_mask + 1u;
    if ((cap & (uint64_t)p->chan_mask) != 0) return fail("vrx fine: chan_mask");
    const uint64_t ocap = (uint64_t)p->out_mask + 1u;
    if ((ocap & (uint64_t)p->out_mask) != 0) return fail("vrx fine: out_mask");
    if ((uint64_t)p->frac0 + (uint64_t)p->count * p->step_rem > 0xFFFFFFFFull)
        return fail("vrx fine: recurrence overflows 32 bits");
    if ((uint64_t)(p->out_rate - 1u) * c->phases > 0xFFFFFFFFull)
        return fail("vrx fine: phase selection overflows 32 bits");
    return 0;
}

int32_t or_vrx_fine(const rv_vrx_fine_config* c, const rv_vrx_fine_params* p, const rv_cf32* chan,
                    uint64_t chan_len, const rv_cf32* taps, uint64_t taps_len, const rv_cf32* nco,
                    uint64_t nco_len, rv_cf32* fine, uint64_t fine_len) {
    if (validate_fine(c, p) != 0) return -1;
    if (taps_len != (uint64_t)c->phases * c->taps + 1u) return fail("vrx fine: tap table size");
    if (nco_len != (1ull << c->nco_log2)) return fail("vrx fine: nco size");
    if (chan_len < (uint64_t)p->chan_base + p->chan_mask + 1u) return fail("vrx fine: channel ring");
    if (fine_len < (uint64_t)p->out_mask + 1u) return fail("vrx fine: output ring");
    if (p->count > (uint64_t)p->out_mask + 1u) return fail("vrx fine: count exceeds output ring");
    if (p->count == 0) return ok();
    flush_scope s;
    flush_begin(&s);
    const uint64_t delta = ((uint64_t)p->nco_delta_high << 32) | p->nco_delta_low;
    const uint64_t phase0 = ((uint64_t)p->nco_phase_high << 32) | p->nco_phase_low;
    for (uint32_t i = 0; i < p->count; ++i) {
        const uint32_t acc = p->frac0 + i * p->step_rem;
        const uint32_t carry = acc / p->out_rate;
        const uint32_t frac = acc - carry * p->out_rate;
        const uint32_t n_rel = i * p->step_whole + carry;
        const uint32_t scaled = frac * c->phases;
        const uint32_t phase = scaled / p->out_rate;
        const uint32_t blend_num = scaled - phase * p->out_rate;
        const float blend = (float)blend_num * p->inv_out_rate;
        const float blend_c = 1.0F - blend;
        const uint32_t base = p->in_offset + n_rel;
        float ar = 0.0F, ai = 0.0F;
        for (uint32_t k = 0; k < c->taps; ++k) {
            const uint32_t slot = phase + k * c->phases;
            const rv_cf32 g0 = taps[slot], g1 = taps[slot + 1u];
            const float tr = g0.re * blend_c + g1.re * blend;
            const float ti = g0.im * blend_c + g1.im * blend;
            const rv_cf32 x = chan[(uint64_t)p->chan_base + ((base - k) & p->chan_mask)];
            ar = ar + (x.re * tr - x.im * ti);
            ai = ai + (x.re * ti + x.im * tr);
        }
        /* phi(i) = phase0 + i * delta mod 2^64 (the kernel's umulExtended /
         * uaddCarry chain is this 64-bit product and sum) */
        const uint64_t phi = phase0 + (uint64_t)i * delta;
        const uint32_t idx = (c->nco_log2 == 0) ? 0u : (uint32_t)(phi >> 32) >> (32u - c->nco_log2);
        const rv_cf32 rot = nco[idx];
        rv_cf32* o = &fine[(p->out_offset + i) & p->out_mask];
        o->re = ar * rot.re - ai * rot.im;
        o->im = ar * rot.im + ai * rot.re;
    }
    flush_end(&s);
    return ok();
}

/* ------------------------------------------------------------------ */
/* demodulators (core/dsp/vrx_reference.cpp:620-917)                   */

static int is_known_mode(uint32_t m) { return m <= 12; }
static int is_complex_mode(uint32_t m) {
    return m == RV_DEMOD_RAW || m == RV_DEMOD_P25P1 || m == RV_DEMOD_DSTAR ||
           m == RV_DEMOD_TETRA || m == RV_DEMOD_DMR;
}

static uint32_t fine_history(const rv_vrx_demod_config* c) {
    const uint32_t det = (c->mode == RV_DEMOD_AM || c->mode == RV_DEMOD_SAM) ? c->dc_taps - 1u
                         : (c->mode == RV_DEMOD_NFM || c->mode == RV_DEMOD_WFM) ? 1u
                                                                                 : 0u;
    const uint32_t audio = c->audio_taps - 1u;
    const uint32_t pilot = c->pilot_taps == 0 ? 0u : c->audio_taps / 2u + c->pilot_taps - 1u;
    return (audio > pilot ? audio : pilot) + det;
}

static int32_t validate_demod(const rv_vrx_demod_config* c, const rv_vrx_demod_params* p) {
    if (!is_known_mode(c->mode)) return fail("vrx demod: unknown mode %u", c->mode);
    const int cx = is_complex_mode(c->mode);
    if (c->decimation == 0) return fail("vrx demod: decimation is zero");
    if (c->audio_taps == 0 || c->audio_taps > 4096) return fail("vrx demod: audio taps");
    if (c->dc_taps == 0 || c->dc_taps > 4096) return fail("vrx demod: dc taps");
    if (cx && (c->decimation != 1u || c->audio_taps != 1u)) return fail("vrx demod: complex tap with a filter");
    if (c->channels != 1u && c->channels != 2u) return fail("vrx demod: channels");
    if (cx && c->channels != 2u) return fail("vrx demod: complex tap is two channels");
    if (c->pilot_taps > 2048) return fail("vrx demod: pilot taps");
    if (c->pilot_taps != 0 && c->mode != RV_DEMOD_WFM) return fail("vrx demod: pilot without WFM");
    if (c->pilot_taps != 0 && c->channels != 2u) return fail("vrx demod: pilot with one channel");
    if (c->channels == 2u && !cx && c->pilot_taps == 0) return fail("vrx demod: stereo without pilot");
    const uint64_t cap = (uint64_t)p->in_mask + 1u;
    if ((cap & (uint64_t)p->in_mask) != 0) return fail("vrx demod: in_mask");
    const uint64_t span = p->count == 0 ? 0 : (uint64_t)(p->count - 1u) * c->decimation + fine_history(c) + 1u;
    if (span > cap) return fail("vrx demod: history does not fit the input ring");
    return 0;
}

typedef struct {
    const rv_vrx_demod_config* c;
    const rv_cf32* ring;
    uint32_t mask;
    const float* w;
} demod_ctx;

static rv_cf32 at(const demod_ctx* d, uint32_t i) { return d->ring[i & d->mask]; }

static float magnitude_at(const demod_ctx* d, uint32_t i) {
    const rv_cf32 z = at(d, i);
    return det_sqrt(z.re * z.re + z.im * z.im);
}

static float detect(const demod_ctx* d, uint32_t index) {
    const rv_vrx_demod_config* c = d->c;
    if (c->mode == RV_DEMOD_AM) {
        float dc = 0.0F;
        for (uint32_t w = 0; w < c->dc_taps; ++w) {
            const float term = magnitude_at(d, index - w) * d->w[c->audio_taps + w];
            dc = dc + term;
        }
        return magnitude_at(d, index) - dc;
    }
    if (c->mode == RV_DEMOD_SAM) {
        float dc = 0.0F;
        for (uint32_t w = 0; w < c->dc_taps; ++w) {
            const float term = at(d, index - w).re * d->w[c->audio_taps + w];
            dc = dc + term;
        }
        return at(d, index).re - dc;
    }
    if (c->mode == RV_DEMOD_NFM || c->mode == RV_DEMOD_WFM) {
        const rv_cf32 z = at(d, index), q = at(d, index - 1u);
        const float pr = z.re * q.re + z.im * q.im;
        const float pi = z.im * q.re - z.re * q.im;
        return det_atan2(pi, pr);
    }
    return at(d, index).re;
}

int32_t or_vrx_demod(const rv_vrx_demod_config* c, const rv_vrx_demod_params* p,
                     const rv_cf32* fine, uint64_t fine_len, const float* weights,
                     uint64_t weights_len, float* audio, uint64_t audio_len) {
    if (validate_demod(c, p) != 0) return -1;
    const uint64_t pilot_base = (uint64_t)c->audio_taps + c->dc_taps;
    const uint64_t rotation_base = pilot_base + 2ull * c->pilot_taps;
    const uint64_t wanted = c->pilot_taps == 0 ? pilot_base : rotation_base + 2ull * c->audio_taps;
    if (weights_len != wanted) return fail("vrx demod: wants %llu weights", (unsigned long long)wanted);
    if (fine_len < (uint64_t)p->in_mask + 1u) return fail("vrx demod: fine ring");
    if (audio_len != (uint64_t)p->count * c->channels) return fail("vrx demod: audio length");
    if (p->count == 0) return ok();
    demod_ctx d = {c, fine, p->in_mask, weights};
    const float kPilotLockPower = 2.0e-5F;
    flush_scope s;
    flush_begin(&s);
    for (uint32_t i = 0; i < p->count; ++i) {
        const uint32_t index = p->in_offset + i * c->decimation;
        if (is_complex_mode(c->mode)) {
            const rv_cf32 z = at(&d, index);
            audio[2u * i] = z.re * p->gain;
            audio[2u * i + 1u] = z.im * p->gain;
            continue;
        }
        if (c->channels == 2u) {
            const uint32_t pilot_at = index - c->audio_taps / 2u;
            float pr = 0.0F, pi = 0.0F;
            for (uint32_t k = 0; k < c->pilot_taps; ++k) {
                const float comp = detect(&d, pilot_at - k);
                const float tr = comp * weights[pilot_base + 2u * k];
                const float ti = comp * weights[pilot_base + 2u * k + 1u];
                pr = pr + tr;
                pi = pi + ti;
            }
            const float sr = pr * p->gain, si = pi * p->gain;
            const float rr = sr * sr, ii = si * si;
            const float power = rr + ii;
            const float inverse = det_recip((power < kPilotLockPower) ? kPilotLockPower : power);
            const float cross = sr * si;
            const float cos_two = (ii - rr) * inverse;
            const float sin_two = (-2.0F * cross) * inverse;
            const float locked = (power >= kPilotLockPower) ? 1.0F : 0.0F;
            float sum = 0.0F, diff = 0.0F;
            for (uint32_t t = 0; t < c->audio_taps; ++t) {
                const float weighted = detect(&d, index - t) * weights[t];
                sum = sum + weighted;
                const float ref = sin_two * weights[rotation_base + 2u * t] -
                                  cos_two * weights[rotation_base + 2u * t + 1u];
                const float term = weighted * ref;
                diff = diff + term;
            }
            const float gated = diff * locked;
            audio[2u * i] = (sum + gated) * p->gain;
            audio[2u * i + 1u] = (sum - gated) * p->gain;
            continue;
        }
        float acc = 0.0F;
        for (uint32_t t = 0; t < c->audio_taps; ++t) {
            const float term = detect(&d, index - t) * weights[t];
            acc = acc + term;
        }
        audio[i] = acc * p->gain;
    }
    flush_end(&s);
    return ok();
}

/* ------------------------------------------------------------------ */
/* carrier loop (core/dsp/vrx_reference.cpp:1040-1187)                 */

static float clampf3(float v, float lo, float hi) {
    const float m = (v < lo) ? lo : v; /* std::max(v, lo) */
    return (hi < m) ? hi : m;          /* std::min(m, hi) */
}

int32_t or_vrx_carrier(const rv_vrx_carrier_config* c, const rv_vrx_carrier_params* p,
                       const rv_cf32* nco, uint64_t nco_len, rv_cf32* fine, uint64_t fine_len,
                       uint32_t* state) {
    if (c->power != 1u && c->power != 2u) return fail("vrx carrier: power");
    if (c->nco_log2 == 0 || c->nco_log2 > 24) return fail("vrx carrier: nco_log2");
    const uint64_t cap = (uint64_t)p->in_mask + 1u;
    if ((cap & (uint64_t)p->in_mask) != 0) return fail("vrx carrier: in_mask");
    if (p->count > cap) return fail("vrx carrier: count exceeds the ring");
    if ((p->flags & ~1u) != 0) return fail("vrx carrier: unknown flags");
    if (!isfinite(p->shift)) return fail("vrx carrier: shift not finite");
    if (!(p->clamp_radians > 0.0F) || !((double)p->clamp_radians <= 0.5 * 3.14159265358979323846))
        return fail("vrx carrier: clamp");
    if (!(p->k1_acquire > 0.0F && p->k1_acquire < 1.0F) || !(p->k1_track > 0.0F && p->k1_track < 1.0F))
        return fail("vrx carrier: proportional gain");
    if (!(p->k2_acquire > 0.0F && p->k2_acquire < 1.0F) || !(p->k2_track > 0.0F && p->k2_track < 1.0F))
        return fail("vrx carrier: integral gain");
    if (!(p->level_alpha > 0.0F && p->level_alpha <= 1.0F) || !(p->lock_alpha > 0.0F && p->lock_alpha <= 1.0F))
        return fail("vrx carrier: one-pole coefficient");
    if (p->hold_in == 0 || p->hold_out == 0) return fail("vrx carrier: zero hold");
    if (nco_len != (1ull << c->nco_log2)) return fail("vrx carrier: nco size");
    if (fine_len < cap) return fail("vrx carrier: fine ring");

    const float kTurnsPerRadian = (float)683565275.576431632;
    const float kLevelFloor = (float)1.0e-24;
    flush_scope s;
    flush_begin(&s);
    const int reset = (p->flags & 1u) != 0;
    uint32_t phase = reset ? 0u : state[0];
    float integrator = reset ? 0.0F : float_of(state[1]);
    float level = reset ? 0.0F : float_of(state[2]);
    float lock_re = reset ? 0.0F : float_of(state[3]);
    float lock_im = reset ? 0.0F : float_of(state[4]);
    uint32_t locked = reset ? 0u : state[5];
    uint32_t held = reset ? 0u : state[6];
    uint32_t primed = reset ? 0u : state[7];
    integrator = clampf3(integrator + p->shift, -p->clamp_radians, p->clamp_radians);
    const uint32_t down = 32u - c->nco_log2;
    for (uint32_t i = 0; i < p->count; ++i) {
        rv_cf32* zp = &fine[(p->in_offset + i) & p->in_mask];
        const rv_cf32 z = *zp;
        const rv_cf32 r = nco[phase >> down];
        const float yr = z.re * r.re - z.im * r.im;
        const float yi = z.re * r.im + z.im * r.re;
        zp->re = yr;
        zp->im = yi;
        const float rr = yr * yr, ii = yi * yi;
        const float power = rr + ii;
        const float cross = yr * yi;
        float wr, wi, mag;
        if (c->power == 1u) {
            wr = yr;
            wi = yi;
            mag = det_sqrt(power);
        } else {
            wr = rr - ii;
            wi = cross + cross;
            mag = power;
        }
        if (primed == 0u) {
            level = mag;
            primed = 1u;
        } else {
            const float step = p->level_alpha * (mag - level);
            level = level + step;
        }
        {
            const float sr = p->lock_alpha * (wr - lock_re);
            const float si = p->lock_alpha * (wi - lock_im);
            lock_re = lock_re + sr;
            lock_im = lock_im + si;
        }
        const float bound = 2.0F * fabsf(lock_im);
        const int inside = lock_re > bound;
        if (locked != 0u) {
            held = inside ? (held > 0u ? held - 1u : 0u) : held + 1u;
            if (held >= p->hold_out) { locked = 0u; held = 0u; }
        } else {
            held = inside ? held + 1u : 0u;
            if (held >= p->hold_in) { locked = 1u; held = 0u; }
        }
        const float inverse = det_recip((level < kLevelFloor) ? kLevelFloor : level);
        const float detected = ((c->power == 1u) ? yi : cross) * inverse;
        const float error = clampf3(detected, -1.0F, 1.0F);
        const float k1 = locked ? p->k1_track : p->k1_acquire;
        const float k2 = locked ? p->k2_track : p->k2_acquire;
        integrator = clampf3(integrator + k2 * error, -p->clamp_radians, p->clamp_radians);
        const float advance = k1 * error + integrator;
        const float turns = advance * kTurnsPerRadian;
        phase = phase + (uint32_t)(int32_t)turns;
    }
    state[0] = phase;
    state[1] = bits_of(integrator);
    state[2] = bits_of(level);
    state[3] = bits_of(lock_re);
    state[4] = bits_of(lock_im);
    state[5] = locked;
    state[6] = held;
    state[7] = primed;
    flush_end(&s);
    return ok();
}

/* ---- front-end correction (core/dsp/front_end_correction_reference.cpp:46-111,
 * core/dsp/front_end_correction.cpp:36-114) ------------------------------- */

int32_t or_iq_moments(const rv_iq_moments_params* p, const rv_cf32* ring, uint64_t ring_len, float* sums,
                      uint64_t sums_len) {
    const uint64_t cap = (uint64_t)p->ring_mask + 1u;
    if ((cap & (uint64_t)p->ring_mask) != 0 || ring_len < cap || p->count > cap) return fail("iq_moments: bad ring");
    const uint32_t chunks = (p->count + 63u) / 64u;
    if (sums_len < (uint64_t)chunks * 5u) return fail("iq_moments: sums too short");
    flush_scope s;
    flush_begin(&s);
    for (uint32_t chunk = 0; chunk < chunks; ++chunk) {
        const uint32_t first = chunk * 64u, last = first + 64u < p->count ? first + 64u : p->count;
        float si = 0.0F, sq = 0.0F, sii = 0.0F, sqq = 0.0F, siq = 0.0F;
        for (uint32_t k = first; k < last; ++k) {
            const rv_cf32 v = ring[(p->src_offset + k) & p->ring_mask];
            si = si + v.re;
            sq = sq + v.im;
            sii = sii + v.re * v.re;
            sqq = sqq + v.im * v.im;
            siq = siq + v.re * v.im;
        }
        float* out = sums + (uint64_t)chunk * 5u;
        out[0] = si;
        out[1] = sq;
        out[2] = sii;
        out[3] = sqq;
        out[4] = siq;
    }
    flush_end(&s);
    return 0;
}

int32_t or_iq_correct(const rv_iq_correct_params* p, const rv_cf32* in, uint64_t in_len, rv_cf32* out,
                      uint64_t out_len) {
    const uint64_t cap = (uint64_t)p->ring_mask + 1u;
    if ((cap & (uint64_t)p->ring_mask) != 0 || in_len < cap || p->count > cap || out_len < in_len)
        return fail("iq_correct: bad ring");
    flush_scope s;
    flush_begin(&s);
    for (uint32_t index = 0; index < p->count; ++index) {
        const uint32_t slot = (p->offset + index) & p->ring_mask;
        const rv_cf32 v = in[slot];
        const float i = v.re - p->dc_i;
        const float q_dc = v.im - p->dc_q;
        const float a = p->cross * i, b = p->scale * q_dc;
        out[slot].re = i;
        out[slot].im = a + b;
    }
    flush_end(&s);
    return 0;
}

/* FrontEndCorrector::update over total_moments of a block's chunk sums. */
int32_t or_front_end_update(rv_front_end* st, const float* sums, uint64_t sums_len, uint32_t count, int64_t rate) {
    if (count == 0) return 0;
    uint64_t chunks = (count + 63u) / 64u;
    if (chunks > sums_len / 5u) chunks = sums_len / 5u;
    double t[5] = {0, 0, 0, 0, 0};
    for (uint64_t c = 0; c < chunks; ++c)
        for (int k = 0; k < 5; ++k) t[k] += (double)sums[c * 5u + k];
    const double n = (double)count;
    const double mean_i = t[0] / n, mean_q = t[1] / n;
    const double c_ii = t[2] / n - mean_i * mean_i;
    const double c_qq = t[3] / n - mean_q * mean_q;
    const double c_iq = t[4] / n - mean_i * mean_q;
    const int first = !st->measured;
    double a_dc = 1.0, a_iq = 1.0;
    if (!first) {
        if (st->dc_time_constant_s > 0.0 && rate > 0)
            a_dc = 1.0 - exp(-(double)count / (st->dc_time_constant_s * (double)rate));
        if (st->iq_time_constant_s > 0.0 && rate > 0)
            a_iq = 1.0 - exp(-(double)count / (st->iq_time_constant_s * (double)rate));
    }
    st->dc_i += a_dc * (mean_i - st->dc_i);
    st->dc_q += a_dc * (mean_q - st->dc_q);
    st->m_ii += a_iq * (c_ii - st->m_ii);
    st->m_qq += a_iq * (c_qq - st->m_qq);
    st->m_iq += a_iq * (c_iq - st->m_iq);
    st->measured = 1;
    st->samples_seen += count;
    if (st->m_ii > 0.0 && st->m_qq > 0.0) {
        st->gain = sqrt(st->m_qq / st->m_ii);
        st->sin_phase = st->m_iq / sqrt(st->m_ii * st->m_qq);
        const double gain_db = fabs(20.0 * log10(st->gain));
        const double sp = st->sin_phase < -1.0 ? -1.0 : (st->sin_phase > 1.0 ? 1.0 : st->sin_phase);
        const double phase_deg = fabs(asin(sp) * 180.0 / 3.141592653589793238462643383279502884);
        st->iq_plausible = isfinite(st->gain) && isfinite(st->sin_phase) && gain_db <= st->max_gain_error_db &&
                           phase_deg <= st->max_phase_error_deg;
    } else {
        st->gain = 1.0;
        st->sin_phase = 0.0;
        st->iq_plausible = 0;
    }
    return 0;
}

int32_t or_front_end_correction(const rv_front_end* st, int32_t dc, int32_t iq, rv_iq_correct_params* out) {
    out->dc_i = 0.0F;
    out->dc_q = 0.0F;
    out->cross = 0.0F;
    out->scale = 1.0F;
    if (!st->measured) return 0;
    if (dc) {
        out->dc_i = (float)st->dc_i;
        out->dc_q = (float)st->dc_q;
    }
    if (iq && st->iq_plausible) {
        const double cos_phase = sqrt(1.0 - st->sin_phase * st->sin_phase);
        out->cross = (float)(-st->sin_phase / cos_phase);
        out->scale = (float)(1.0 / (st->gain * cos_phase));
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* impulse excision: core/dsp/impulse_excision_reference.cpp          */

static uint64_t ring_size(uint32_t mask) { return (uint64_t)mask + 1u; }

static uint32_t bit_ceil_u32(uint32_t v) {
    uint32_t p = 1;
    while (p < v) p <<= 1;
    return p;
}

static uint64_t bit_ceil_u64(uint64_t v) {
    uint64_t p = 1;
    while (p < v) p <<= 1;
    return p;
}

static double clampd(double v, double lo, double hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* design_excision (impulse_excision_reference.cpp:57-80) */
int32_t or_design_excision(int64_t source_rate, double max_width_seconds, rv_excision_config* out) {
    const double rate = (double)(source_rate > 1 ? source_rate : 1);
    memset(out, 0, sizeof *out);
    out->max_width = (uint32_t)clampd(round(max_width_seconds * rate), 1.0, (double)RV_EXCISE_MAX_WIDTH);
    out->hang = (uint32_t)clampd(round(0.1e-6 * rate), 2.0, 16.0);
    out->lead = out->hang;
    const uint32_t quarter = (out->max_width + 3u) / 4u > 16u ? (out->max_width + 3u) / 4u : 16u;
    uint32_t log2 = 0;
    while ((1u << log2) < bit_ceil_u32(quarter)) ++log2;
    out->seg_log2 = log2 < RV_EXCISE_MAX_SEG_LOG2 ? log2 : RV_EXCISE_MAX_SEG_LOG2;
    out->segments = 32;
    return ok();
}

/* excision_threshold (:82-84) */
float or_excision_threshold(double threshold_db) { return (float)pow(10.0, threshold_db / 10.0); }

static int is_mask32(uint32_t m) { return is_pow2_u64(ring_size(m)); }

/* validate (:86-140) */
static int32_t excise_validate(const rv_excision_config* c, const rv_excision_params* p) {
    if (c->pass > RV_EXCISE_APPLY) return fail("excision: bad pass");
    if (c->seg_log2 < 2 || c->seg_log2 > RV_EXCISE_MAX_SEG_LOG2) return fail("excision: bad segment");
    if (c->segments < 2 || c->segments > RV_EXCISE_MAX_SEGMENTS) return fail("excision: bad segments");
    if (c->max_width < 1 || c->max_width > RV_EXCISE_MAX_WIDTH) return fail("excision: bad width");
    if (c->hang > RV_EXCISE_MAX_GUARD || c->lead > RV_EXCISE_MAX_GUARD) return fail("excision: bad guard");
    if (!is_mask32(p->ring_mask) || !is_mask32(p->seg_mask) || !is_mask32(p->flag_mask) || !is_mask32(p->removed_mask))
        return fail("excision: masks");
    const uint64_t ring = ring_size(p->ring_mask);
    if ((ring_size(p->seg_mask) << c->seg_log2) > ring || ring_size(p->flag_mask) > ring ||
        ring_size(p->removed_mask) > ring)
        return fail("excision: rings larger than the sample ring");
    if (c->pass == RV_EXCISE_SEGMENT || c->pass == RV_EXCISE_REFERENCE) {
        if ((p->first & ((1u << c->seg_log2) - 1u)) != 0u) return fail("excision: segment boundary");
        if ((uint64_t)p->count + c->segments + 2u > ring_size(p->seg_mask)) return fail("excision: segment ring");
    } else {
        const uint64_t reach = (uint64_t)p->count + 2u * (uint64_t)c->max_width + c->hang + c->lead;
        if (reach >= ring_size(p->flag_mask) || (c->pass == RV_EXCISE_APPLY && p->count > ring_size(p->removed_mask)))
            return fail("excision: flag or removed ring");
    }
    if (!(p->threshold > 0.0F)) return fail("excision: threshold");
    return 0;
}

/* size_excision_rings (:142-172) */
int32_t or_size_excision_rings(const rv_excision_config* c, uint64_t max_block, uint32_t frames_in_flight,
                               uint32_t ring_mask, rv_excision_rings* out) {
    const uint64_t frames = frames_in_flight > 1u ? frames_in_flight : 1u;
    const uint64_t segment = 1ull << c->seg_log2;
    const uint64_t reach = (uint64_t)c->max_width + c->lead;
    const uint64_t lag = reach > segment ? reach : segment;
    const uint64_t in_flight = max_block * frames;
    const uint64_t flags = bit_ceil_u64(in_flight + lag + 2u * (uint64_t)c->max_width + c->hang + c->lead + 1u);
    const uint64_t segs = bit_ceil_u64(in_flight / segment + c->segments + 4u);
    const uint64_t removed = bit_ceil_u64((max_block + lag) * frames);
    const uint64_t ring = ring_size(ring_mask);
    if (flags > ring || removed > ring || (segs << c->seg_log2) > ring) return fail("excision: ring too small");
    out->seg_mask = (uint32_t)(segs - 1u);
    out->flag_mask = (uint32_t)(flags - 1u);
    out->removed_mask = (uint32_t)(removed - 1u);
    return ok();
}

/* ExcisionCursor (:175-245) */
int32_t or_excision_cursor_init(rv_excision_cursor* k, const rv_excision_config* c, uint32_t ring_mask,
                                const rv_excision_rings* rings, float threshold) {
    memset(k, 0, sizeof *k);
    k->config = *c;
    k->ring_mask = ring_mask;
    k->rings = *rings;
    k->threshold = threshold;
    return ok();
}

static rv_excision_params cursor_params(const rv_excision_cursor* k, uint64_t first, uint32_t count) {
    rv_excision_params o;
    o.ring_mask = k->ring_mask;
    o.first = (uint32_t)(first & k->ring_mask);
    o.count = count;
    o.seg_mask = k->rings.seg_mask;
    o.flag_mask = k->rings.flag_mask;
    o.removed_mask = k->rings.removed_mask;
    const int64_t clamp = (int64_t)1 << 30;
    int64_t h = (int64_t)first - (int64_t)k->valid_from;
    h = h < -clamp ? -clamp : (h > clamp ? clamp : h);
    o.history = (int32_t)h;
    o.threshold = k->threshold;
    return o;
}

int32_t or_excision_plan_block(rv_excision_cursor* k, uint64_t start, uint32_t count, rv_excision_plan* out) {
    memset(out, 0, sizeof *out);
    out->segment.threshold = out->reference.threshold = out->flag.threshold = out->apply.threshold = 31.622776F;
    const uint64_t segment = 1ull << k->config.seg_log2;
    if (!k->running || start != k->next_in) {
        k->running = 1;
        out->restarted = 1;
        k->valid_from = start;
        k->seg_next = (start + segment - 1u) / segment;
        k->flag_next = start;
        k->apply_next = start;
    }
    const uint64_t end = start + count;
    k->next_in = end;
    const uint64_t seg_end = end / segment;
    if (seg_end > k->seg_next) {
        out->segment = cursor_params(k, k->seg_next * segment, (uint32_t)(seg_end - k->seg_next));
        k->seg_next = seg_end;
    }
    if (end > k->flag_next) {
        const uint64_t lo = k->flag_next / segment, hi = (end - 1u) / segment;
        out->reference = cursor_params(k, lo * segment, (uint32_t)(hi - lo + 1u));
        out->flag = cursor_params(k, k->flag_next, (uint32_t)(end - k->flag_next));
        k->flag_next = end;
    }
    const uint64_t reach = (uint64_t)k->config.max_width + k->config.lead;
    const uint64_t by_scan = end > reach ? end - reach : 0;
    const uint64_t by_segment = (end / segment) * segment;
    const uint64_t apply_end = by_scan < by_segment ? by_scan : by_segment;
    if (apply_end > k->apply_next) {
        out->apply = cursor_params(k, k->apply_next, (uint32_t)(apply_end - k->apply_next));
        k->apply_next = apply_end;
    }
    out->cleaned_end = k->apply_next;
    return ok();
}

static rv_excision_config with_pass(const rv_excision_config* c, uint32_t pass) {
    rv_excision_config o = *c;
    o.pass = pass;
    return o;
}

/* reference_excise_segment (:248-270): sequential fp32 sum of |x|^2 */
int32_t or_excise_segment(const rv_excision_config* c0, const rv_excision_params* p, const rv_cf32* raw,
                          uint64_t raw_len, float* seg_power, uint64_t seg_len) {
    const rv_excision_config c = with_pass(c0, RV_EXCISE_SEGMENT);
    if (excise_validate(&c, p)) return -1;
    if (raw_len < ring_size(p->ring_mask) || seg_len < ring_size(p->seg_mask)) return fail("excise_segment: short");
    flush_scope s;
    flush_begin(&s);
    const uint32_t n = 1u << c.seg_log2;
    for (uint32_t j = 0; j < p->count; ++j) {
        const uint32_t base = (p->first + (j << c.seg_log2)) & p->ring_mask;
        float sum = 0.0F;
        for (uint32_t m = 0; m < n; ++m) {
            const rv_cf32 v = raw[(base + m) & p->ring_mask];
            const float q = v.re * v.re + v.im * v.im;
            sum = sum + q;
        }
        seg_power[(base >> c.seg_log2) & p->seg_mask] = sum;
    }
    flush_end(&s);
    return ok();
}

/* reference_excise_reference (:272-306): the median (element K/2 after an
 * insertion sort) of the K segments before the guard segment */
int32_t or_excise_reference(const rv_excision_config* c0, const rv_excision_params* p, const float* seg_power,
                            float* seg_level, uint64_t seg_len) {
    const rv_excision_config c = with_pass(c0, RV_EXCISE_REFERENCE);
    if (excise_validate(&c, p)) return -1;
    if (seg_len < ring_size(p->seg_mask)) return fail("excise_reference: short");
    const int64_t segment = (int64_t)1 << c.seg_log2, window = c.segments;
    for (uint32_t j = 0; j < p->count; ++j) {
        const uint32_t base = (p->first + (j << c.seg_log2)) & p->ring_mask;
        const uint32_t slot = base >> c.seg_log2;
        const int64_t rel = (int64_t)j * segment;
        if (rel - (window + 1) * segment + p->history < 0) {
            seg_level[slot & p->seg_mask] = 0.0F;
            continue;
        }
        float v[RV_EXCISE_MAX_SEGMENTS];
        for (uint32_t m = 0; m < c.segments; ++m) v[m] = seg_power[(slot - 1u - c.segments + m) & p->seg_mask];
        for (uint32_t a = 1; a < c.segments; ++a) {
            const float x = v[a];
            uint32_t b = a;
            while (b > 0 && v[b - 1u] > x) {
                v[b] = v[b - 1u];
                --b;
            }
            v[b] = x;
        }
        seg_level[slot & p->seg_mask] = v[c.segments / 2u];
    }
    return ok();
}

/* reference_excise_flag (:308-330) */
int32_t or_excise_flag(const rv_excision_config* c0, const rv_excision_params* p, const rv_cf32* raw,
                       uint64_t raw_len, const float* seg_level, uint64_t seg_len, uint32_t* flags,
                       uint64_t flags_len) {
    const rv_excision_config c = with_pass(c0, RV_EXCISE_FLAG);
    if (excise_validate(&c, p)) return -1;
    if (raw_len < ring_size(p->ring_mask) || seg_len < ring_size(p->seg_mask) || flags_len < ring_size(p->flag_mask))
        return fail("excise_flag: short");
    flush_scope s;
    flush_begin(&s);
    const float samples = (float)(1u << c.seg_log2);
    for (uint32_t j = 0; j < p->count; ++j) {
        const uint32_t slot = (p->first + j) & p->ring_mask;
        const rv_cf32 v = raw[slot];
        const float pw = v.re * v.re + v.im * v.im;
        const float level = seg_level[(slot >> c.seg_log2) & p->seg_mask];
        const float lhs = pw * samples;
        const float rhs = p->threshold * level;
        flags[(p->first + j) & p->flag_mask] = (level > 0.0F && lhs > rhs) ? 1u : 0u;
    }
    flush_end(&s);
    return ok();
}

static int excise_flag_at(const rv_excision_params* p, const uint32_t* flags, int64_t rel) {
    if (rel + p->history < 0) return 0;
    return flags[(p->first + (uint32_t)rel) & p->flag_mask] != 0u;
}

static int excise_marked(const rv_excision_config* c, const rv_excision_params* p, const uint32_t* flags,
                         int64_t rel) {
    for (uint32_t m = 0; m <= c->hang + c->lead; ++m)
        if (excise_flag_at(p, flags, rel - (int64_t)c->hang + m)) return 1;
    return 0;
}

/* reference_excise_apply (:332-378) */
int32_t or_excise_apply(const rv_excision_config* c0, const rv_excision_params* p, const rv_cf32* raw,
                        uint64_t raw_len, const uint32_t* flags, uint64_t flags_len, rv_cf32* cleaned,
                        rv_cf32* removed, uint64_t removed_len, uint32_t* counters) {
    const rv_excision_config c = with_pass(c0, RV_EXCISE_APPLY);
    if (excise_validate(&c, p)) return -1;
    if (raw_len < ring_size(p->ring_mask) || flags_len < ring_size(p->flag_mask) ||
        removed_len < ring_size(p->removed_mask))
        return fail("excise_apply: short");
    rv_cf32 nothing;
    const uint32_t neg_zero = 0x80000000u;
    memcpy(&nothing.re, &neg_zero, 4);
    memcpy(&nothing.im, &neg_zero, 4);
    for (uint32_t j = 0; j < p->count; ++j) {
        const int64_t rel = j;
        const uint32_t slot = (p->first + j) & p->ring_mask;
        const rv_cf32 x = raw[slot];
        int excise = 0;
        if (excise_marked(&c, p, flags, rel)) {
            uint32_t left = 0, right = 0;
            for (uint32_t k = 1; k <= c.max_width; ++k) {
                if (!excise_marked(&c, p, flags, rel - k)) break;
                ++left;
            }
            for (uint32_t k = 1; k <= c.max_width; ++k) {
                if (!excise_marked(&c, p, flags, rel + k)) break;
                ++right;
            }
            excise = left + right + 1u <= c.max_width;
            if (left == 0u) counters[excise ? RV_EXCISE_COUNTER_EVENTS : RV_EXCISE_COUNTER_SPARED] += 1u;
        }
        if (excise) counters[RV_EXCISE_COUNTER_SAMPLES] += 1u;
        cleaned[slot] = excise ? nothing : x;
        removed[(p->first + j) & p->removed_mask] = excise ? x : nothing;
    }
    return ok();
}

/* ------------------------------------------------------------------ */
/* per-receiver noise stages: core/dsp/noise_reference.cpp            */

/* design_blanker (:112-121) */
int32_t or_design_blanker(int64_t channel_rate, rv_blanker_config* out) {
    memset(out, 0, sizeof *out);
    out->window = (uint32_t)clampd(round(0.5e-3 * (double)channel_rate), 16.0, 256.0);
    out->hang = 2;
    out->lead = 2;
    out->guard = out->lead + 2u;
    return ok();
}

float or_blanker_threshold(double threshold_db) { return (float)pow(10.0, threshold_db / 10.0); }

static int32_t blanker_valid(const rv_blanker_config* c, const rv_blanker_params* p) {
    if (c->pass > 1u) return fail("blanker: pass");
    if (c->window < 16u || c->window > 256u) return fail("blanker: window");
    if (!is_mask32(p->chan_mask) || !is_mask32(p->out_mask)) return fail("blanker: masks");
    const uint64_t reach = (uint64_t)c->hang + c->guard + c->window + c->lead + p->count;
    const uint64_t smaller = (uint64_t)(p->chan_mask < p->out_mask ? p->chan_mask : p->out_mask) + 1u;
    if (reach >= smaller) return fail("blanker: reach");
    if (!(p->threshold > 0.0F)) return fail("blanker: threshold");
    return 0;
}

/* reference_blank_detect (:158-195) */
int32_t or_blank_detect(const rv_blanker_config* c0, const rv_blanker_params* p, const rv_cf32* chan,
                        uint64_t chan_len, float* flags, uint64_t flags_len) {
    rv_blanker_config c = *c0;
    c.pass = 0;
    if (blanker_valid(&c, p)) return -1;
    if (flags_len < (uint64_t)p->out_mask + 1u || chan_len < (uint64_t)p->chan_base + p->chan_mask + 1u)
        return fail("blank_detect: short");
    flush_scope s;
    flush_begin(&s);
    const float window = (float)c.window;
    for (uint32_t i = 0; i < p->count; ++i) {
        const uint32_t ch = (p->chan_first + i) & p->chan_mask;
        const uint32_t o = (p->out_first + i) & p->out_mask;
        const rv_cf32 x = chan[p->chan_base + ch];
        const float pw = x.re * x.re + x.im * x.im;
        float sum = 0.0F;
        for (uint32_t m = 0; m < c.window; ++m) {
            const rv_cf32 r = chan[p->chan_base + ((ch - c.guard - c.window + m) & p->chan_mask)];
            const float q = r.re * r.re + r.im * r.im;
            sum = sum + q;
        }
        const float lhs = pw * window;
        const float rhs = p->threshold * sum;
        flags[o] = (sum > 0.0F && lhs > rhs) ? 1.0F : 0.0F;
    }
    flush_end(&s);
    return ok();
}

/* reference_blank_apply (:197-225) */
int32_t or_blank_apply(const rv_blanker_config* c0, const rv_blanker_params* p, const rv_cf32* chan,
                       uint64_t chan_len, const float* flags, uint64_t flags_len, rv_cf32* blanked,
                       uint64_t blanked_len) {
    rv_blanker_config c = *c0;
    c.pass = 1;
    if (blanker_valid(&c, p)) return -1;
    if (flags_len < (uint64_t)p->out_mask + 1u || blanked_len < (uint64_t)p->out_mask + 1u ||
        chan_len < (uint64_t)p->chan_base + p->chan_mask + 1u)
        return fail("blank_apply: short");
    for (uint32_t i = 0; i < p->count; ++i) {
        const uint32_t ch = (p->chan_first + i) & p->chan_mask;
        const uint32_t o = (p->out_first + i) & p->out_mask;
        int hit = 0;
        for (uint32_t m = 0; m <= c.hang + c.lead; ++m)
            if (flags[(o - c.hang + m) & p->out_mask] != 0.0F) hit = 1;
        if (hit) {
            blanked[o].re = 0.0F;
            blanked[o].im = 0.0F;
        } else {
            blanked[o] = chan[p->chan_base + ch];
        }
    }
    return ok();
}

static uint32_t line_sections_of(uint32_t flags) {
    return (flags & RV_LINE_NOTCH) == 0u ? 0u : 1u + ((flags >> RV_LINE_NOTCH_COUNT_SHIFT) & 3u);
}

static float biquad_step(float* st, float b0, float b1, float b2, float a1, float a2, float x) {
    const float t0 = b0 * x;
    const float t1 = b1 * st[0];
    const float t2 = b2 * st[1];
    const float t3 = a1 * st[2];
    const float t4 = a2 * st[3];
    float acc = t0 + t1;
    acc = acc + t2;
    acc = acc - t3;
    acc = acc - t4;
    st[1] = st[0];
    st[0] = x;
    st[3] = st[2];
    st[2] = acc;
    return acc;
}

/* reference_line (:265-420) */
int32_t or_noise_line(const rv_line_config* c, const rv_line_params* p, float* audio, uint64_t audio_len,
                      float* state, uint64_t state_len) {
    if (c->lanes == 0 || c->taps == 0 || c->taps % c->lanes != 0) return fail("line: lanes");
    if (!is_pow2_u64(c->history)) return fail("line: history");
    if (p->stride == 0 || p->stride > RV_LINE_MAX_STRIDE) return fail("line: stride");
    if (p->delay == 0) return fail("line: delay");
    if ((uint64_t)p->delay + (uint64_t)(c->taps - 1u) * p->stride >= c->history) return fail("line: reach");
    if (!(p->eps > 0.0F)) return fail("line: eps");
    if ((p->flags & ~(uint32_t)(RV_LINE_NOTCH | RV_LINE_ALE | RV_LINE_GUARD | (3u << RV_LINE_NOTCH_COUNT_SHIFT))) != 0u)
        return fail("line: flags");
    if (audio_len < p->count || state_len < (uint64_t)RV_LINE_STATE_WEIGHTS + c->taps + c->history)
        return fail("line: short");
    flush_scope s;
    flush_begin(&s);
    const int notch = (p->flags & RV_LINE_NOTCH) != 0u;
    const int ale = (p->flags & RV_LINE_ALE) != 0u;
    const int guard = ale && (p->flags & RV_LINE_GUARD) != 0u;
    const uint32_t sections = line_sections_of(p->flags);
    const uint32_t per_lane = c->taps / c->lanes, hmask = c->history - 1u;
    float* w = state + RV_LINE_STATE_WEIGHTS;
    float* hist = w + c->taps;
    float* ref = (float*)malloc(sizeof(float) * c->taps);
    float* part_y = (float*)malloc(sizeof(float) * c->lanes);
    float* part_p = (float*)malloc(sizeof(float) * c->lanes);
    float n0[4] = {state[0], state[1], state[2], state[3]};
    float more[3][4];
    for (uint32_t k = 0; k + 1u < sections; ++k)
        for (int j = 0; j < 4; ++j) more[k][j] = state[RV_LINE_STATE_MORE + 4 * k + j];
    float g[4] = {state[RV_LINE_STATE_GUARD], state[RV_LINE_STATE_GUARD + 1], state[RV_LINE_STATE_GUARD + 2],
                  state[RV_LINE_STATE_GUARD + 3]};
    uint32_t position = (uint32_t)state[RV_LINE_STATE_POSITION];
    for (uint32_t n = 0; n < p->count; ++n) {
        const float x = audio[n];
        float v = x;
        if (notch) {
            v = biquad_step(n0, p->b0, p->b1, p->b2, p->a1, p->a2, x);
            for (uint32_t k = 0; k + 1u < sections; ++k)
                v = biquad_step(more[k], p->more[k].b0, p->more[k].b1, p->more[k].b2, p->more[k].a1, p->more[k].a2, v);
        }
        float out = v;
        if (ale) {
            for (uint32_t lane = 0; lane < c->lanes; ++lane) {
                float py = 0.0F, pp = 0.0F;
                for (uint32_t j = 0; j < per_lane; ++j) {
                    const uint32_t k = lane + j * c->lanes;
                    const float r = hist[(position - p->delay - k * p->stride) & hmask];
                    ref[k] = r;
                    const float wy = w[k] * r;
                    py = py + wy;
                    const float rr = r * r;
                    pp = pp + rr;
                }
                part_y[lane] = py;
                part_p[lane] = pp;
            }
            float y = 0.0F, pw = 0.0F;
            for (uint32_t lane = 0; lane < c->lanes; ++lane) {
                y = y + part_y[lane];
                pw = pw + part_p[lane];
            }
            const float e = v - y;
            const float gain = p->mu * det_recip(pw + p->eps);
            const float ge = gain * e;
            for (uint32_t k = 0; k < c->taps; ++k) {
                const float kept = p->leak * w[k];
                const float step = ge * ref[k];
                w[k] = kept + step;
            }
            hist[position & hmask] = v;
            out = e;
            if (guard) out = v - biquad_step(g, p->gb0, p->gb1, p->gb2, p->ga1, p->ga2, y);
        }
        audio[n] = out;
        position = position + 1u;
    }
    state[0] = n0[0];
    state[1] = n0[1];
    state[2] = n0[2];
    state[3] = n0[3];
    for (uint32_t k = 0; k + 1u < sections; ++k)
        for (int j = 0; j < 4; ++j) state[RV_LINE_STATE_MORE + 4 * k + j] = more[k][j];
    state[RV_LINE_STATE_POSITION] = (float)(position & hmask);
    for (int j = 0; j < 4; ++j) state[RV_LINE_STATE_GUARD + j] = g[j];
    free(ref);
    free(part_y);
    free(part_p);
    flush_end(&s);
    return ok();
}

/* design_notch (:424-459) */
int32_t or_design_notch(double audio_hz, double depth_db, double width_hz, int64_t audio_rate, rv_notch_design* d) {
    if (audio_rate <= 0) return fail("notch: rate");
    const double fa = (double)audio_rate, pi = 3.14159265358979323846;
    if (!(audio_hz > 0.0) || !(audio_hz < 0.5 * fa)) return fail("notch: frequency");
    if (!(width_hz > 0.0) || !(width_hz < 0.25 * fa)) return fail("notch: width");
    const double omega = 2.0 * pi * audio_hz / fa;
    const double rp = 1.0 - pi * width_hz / fa;
    const double rz = 1.0 - (1.0 - rp) * pow(10.0, -depth_db / 20.0);
    const double cs = cos(omega);
    d->b0 = 1.0;
    d->b1 = -2.0 * rz * cs;
    d->b2 = rz * rz;
    d->a1 = -2.0 * rp * cs;
    d->a2 = rp * rp;
    const double z = (omega < 0.5 * pi) ? -1.0 : 1.0;
    const double scale = (1.0 + d->a1 * z + d->a2) / (d->b0 + d->b1 * z + d->b2);
    d->b0 *= scale;
    d->b1 *= scale;
    d->b2 *= scale;
    return ok();
}

/* spectral_config_for (:493-501) */
int32_t or_spectral_config_for(int64_t audio_rate, rv_spectral_config* out) {
    const uint64_t wanted = audio_rate > 0 ? (uint64_t)audio_rate / 90u : 64u;
    uint64_t f = 1;
    while (f * 2u <= (wanted > 1u ? wanted : 1u)) f *= 2u;
    out->frame = (uint32_t)(f < 64u ? 64u : (f > 512u ? 512u : f));
    return ok();
}

/* design_spectral_tables (:503-539) */
int32_t or_design_spectral_tables(const rv_spectral_config* c, float* t, uint64_t len) {
    const uint32_t n = c->frame;
    if (len < 4ull * n) return fail("spectral tables: short");
    const double pi = 3.14159265358979323846, step = 2.0 * pi / (double)n;
    for (uint32_t k = 0; k < n; ++k) {
        double cs = cos(step * (double)k), sn = sin(step * (double)k);
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
        t[k] = (float)cs;
        t[n + k] = (float)sn;
        const double w = sin(pi * ((double)k + 0.5) / (double)n);
        t[2u * n + k] = (float)w;
        t[3u * n + k] = (float)(w / (double)n);
    }
    return ok();
}

/* spectral_params (:541-554) */
int32_t or_design_spectral_params(double strength, rv_spectral_params* o) {
    const double s = strength < 0.0 ? 0.0 : (strength > 1.0 ? 1.0 : strength);
    memset(o, 0, sizeof *o);
    o->smoothing = (float)0.7;
    o->smoothing_complement = (float)(1.0 - 0.7);
    o->gamma = (float)0.998;
    o->beta = (float)0.96;
    o->rise = (float)((1.0 - 0.998) / (1.0 - 0.96));
    o->bias = (float)2.4;
    o->alpha = (float)(1.0 + s);
    o->floor_gain = (float)pow(10.0, -(6.0 + 12.0 * s) / 20.0);
    o->eps = (float)1.0e-12;
    return ok();
}

/* reference_spectral (:568-684) */
int32_t or_noise_spectral(const rv_spectral_config* c, const rv_spectral_params* p, const float* tables,
                          uint64_t tables_len, float* audio, uint64_t audio_len, float* state, uint64_t state_len) {
    const uint32_t n = c->frame, h = n / 2u, bins = h + 1u, mask = n - 1u;
    if (!is_pow2_u64(n) || n < 64u || n > 512u) return fail("spectral: frame");
    if (!(p->eps > 0.0F)) return fail("spectral: eps");
    if (tables_len < 4ull * n || audio_len < p->count || state_len < 2u + n + h + h + 2u * bins)
        return fail("spectral: short");
    flush_scope sc;
    flush_begin(&sc);
    const float* cosine = tables;
    const float* sine = tables + n;
    const float* analysis = sine + n;
    const float* synthesis = analysis + n;
    float* hist = state + 2;
    float* tail = hist + n;
    float* queue = tail + h;
    float* smoothed = queue + h;
    float* minimum = smoothed + bins;
    uint32_t phase = (uint32_t)state[0];
    float seen = state[1];
    float work[512], y_re[257], y_im[257];
    uint32_t s = 0;
    while (s < p->count) {
        const uint32_t length = (h - phase) < (p->count - s) ? (h - phase) : (p->count - s);
        for (uint32_t i = 0; i < length; ++i) {
            const float x = audio[s + i];
            hist[h + phase + i] = x;
            audio[s + i] = queue[phase + i];
        }
        phase += length;
        s += length;
        if (phase != h) continue;
        for (uint32_t t = 0; t < n; ++t) work[t] = hist[t] * analysis[t];
        for (uint32_t k = 0; k < bins; ++k) {
            float re = 0.0F, im = 0.0F;
            for (uint32_t t = 0; t < n; ++t) {
                const uint32_t at = (k * t) & mask;
                const float xc = work[t] * cosine[at];
                re = re + xc;
                const float xs = work[t] * sine[at];
                im = im - xs;
            }
            const float rr = re * re;
            const float ii = im * im;
            const float power = rr + ii;
            float level = power, floor_power = power;
            if (seen != 0.0F) {
                const float previous = smoothed[k];
                const float kept = p->smoothing * previous;
                const float fresh = p->smoothing_complement * power;
                level = kept + fresh;
                const float held = minimum[k];
                if (held < level) {
                    const float decayed = p->gamma * held;
                    const float lagged = p->beta * previous;
                    const float lift = level - lagged;
                    const float risen = p->rise * lift;
                    floor_power = decayed + risen;
                } else {
                    floor_power = level;
                }
            }
            smoothed[k] = level;
            minimum[k] = floor_power;
            const float noise = p->bias * floor_power;
            const float ratio = noise * det_recip(level + p->eps);
            const float cut = p->alpha * ratio;
            float gain = 1.0F - cut;
            if (gain < p->floor_gain) gain = p->floor_gain;
            y_re[k] = gain * re;
            y_im[k] = gain * im;
        }
        for (uint32_t t = 0; t < n; ++t) {
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
        for (uint32_t t = 0; t < h; ++t) {
            queue[t] = tail[t] + work[t];
            tail[t] = work[h + t];
            hist[t] = hist[h + t];
        }
        phase = 0;
        seen = seen + 1.0F < 2.0F ? seen + 1.0F : 2.0F;
    }
    state[0] = (float)phase;
    state[1] = seen;
    flush_end(&sc);
    return ok();
}

/* ------------------------------------------------------------------ */
/* comb cancellation: core/dsp/comb_kernels_reference.cpp             */

uint32_t or_comb_step(double frequency_hz, int64_t rate) {
    if (rate <= 0 || !isfinite(frequency_hz)) return 0;
    const double cycle = 4294967296.0;
    double steps = round(frequency_hz / (double)rate * cycle);
    steps = fmod(steps, cycle);
    if (steps < 0.0) steps += cycle;
    return (uint32_t)(uint64_t)steps;
}

int32_t or_comb_table(rv_cf32* t, uint64_t len) {
    if (len < RV_COMB_TABLE_SIZE) return fail("comb table: short");
    const double pi = 3.14159265358979323846;
    for (uint32_t i = 0; i < RV_COMB_TABLE_SIZE; ++i) {
        const double angle = 2.0 * pi * (double)i / (double)RV_COMB_TABLE_SIZE;
        t[i].re = (float)cos(angle);
        t[i].im = (float)sin(angle);
    }
    return ok();
}

static int32_t comb_valid(const rv_comb_params* p) {
    if (!is_mask32(p->ring_mask) || !is_mask32(p->removed_mask)) return fail("comb: masks");
    if (p->removed_mask > p->ring_mask) return fail("comb: removed ring");
    if (p->lines > RV_COMB_MAX_LINES) return fail("comb: lines");
    if (p->sub_blocks < 1 || p->sub_blocks > RV_COMB_MAX_SUB_BLOCKS) return fail("comb: sub-blocks");
    if (p->count == 0 || p->count % p->sub_blocks != 0) return fail("comb: count");
    if ((uint64_t)p->count > (uint64_t)p->removed_mask + 1u) return fail("comb: removed ring too short");
    return 0;
}

static rv_cf32 comb_tone(const rv_cf32* table, const rv_comb_line* l, uint32_t n) {
    return table[(l->phase0 + n * l->step) >> (32u - RV_COMB_TABLE_LOG2)];
}

/* reference_comb_project */
int32_t or_comb_project(const rv_comb_params* p, const rv_cf32* raw, uint64_t raw_len, const rv_comb_line* lines,
                        uint64_t lines_len, const rv_cf32* table, uint64_t table_len, rv_cf32* proj,
                        uint64_t proj_len) {
    if (comb_valid(p)) return -1;
    if (raw_len < (uint64_t)p->ring_mask + 1u || lines_len < p->lines || table_len != RV_COMB_TABLE_SIZE ||
        proj_len < (uint64_t)p->lines * p->sub_blocks)
        return fail("comb_project: short");
    flush_scope s;
    flush_begin(&s);
    const uint32_t length = p->count / p->sub_blocks;
    for (uint32_t l = 0; l < p->lines; ++l)
        for (uint32_t sb = 0; sb < p->sub_blocks; ++sb) {
            const uint32_t begin = sb * length;
            float tr = 0.0F, ti = 0.0F;
            for (uint32_t c = 0; c < length; c += 64u) {
                const uint32_t end = c + 64u < length ? c + 64u : length;
                float cr = 0.0F, ci = 0.0F;
                for (uint32_t m = c; m < end; ++m) {
                    const uint32_t n = begin + m;
                    const rv_cf32 x = raw[(p->first + n) & p->ring_mask];
                    const rv_cf32 t = comb_tone(table, &lines[l], n);
                    const float re = x.re * t.re + x.im * t.im;
                    const float im = x.im * t.re - x.re * t.im;
                    cr = cr + re;
                    ci = ci + im;
                }
                tr = tr + cr;
                ti = ti + ci;
            }
            proj[(uint64_t)l * p->sub_blocks + sb].re = tr;
            proj[(uint64_t)l * p->sub_blocks + sb].im = ti;
        }
    flush_end(&s);
    return ok();
}

/* reference_comb_subtract */
int32_t or_comb_subtract(const rv_comb_params* p, const rv_cf32* raw, uint64_t raw_len, const rv_comb_line* lines,
                         uint64_t lines_len, const rv_cf32* table, uint64_t table_len, rv_cf32* cleaned,
                         uint64_t cleaned_len, rv_cf32* removed, uint64_t removed_len) {
    if (comb_valid(p)) return -1;
    if (raw_len < (uint64_t)p->ring_mask + 1u || cleaned_len < (uint64_t)p->ring_mask + 1u || lines_len < p->lines ||
        table_len != RV_COMB_TABLE_SIZE || removed_len < (uint64_t)p->removed_mask + 1u)
        return fail("comb_subtract: short");
    flush_scope s;
    flush_begin(&s);
    for (uint32_t n = 0; n < p->count; ++n) {
        const uint32_t slot = (p->first + n) & p->ring_mask;
        const rv_cf32 x = raw[slot];
        float sr = -0.0F, si = -0.0F;
        for (uint32_t l = 0; l < p->lines; ++l) {
            const rv_cf32 t = comb_tone(table, &lines[l], n);
            const rv_cf32 a = lines[l].amplitude;
            const float re = a.re * t.re - a.im * t.im;
            const float im = a.re * t.im + a.im * t.re;
            sr = sr + re;
            si = si + im;
        }
        if (p->lines == 0) {
            cleaned[slot] = x;
        } else {
            cleaned[slot].re = x.re - sr;
            cleaned[slot].im = x.im - si;
        }
        removed[(p->first + n) & p->removed_mask].re = sr;
        removed[(p->first + n) & p->removed_mask].im = si;
    }
    flush_end(&s);
    return ok();
}

/* ---- scene noise: siggen::Scene::fill_noise ------------------------------
 * core/dsp/synth/wideband.cpp:535-580 restated: 4096-sample noise blocks,
 * block b drawing from an MT19937-64 (the C++ standard's mt19937_64, the
 * published algorithm of Matsumoto and Nishimura) seeded with
 * derive_stream_seed(seed ^ b, noise domain) (wideband.cpp:46-53), two draws
 * per sample, Box-Muller in FP64 with the C library's log, sqrt, cos, sin. */

#define OR_NOISE_BLOCK 4096u
#define OR_MT_N 312u
#define OR_MT_M 156u

static uint64_t or_derive_stream_seed(uint64_t master, uint64_t domain) {
    uint64_t z = master + domain * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

typedef struct {
    uint64_t mt[OR_MT_N];
    uint32_t index;
} or_mt64;

static void or_mt64_seed(or_mt64* g, uint64_t seed) {
    g->mt[0] = seed;
    for (uint32_t i = 1; i < OR_MT_N; ++i) g->mt[i] = 6364136223846793005ull * (g->mt[i - 1] ^ (g->mt[i - 1] >> 62)) + i;
    g->index = OR_MT_N;
}

static uint64_t or_mt64_next(or_mt64* g) {
    if (g->index >= OR_MT_N) {
        for (uint32_t i = 0; i < OR_MT_N; ++i) {
            const uint64_t y = (g->mt[i] & 0xFFFFFFFF80000000ull) | (g->mt[(i + 1) % OR_MT_N] & 0x7FFFFFFFull);
            g->mt[i] = g->mt[(i + OR_MT_M) % OR_MT_N] ^ (y >> 1) ^ ((y & 1ull) ? 0xB5026F5AA96619E9ull : 0ull);
        }
        g->index = 0;
    }
    uint64_t y = g->mt[g->index++];
    y ^= (y >> 29) & 0x5555555555555555ull;
    y ^= (y << 17) & 0x71D67FFFEDA60000ull;
    y ^= (y << 37) & 0xFFF7EEE000000000ull;
    return y ^ (y >> 43);
}

double or_scene_noise_sigma(double dbfs) { return sqrt(pow(10.0, dbfs * 0.1) * 0.5); }

/* draws (2 per sample) or samples of [start, start + count) */
static int32_t scene_noise_any(uint64_t seed, double sigma, uint64_t start, uint64_t count, rv_cf32* out,
                               uint64_t* draws) {
    const double step = 1.0 / 9007199254740992.0, two_pi = 6.283185307179586476925286766559;
    const uint64_t end = start + count;
    uint64_t index = start;
    or_mt64* g = (or_mt64*)malloc(sizeof(or_mt64));
    if (g == NULL) return fail("scene noise: out of memory");
    while (index < end) {
        const uint64_t block = index / OR_NOISE_BLOCK, block_start = block * OR_NOISE_BLOCK;
        const uint64_t stop = end < block_start + OR_NOISE_BLOCK ? end : block_start + OR_NOISE_BLOCK;
        or_mt64_seed(g, or_derive_stream_seed(seed ^ block, 0x1a59017e55ce0d02ull));
        for (uint64_t skipped = block_start; skipped < index; ++skipped) {
            (void)or_mt64_next(g);
            (void)or_mt64_next(g);
        }
        for (; index < stop; ++index) {
            const uint64_t first = or_mt64_next(g), second = or_mt64_next(g);
            if (draws) {
                draws[2 * (index - start)] = first;
                draws[2 * (index - start) + 1] = second;
                continue;
            }
            const double radial = (double)((first >> 11) + 1ull) * step;
            const double angular = (double)(second >> 11) * step;
            const double magnitude = sigma * sqrt(-2.0 * log(radial));
            const double angle = two_pi * angular;
            out[index - start].re = (float)(magnitude * cos(angle));
            out[index - start].im = (float)(magnitude * sin(angle));
        }
    }
    free(g);
    return ok();
}

int32_t or_scene_noise(uint64_t seed, double sigma, uint64_t start, uint64_t count, rv_cf32* out) {
    return scene_noise_any(seed, sigma, start, count, out, NULL);
}

int32_t or_scene_noise_draws(uint64_t seed, uint64_t start, uint64_t count, uint64_t* draws) {
    return scene_noise_any(seed, 0.0, start, count, NULL, draws);
}

/* ---- tone emitters: siggen::Modulator::accumulate_am / _nfm / _ssb -------
 * core/dsp/synth/modulators.cpp:1244-1366 restated, with walk_anchored
 * (:99-122: phasors re-anchored every 1024 emitter samples from exact_phase,
 * :439-449, and advanced by complex multiply) and Phasor (:58-83). */

static double or_exact_phase(int64_t frequency, int64_t rate, uint64_t index) {
    int64_t reduced = frequency % rate;
    if (reduced < 0) reduced += rate;
    const int64_t position = (int64_t)(index % (uint64_t)rate);
    const int64_t turns = (reduced * position) % rate;
    return 6.283185307179586476925286766559 * (double)turns / (double)rate;
}

/* CW: Morse (ITU-R M.1677, the reference's character set) and the keyed
 * elements of one message cycle (modulators.cpp:124-161, :675-741). */
static const char* or_morse(char c) {
    static const char* const letters[26] = {".-", "-...", "-.-.", "-..", ".", "..-.", "--.", "....", "..", ".---",
                                            "-.-", ".-..", "--", "-.", "---", ".--.", "--.-", ".-.", "...", "-",
                                            "..-", "...-", ".--", "-..-", "-.--", "--.."};
    static const char* const digits[10] = {"-----", ".----", "..---", "...--", "....-",
                                           ".....", "-....", "--...", "---..", "----."};
    if (c >= 'a' && c <= 'z') c = (char)(c - 'a' + 'A');
    if (c >= 'A' && c <= 'Z') return letters[c - 'A'];
    if (c >= '0' && c <= '9') return digits[c - '0'];
    switch (c) {
        case '.': return ".-.-.-";
        case ',': return "--..--";
        case '?': return "..--..";
        case '/': return "-..-.";
        case '=': return "-...-";
        case '+': return ".-.-.";
        case '-': return "-....-";
        case ':': return "---...";
        default: return NULL;
    }
}

typedef struct {
    int64_t start, stop;
    int keyed;
} or_cw_element;

static uint32_t or_cw_elements(const char* text, double dot, double gap, or_cw_element* out, uint32_t cap) {
    int on[1024];
    double dots[1024];
    uint32_t n = 0;
#define OFF(d)                                           \
    do {                                                 \
        const double dd = (d);                           \
        if (dd > 0.0) {                                  \
            if (n > 0 && !on[n - 1]) dots[n - 1] += dd;  \
            else if (n < 1024) on[n] = 0, dots[n++] = dd; \
        }                                                \
    } while (0)
    for (const char* c = text; *c; ++c) {
        if (*c == ' ') {
            OFF(4.0);
            continue;
        }
        for (const char* m = or_morse(*c); *m; ++m) {
            if (n < 1024) on[n] = 1, dots[n++] = (*m == '.') ? 1.0 : 3.0;
            OFF(1.0);
        }
        OFF(2.0);
    }
    OFF(gap - 3.0 > 0.0 ? gap - 3.0 : 0.0);
#undef OFF
    double cumulative = 0.0;
    int64_t previous = 0;
    uint32_t k = 0;
    for (uint32_t i = 0; i < n && k < cap; ++i) {
        cumulative += dots[i];
        int64_t edge = (int64_t)llround(cumulative * dot);
        if (edge <= previous) edge = previous + 1;
        out[k].start = previous;
        out[k].stop = edge;
        out[k].keyed = on[i];
        ++k;
        previous = edge;
    }
    return k;
}

static double or_cw_envelope(const or_cw_element* el, uint32_t n, double ramp_samples, uint64_t index) {
    const double pi = 3.141592653589793238462643383279502884;
    const int64_t position = (int64_t)(index % (uint64_t)el[n - 1].stop);
    uint32_t i = 0;
    while (i + 1 < n && el[i].stop <= position) ++i;
    if (!el[i].keyed) return 0.0;
    const double length = (double)(el[i].stop - el[i].start);
    const double ramp = ramp_samples < length * 0.5 ? ramp_samples : length * 0.5;
    if (ramp <= 0.0) return 1.0;
    const double from_start = (double)(position - el[i].start), to_end = (double)(el[i].stop - position);
    double envelope = 1.0;
    if (from_start < ramp) envelope *= 0.5 - 0.5 * cos(pi * from_start / ramp);
    if (to_end <= ramp) envelope *= 0.5 - 0.5 * cos(pi * to_end / ramp);
    return envelope;
}

/* FSK2 (modulators.cpp:216-257 symbol clock, :402-423 index_at, :454-472
 * random_bits, :850-882 phase prefix, :1393-1441 accumulate_fsk) */
static int32_t or_fsk_accumulate(const rv_tone_emitter* e, uint64_t first, uint64_t count, double gain, rv_cf32* io) {
    const double two_pi = 6.283185307179586476925286766559;
    const uint64_t symbols = e->symbol_count;
    if (symbols == 0 || symbols > 1000000) return fail("fsk: symbol count");
    const double rate = (double)e->rate;
    const double real = (double)symbols * (rate / e->symbol_rate);
    const int64_t cycle = (int64_t)llround(real);
    if (cycle < (int64_t)symbols * 2) return fail("fsk: under two samples per symbol");
    uint8_t* bits = (uint8_t*)malloc(symbols);
    int64_t* boundary = (int64_t*)malloc((symbols + 1) * sizeof(int64_t));
    double* prefix = (double*)malloc((symbols + 1) * sizeof(double));
    or_mt64* g = (or_mt64*)malloc(sizeof(or_mt64));
    if (!bits || !boundary || !prefix || !g) return fail("fsk: out of memory");
    or_mt64_seed(g, e->seed);
    uint64_t word = 0;
    unsigned remaining = 0;
    for (uint64_t i = 0; i < symbols; ++i) {
        if (remaining == 0) word = or_mt64_next(g), remaining = 64;
        bits[i] = (uint8_t)(word & 1u);
        word >>= 1;
        --remaining;
    }
    for (uint64_t k = 0; k <= symbols; ++k) boundary[k] = ((int64_t)k * cycle) / (int64_t)symbols;
    const double upper = two_pi * (double)e->deviation / rate, lower = -upper;
    double accumulated = 0.0;
    for (uint64_t k = 0; k < symbols; ++k) {
        prefix[k] = accumulated;
        accumulated += (bits[k] != 0 ? upper : lower) * (double)(boundary[k + 1] - boundary[k]);
        accumulated = fmod(accumulated, two_pi);
    }
    const double cycle_phase = accumulated, level = gain * e->amplitude;
    const double carrier_step = two_pi * (double)e->carrier_offset / rate;
    const uint64_t end = first + count;
    uint64_t index = first;
    while (index < end) {
        const int64_t repeat = (int64_t)index / cycle, position = (int64_t)index - repeat * cycle;
        uint64_t sym = (uint64_t)((position * (int64_t)symbols) / cycle);
        if (sym >= symbols) sym = symbols - 1;
        while (sym + 1 < symbols && boundary[sym + 1] <= position) ++sym;
        while (sym > 0 && boundary[sym] > position) --sym;
        const uint64_t ss = (uint64_t)(repeat * cycle + boundary[sym]), se = (uint64_t)(repeat * cycle + boundary[sym + 1]);
        const uint64_t grid = index - index % 1024u;
        const uint64_t anchor = grid > ss ? grid : ss;
        uint64_t stop = end < se ? end : se;
        if (grid + 1024u < stop) stop = grid + 1024u;
        const double sense = bits[sym] != 0 ? 1.0 : -1.0;
        const double phase = e->initial_phase + or_exact_phase(e->carrier_offset, e->rate, anchor) +
                             fmod((double)repeat * cycle_phase, two_pi) + prefix[sym] +
                             sense * upper * (double)(anchor - ss);
        const double step = carrier_step + sense * upper;
        double re = cos(phase), im = sin(phase);
        const double sr = cos(step), si = sin(step);
        for (uint64_t k = anchor; k < stop; ++k) {
            if (k >= index) {
                io[k - first].re = io[k - first].re + (float)(level * re);
                io[k - first].im = io[k - first].im + (float)(level * im);
            }
            const double nre = re * sr - im * si, nim = re * si + im * sr;
            re = nre, im = nim;
        }
        index = stop;
    }
    free(bits), free(boundary), free(prefix), free(g);
    return ok();
}

/* BPSK/QPSK (modulators.cpp:172-196 root_raised_cosine, :885-1016 the
 * tables, :1092-1156 the pulse lookup and envelope, :1443-1527 accumulate) */
typedef struct {
    uint64_t symbols, span;
    int64_t cycle, stride;
    int64_t* boundary;
    double* boundary_d;
    float *re, *im, *rrc;
    double scale, base, limit, cycle_span, gain;
} or_psk;

static double or_rrc(double t, double beta) {
    const double pi = 3.141592653589793238462643383279502884;
    if (fabs(t) < 1e-9) return 1.0 + beta * (4.0 / pi - 1.0);
    if (beta <= 0.0) return sin(pi * t) / (pi * t);
    const double quarter = 1.0 / (4.0 * beta);
    if (fabs(fabs(t) - quarter) < 1e-9) {
        const double leading = (1.0 + 2.0 / pi) * sin(pi / (4.0 * beta));
        const double trailing = (1.0 - 2.0 / pi) * cos(pi / (4.0 * beta));
        return (beta / sqrt(2.0)) * (leading + trailing);
    }
    const double fbt = 4.0 * beta * t;
    return (sin(pi * t * (1.0 - beta)) + fbt * cos(pi * t * (1.0 + beta))) / (pi * t * (1.0 - fbt * fbt));
}

static double or_rrc_tap(const or_psk* p, double position) {
    if (position <= 0.0 || position >= p->limit) return 0.0;
    const size_t lower = (size_t)position;
    const double fraction = position - (double)lower;
    const double a = (double)p->rrc[lower], b = (double)p->rrc[lower + 1];
    return a + fraction * (b - a);
}

static uint64_t or_psk_index(const or_psk* p, int64_t position) {
    uint64_t e = (uint64_t)((position * (int64_t)p->symbols) / p->cycle);
    if (e >= p->symbols) e = p->symbols - 1;
    while (e + 1 < p->symbols && p->boundary[e + 1] <= position) ++e;
    while (e > 0 && p->boundary[e] > position) --e;
    return e;
}

static void or_psk_env(const or_psk* p, int64_t pos_in_cycle, uint64_t symbol, float* er, float* ei) {
    const int64_t symbols = (int64_t)p->symbols, span = (int64_t)p->span;
    const double position = (double)pos_in_cycle;
    double ip = 0.0, qd = 0.0;
    for (int64_t off = -span; off <= span; ++off) {
        int64_t w = (int64_t)symbol + off;
        double shift = 0.0;
        if (w < 0) w += symbols, shift = -p->cycle_span;
        else if (w >= symbols) w -= symbols, shift = p->cycle_span;
        const double tap = or_rrc_tap(p, (position - (p->boundary_d[w] + shift)) * p->scale + p->base);
        if (tap == 0.0) continue;
        ip += (double)p->re[w] * tap;
        qd += (double)p->im[w] * tap;
    }
    *er = (float)(ip * p->gain);
    *ei = (float)(qd * p->gain);
}

static void or_psk_env_at(const or_psk* p, uint64_t index, float* er, float* ei) {
    const int64_t position = (int64_t)(index % (uint64_t)p->cycle);
    or_psk_env(p, position, or_psk_index(p, position), er, ei);
}

static int32_t or_psk_accumulate(const rv_tone_emitter* e, uint64_t first, uint64_t count, double gain, rv_cf32* io) {
    const double two_pi = 6.283185307179586476925286766559;
    const int quad = e->modulation == RV_EMITTER_QPSK;
    const uint64_t bps = quad ? 2 : 1, nbits = e->symbol_count * bps, symbols = e->symbol_count;
    if (symbols == 0 || e->span_symbols >= symbols) return fail("psk: payload shorter than the pulse");
    or_psk p;
    memset(&p, 0, sizeof p);
    p.symbols = symbols, p.span = e->span_symbols;
    const double real = (double)symbols * ((double)e->rate / e->symbol_rate);
    p.cycle = (int64_t)llround(real);
    if (p.cycle < (int64_t)symbols * 2) return fail("psk: under two samples per symbol");
    uint8_t* bits = (uint8_t*)malloc(nbits);
    p.boundary = (int64_t*)malloc((symbols + 1) * sizeof(int64_t));
    p.boundary_d = (double*)malloc(symbols * sizeof(double));
    p.re = (float*)malloc(symbols * sizeof(float));
    p.im = (float*)malloc(symbols * sizeof(float));
    const size_t table = 2 * p.span * 512 + 1;
    p.rrc = (float*)malloc(table * sizeof(float));
    or_mt64* g = (or_mt64*)malloc(sizeof(or_mt64));
    if (!bits || !p.boundary || !p.boundary_d || !p.re || !p.im || !p.rrc || !g) return fail("psk: out of memory");
    or_mt64_seed(g, e->seed);
    uint64_t word = 0;
    unsigned remaining = 0;
    for (uint64_t i = 0; i < nbits; ++i) {
        if (remaining == 0) word = or_mt64_next(g), remaining = 64;
        bits[i] = (uint8_t)(word & 1u);
        word >>= 1;
        --remaining;
    }
    for (uint64_t k = 0; k <= symbols; ++k) p.boundary[k] = ((int64_t)k * p.cycle) / (int64_t)symbols;
    const double unit = 1.0 / sqrt(2.0);
    for (uint64_t k = 0; k < symbols; ++k) {
        p.boundary_d[k] = (double)p.boundary[k];
        if (quad) {
            p.re[k] = (float)(bits[2 * k] ? -unit : unit);
            p.im[k] = (float)(bits[2 * k + 1] ? -unit : unit);
        } else {
            p.re[k] = bits[k] ? 1.0f : -1.0f;
            p.im[k] = 0.0f;
        }
    }
    for (size_t i = 0; i < table; ++i) p.rrc[i] = (float)or_rrc((double)i / 512.0 - (double)p.span, e->rolloff);
    p.rrc[0] = 0.0f;
    p.rrc[table - 1] = 0.0f;
    const double sps = (double)p.cycle / (double)symbols;
    p.scale = 512.0 / sps, p.base = (double)p.span * 512.0, p.limit = (double)(table - 1);
    p.cycle_span = (double)p.cycle;
    const int64_t reach = (int64_t)ceil((double)p.span * sps);
    double energy = 0.0;
    for (int64_t off = -reach; off <= reach; ++off) {
        const double tap = or_rrc_tap(&p, ((double)off / sps) * 512.0 + p.base);
        energy += tap * tap;
    }
    p.gain = energy > 0.0 ? sqrt(sps / energy) : 1.0;
    p.stride = 1;
    while (p.stride * 2 <= 1024 && (double)(p.stride * 2) <= sps / 1024.0) p.stride *= 2;
    const double level = gain * e->amplitude;
    const double cs = two_pi * (double)e->carrier_offset / (double)e->rate, sr = cos(cs), si = sin(cs);
    const uint64_t end = first + count;
    uint64_t index = first;
    while (index < end) {
        const uint64_t anchor = index - index % 1024u, stop = end < anchor + 1024u ? end : anchor + 1024u;
        const double cp = e->initial_phase + or_exact_phase(e->carrier_offset, e->rate, anchor);
        double cr = cos(cp), ci = sin(cp);
        for (uint64_t k = anchor; k < index; ++k) {
            const double a = cr * sr - ci * si, b = cr * si + ci * sr;
            cr = a, ci = b;
        }
        float nr = 0, ni = 0, fr = 0, fi = 0;
        int64_t position = 0;
        uint64_t symbol = 0, node = 0;
        const double inverse = 1.0 / (double)p.stride;
        if (p.stride == 1) {
            position = (int64_t)(index % (uint64_t)p.cycle);
            symbol = or_psk_index(&p, position);
        } else {
            node = index - index % (uint64_t)p.stride;
            or_psk_env_at(&p, node, &nr, &ni);
            or_psk_env_at(&p, node + (uint64_t)p.stride, &fr, &fi);
        }
        for (; index < stop; ++index) {
            double ip, qd;
            if (p.stride == 1) {
                float er, ei;
                or_psk_env(&p, position, symbol, &er, &ei);
                ip = (double)er, qd = (double)ei;
            } else {
                if (index >= node + (uint64_t)p.stride) {
                    node += (uint64_t)p.stride;
                    nr = fr, ni = fi;
                    or_psk_env_at(&p, node + (uint64_t)p.stride, &fr, &fi);
                }
                const double w = (double)(index - node) * inverse;
                ip = (double)nr + w * ((double)fr - (double)nr);
                qd = (double)ni + w * ((double)fi - (double)ni);
            }
            const double re = ip * cr - qd * ci, im = ip * ci + qd * cr;
            io[index - first].re = io[index - first].re + (float)(level * re);
            io[index - first].im = io[index - first].im + (float)(level * im);
            const double a = cr * sr - ci * si, b = cr * si + ci * sr;
            cr = a, ci = b;
            if (p.stride == 1) {
                ++position;
                if (position >= p.cycle) position = 0, symbol = 0;
                else if (position >= p.boundary[symbol + 1]) ++symbol;
            }
        }
    }
    free(bits), free(p.boundary), free(p.boundary_d), free(p.re), free(p.im), free(p.rrc), free(g);
    return ok();
}

int32_t or_emitter_accumulate(const rv_tone_emitter* e, uint64_t first, uint64_t count, double gain, rv_cf32* io) {
    const double two_pi = 6.283185307179586476925286766559;
    if (e->modulation == RV_EMITTER_FSK2) return or_fsk_accumulate(e, first, count, gain, io);
    if (e->modulation == RV_EMITTER_BPSK || e->modulation == RV_EMITTER_QPSK)
        return or_psk_accumulate(e, first, count, gain, io);
    if (e->modulation < RV_EMITTER_CW || e->modulation > RV_EMITTER_LSB) return fail("emitter: modulation");
    or_cw_element* elements = NULL;
    uint32_t nel = 0;
    const int cw = e->modulation == RV_EMITTER_CW;
    if (cw) {
        elements = (or_cw_element*)malloc(1024 * sizeof(or_cw_element));
        if (elements == NULL) return fail("emitter: out of memory");
        nel = or_cw_elements(e->text, 1.2 * (double)e->rate / e->words_per_minute, e->message_gap_dots, elements,
                             1024);
    }
    /* tone SSB (modulators.cpp:789-803, :1329-1366): one rotation per tone at
     * carrier +/- tone, both anchored with the initial phase */
    const int ssb = e->modulation == RV_EMITTER_USB || e->modulation == RV_EMITTER_LSB;
    const int64_t sense = e->modulation == RV_EMITTER_LSB ? -1 : 1;
    const int64_t f1 = ssb ? e->carrier_offset + sense * e->tone_hz : e->carrier_offset;
    const int64_t f2 = ssb ? e->carrier_offset + sense * e->tone2_hz : e->tone_hz;
    const int two_tone = ssb && e->tone2_hz != 0;
    double level = gain * e->amplitude;
    if (two_tone) level = 0.5 * level;
    const double cs = two_pi * (double)f1 / (double)e->rate;
    const double ts = two_pi * (double)f2 / (double)e->rate;
    const double c_re = cos(cs), c_im = sin(cs), t_re = cos(ts), t_im = sin(ts);
    const double beta = (double)e->deviation / (double)e->tone_hz;
    const uint64_t end = first + count;
    uint64_t index = first;
    while (index < end) {
        const uint64_t anchor = index - index % 1024u;
        const uint64_t stop = end < anchor + 1024u ? end : anchor + 1024u;
        const double cp = e->initial_phase + or_exact_phase(f1, e->rate, anchor);
        const double tp = ssb ? e->initial_phase + or_exact_phase(f2, e->rate, anchor)
                              : or_exact_phase(f2, e->rate, anchor);
        double cr = cos(cp), ci = sin(cp), tr = cos(tp), ti = sin(tp);
        for (uint64_t k = anchor; k < stop; ++k) {
            if (k >= index) {
                float ar, ai;
                if (cw) {
                    const double envelope =
                        level * or_cw_envelope(elements, nel, e->rise_fall_ms * 0.001 * (double)e->rate, k);
                    ar = (float)(envelope * cr);
                    ai = (float)(envelope * ci);
                } else if (e->modulation == RV_EMITTER_AM) {
                    const double envelope = level * (1.0 + e->modulation_index * tr);
                    ar = (float)(envelope * cr);
                    ai = (float)(envelope * ci);
                } else if (ssb) {
                    double re = cr, im = ci;
                    if (two_tone) {
                        re += tr;
                        im += ti;
                    }
                    ar = (float)(level * re);
                    ai = (float)(level * im);
                } else {
                    const double deviation = beta * ti;
                    const double cosine = cos(deviation), sine = sin(deviation);
                    const double re = cr * cosine - ci * sine;
                    const double im = cr * sine + ci * cosine;
                    ar = (float)(level * re);
                    ai = (float)(level * im);
                }
                io[k - first].re = io[k - first].re + ar;
                io[k - first].im = io[k - first].im + ai;
            }
            const double ncr = cr * c_re - ci * c_im, nci = cr * c_im + ci * c_re;
            const double ntr = tr * t_re - ti * t_im, nti = tr * t_im + ti * t_re;
            cr = ncr, ci = nci, tr = ntr, ti = nti;
        }
        index = stop;
    }
    free(elements);
    return ok();
}

/* supplied audio (modulators.cpp:1048-1053 audio_at, :756-781 the FM phase
 * integral, :807-836 and :1169-1193 the Hilbert phasing network, with the
 * accumulate functions' audio paths) */
int32_t or_emitter_accumulate_audio(const rv_tone_emitter* e, const float* audio, uint64_t len, uint32_t taps,
                                    uint64_t first, uint64_t count, double gain, rv_cf32* io) {
    const double two_pi = 6.283185307179586476925286766559, pi = 3.141592653589793238462643383279502884;
    const int m = e->modulation;
    const double rate = (double)e->rate, level = gain * e->amplitude;
    double* phase = NULL;
    double* hilbert = NULL;
    if (m == RV_EMITTER_NFM) {
        phase = (double*)calloc(len + 1, sizeof(double));
        const double scale = two_pi * (double)e->deviation / rate;
        double acc = 0.0;
        for (uint64_t i = 0; i < len; ++i) {
            acc += scale * (double)audio[i];
            acc = fmod(acc, two_pi);
            phase[i + 1] = acc;
        }
    }
    if (m == RV_EMITTER_USB || m == RV_EMITTER_LSB) {
        hilbert = (double*)calloc(taps, sizeof(double));
        const int64_t half = (int64_t)(taps / 2);
        for (uint32_t i = 0; i < taps; ++i) {
            const int64_t lag = (int64_t)i - half;
            if (lag == 0 || lag % 2 == 0) continue;
            const double position = (double)i / (double)(taps - 1);
            hilbert[i] = (2.0 / (pi * (double)lag)) *
                         (0.42 - 0.5 * cos(two_pi * position) + 0.08 * cos(2.0 * two_pi * position));
        }
    }
    const double cs = two_pi * (double)e->carrier_offset / rate, sr = cos(cs), si = sin(cs);
    const double sense = m == RV_EMITTER_LSB ? -1.0 : 1.0;
    const uint64_t end = first + count;
    uint64_t index = first;
    while (index < end) {
        const uint64_t anchor = index - index % 1024u, stop = end < anchor + 1024u ? end : anchor + 1024u;
        const double cp = e->initial_phase + or_exact_phase(e->carrier_offset, e->rate, anchor);
        double cr = cos(cp), ci = sin(cp);
        for (uint64_t k = anchor; k < stop; ++k) {
            if (k >= index) {
                double re, im;
                const double a = k < len ? (double)audio[k] : 0.0;
                if (m == RV_EMITTER_AM) {
                    const double envelope = level * (1.0 + e->modulation_index * a);
                    re = envelope * cr, im = envelope * ci;
                } else if (m == RV_EMITTER_NFM) {
                    const double dev = phase[k < len ? k : len];
                    const double c = cos(dev), s = sin(dev);
                    re = level * (cr * c - ci * s), im = level * (cr * s + ci * c);
                } else {
                    const int64_t half = (int64_t)(taps / 2);
                    double total = 0.0;
                    for (uint64_t i = (half % 2) == 0 ? 1u : 0u; i < taps; i += 2) {
                        const int64_t source = (int64_t)k + half - (int64_t)i;
                        if (source < 0) continue;
                        total += hilbert[i] * ((uint64_t)source < len ? (double)audio[source] : 0.0);
                    }
                    const double q = sense * total;
                    re = level * (a * cr - q * ci), im = level * (a * ci + q * cr);
                }
                io[k - first].re = io[k - first].re + (float)re;
                io[k - first].im = io[k - first].im + (float)im;
            }
            const double ncr = cr * sr - ci * si, nci = cr * si + ci * sr;
            cr = ncr, ci = nci;
        }
        index = stop;
    }
    free(phase);
    free(hilbert);
    return ok();
}
