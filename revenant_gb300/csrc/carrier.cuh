// The serial carrier loop (second-order PLL for SAM, Costas for DSB), shared
// by the plain kernel and the batched receiver path.
//
// core/shaders/vrx_carrier.comp:169-296, twin core/dsp/vrx_reference.cpp:1083-1187:
// rotate each fine sample by the loop's 0.32 phase, update the level and lock
// filters, gear-shift between acquire and track gains, advance the phase by
// the clamped proportional + integral correction. State is eight words.
#pragma once

#include "common.cuh"

namespace rv {

__device__ __forceinline__ float clamp3(float v, float lo, float hi) {
    const float m = (v < lo) ? lo : v;  // std::max(v, lo)
    return (hi < m) ? hi : m;           // std::min(m, hi)
}

__device__ inline void carrier_loop(const rv_cf32* __restrict__ nco, rv_cf32* __restrict__ fine, uint32_t* state,
                                    uint32_t power, uint32_t nco_log2, const rv_vrx_carrier_params& p) {
    const bool reset = (p.flags & 1u) != 0;
    uint32_t phase = reset ? 0u : state[0];
    float integrator = reset ? 0.0F : __uint_as_float(state[1]);
    float level = reset ? 0.0F : __uint_as_float(state[2]);
    float lock_re = reset ? 0.0F : __uint_as_float(state[3]);
    float lock_im = reset ? 0.0F : __uint_as_float(state[4]);
    uint32_t locked = reset ? 0u : state[5];
    uint32_t held = reset ? 0u : state[6];
    uint32_t primed = reset ? 0u : state[7];
    integrator = clamp3(integrator + p.shift, -p.clamp_radians, p.clamp_radians);
    const uint32_t down = 32u - nco_log2;
    for (uint32_t i = 0; i < p.count; ++i) {
        rv_cf32* zp = &fine[(p.in_offset + i) & p.in_mask];
        const float2 z = ld_cf32(zp);
        const float2 r = ld_cf32(&nco[phase >> down]);
        const float yr = z.x * r.x - z.y * r.y;
        const float yi = z.x * r.y + z.y * r.x;
        st_cf32(zp, make_float2(yr, yi));
        const float rr = yr * yr, ii = yi * yi;
        const float pw = rr + ii;
        const float cross = yr * yi;
        float wr, wi, mag;
        if (power == 1u) {
            wr = yr;
            wi = yi;
            mag = det_sqrt(pw);
        } else {
            wr = rr - ii;
            wi = cross + cross;
            mag = pw;
        }
        if (primed == 0u) {
            level = mag;
            primed = 1u;
        } else {
            const float step = p.level_alpha * (mag - level);
            level = level + step;
        }
        const float sr = p.lock_alpha * (wr - lock_re);
        const float si = p.lock_alpha * (wi - lock_im);
        lock_re = lock_re + sr;
        lock_im = lock_im + si;
        const float bound = 2.0F * fabsf(lock_im);
        const bool inside = lock_re > bound;
        if (locked != 0u) {
            held = inside ? (held > 0u ? held - 1u : 0u) : held + 1u;
            if (held >= p.hold_out) {
                locked = 0u;
                held = 0u;
            }
        } else {
            held = inside ? held + 1u : 0u;
            if (held >= p.hold_in) {
                locked = 1u;
                held = 0u;
            }
        }
        const float inverse = det_recip((level < (float)1.0e-24) ? (float)1.0e-24 : level);
        const float detected = ((power == 1u) ? yi : cross) * inverse;
        const float error = clamp3(detected, -1.0F, 1.0F);
        const float k1 = locked ? p.k1_track : p.k1_acquire;
        const float k2 = locked ? p.k2_track : p.k2_acquire;
        integrator = clamp3(integrator + k2 * error, -p.clamp_radians, p.clamp_radians);
        const float advance = k1 * error + integrator;
        const float turns = advance * (float)683565275.576431632;
        phase = phase + (uint32_t)__float2int_rz(turns);
    }
    state[0] = phase;
    state[1] = __float_as_uint(integrator);
    state[2] = __float_as_uint(level);
    state[3] = __float_as_uint(lock_re);
    state[4] = __float_as_uint(lock_im);
    state[5] = locked;
    state[6] = held;
    state[7] = primed;
}

}  // namespace rv
