// The plain path: one CUDA kernel per reference dispatch.
//
// Each kernel computes what its reference shader computes, in the same
// per-output operation order, so its output is bit-identical to the
// reference's CPU twin (the twins transcribe the shaders; see the citation on
// each kernel). These are the correctness anchor and the "one dispatch per
// stage" baseline the fused kernels are measured against. Launch shapes are
// plain CUDA: a grid-stride loop over outputs (or one CTA per transform), not
// the reference's workgroup tiling.
//
// Every launcher validates on the host with the rules of the matching twin's
// validate(), plus bounds checks of every device buffer it is handed, so no
// launch can index outside the buffers it was given.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "carrier.cuh"
#include "common.cuh"
#include "revenant_gb300.h"

namespace rv {
namespace {

constexpr int kThreads = 256;

inline unsigned grid_for(uint64_t n, int threads = kThreads) {
    const uint64_t blocks = (n + threads - 1) / threads;
    const uint64_t cap = 152ull * 64ull;
    return (unsigned)(blocks == 0 ? 1 : (blocks < cap ? blocks : cap));
}

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

int32_t launched(const char* what) { return cuda_status(cudaGetLastError(), what); }

// ---------------------------------------------------------------------
// convert: core/shaders/convert_*_cf32.comp, twins core/dsp/convert.cpp.
// One thread per sample; samples are assembled from 32-bit words exactly as
// the twins assemble them (little-endian fields, sign-extended).

__device__ __forceinline__ int32_t sext(uint32_t raw, int bits) {
    return ((int32_t)(raw << (32 - bits))) >> (32 - bits);
}

template <int FMT>
__global__ void k_convert(const uint32_t* __restrict__ words, rv_cf32* __restrict__ ring,
                          rv_convert_params p) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < p.count; g += stride) {
        const uint32_t index = (uint32_t)g;
        const uint32_t src = p.src_offset + index;
        float iv, qv;
        if (FMT == RV_FORMAT_CU8 || FMT == RV_FORMAT_CS8) {
            const uint32_t word = words[src >> 1];
            const int shift = (int)((src & 1u) << 4);
            const uint32_t i_raw = (word >> shift) & 0xFFu;
            const uint32_t q_raw = (word >> (shift + 8)) & 0xFFu;
            if (FMT == RV_FORMAT_CU8) {
                // (code - 127.5) * 0x3C008081, core/dsp/convert.h:43-72
                iv = ((float)i_raw - 127.5F) * 0.00784313772F;
                qv = ((float)q_raw - 127.5F) * 0.00784313772F;
            } else {
                iv = (float)sext(i_raw, 8) * 0.0078125F;
                qv = (float)sext(q_raw, 8) * 0.0078125F;
            }
        } else if (FMT == RV_FORMAT_CS16) {
            const uint32_t word = words[src];
            iv = (float)sext(word & 0xFFFFu, 16) * 0.000030517578125F;
            qv = (float)sext(word >> 16, 16) * 0.000030517578125F;
        } else {
            // six bytes a sample straddling words (convert_cs24_cf32.comp:88)
            const uint32_t wi = src + (src >> 1);
            const uint32_t lo = words[wi];
            const uint32_t hi = words[wi + 1u];
            const uint32_t shift = (src & 1u) << 4;
            const uint32_t window = (lo >> shift) | ((hi << 16) << (16u - shift));
            const uint32_t q_raw = (window >> 24) | ((hi >> shift) << 8);
            iv = (float)sext(window & 0xFFFFFFu, 24) * 0.00000011920928955078125F;
            qv = (float)sext(q_raw & 0xFFFFFFu, 24) * 0.00000011920928955078125F;
        }
        st_cf32(&ring[(p.dst_offset + index) & p.ring_mask], make_float2(iv, qv));
    }
}

// ---------------------------------------------------------------------
// branch FIR: core/shaders/pfb_branch.comp:98-149, twin
// core/dsp/pfb_branch_reference.cpp:98-141. One thread per (block, r).

__global__ void k_pfb_branch(const float* __restrict__ taps, const rv_cf32* __restrict__ ring,
                             rv_cf32* __restrict__ out, uint32_t M, uint32_t T, uint32_t D,
                             rv_pfb_branch_params p) {
    const uint64_t total = (uint64_t)p.block_count * M;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t id = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; id < total; id += stride) {
        const uint32_t block = (uint32_t)(id / M);
        const uint32_t r = (uint32_t)(id % M);
        const uint32_t base = p.base_offset + block * D;
        float ar = 0.0F, ai = 0.0F;
        for (uint32_t q = 0; q < T; ++q) {
            const uint32_t n = q * M + r;
            const float2 s = ld_cf32(&ring[(base - n) & p.ring_mask]);
            const float c = taps[n];
            ar = ar + s.x * c;
            ai = ai + s.y * c;
        }
        st_cf32(&out[(uint64_t)block * M + ((M - r) & (M - 1u))], make_float2(ar, ai));
    }
}

// ---------------------------------------------------------------------
// M-point FFT + phase correction + channel-major scatter:
// core/shaders/pfb_fft.comp:274-363, twin core/dsp/pfb_fft_reference.cpp.
// One CTA per block, the transform in shared memory.

__device__ __forceinline__ void shared_fft(float2* x, const rv_cf32* __restrict__ tw, uint32_t n,
                                           uint32_t stages) {
    const uint32_t butterflies = n >> 1;
    for (uint32_t st = 0; st < stages; ++st) {
        const uint32_t half = 1u << st;
        const uint32_t step = n >> (st + 1u);
        for (uint32_t b = threadIdx.x; b < butterflies; b += blockDim.x) {
            const uint32_t j = b & (half - 1u);
            const uint32_t ia = ((b >> st) << (st + 1u)) + j;
            butterfly(x[ia], x[ia + half], ld_cf32(&tw[j * step]));
        }
        __syncthreads();
    }
}

// A CTA transforms the blocks of one pair (2j, 2j + 1), each as the
// reference does, and writes each channel's two ring slots together: they
// are adjacent in the channel-major ring, so one 16-byte store replaces two
// scattered 8-byte ones when the first slot is even (a pair that straddles
// the ring's wrap, or a lone last block, is stored element by element).
// `paired` is false when two blocks do not fit in shared memory.
__global__ void k_pfb_fft(const rv_cf32* __restrict__ branch, const rv_cf32* __restrict__ tw,
                          rv_cf32* __restrict__ ring, rv_pfb_fft_params p, bool paired) {
    extern __shared__ float2 x[];
    const uint32_t M = p.channels, per = paired ? 2u : 1u;
    const uint32_t groups = (p.block_count + per - 1u) / per;
    float2* const x1 = x + M;
    const bool aligned = (reinterpret_cast<uintptr_t>(ring) & 15u) == 0u;
    for (uint32_t gi = blockIdx.x; gi < groups; gi += gridDim.x) {
        const uint32_t b0 = gi * per, nb = (p.block_count - b0 < per) ? p.block_count - b0 : per;
        for (uint32_t h = 0; h < nb; ++h) {
            const rv_cf32* in = branch + (uint64_t)(b0 + h) * M;
            float2* xh = h ? x1 : x;
            for (uint32_t i = threadIdx.x; i < M; i += blockDim.x) xh[i] = ld_cf32(&in[brev(i, p.stages)]);
        }
        __syncthreads();
        shared_fft(x, tw, M, p.stages);
        if (nb == 2u) shared_fft(x1, tw, M, p.stages);
        const uint32_t m0 = p.block_base + b0, m1 = m0 + 1u;
        const uint32_t slot0 = m0 & p.out_ring_mask, slot1 = m1 & p.out_ring_mask;
        const uint32_t dm0 = ((m0 & (M - 1u)) * p.decimation) & (M - 1u);
        const uint32_t dm1 = ((m1 & (M - 1u)) * p.decimation) & (M - 1u);
        const bool pair = nb == 2u && aligned && slot1 == slot0 + 1u && (slot0 & 1u) == 0u;
        for (uint32_t k = threadIdx.x; k < M; k += blockDim.x) {
            float2 v0 = x[k];
            if (p.decimation != M) v0 = cmul(v0, ld_cf32(&tw[(k * dm0) & (M - 1u)]));
            rv_cf32* row = ring + (uint64_t)k * p.out_ring_blocks;
            if (nb == 2u) {
                float2 v1 = x1[k];
                if (p.decimation != M) v1 = cmul(v1, ld_cf32(&tw[(k * dm1) & (M - 1u)]));
                if (pair) {
                    *reinterpret_cast<float4*>(row + slot0) = make_float4(v0.x, v0.y, v1.x, v1.y);
                } else {
                    st_cf32(&row[slot0], v0);
                    st_cf32(&row[slot1], v1);
                }
            } else {
                st_cf32(&row[slot0], v0);
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------
// spectrum: core/shaders/spectrum.comp:252, twin
// core/dsp/spectrum_reference.cpp:286. One CTA per channel.

__global__ void k_spectrum(const rv_cf32* __restrict__ ring, const rv_cf32* __restrict__ tw,
                           const float* __restrict__ window, float* __restrict__ frame,
                           rv_spectrum_params p) {
    extern __shared__ float2 x[];
    const uint32_t N = p.transform, M = p.channels, half = N / 2;
    const uint32_t ch = blockIdx.x;
    const uint64_t origin = (uint64_t)ch * p.chan_blocks;
    for (uint32_t n = threadIdx.x; n < N; n += blockDim.x) {
        const float2 v = ld_cf32(&ring[origin + ((p.in_offset + n) & p.chan_mask)]);
        const float gain = window[n];
        x[brev(n, p.stages)] = make_float2(v.x * gain, v.y * gain);
    }
    __syncthreads();
    shared_fft(x, tw, N, p.stages);
    const uint64_t out_origin = (uint64_t)((ch + M / 2) & (M - 1u)) * half;
    for (uint32_t bin = threadIdx.x; bin < half; bin += blockDim.x) {
        const float2 v = x[(bin + N - N / 4) & (N - 1u)];
        const float power = v.x * v.x + v.y * v.y;
        const float flattened = power * window[N + bin];
        const float floored = (flattened < 1.0e-20F) ? 1.0e-20F : flattened;
        frame[out_origin + bin] = det_log2(floored) * 3.01029995663981195F;
    }
}

// ---------------------------------------------------------------------
// spectrum levels: core/shaders/spectrum_levels.comp:146, twin
// core/dsp/spectrum_levels_reference.cpp:75. One CTA, shared histogram.

__device__ __forceinline__ uint32_t rank_of(uint32_t count, uint32_t permille) {
    return (count / 1000u) * permille + ((count % 1000u) * permille) / 1000u;
}

__global__ void k_spectrum_levels(const float* __restrict__ frame, float* __restrict__ levels,
                                  rv_spectrum_levels_params p) {
    __shared__ uint32_t hist[1024];
    for (uint32_t b = threadIdx.x; b < 1024; b += blockDim.x) hist[b] = 0;
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < p.bins; i += blockDim.x) {
        float t = (frame[i] - (-200.0F)) * 4.26666666666666666F;
        t = (t < 0.0F) ? 0.0F : t;
        t = (t > 1023.0F) ? 1023.0F : t;
        atomicAdd(&hist[(uint32_t)t], 1u);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t lo = rank_of(p.bins, p.low_permille), hi = rank_of(p.bins, p.high_permille);
        if (lo > p.bins - 1u) lo = p.bins - 1u;
        if (hi > p.bins - 1u) hi = p.bins - 1u;
        uint32_t lb = 0, hb = 0, cum = 0;
        bool lf = false, hf = false;
        for (uint32_t b = 0; b < 1024; ++b) {
            cum += hist[b];
            if (!lf && cum > lo) { lb = b; lf = true; }
            if (!hf && cum > hi) { hb = b; hf = true; }
        }
        levels[0] = -200.0F + ((float)lb + 0.5F) * 0.234375F;
        levels[1] = -200.0F + ((float)hb + 0.5F) * 0.234375F;
    }
}

// ---------------------------------------------------------------------
// fine stage: core/shaders/vrx_fine.comp:270-369, twin
// core/dsp/vrx_reference.cpp:560-618. One thread per fine output: exact
// integer resampler recurrence, lerped polyphase taps, complex FIR, then the
// 0.64 NCO rotation phi(i) = phase0 + i*delta mod 2^64.

__global__ void k_vrx_fine(const rv_cf32* __restrict__ chan, const rv_cf32* __restrict__ taps,
                           const rv_cf32* __restrict__ nco, rv_cf32* __restrict__ fine,
                           rv_vrx_fine_config c, rv_vrx_fine_params p) {
    const uint64_t delta = ((uint64_t)p.nco_delta_high << 32) | p.nco_delta_low;
    const uint64_t phase0 = ((uint64_t)p.nco_phase_high << 32) | p.nco_phase_low;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < p.count; g += stride) {
        const uint32_t i = (uint32_t)g;
        const uint32_t acc = p.frac0 + i * p.step_rem;
        const uint32_t carry = acc / p.out_rate;
        const uint32_t frac = acc - carry * p.out_rate;
        const uint32_t n_rel = i * p.step_whole + carry;
        const uint32_t scaled = frac * c.phases;
        const uint32_t phase = scaled / p.out_rate;
        const uint32_t blend_num = scaled - phase * p.out_rate;
        const float blend = (float)blend_num * p.inv_out_rate;
        const float blend_c = 1.0F - blend;
        const uint32_t base = p.in_offset + n_rel;
        float ar = 0.0F, ai = 0.0F;
        for (uint32_t k = 0; k < c.taps; ++k) {
            const uint32_t slot = phase + k * c.phases;
            const float2 g0 = ld_cf32(&taps[slot]);
            const float2 g1 = ld_cf32(&taps[slot + 1u]);
            const float tr = g0.x * blend_c + g1.x * blend;
            const float ti = g0.y * blend_c + g1.y * blend;
            const float2 s = ld_cf32(&chan[(uint64_t)p.chan_base + ((base - k) & p.chan_mask)]);
            ar = ar + (s.x * tr - s.y * ti);
            ai = ai + (s.x * ti + s.y * tr);
        }
        const uint64_t phi = phase0 + (uint64_t)i * delta;
        const uint32_t idx = (c.nco_log2 == 0) ? 0u : ((uint32_t)(phi >> 32) >> (32u - c.nco_log2));
        const float2 rot = ld_cf32(&nco[idx]);
        st_cf32(&fine[(p.out_offset + i) & p.out_mask],
                make_float2(ar * rot.x - ai * rot.y, ar * rot.y + ai * rot.x));
    }
}

// ---------------------------------------------------------------------
// demodulators: core/shaders/vrx_demod.comp:445-659, twin
// core/dsp/vrx_reference.cpp:714-917. One thread per audio frame; the
// detector is evaluated per tap, as the reference kernel does.

__device__ __forceinline__ bool complex_mode(uint32_t m) {
    return m == RV_DEMOD_RAW || m == RV_DEMOD_P25P1 || m == RV_DEMOD_DSTAR || m == RV_DEMOD_TETRA ||
           m == RV_DEMOD_DMR;
}

struct DemodView {
    const rv_cf32* ring;
    uint32_t mask;
    const float* w;
    rv_vrx_demod_config c;

    __device__ __forceinline__ float2 at(uint32_t i) const { return ld_cf32(&ring[i & mask]); }
    __device__ __forceinline__ float magnitude_at(uint32_t i) const {
        const float2 z = at(i);
        return det_sqrt(z.x * z.x + z.y * z.y);
    }
    __device__ float detect(uint32_t index) const {
        if (c.mode == RV_DEMOD_AM) {
            float dc = 0.0F;
            for (uint32_t k = 0; k < c.dc_taps; ++k) {
                const float term = magnitude_at(index - k) * w[c.audio_taps + k];
                dc = dc + term;
            }
            return magnitude_at(index) - dc;
        }
        if (c.mode == RV_DEMOD_SAM) {
            float dc = 0.0F;
            for (uint32_t k = 0; k < c.dc_taps; ++k) {
                const float term = at(index - k).x * w[c.audio_taps + k];
                dc = dc + term;
            }
            return at(index).x - dc;
        }
        if (c.mode == RV_DEMOD_NFM || c.mode == RV_DEMOD_WFM) {
            const float2 z = at(index), q = at(index - 1u);
            const float pr = z.x * q.x + z.y * q.y;
            const float pi = z.y * q.x - z.x * q.y;
            return det_atan2(pi, pr);
        }
        return at(index).x;
    }
};

__global__ void k_vrx_demod(DemodView v, rv_vrx_demod_params p, float* __restrict__ audio) {
    const rv_vrx_demod_config& c = v.c;
    const uint32_t pilot_base = c.audio_taps + c.dc_taps;
    const uint32_t rotation_base = pilot_base + 2u * c.pilot_taps;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < p.count; g += stride) {
        const uint32_t i = (uint32_t)g;
        const uint32_t index = p.in_offset + i * c.decimation;
        if (complex_mode(c.mode)) {
            const float2 z = v.at(index);
            audio[2u * i] = z.x * p.gain;
            audio[2u * i + 1u] = z.y * p.gain;
            continue;
        }
        if (c.channels == 2u) {
            const uint32_t pilot_at = index - c.audio_taps / 2u;
            float pr = 0.0F, pi = 0.0F;
            for (uint32_t k = 0; k < c.pilot_taps; ++k) {
                const float comp = v.detect(pilot_at - k);
                const float tr = comp * v.w[pilot_base + 2u * k];
                const float ti = comp * v.w[pilot_base + 2u * k + 1u];
                pr = pr + tr;
                pi = pi + ti;
            }
            const float sr = pr * p.gain, si = pi * p.gain;
            const float rr = sr * sr, ii = si * si;
            const float power = rr + ii;
            const float inverse = det_recip((power < 2.0e-5F) ? 2.0e-5F : power);
            const float cross = sr * si;
            const float cos_two = (ii - rr) * inverse;
            const float sin_two = (-2.0F * cross) * inverse;
            const float locked = (power >= 2.0e-5F) ? 1.0F : 0.0F;
            float sum = 0.0F, diff = 0.0F;
            for (uint32_t t = 0; t < c.audio_taps; ++t) {
                const float weighted = v.detect(index - t) * v.w[t];
                sum = sum + weighted;
                const float ref = sin_two * v.w[rotation_base + 2u * t] -
                                  cos_two * v.w[rotation_base + 2u * t + 1u];
                const float term = weighted * ref;
                diff = diff + term;
            }
            const float gated = diff * locked;
            audio[2u * i] = (sum + gated) * p.gain;
            audio[2u * i + 1u] = (sum - gated) * p.gain;
            continue;
        }
        float acc = 0.0F;
        for (uint32_t t = 0; t < c.audio_taps; ++t) {
            const float term = v.detect(index - t) * v.w[t];
            acc = acc + term;
        }
        audio[i] = acc * p.gain;
    }
}

// ---------------------------------------------------------------------
// carrier loop: core/shaders/vrx_carrier.comp:169-296, twin
// core/dsp/vrx_reference.cpp:1083-1187. Serial by construction: one thread.

__global__ void k_vrx_carrier(const rv_cf32* __restrict__ nco, rv_cf32* __restrict__ fine,
                              uint32_t* __restrict__ state, rv_vrx_carrier_config c,
                              rv_vrx_carrier_params p) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    carrier_loop(nco, fine, state, c.power, c.nco_log2, p);
}

}  // namespace

// ---------------------------------------------------------------------
// host-side validation shared with the fused paths

// The reference's grid rules (core/dsp/pfb_design.cpp:301-380) with its
// channel cap, kMaxChannels = 2048, or a wider one for the *_wide entry
// points (C4's M = 4096, which the reference refuses).
int32_t validate_grid_upto(const rv_grid_params* g, uint32_t max_channels) {
    if (g == nullptr) return set_error_fmt(RV_ERR_INVALID, "grid: NULL");
    if (g->channels < 2) return set_error_fmt(RV_ERR_INVALID, "grid: channel count %u is below the minimum of 2", g->channels);
    if (!is_pow2(g->channels)) return set_error_fmt(RV_ERR_INVALID, "grid: channel count %u is not a power of two", g->channels);
    if (g->channels > max_channels)
        return set_error_fmt(RV_ERR_INVALID, "grid: channel count %u exceeds %u", g->channels, max_channels);
    if (g->taps_per_branch == 0) return set_error_fmt(RV_ERR_INVALID, "grid: zero taps per branch");
    if (g->decimation == 0) return set_error_fmt(RV_ERR_INVALID, "grid: zero decimation");
    if (g->channels % g->decimation != 0)
        return set_error_fmt(RV_ERR_INVALID, "grid: decimation %u does not divide %u channels", g->decimation, g->channels);
    if ((uint64_t)g->channels * g->taps_per_branch > (1ull << 20))
        return set_error_fmt(RV_ERR_INVALID, "grid: prototype of %llu taps exceeds 1048576",
                             (unsigned long long)g->channels * g->taps_per_branch);
    return RV_OK;
}

int32_t validate_grid(const rv_grid_params* g) { return validate_grid_upto(g, 2048); }

int32_t validate_fft(const rv_pfb_fft_params* p) {
    if (!is_pow2(p->channels) || p->channels < 2)
        return set_error_fmt(RV_ERR_INVALID, "pfb fft: channels must be a power of two of at least 2, got %u", p->channels);
    if (p->stages >= 32 || (1u << p->stages) != p->channels)
        return set_error_fmt(RV_ERR_INVALID, "pfb fft: stages must be log2(channels), got %u", p->stages);
    if (p->decimation == 0 || p->decimation > p->channels || p->channels % p->decimation != 0)
        return set_error_fmt(RV_ERR_INVALID, "pfb fft: decimation %u must divide %u", p->decimation, p->channels);
    if (!is_pow2(p->out_ring_blocks))
        return set_error_fmt(RV_ERR_INVALID, "pfb fft: out_ring_blocks must be a non-zero power of two, got %u", p->out_ring_blocks);
    if (p->out_ring_mask != p->out_ring_blocks - 1u)
        return set_error_fmt(RV_ERR_INVALID, "pfb fft: out_ring_mask must be out_ring_blocks - 1");
    if (p->block_count > p->out_ring_blocks)
        return set_error_fmt(RV_ERR_INVALID, "pfb fft: dispatch of %u blocks overruns a %u-block ring",
                             p->block_count, p->out_ring_blocks);
    return RV_OK;
}

int32_t validate_fine(const rv_vrx_fine_config* c, const rv_vrx_fine_params* p) {
    if (c->taps < 2 || c->taps > 256) return set_error_fmt(RV_ERR_INVALID, "vrx fine: %u taps is outside [2, 256]", c->taps);
    if (c->phases < 1 || c->phases > 4096) return set_error_fmt(RV_ERR_INVALID, "vrx fine: %u phases is outside [1, 4096]", c->phases);
    if (c->nco_log2 > 24) return set_error_fmt(RV_ERR_INVALID, "vrx fine: NCO log2 size %u exceeds 24", c->nco_log2);
    if (p->out_rate == 0) return set_error_fmt(RV_ERR_INVALID, "vrx fine: output rate is zero");
    if (p->frac0 >= p->out_rate) return set_error_fmt(RV_ERR_INVALID, "vrx fine: frac0 %u must be below the output rate %u", p->frac0, p->out_rate);
    const uint64_t cap = (uint64_t)p->chan_mask + 1u;
    if ((cap & (uint64_t)p->chan_mask) != 0) return set_error_fmt(RV_ERR_INVALID, "vrx fine: channel ring mask %u is not a power of two minus one", p->chan_mask);
    const uint64_t ocap = (uint64_t)p->out_mask + 1u;
    if ((ocap & (uint64_t)p->out_mask) != 0) return set_error_fmt(RV_ERR_INVALID, "vrx fine: output ring mask %u is not a power of two minus one", p->out_mask);
    if ((uint64_t)p->frac0 + (uint64_t)p->count * p->step_rem > 0xFFFFFFFFull)
        return set_error_fmt(RV_ERR_INVALID, "vrx fine: recurrence overflows 32 bits; dispatch fewer outputs");
    if ((uint64_t)(p->out_rate - 1u) * c->phases > 0xFFFFFFFFull)
        return set_error_fmt(RV_ERR_INVALID, "vrx fine: phase selection overflows 32 bits");
    return RV_OK;
}

bool is_complex_mode(uint32_t m) {
    return m == RV_DEMOD_RAW || m == RV_DEMOD_P25P1 || m == RV_DEMOD_DSTAR || m == RV_DEMOD_TETRA ||
           m == RV_DEMOD_DMR;
}

uint32_t demod_fine_history(const rv_vrx_demod_config* c) {
    const uint32_t det = (c->mode == RV_DEMOD_AM || c->mode == RV_DEMOD_SAM) ? c->dc_taps - 1u
                         : (c->mode == RV_DEMOD_NFM || c->mode == RV_DEMOD_WFM) ? 1u
                                                                                 : 0u;
    const uint32_t audio = c->audio_taps - 1u;
    const uint32_t pilot = c->pilot_taps == 0 ? 0u : c->audio_taps / 2u + c->pilot_taps - 1u;
    return (audio > pilot ? audio : pilot) + det;
}

int32_t validate_demod(const rv_vrx_demod_config* c, const rv_vrx_demod_params* p) {
    if (c->mode > 12) return set_error_fmt(RV_ERR_INVALID, "vrx demod: mode %u is not a demodulator", c->mode);
    const bool cx = is_complex_mode(c->mode);
    if (c->decimation == 0) return set_error_fmt(RV_ERR_INVALID, "vrx demod: audio decimation is zero");
    if (c->audio_taps == 0 || c->audio_taps > 4096) return set_error_fmt(RV_ERR_INVALID, "vrx demod: %u audio taps is outside [1, 4096]", c->audio_taps);
    if (c->dc_taps == 0 || c->dc_taps > 4096) return set_error_fmt(RV_ERR_INVALID, "vrx demod: %u DC taps is outside [1, 4096]", c->dc_taps);
    if (cx && (c->decimation != 1u || c->audio_taps != 1u)) return set_error_fmt(RV_ERR_INVALID, "vrx demod: a complex tap carries no audio filter");
    if (c->channels != 1u && c->channels != 2u) return set_error_fmt(RV_ERR_INVALID, "vrx demod: %u channels", c->channels);
    if (cx && c->channels != 2u) return set_error_fmt(RV_ERR_INVALID, "vrx demod: a complex tap is two channels");
    if (c->pilot_taps > 2048) return set_error_fmt(RV_ERR_INVALID, "vrx demod: %u pilot taps is above 2048", c->pilot_taps);
    if (c->pilot_taps != 0 && c->mode != RV_DEMOD_WFM) return set_error_fmt(RV_ERR_INVALID, "vrx demod: a pilot bandpass belongs to wideband FM");
    if (c->pilot_taps != 0 && c->channels != 2u) return set_error_fmt(RV_ERR_INVALID, "vrx demod: a pilot bandpass needs two channels");
    if (c->channels == 2u && !cx && c->pilot_taps == 0) return set_error_fmt(RV_ERR_INVALID, "vrx demod: two channels without a pilot bandpass");
    const uint64_t cap = (uint64_t)p->in_mask + 1u;
    if ((cap & (uint64_t)p->in_mask) != 0) return set_error_fmt(RV_ERR_INVALID, "vrx demod: input ring mask %u is not a power of two minus one", p->in_mask);
    const uint64_t span = p->count == 0 ? 0 : (uint64_t)(p->count - 1u) * c->decimation + demod_fine_history(c) + 1u;
    if (span > cap) return set_error_fmt(RV_ERR_INVALID, "vrx demod: %u audio samples need %llu fine samples of history, the ring holds %llu",
                                         p->count, (unsigned long long)span, (unsigned long long)cap);
    return RV_OK;
}

uint64_t demod_weight_count(const rv_vrx_demod_config* c) {
    const uint64_t pilot_base = (uint64_t)c->audio_taps + c->dc_taps;
    return c->pilot_taps == 0 ? pilot_base : pilot_base + 2ull * c->pilot_taps + 2ull * c->audio_taps;
}

int32_t validate_carrier(const rv_vrx_carrier_config* c, const rv_vrx_carrier_params* p) {
    if (c->power != 1u && c->power != 2u) return set_error_fmt(RV_ERR_INVALID, "vrx carrier: power %u is neither PLL (1) nor Costas (2)", c->power);
    if (c->nco_log2 == 0 || c->nco_log2 > 24) return set_error_fmt(RV_ERR_INVALID, "vrx carrier: NCO log2 %u outside [1, 24]", c->nco_log2);
    const uint64_t cap = (uint64_t)p->in_mask + 1u;
    if ((cap & (uint64_t)p->in_mask) != 0) return set_error_fmt(RV_ERR_INVALID, "vrx carrier: ring mask is not a power of two minus one");
    if (p->count > cap) return set_error_fmt(RV_ERR_INVALID, "vrx carrier: %u samples in a ring of %llu", p->count, (unsigned long long)cap);
    if ((p->flags & ~1u) != 0) return set_error_fmt(RV_ERR_INVALID, "vrx carrier: flags carry unknown bits");
    if (!isfinite(p->shift)) return set_error_fmt(RV_ERR_INVALID, "vrx carrier: the retune shift is not finite");
    if (!(p->clamp_radians > 0.0F) || !((double)p->clamp_radians <= 0.5 * 3.14159265358979323846))
        return set_error_fmt(RV_ERR_INVALID, "vrx carrier: integrator bound outside (0, pi/2]");
    if (!(p->k1_acquire > 0.0F && p->k1_acquire < 1.0F) || !(p->k1_track > 0.0F && p->k1_track < 1.0F))
        return set_error_fmt(RV_ERR_INVALID, "vrx carrier: proportional gain outside (0, 1)");
    if (!(p->k2_acquire > 0.0F && p->k2_acquire < 1.0F) || !(p->k2_track > 0.0F && p->k2_track < 1.0F))
        return set_error_fmt(RV_ERR_INVALID, "vrx carrier: integral gain outside (0, 1)");
    if (!(p->level_alpha > 0.0F && p->level_alpha <= 1.0F) || !(p->lock_alpha > 0.0F && p->lock_alpha <= 1.0F))
        return set_error_fmt(RV_ERR_INVALID, "vrx carrier: one-pole coefficient outside (0, 1]");
    if (p->hold_in == 0 || p->hold_out == 0) return set_error_fmt(RV_ERR_INVALID, "vrx carrier: a lock hold of zero samples");
    return RV_OK;
}

// Launch entry points used by the chain runner as well as the C ABI.

int32_t launch_convert(cudaStream_t s, int32_t format, const rv_convert_params& p, const void* packed,
                       rv_cf32* ring) {
    if (p.count == 0) return RV_OK;
    const unsigned grid = grid_for(p.count);
    const uint32_t* w = static_cast<const uint32_t*>(packed);
    switch (format) {
        case RV_FORMAT_CU8: k_convert<RV_FORMAT_CU8><<<grid, kThreads, 0, s>>>(w, ring, p); break;
        case RV_FORMAT_CS8: k_convert<RV_FORMAT_CS8><<<grid, kThreads, 0, s>>>(w, ring, p); break;
        case RV_FORMAT_CS16: k_convert<RV_FORMAT_CS16><<<grid, kThreads, 0, s>>>(w, ring, p); break;
        default: k_convert<RV_FORMAT_CS24><<<grid, kThreads, 0, s>>>(w, ring, p); break;
    }
    return launched("convert");
}

int32_t launch_pfb_fft(cudaStream_t s, const rv_pfb_fft_params& p, const rv_cf32* branch,
                       const rv_cf32* tw, rv_cf32* ring) {
    if (p.block_count == 0) return RV_OK;
    const size_t one = (size_t)p.channels * sizeof(float2);
    const bool paired = 2 * one <= 160 * 1024 && p.block_count > 1;  // two blocks in shared memory
    const size_t shared = paired ? 2 * one : one;
    if (shared > 48 * 1024) {
        if (int32_t st = cuda_status(cudaFuncSetAttribute(k_pfb_fft, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                          (int)shared), "pfb_fft shared"))
            return st;
    }
    const unsigned threads = p.channels / 2 < 256 ? (p.channels / 2 < 32 ? 32 : p.channels / 2) : 256;
    const uint32_t groups = paired ? (p.block_count + 1u) / 2u : p.block_count;
    const unsigned grid = groups < 152u * 16u ? groups : 152u * 16u;
    k_pfb_fft<<<grid, threads, shared, s>>>(branch, tw, ring, p, paired);
    return launched("pfb_fft");
}

}  // namespace rv

using namespace rv;

extern "C" {

int32_t rv_validate_grid(const rv_grid_params* grid) {
    if (int32_t st = validate_grid(grid)) return st;
    return clear_error();
}

int32_t rv_convert(void* stream, int32_t format, const rv_convert_params* p, const void* packed_dev,
                   uint64_t packed_bytes, rv_cf32* ring_dev, uint64_t ring_len) {
    if (p == nullptr || packed_dev == nullptr || ring_dev == nullptr)
        return set_error_fmt(RV_ERR_INVALID, "rv_convert: NULL argument");
    uint64_t bps;
    switch (format) {
        case RV_FORMAT_CU8:
        case RV_FORMAT_CS8: bps = 2; break;
        case RV_FORMAT_CS16: bps = 4; break;
        case RV_FORMAT_CS24: bps = 6; break;
        default: return set_error_fmt(RV_ERR_INVALID, "rv_convert: unknown format %d", format);
    }
    if (((uintptr_t)packed_dev & 3u) != 0) return set_error_fmt(RV_ERR_INVALID, "rv_convert: staging buffer is not 4-byte aligned");
    const uint64_t capacity = (uint64_t)p->ring_mask + 1u;
    if ((capacity & (uint64_t)p->ring_mask) != 0)
        return set_error_fmt(RV_ERR_INVALID, "convert: ring_mask %u is not a power of two minus one", p->ring_mask);
    if (ring_len < capacity)
        return set_error_fmt(RV_ERR_INVALID, "convert: ring holds %llu samples, mask %u implies %llu",
                             (unsigned long long)ring_len, p->ring_mask, (unsigned long long)capacity);
    if (p->count > capacity)
        return set_error_fmt(RV_ERR_INVALID, "convert: %u samples into a ring of %llu would alias", p->count,
                             (unsigned long long)capacity);
    const uint64_t last = (uint64_t)p->src_offset + p->count;
    if (last > 0xFFFFFFFFull) return set_error_fmt(RV_ERR_INVALID, "convert: src_offset plus count overflows 32 bits");
    const uint64_t words = (last * bps + 3u) / 4u;
    if (words > 0x100000000ull) return set_error_fmt(RV_ERR_INVALID, "convert: request passes the 32-bit word index");
    if (packed_bytes < words * 4u)
        return set_error_fmt(RV_ERR_INVALID, "convert: reads %llu whole words, the source holds %llu bytes",
                             (unsigned long long)words, (unsigned long long)packed_bytes);
    if (int32_t st = launch_convert(as_stream(stream), format, *p, packed_dev, ring_dev)) return st;
    return clear_error();
}

static int32_t pfb_branch(void* stream, const rv_grid_params* g, const rv_pfb_branch_params* p, const float* taps,
                          uint64_t taps_len, const rv_cf32* ring, uint64_t ring_len, rv_cf32* out, uint64_t out_len,
                          uint32_t max_channels);

int32_t rv_pfb_branch(void* stream, const rv_grid_params* g, const rv_pfb_branch_params* p,
                      const float* taps, uint64_t taps_len, const rv_cf32* ring, uint64_t ring_len,
                      rv_cf32* out, uint64_t out_len) {
    return pfb_branch(stream, g, p, taps, taps_len, ring, ring_len, out, out_len, 2048);
}

int32_t rv_pfb_branch_wide(void* stream, const rv_grid_params* g, const rv_pfb_branch_params* p, const float* taps,
                           uint64_t taps_len, const rv_cf32* ring, uint64_t ring_len, rv_cf32* out, uint64_t out_len) {
    return pfb_branch(stream, g, p, taps, taps_len, ring, ring_len, out, out_len, 16384);
}

static int32_t pfb_branch(void* stream, const rv_grid_params* g, const rv_pfb_branch_params* p, const float* taps,
                          uint64_t taps_len, const rv_cf32* ring, uint64_t ring_len, rv_cf32* out, uint64_t out_len,
                          uint32_t max_channels) {
    if (p == nullptr || taps == nullptr || ring == nullptr || out == nullptr)
        return set_error_fmt(RV_ERR_INVALID, "rv_pfb_branch: NULL argument");
    if (int32_t st = validate_grid_upto(g, max_channels)) return st;
    const uint32_t M = g->channels, T = g->taps_per_branch, D = g->decimation;
    if (taps_len != (uint64_t)M * T) return set_error_fmt(RV_ERR_INVALID, "pfb branch: wants %u prototype taps, got %llu", M * T, (unsigned long long)taps_len);
    if (out_len < (uint64_t)p->block_count * M) return set_error_fmt(RV_ERR_INVALID, "pfb branch: output holds %llu values, %llu needed",
                                                                   (unsigned long long)out_len, (unsigned long long)p->block_count * M);
    if (p->block_count == 0) return clear_error();
    const uint64_t cap = (uint64_t)p->ring_mask + 1u;
    if ((cap & (uint64_t)p->ring_mask) != 0) return set_error_fmt(RV_ERR_INVALID, "pfb branch: ring_mask %u is not a power of two minus one", p->ring_mask);
    if (ring_len < cap) return set_error_fmt(RV_ERR_INVALID, "pfb branch: ring holds %llu samples, mask implies %llu", (unsigned long long)ring_len, (unsigned long long)cap);
    const uint64_t span = (uint64_t)M * T + (uint64_t)(p->block_count - 1u) * D;
    if (span > cap) return set_error_fmt(RV_ERR_INVALID, "pfb branch: needs %llu samples of history, ring capacity is %llu",
                                         (unsigned long long)span, (unsigned long long)cap);
    const uint64_t total = (uint64_t)p->block_count * M;
    k_pfb_branch<<<grid_for(total), kThreads, 0, as_stream(stream)>>>(taps, ring, out, M, T, D, *p);
    if (int32_t st = launched("pfb_branch")) return st;
    return clear_error();
}

int32_t rv_pfb_fft(void* stream, const rv_pfb_fft_params* p, const rv_cf32* branch, uint64_t branch_len,
                   const rv_cf32* tw, uint64_t tw_len, rv_cf32* ring, uint64_t ring_len) {
    if (p == nullptr || branch == nullptr || tw == nullptr || ring == nullptr)
        return set_error_fmt(RV_ERR_INVALID, "rv_pfb_fft: NULL argument");
    if (int32_t st = validate_fft(p)) return st;
    if (p->channels > 16384) return set_error_fmt(RV_ERR_UNSUPPORTED, "pfb fft: %u channels exceeds the 16384 one CTA holds", p->channels);
    if (tw_len != p->channels) return set_error_fmt(RV_ERR_INVALID, "pfb fft: needs exactly %u twiddles", p->channels);
    if (branch_len < (uint64_t)p->block_count * p->channels) return set_error_fmt(RV_ERR_INVALID, "pfb fft: branch buffer too short");
    if (ring_len < (uint64_t)p->channels * p->out_ring_blocks) return set_error_fmt(RV_ERR_INVALID, "pfb fft: channel ring too short");
    if (int32_t st = launch_pfb_fft(as_stream(stream), *p, branch, tw, ring)) return st;
    return clear_error();
}

int32_t rv_spectrum(void* stream, const rv_spectrum_params* p, const rv_cf32* ring, uint64_t ring_len,
                    const rv_cf32* tw, uint64_t tw_len, const float* window, uint64_t window_len,
                    float* frame, uint64_t frame_len) {
    if (p == nullptr || ring == nullptr || tw == nullptr || window == nullptr || frame == nullptr)
        return set_error_fmt(RV_ERR_INVALID, "rv_spectrum: NULL argument");
    if (!is_pow2(p->channels) || p->channels < 2) return set_error_fmt(RV_ERR_INVALID, "spectrum: channels must be a power of two of at least 2");
    if (!is_pow2(p->transform) || p->transform < 4) return set_error_fmt(RV_ERR_INVALID, "spectrum: transform must be a power of two of at least 4");
    if (p->transform > 2048) return set_error_fmt(RV_ERR_INVALID, "spectrum: a %u-point transform exceeds 2048", p->transform);
    if (p->stages >= 32 || (1u << p->stages) != p->transform) return set_error_fmt(RV_ERR_INVALID, "spectrum: stages must be log2(transform)");
    if (!is_pow2(p->chan_blocks)) return set_error_fmt(RV_ERR_INVALID, "spectrum: chan_blocks must be a power of two");
    if (p->chan_mask != p->chan_blocks - 1u) return set_error_fmt(RV_ERR_INVALID, "spectrum: chan_mask must be chan_blocks - 1");
    if (p->transform > p->chan_blocks) return set_error_fmt(RV_ERR_INVALID, "spectrum: a %u-point window does not fit %u blocks", p->transform, p->chan_blocks);
    const uint32_t N = p->transform;
    if (tw_len != N) return set_error_fmt(RV_ERR_INVALID, "spectrum: needs exactly %u twiddles", N);
    if (window_len != (uint64_t)N + N / 2) return set_error_fmt(RV_ERR_INVALID, "spectrum: window must hold %u floats", N + N / 2);
    if (ring_len < (uint64_t)p->channels * p->chan_blocks) return set_error_fmt(RV_ERR_INVALID, "spectrum: channel ring too short");
    if (frame_len < (uint64_t)p->channels * (N / 2)) return set_error_fmt(RV_ERR_INVALID, "spectrum: frame too short");
    k_spectrum<<<p->channels, 256, N * sizeof(float2), as_stream(stream)>>>(ring, tw, window, frame, *p);
    if (int32_t st = launched("spectrum")) return st;
    return clear_error();
}

int32_t rv_spectrum_levels(void* stream, const rv_spectrum_levels_params* p, const float* frame,
                           uint64_t frame_len, float* levels) {
    if (p == nullptr || frame == nullptr || levels == nullptr)
        return set_error_fmt(RV_ERR_INVALID, "rv_spectrum_levels: NULL argument");
    if (p->bins == 0) return set_error_fmt(RV_ERR_INVALID, "spectrum levels needs at least one bin");
    if (p->low_permille > 1000 || p->high_permille > 1000) return set_error_fmt(RV_ERR_INVALID, "spectrum levels: a permille above 1000");
    if (p->low_permille >= p->high_permille) return set_error_fmt(RV_ERR_INVALID, "spectrum levels: the low percentile must sit below the high one");
    if (frame_len < p->bins) return set_error_fmt(RV_ERR_INVALID, "spectrum levels: frame shorter than bins");
    k_spectrum_levels<<<1, 1024, 0, as_stream(stream)>>>(frame, levels, *p);
    if (int32_t st = launched("spectrum_levels")) return st;
    return clear_error();
}

int32_t rv_vrx_fine(void* stream, const rv_vrx_fine_config* c, const rv_vrx_fine_params* p,
                    const rv_cf32* chan, uint64_t chan_len, const rv_cf32* taps, uint64_t taps_len,
                    const rv_cf32* nco, uint64_t nco_len, rv_cf32* fine, uint64_t fine_len) {
    if (c == nullptr || p == nullptr || chan == nullptr || taps == nullptr || nco == nullptr || fine == nullptr)
        return set_error_fmt(RV_ERR_INVALID, "rv_vrx_fine: NULL argument");
    if (int32_t st = validate_fine(c, p)) return st;
    if (taps_len != (uint64_t)c->phases * c->taps + 1u) return set_error_fmt(RV_ERR_INVALID, "vrx fine: wants %llu tap entries", (unsigned long long)c->phases * c->taps + 1u);
    if (nco_len != (1ull << c->nco_log2)) return set_error_fmt(RV_ERR_INVALID, "vrx fine: wants %llu NCO entries", 1ull << c->nco_log2);
    if (chan_len < (uint64_t)p->chan_base + p->chan_mask + 1u) return set_error_fmt(RV_ERR_INVALID, "vrx fine: channel ring too short for base %u", p->chan_base);
    if (fine_len < (uint64_t)p->out_mask + 1u) return set_error_fmt(RV_ERR_INVALID, "vrx fine: output ring too short");
    if (p->count > (uint64_t)p->out_mask + 1u) return set_error_fmt(RV_ERR_INVALID, "vrx fine: %u outputs do not fit the output ring", p->count);
    if (p->count == 0) return clear_error();
    k_vrx_fine<<<grid_for(p->count, 128), 128, 0, as_stream(stream)>>>(chan, taps, nco, fine, *c, *p);
    if (int32_t st = launched("vrx_fine")) return st;
    return clear_error();
}

int32_t rv_vrx_demod(void* stream, const rv_vrx_demod_config* c, const rv_vrx_demod_params* p,
                     const rv_cf32* fine, uint64_t fine_len, const float* weights, uint64_t weights_len,
                     float* audio, uint64_t audio_len) {
    if (c == nullptr || p == nullptr || fine == nullptr || weights == nullptr || audio == nullptr)
        return set_error_fmt(RV_ERR_INVALID, "rv_vrx_demod: NULL argument");
    if (int32_t st = validate_demod(c, p)) return st;
    if (weights_len != demod_weight_count(c)) return set_error_fmt(RV_ERR_INVALID, "vrx demod: wants %llu weights", (unsigned long long)demod_weight_count(c));
    if (fine_len < (uint64_t)p->in_mask + 1u) return set_error_fmt(RV_ERR_INVALID, "vrx demod: fine ring too short");
    if (audio_len < (uint64_t)p->count * c->channels) return set_error_fmt(RV_ERR_INVALID, "vrx demod: audio buffer too short");
    if (p->count == 0) return clear_error();
    DemodView v{fine, p->in_mask, weights, *c};
    k_vrx_demod<<<grid_for(p->count, 64), 64, 0, as_stream(stream)>>>(v, *p, audio);
    if (int32_t st = launched("vrx_demod")) return st;
    return clear_error();
}

int32_t rv_vrx_carrier(void* stream, const rv_vrx_carrier_config* c, const rv_vrx_carrier_params* p,
                       const rv_cf32* nco, uint64_t nco_len, rv_cf32* fine, uint64_t fine_len,
                       uint32_t* state) {
    if (c == nullptr || p == nullptr || nco == nullptr || fine == nullptr || state == nullptr)
        return set_error_fmt(RV_ERR_INVALID, "rv_vrx_carrier: NULL argument");
    if (int32_t st = validate_carrier(c, p)) return st;
    if (nco_len != (1ull << c->nco_log2)) return set_error_fmt(RV_ERR_INVALID, "vrx carrier: NCO table size");
    if (fine_len < (uint64_t)p->in_mask + 1u) return set_error_fmt(RV_ERR_INVALID, "vrx carrier: fine ring too short");
    k_vrx_carrier<<<1, 1, 0, as_stream(stream)>>>(nco, fine, state, *c, *p);
    if (int32_t st = launched("vrx_carrier")) return st;
    return clear_error();
}

uint32_t rv_demod_fine_history(const rv_vrx_demod_config* c) { return c ? demod_fine_history(c) : 0u; }

}  // extern "C"
