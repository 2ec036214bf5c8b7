// Front-end DC and IQ-imbalance correction: the moments and correction
// kernels (core/shaders/iq_moments.comp, iq_correct.comp; twins
// core/dsp/front_end_correction_reference.cpp:46-111) and the host estimator
// (FrontEndCorrector, core/dsp/front_end_correction.cpp). The kernels keep the
// twins' arithmetic: the chunk sums accumulate in sample order with a rounded
// multiply and a rounded add each, and the correction is two rounded
// differences, two rounded products and a rounded sum.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "revenant_gb300.h"

namespace rv {
namespace {

__global__ void k_iq_moments(const rv_cf32* __restrict__ ring, rv_iq_moments_params p, float* __restrict__ sums) {
    const uint32_t chunk = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t chunks = (p.count + RV_IQ_MOMENTS_CHUNK - 1u) / RV_IQ_MOMENTS_CHUNK;
    if (chunk >= chunks) return;
    const uint32_t first = chunk * RV_IQ_MOMENTS_CHUNK;
    const uint32_t last = min(first + RV_IQ_MOMENTS_CHUNK, p.count);
    float si = 0.0F, sq = 0.0F, sii = 0.0F, sqq = 0.0F, siq = 0.0F;
    for (uint32_t k = first; k < last; ++k) {
        const float2 v = ld_cf32(&ring[(p.src_offset + k) & p.ring_mask]);
        si = si + v.x;
        sq = sq + v.y;
        sii = sii + v.x * v.x;
        sqq = sqq + v.y * v.y;
        siq = siq + v.x * v.y;
    }
    float* out = sums + (uint64_t)chunk * RV_IQ_MOMENTS_PER_CHUNK;
    out[0] = si;
    out[1] = sq;
    out[2] = sii;
    out[3] = sqq;
    out[4] = siq;
}

__global__ void k_iq_correct(const rv_cf32* __restrict__ in, rv_iq_correct_params p, rv_cf32* __restrict__ out) {
    const uint32_t index = blockIdx.x * blockDim.x + threadIdx.x;
    if (index >= p.count) return;
    const uint32_t slot = (p.offset + index) & p.ring_mask;
    const float2 v = ld_cf32(&in[slot]);
    const float i = v.x - p.dc_i;
    const float q_dc = v.y - p.dc_q;
    const float q = p.cross * i + p.scale * q_dc;
    st_cf32(&out[slot], make_float2(i, q));
}

// The same sums over a native-format ring (the batched chain's raw ring),
// each sample converted as the convert kernel would.
template <int FMT>
__global__ void k_iq_moments_raw(const uint32_t* __restrict__ raw, rv_iq_moments_params p, float* __restrict__ sums) {
    const uint32_t chunk = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t chunks = (p.count + RV_IQ_MOMENTS_CHUNK - 1u) / RV_IQ_MOMENTS_CHUNK;
    if (chunk >= chunks) return;
    const uint32_t first = chunk * RV_IQ_MOMENTS_CHUNK;
    const uint32_t last = min(first + RV_IQ_MOMENTS_CHUNK, p.count);
    float si = 0.0F, sq = 0.0F, sii = 0.0F, sqq = 0.0F, siq = 0.0F;
    for (uint32_t k = first; k < last; ++k) {
        const float2 v = convert_raw<FMT>(raw, (p.src_offset + k) & p.ring_mask);
        si = si + v.x;
        sq = sq + v.y;
        sii = sii + v.x * v.x;
        sqq = sqq + v.y * v.y;
        siq = siq + v.x * v.y;
    }
    float* out = sums + (uint64_t)chunk * RV_IQ_MOMENTS_PER_CHUNK;
    out[0] = si;
    out[1] = sq;
    out[2] = sii;
    out[3] = sqq;
    out[4] = siq;
}

int32_t check_ring(uint64_t ring_len, uint32_t mask, uint32_t count, const char* what) {
    const uint64_t cap = (uint64_t)mask + 1u;
    if ((cap & (uint64_t)mask) != 0) return set_error_fmt(RV_ERR_INVALID, "%s: ring_mask %u is not a power of two less one", what, mask);
    if (ring_len < cap) return set_error_fmt(RV_ERR_INVALID, "%s: the ring holds %llu samples and the mask names %llu", what,
                                             (unsigned long long)ring_len, (unsigned long long)cap);
    if (count > cap) return set_error_fmt(RV_ERR_INVALID, "%s: a block of %u samples is longer than the ring", what, count);
    return RV_OK;
}

double weight_of(uint64_t samples, double tau_s, int64_t rate) {
    if (tau_s <= 0.0 || rate <= 0) return 1.0;
    return 1.0 - std::exp(-(double)samples / (tau_s * (double)rate));
}

}  // namespace

int32_t launch_iq_moments(cudaStream_t s, const rv_iq_moments_params& p, const rv_cf32* ring, float* sums) {
    const uint32_t chunks = (p.count + RV_IQ_MOMENTS_CHUNK - 1u) / RV_IQ_MOMENTS_CHUNK;
    if (chunks == 0) return RV_OK;
    k_iq_moments<<<(chunks + 255u) / 256u, 256, 0, s>>>(ring, p, sums);
    return cuda_status(cudaGetLastError(), "iq moments");
}

int32_t launch_iq_moments_raw(cudaStream_t s, int32_t format, const rv_iq_moments_params& p, const void* raw,
                              float* sums) {
    const uint32_t chunks = (p.count + RV_IQ_MOMENTS_CHUNK - 1u) / RV_IQ_MOMENTS_CHUNK;
    if (chunks == 0) return RV_OK;
    const uint32_t* w = static_cast<const uint32_t*>(raw);
    if (format == RV_FORMAT_CS16)
        k_iq_moments_raw<RV_FORMAT_CS16><<<(chunks + 255u) / 256u, 256, 0, s>>>(w, p, sums);
    else if (format == RV_FORMAT_CU8)
        k_iq_moments_raw<RV_FORMAT_CU8><<<(chunks + 255u) / 256u, 256, 0, s>>>(w, p, sums);
    else
        return set_error_fmt(RV_ERR_UNSUPPORTED, "iq moments: format %d", format);
    return cuda_status(cudaGetLastError(), "iq moments");
}

// total_moments + FrontEndCorrector::update, in the reference's order.
void front_end_update(rv_front_end* st, const double totals[5], uint64_t samples, int64_t rate) {
    if (samples == 0) return;
    const double n = (double)samples;
    const double mean_i = totals[0] / n, mean_q = totals[1] / n;
    const double c_ii = totals[2] / n - mean_i * mean_i;
    const double c_qq = totals[3] / n - mean_q * mean_q;
    const double c_iq = totals[4] / n - mean_i * mean_q;
    const bool first = !st->measured;
    const double a_dc = first ? 1.0 : weight_of(samples, st->dc_time_constant_s, rate);
    const double a_iq = first ? 1.0 : weight_of(samples, st->iq_time_constant_s, rate);
    st->dc_i += a_dc * (mean_i - st->dc_i);
    st->dc_q += a_dc * (mean_q - st->dc_q);
    st->m_ii += a_iq * (c_ii - st->m_ii);
    st->m_qq += a_iq * (c_qq - st->m_qq);
    st->m_iq += a_iq * (c_iq - st->m_iq);
    st->measured = 1;
    st->samples_seen += samples;
    if (st->m_ii > 0.0 && st->m_qq > 0.0) {
        st->gain = std::sqrt(st->m_qq / st->m_ii);
        st->sin_phase = st->m_iq / std::sqrt(st->m_ii * st->m_qq);
        const double gain_db = std::abs(20.0 * std::log10(st->gain));
        const double phase_deg = std::abs(std::asin(std::clamp(st->sin_phase, -1.0, 1.0)) * 180.0 /
                                          3.141592653589793238462643383279502884);
        st->iq_plausible = std::isfinite(st->gain) && std::isfinite(st->sin_phase) &&
                           gain_db <= st->max_gain_error_db && phase_deg <= st->max_phase_error_deg;
    } else {
        st->gain = 1.0;
        st->sin_phase = 0.0;
        st->iq_plausible = 0;
    }
}

// total_moments: the chunk sums added in chunk order, in double.
void total_moments(const float* sums, uint64_t chunks, double totals[5]) {
    for (int k = 0; k < 5; ++k) totals[k] = 0.0;
    for (uint64_t c = 0; c < chunks; ++c)
        for (int k = 0; k < 5; ++k) totals[k] += (double)sums[c * RV_IQ_MOMENTS_PER_CHUNK + k];
}

}  // namespace rv

extern "C" {

int32_t rv_iq_moments(void* stream, const rv_iq_moments_params* p, const rv_cf32* ring_dev, uint64_t ring_len,
                      float* sums_dev, uint64_t sums_len) {
    if (p == nullptr || ring_dev == nullptr || sums_dev == nullptr)
        return rv::set_error_fmt(RV_ERR_INVALID, "rv_iq_moments: NULL argument");
    if (int32_t st = rv::check_ring(ring_len, p->ring_mask, p->count, "rv_iq_moments")) return st;
    const uint64_t chunks = (p->count + RV_IQ_MOMENTS_CHUNK - 1u) / RV_IQ_MOMENTS_CHUNK;
    if (sums_len < chunks * RV_IQ_MOMENTS_PER_CHUNK)
        return rv::set_error_fmt(RV_ERR_INVALID, "rv_iq_moments: %llu chunks need %llu floats", (unsigned long long)chunks,
                                 (unsigned long long)(chunks * RV_IQ_MOMENTS_PER_CHUNK));
    if (int32_t st = rv::launch_iq_moments(reinterpret_cast<cudaStream_t>(stream), *p, ring_dev, sums_dev)) return st;
    return rv::clear_error();
}

int32_t rv_iq_correct(void* stream, const rv_iq_correct_params* p, const rv_cf32* in_dev, uint64_t in_len,
                      rv_cf32* out_dev, uint64_t out_len) {
    if (p == nullptr || in_dev == nullptr || out_dev == nullptr)
        return rv::set_error_fmt(RV_ERR_INVALID, "rv_iq_correct: NULL argument");
    if (int32_t st = rv::check_ring(in_len, p->ring_mask, p->count, "rv_iq_correct")) return st;
    if (out_len < in_len) return rv::set_error_fmt(RV_ERR_INVALID, "rv_iq_correct: the output ring is shorter than the input");
    if (p->count == 0) return rv::clear_error();
    rv::k_iq_correct<<<(p->count + 255u) / 256u, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(in_dev, *p, out_dev);
    if (int32_t st = rv::cuda_status(cudaGetLastError(), "iq correct")) return st;
    return rv::clear_error();
}

int32_t rv_front_end_init(rv_front_end* st) {
    if (st == nullptr) return rv::set_error_fmt(RV_ERR_INVALID, "rv_front_end_init: NULL");
    st->dc_time_constant_s = 0.1;
    st->iq_time_constant_s = 1.0;
    st->max_gain_error_db = 6.0;
    st->max_phase_error_deg = 30.0;
    return rv_front_end_reset(st);
}

int32_t rv_front_end_reset(rv_front_end* st) {
    if (st == nullptr) return rv::set_error_fmt(RV_ERR_INVALID, "rv_front_end_reset: NULL");
    st->measured = 0;
    st->iq_plausible = 0;
    st->samples_seen = 0;
    st->dc_i = st->dc_q = 0.0;
    st->gain = 1.0;
    st->sin_phase = 0.0;
    st->m_ii = st->m_qq = st->m_iq = 0.0;
    return rv::clear_error();
}

int32_t rv_front_end_update(rv_front_end* st, const float* sums, uint64_t sums_len, uint32_t count, int64_t rate) {
    if (st == nullptr || (sums == nullptr && count > 0)) return rv::set_error_fmt(RV_ERR_INVALID, "rv_front_end_update: NULL");
    const uint64_t chunks = std::min<uint64_t>((count + RV_IQ_MOMENTS_CHUNK - 1u) / RV_IQ_MOMENTS_CHUNK,
                                               sums_len / RV_IQ_MOMENTS_PER_CHUNK);
    double totals[5];
    rv::total_moments(sums, chunks, totals);
    rv::front_end_update(st, totals, count, rate);
    return rv::clear_error();
}

int32_t rv_front_end_correction(const rv_front_end* st, int32_t dc, int32_t iq, rv_iq_correct_params* out) {
    if (st == nullptr || out == nullptr) return rv::set_error_fmt(RV_ERR_INVALID, "rv_front_end_correction: NULL");
    out->dc_i = 0.0F;
    out->dc_q = 0.0F;
    out->cross = 0.0F;
    out->scale = 1.0F;
    if (!st->measured) return rv::clear_error();
    if (dc) {
        out->dc_i = (float)st->dc_i;
        out->dc_q = (float)st->dc_q;
    }
    if (iq && st->iq_plausible) {
        const double cos_phase = std::sqrt(1.0 - st->sin_phase * st->sin_phase);
        out->cross = (float)(-st->sin_phase / cos_phase);
        out->scale = (float)(1.0 / (st->gain * cos_phase));
    }
    return rv::clear_error();
}

}  // extern "C"
