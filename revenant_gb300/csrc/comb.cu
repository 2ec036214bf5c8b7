// Comb / spur cancellation on the sample ring (core/dsp/comb_cancel.h,
// comb_kernels_reference.cpp, core/shaders/comb_project.comp and
// comb_subtract.comp).
//
//   project   one block per (line, sub-block): each thread sums one
//             64-sample chunk of x(n) conj(tone(n)) in sample order, then one
//             thread adds the chunk sums in chunk order (the twin's order)
//   subtract  one thread per sample: the lines' tones times their amplitudes
//             summed in line order from -0, subtracted from the sample; the
//             removed ring gets the sum (cleaned + removed is raw where no
//             line runs, and the sum's own bits where one does)
// The tone of line l at sample n is table[(phase0 + n step) >> 20], the
// phase wrapping in 32 bits.
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

constexpr uint32_t kChunk = 64;
constexpr uint32_t kShift = 32u - RV_COMB_TABLE_LOG2;

bool is_mask(uint32_t m) { return rv::is_pow2((uint64_t)m + 1u); }

// validate (comb_kernels_reference.cpp)
int32_t validate(const rv_comb_params& p, const char* who) {
    if (!is_mask(p.ring_mask) || !is_mask(p.removed_mask))
        return set_error_fmt(RV_ERR_INVALID, "%s: the ring and removed masks must each be a power of two minus one", who);
    if ((uint64_t)p.removed_mask > (uint64_t)p.ring_mask)
        return set_error_fmt(RV_ERR_INVALID, "%s: the removed ring must be no larger than the sample ring", who);
    if (p.lines > RV_COMB_MAX_LINES)
        return set_error_fmt(RV_ERR_INVALID, "%s: %u lines is more than the %u the stage cancels", who, p.lines,
                             RV_COMB_MAX_LINES);
    if (p.sub_blocks < 1 || p.sub_blocks > RV_COMB_MAX_SUB_BLOCKS)
        return set_error_fmt(RV_ERR_INVALID, "%s: %u sub-blocks is outside [1, %u]", who, p.sub_blocks,
                             RV_COMB_MAX_SUB_BLOCKS);
    if (p.count == 0 || p.count % p.sub_blocks != 0)
        return set_error_fmt(RV_ERR_INVALID, "%s: %u samples do not split into %u equal non-empty sub-blocks", who,
                             p.count, p.sub_blocks);
    if ((uint64_t)p.count > (uint64_t)p.removed_mask + 1u)
        return set_error_fmt(RV_ERR_INVALID, "%s: %u samples do not fit the removed ring of %llu", who, p.count,
                             (unsigned long long)p.removed_mask + 1u);
    return RV_OK;
}

__device__ __forceinline__ float2 tone(const float2* table, const rv_comb_line& l, uint32_t n) {
    return table[(l.phase0 + n * l.step) >> kShift];
}

// Dynamic shared memory: one float2 per chunk of the sub-block.
__global__ void k_comb_project(rv_comb_params p, const float2* __restrict__ raw, const rv_comb_line* __restrict__ lines,
                               const float2* __restrict__ table, float2* __restrict__ out) {
    extern __shared__ float2 chunk_sums[];
    const uint32_t l = blockIdx.x / p.sub_blocks, s = blockIdx.x % p.sub_blocks;
    const rv_comb_line line = lines[l];
    const uint32_t length = p.count / p.sub_blocks, begin = s * length;
    const uint32_t chunks = (length + kChunk - 1u) / kChunk;
    for (uint32_t c = threadIdx.x; c < chunks; c += blockDim.x) {
        const uint32_t m0 = c * kChunk, m1 = min(m0 + kChunk, length);
        float re_sum = 0.0F, im_sum = 0.0F;
        for (uint32_t m = m0; m < m1; ++m) {
            const uint32_t n = begin + m;
            const float2 x = __ldg(raw + ((p.first + n) & p.ring_mask));
            const float2 t = tone(table, line, n);
            const float re = x.x * t.x + x.y * t.y;
            const float im = x.y * t.x - x.x * t.y;
            re_sum = re_sum + re;
            im_sum = im_sum + im;
        }
        chunk_sums[c] = make_float2(re_sum, im_sum);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float re = 0.0F, im = 0.0F;
        for (uint32_t c = 0; c < chunks; ++c) {
            re = re + chunk_sums[c].x;
            im = im + chunk_sums[c].y;
        }
        out[(size_t)l * p.sub_blocks + s] = make_float2(re, im);
    }
}

// Lines in shared memory (at most RV_COMB_MAX_LINES * 24 bytes).
__global__ void k_comb_subtract(rv_comb_params p, const float2* raw, const rv_comb_line* __restrict__ lines_g,
                                const float2* __restrict__ table, float2* cleaned, float2* __restrict__ removed) {
    extern __shared__ rv_comb_line lines[];
    for (uint32_t i = threadIdx.x; i < p.lines; i += blockDim.x) lines[i] = lines_g[i];
    __syncthreads();
    const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= p.count) return;
    const uint32_t slot = (p.first + n) & p.ring_mask;
    const float2 x = raw[slot];
    float sum_re = -0.0F, sum_im = -0.0F;
    for (uint32_t l = 0; l < p.lines; ++l) {
        const float2 t = tone(table, lines[l], n);
        const rv_cf32 a = lines[l].amplitude;
        const float re = a.re * t.x - a.im * t.y;
        const float im = a.re * t.y + a.im * t.x;
        sum_re = sum_re + re;
        sum_im = sum_im + im;
    }
    cleaned[slot] = p.lines == 0 ? x : make_float2(x.x - sum_re, x.y - sum_im);
    removed[(p.first + n) & p.removed_mask] = make_float2(sum_re, sum_im);
}

}  // namespace

extern "C" {

uint32_t rv_comb_step(double frequency_hz, int64_t rate) {
    if (rate <= 0 || !std::isfinite(frequency_hz)) return 0;
    const double cycle = 4294967296.0;
    double steps = std::round(frequency_hz / (double)rate * cycle);
    steps = std::fmod(steps, cycle);
    if (steps < 0.0) steps += cycle;
    return (uint32_t)(uint64_t)steps;
}

int32_t rv_comb_table(rv_cf32* table, uint64_t len) {
    if (table == nullptr || len < RV_COMB_TABLE_SIZE)
        return set_error_fmt(RV_ERR_INVALID, "rv_comb_table: %llu entries, %u wanted", (unsigned long long)len,
                             RV_COMB_TABLE_SIZE);
    const double two_pi = 6.283185307179586476925286766559;
    for (uint32_t i = 0; i < RV_COMB_TABLE_SIZE; ++i) {
        const double angle = two_pi * (double)i / (double)RV_COMB_TABLE_SIZE;
        table[i].re = (float)std::cos(angle);
        table[i].im = (float)std::sin(angle);
    }
    return rv::clear_error();
}

int32_t rv_comb_project(void* stream, const rv_comb_params* params, const rv_cf32* raw, uint64_t raw_len,
                        const rv_comb_line* lines, uint64_t lines_len, const rv_cf32* table, uint64_t table_len,
                        rv_cf32* projections, uint64_t projections_len) {
    if (params == nullptr || raw == nullptr || table == nullptr || projections == nullptr ||
        (lines == nullptr && params->lines > 0))
        return set_error_fmt(RV_ERR_INVALID, "rv_comb_project: NULL argument");
    if (int32_t st = validate(*params, "rv_comb_project")) return st;
    if (raw_len < (uint64_t)params->ring_mask + 1u || lines_len < params->lines || table_len != RV_COMB_TABLE_SIZE ||
        projections_len < (uint64_t)params->lines * params->sub_blocks)
        return set_error_fmt(RV_ERR_INVALID, "rv_comb_project: a buffer is shorter than its parameters");
    if (params->lines == 0) return rv::clear_error();
    const uint32_t chunks = (params->count / params->sub_blocks + kChunk - 1u) / kChunk;
    const size_t smem = (size_t)chunks * sizeof(float2);
    if (smem > 200u * 1024u) return set_error_fmt(RV_ERR_UNSUPPORTED, "rv_comb_project: %u chunks per sub-block", chunks);
    if (smem > 48u * 1024u)
        if (int32_t st = cuda_status(cudaFuncSetAttribute(k_comb_project, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                          (int)smem),
                                     "rv_comb_project"))
            return st;
    k_comb_project<<<params->lines * params->sub_blocks, 256, smem, (cudaStream_t)stream>>>(
        *params, reinterpret_cast<const float2*>(raw), lines, reinterpret_cast<const float2*>(table),
        reinterpret_cast<float2*>(projections));
    if (int32_t st = cuda_status(cudaGetLastError(), "rv_comb_project")) return st;
    return rv::clear_error();
}

int32_t rv_comb_subtract(void* stream, const rv_comb_params* params, const rv_cf32* raw, uint64_t raw_len,
                         const rv_comb_line* lines, uint64_t lines_len, const rv_cf32* table, uint64_t table_len,
                         rv_cf32* cleaned, uint64_t cleaned_len, rv_cf32* removed, uint64_t removed_len) {
    if (params == nullptr || raw == nullptr || table == nullptr || cleaned == nullptr || removed == nullptr ||
        (lines == nullptr && params->lines > 0))
        return set_error_fmt(RV_ERR_INVALID, "rv_comb_subtract: NULL argument");
    if (int32_t st = validate(*params, "rv_comb_subtract")) return st;
    if (raw_len < (uint64_t)params->ring_mask + 1u || cleaned_len < (uint64_t)params->ring_mask + 1u ||
        lines_len < params->lines || table_len != RV_COMB_TABLE_SIZE ||
        removed_len < (uint64_t)params->removed_mask + 1u)
        return set_error_fmt(RV_ERR_INVALID, "rv_comb_subtract: a buffer is shorter than its parameters");
    const size_t smem = (size_t)params->lines * sizeof(rv_comb_line);
    if (smem > 48u * 1024u)
        if (int32_t st = cuda_status(cudaFuncSetAttribute(k_comb_subtract, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                          (int)smem),
                                     "rv_comb_subtract"))
            return st;
    k_comb_subtract<<<(params->count + 255u) / 256u, 256, smem, (cudaStream_t)stream>>>(
        *params, reinterpret_cast<const float2*>(raw), lines, reinterpret_cast<const float2*>(table),
        reinterpret_cast<float2*>(cleaned), reinterpret_cast<float2*>(removed));
    if (int32_t st = cuda_status(cudaGetLastError(), "rv_comb_subtract")) return st;
    return rv::clear_error();
}

}  // extern "C"
