// Span-wide impulse excision on the cf32 sample ring
// (core/dsp/impulse_excision.h, impulse_excision_reference.cpp,
// core/shaders/impulse_excise.comp).
//
//   segment    p[s] = sum over the segment's 2^L samples of |x|^2, in sample
//              order (one thread per segment; a segment is contiguous in the
//              ring because the ring is a whole number of segments)
//   reference  r[s] = element K/2 of the K segments before the guard segment,
//              sorted by insertion as the reference sorts them
//   flag       f[i] = r > 0 and |x|^2 * 2^L > T * r, one thread per sample
//   apply      a sample is marked when a flag lies in [i - hang, i + lead];
//              a marked sample whose run of marked neighbours (at most
//              max_width each side) is no longer than max_width becomes -0
//              and moves to the removed ring, every other sample stays and
//              the removed ring gets -0.
// The apply pass works in tiles of kTile samples: the tile's flags with
// max_width + guard either side are staged in shared memory as bytes, the
// marks computed once per position from them, and each marked sample walks
// the marks in shared memory. Counters are added once per warp.
//
// Every multiply and add is a rounded fp32 operation in the reference's
// order, so powers, levels and flags are the reference's bits.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>

#include "common.cuh"

namespace {

using rv::cuda_status;
using rv::set_error_fmt;

constexpr uint32_t kTile = 1024;
constexpr uint32_t kThreads = 256;

uint64_t ring_size(uint32_t mask) { return (uint64_t)mask + 1u; }
bool is_mask(uint32_t m) { return rv::is_pow2(ring_size(m)); }

// validate (impulse_excision_reference.cpp:86-140)
int32_t validate(const rv_excision_config& c, const rv_excision_params& p, const char* who) {
    if (c.pass > RV_EXCISE_APPLY) return set_error_fmt(RV_ERR_INVALID, "%s: pass %u is not one of the four", who, c.pass);
    if (c.seg_log2 < 2 || c.seg_log2 > RV_EXCISE_MAX_SEG_LOG2)
        return set_error_fmt(RV_ERR_INVALID, "%s: a segment of 2^%u samples is outside [4, %u]", who, c.seg_log2,
                             1u << RV_EXCISE_MAX_SEG_LOG2);
    if (c.segments < 2 || c.segments > RV_EXCISE_MAX_SEGMENTS)
        return set_error_fmt(RV_ERR_INVALID, "%s: %u reference segments is outside [2, %u]", who, c.segments,
                             RV_EXCISE_MAX_SEGMENTS);
    if (c.max_width < 1 || c.max_width > RV_EXCISE_MAX_WIDTH)
        return set_error_fmt(RV_ERR_INVALID, "%s: a %u sample maximum width is outside [1, %u]", who, c.max_width,
                             RV_EXCISE_MAX_WIDTH);
    if (c.hang > RV_EXCISE_MAX_GUARD || c.lead > RV_EXCISE_MAX_GUARD)
        return set_error_fmt(RV_ERR_INVALID, "%s: hang %u and lead %u must each be at most %u", who, c.hang, c.lead,
                             RV_EXCISE_MAX_GUARD);
    if (!is_mask(p.ring_mask) || !is_mask(p.seg_mask) || !is_mask(p.flag_mask) || !is_mask(p.removed_mask))
        return set_error_fmt(RV_ERR_INVALID, "%s: every mask must be a power of two minus one", who);
    const uint64_t ring = ring_size(p.ring_mask);
    if ((ring_size(p.seg_mask) << c.seg_log2) > ring || ring_size(p.flag_mask) > ring || ring_size(p.removed_mask) > ring)
        return set_error_fmt(RV_ERR_INVALID,
                             "%s: the segment, flag and removed rings must each be no larger than the sample ring", who);
    if (c.pass == RV_EXCISE_SEGMENT || c.pass == RV_EXCISE_REFERENCE) {
        if ((p.first & ((1u << c.seg_log2) - 1u)) != 0u)
            return set_error_fmt(RV_ERR_INVALID, "%s: a segment pass must start on a segment boundary", who);
        if ((uint64_t)p.count + c.segments + 2u > ring_size(p.seg_mask))
            return set_error_fmt(RV_ERR_INVALID, "%s: %u segments and a %u segment reference do not fit a %llu segment ring",
                                 who, p.count, c.segments, (unsigned long long)ring_size(p.seg_mask));
    } else {
        const uint64_t reach = (uint64_t)p.count + 2u * (uint64_t)c.max_width + c.hang + c.lead;
        if (reach >= ring_size(p.flag_mask) || (c.pass == RV_EXCISE_APPLY && p.count > ring_size(p.removed_mask)))
            return set_error_fmt(RV_ERR_INVALID,
                                 "%s: %u samples and their scan do not fit the flag ring of %llu or the removed ring of %llu",
                                 who, p.count, (unsigned long long)ring_size(p.flag_mask),
                                 (unsigned long long)ring_size(p.removed_mask));
    }
    if (!(p.threshold > 0.0F)) return set_error_fmt(RV_ERR_INVALID, "%s: the threshold must be a positive power ratio", who);
    return RV_OK;
}

// ---- kernels -----------------------------------------------------------

__global__ void k_excise_segment(rv_excision_params p, uint32_t seg_log2, const float2* __restrict__ raw,
                                 float* __restrict__ seg_power) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= p.count) return;
    const uint32_t base = (p.first + (j << seg_log2)) & p.ring_mask;
    // base is a multiple of the (power of two) segment and the ring a whole
    // number of segments: the segment is contiguous and 16-byte aligned
    const float4* q = reinterpret_cast<const float4*>(raw + base);
    const uint32_t pairs = 1u << (seg_log2 - 1u);
    float sum = 0.0F;
    for (uint32_t m = 0; m < pairs; ++m) {
        const float4 v = __ldg(q + m);
        const float a = v.x * v.x + v.y * v.y;
        sum = sum + a;
        const float b = v.z * v.z + v.w * v.w;
        sum = sum + b;
    }
    seg_power[(base >> seg_log2) & p.seg_mask] = sum;
}

__global__ void k_excise_reference(rv_excision_params p, uint32_t seg_log2, uint32_t segments,
                                   const float* __restrict__ seg_power, float* __restrict__ seg_level) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= p.count) return;
    const uint32_t base = (p.first + (j << seg_log2)) & p.ring_mask;
    const uint32_t slot = base >> seg_log2;
    const int64_t segment = (int64_t)1 << seg_log2;
    const int64_t rel = (int64_t)j * segment;
    if (rel - ((int64_t)segments + 1) * segment + p.history < 0) {
        seg_level[slot & p.seg_mask] = 0.0F;
        return;
    }
    float v[RV_EXCISE_MAX_SEGMENTS];
    for (uint32_t m = 0; m < segments; ++m) v[m] = seg_power[(slot - 1u - segments + m) & p.seg_mask];
    for (uint32_t a = 1; a < segments; ++a) {
        const float x = v[a];
        uint32_t b = a;
        while (b > 0 && v[b - 1u] > x) {
            v[b] = v[b - 1u];
            --b;
        }
        v[b] = x;
    }
    seg_level[slot & p.seg_mask] = v[segments / 2u];
}

__global__ void k_excise_flag(rv_excision_params p, uint32_t seg_log2, const float2* __restrict__ raw,
                              const float* __restrict__ seg_level, uint32_t* __restrict__ flags) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= p.count) return;
    const uint32_t slot = (p.first + j) & p.ring_mask;
    const float2 s = __ldg(raw + slot);
    const float pw = s.x * s.x + s.y * s.y;
    const float level = __ldg(seg_level + ((slot >> seg_log2) & p.seg_mask));
    const float lhs = pw * (float)(1u << seg_log2);
    const float rhs = p.threshold * level;
    flags[(p.first + j) & p.flag_mask] = (level > 0.0F && lhs > rhs) ? 1u : 0u;
}

// Dynamic shared memory: flags[kTile + 2W + hang + lead] then marks[kTile + 2W],
// bytes. Position 0 of `flags` is rel = t0 - W - hang, of `marks` rel = t0 - W.
__global__ void __launch_bounds__(kThreads)
k_excise_apply(rv_excision_params p, rv_excision_config c, const float2* raw, const uint32_t* __restrict__ flags,
               float2* cleaned, float2* __restrict__ removed, uint32_t* __restrict__ counters) {
    extern __shared__ uint8_t sm[];
    const uint32_t W = c.max_width, H = c.hang, L = c.lead;
    const int64_t t0 = (int64_t)blockIdx.x * kTile;
    const uint32_t nflags = kTile + 2u * W + H + L;
    const uint32_t nmarks = kTile + 2u * W;
    uint8_t* f = sm;
    uint8_t* mk = sm + nflags;
    for (uint32_t i = threadIdx.x; i < nflags; i += blockDim.x) {
        const int64_t rel = t0 - (int64_t)W - (int64_t)H + (int64_t)i;
        uint8_t v = 0;
        if (rel + p.history >= 0) v = flags[(p.first + (uint32_t)rel) & p.flag_mask] != 0u ? 1 : 0;
        f[i] = v;
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < nmarks; i += blockDim.x) {
        uint8_t v = 0;
        for (uint32_t m = 0; m <= H + L; ++m) v |= f[i + m];  // flags at [rel - hang, rel + lead]
        mk[i] = v;
    }
    __syncthreads();
    uint32_t n_samples = 0, n_events = 0, n_spared = 0;
    const float nz = __uint_as_float(0x80000000u);
    const float2 nothing = make_float2(nz, nz);
    for (uint32_t u = threadIdx.x; u < kTile; u += blockDim.x) {
        const int64_t j = t0 + u;
        if (j >= (int64_t)p.count) break;
        const uint32_t slot = (p.first + (uint32_t)j) & p.ring_mask;
        const float2 x = raw[slot];
        const uint32_t at = W + u;  // this sample in `mk`
        bool excise = false;
        if (mk[at]) {
            uint32_t left = 0, right = 0;
            while (left < W && mk[at - 1u - left]) ++left;
            while (right < W && mk[at + 1u + right]) ++right;
            excise = left + right + 1u <= W;
            if (left == 0u) {
                if (excise)
                    ++n_events;
                else
                    ++n_spared;
            }
        }
        if (excise) ++n_samples;
        cleaned[slot] = excise ? nothing : x;
        removed[(p.first + (uint32_t)j) & p.removed_mask] = excise ? x : nothing;
    }
    // one add per warp and counter
    for (int o = 16; o > 0; o >>= 1) {
        n_samples += __shfl_xor_sync(0xFFFFFFFFu, n_samples, o);
        n_events += __shfl_xor_sync(0xFFFFFFFFu, n_events, o);
        n_spared += __shfl_xor_sync(0xFFFFFFFFu, n_spared, o);
    }
    if ((threadIdx.x & 31u) == 0) {
        if (n_samples) atomicAdd(&counters[RV_EXCISE_COUNTER_SAMPLES], n_samples);
        if (n_events) atomicAdd(&counters[RV_EXCISE_COUNTER_EVENTS], n_events);
        if (n_spared) atomicAdd(&counters[RV_EXCISE_COUNTER_SPARED], n_spared);
    }
}

uint32_t apply_smem(const rv_excision_config& c) {
    return (kTile + 2u * c.max_width + c.hang + c.lead) + (kTile + 2u * c.max_width);
}

rv_excision_config with_pass(const rv_excision_config* c, uint32_t pass) {
    rv_excision_config o = *c;
    o.pass = pass;
    return o;
}

uint32_t grid_for(uint64_t n, uint32_t per) { return (uint32_t)((n + per - 1u) / per); }

int32_t launch_segment(cudaStream_t s, const rv_excision_config& c, const rv_excision_params& p, const rv_cf32* raw,
                       float* seg) {
    if (p.count == 0) return RV_OK;
    k_excise_segment<<<grid_for(p.count, kThreads), kThreads, 0, s>>>(p, c.seg_log2,
                                                                      reinterpret_cast<const float2*>(raw), seg);
    return cuda_status(cudaGetLastError(), "rv_excise_segment");
}

int32_t launch_reference(cudaStream_t s, const rv_excision_config& c, const rv_excision_params& p, const float* seg,
                         float* level) {
    if (p.count == 0) return RV_OK;
    k_excise_reference<<<grid_for(p.count, 128), 128, 0, s>>>(p, c.seg_log2, c.segments, seg, level);
    return cuda_status(cudaGetLastError(), "rv_excise_reference");
}

int32_t launch_flag(cudaStream_t s, const rv_excision_config& c, const rv_excision_params& p, const rv_cf32* raw,
                    const float* level, uint32_t* flags) {
    if (p.count == 0) return RV_OK;
    k_excise_flag<<<grid_for(p.count, kThreads), kThreads, 0, s>>>(p, c.seg_log2, reinterpret_cast<const float2*>(raw),
                                                                   level, flags);
    return cuda_status(cudaGetLastError(), "rv_excise_flag");
}

int32_t launch_apply(cudaStream_t s, const rv_excision_config& c, const rv_excision_params& p, const rv_cf32* raw,
                     const uint32_t* flags, rv_cf32* cleaned, rv_cf32* removed, uint32_t* counters) {
    if (p.count == 0) return RV_OK;
    const uint32_t smem = apply_smem(c);  // <= 1024 + 8192 + 32 + 1024 + 8192 bytes
    if (smem > 48u * 1024u)
        if (int32_t st = cuda_status(cudaFuncSetAttribute(k_excise_apply, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                          (int)smem),
                                     "rv_excise_apply"))
            return st;
    k_excise_apply<<<grid_for(p.count, kTile), kThreads, smem, s>>>(
        p, c, reinterpret_cast<const float2*>(raw), flags, reinterpret_cast<float2*>(cleaned),
        reinterpret_cast<float2*>(removed), counters);
    return cuda_status(cudaGetLastError(), "rv_excise_apply");
}

// ---- host bookkeeping (impulse_excision_reference.cpp:57-245) ----------

uint64_t bit_ceil64(uint64_t v) {
    uint64_t p = 1;
    while (p < v) p <<= 1;
    return p;
}

rv_excision_params cursor_params(const rv_excision_cursor& k, uint64_t first, uint32_t count) {
    rv_excision_params o;
    o.ring_mask = k.ring_mask;
    o.first = (uint32_t)(first & k.ring_mask);
    o.count = count;
    o.seg_mask = k.rings.seg_mask;
    o.flag_mask = k.rings.flag_mask;
    o.removed_mask = k.rings.removed_mask;
    const int64_t clamp = (int64_t)1 << 30;
    o.history = (int32_t)std::clamp((int64_t)first - (int64_t)k.valid_from, -clamp, clamp);
    o.threshold = k.threshold;
    return o;
}

rv_excision_params idle_params() {
    rv_excision_params o;
    memset(&o, 0, sizeof o);
    o.threshold = 31.622776F;  // ExcisionParams' default member
    return o;
}

}  // namespace

extern "C" {

int32_t rv_design_excision(int64_t source_rate, double max_width_seconds, rv_excision_config* out) {
    if (out == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_design_excision: NULL");
    const double rate = (double)std::max<int64_t>(source_rate, 1);
    memset(out, 0, sizeof *out);
    out->max_width = (uint32_t)std::clamp(std::round(max_width_seconds * rate), 1.0, (double)RV_EXCISE_MAX_WIDTH);
    // hang and lead: 0.1 us either side, 2 to 16 samples
    out->hang = (uint32_t)std::clamp(std::round(0.1e-6 * rate), 2.0, (double)RV_EXCISE_MAX_GUARD);
    out->lead = out->hang;
    // a segment of at least a quarter of the widest impulse, 16 samples or more
    const uint32_t quarter = std::max(16u, (out->max_width + 3u) / 4u);
    uint32_t log2 = 0;
    while ((1u << log2) < quarter) ++log2;
    out->seg_log2 = std::min<uint32_t>(log2, RV_EXCISE_MAX_SEG_LOG2);
    out->segments = 32;
    return rv::clear_error();
}

float rv_excision_threshold(double threshold_db) { return (float)std::pow(10.0, threshold_db / 10.0); }

int32_t rv_size_excision_rings(const rv_excision_config* c, uint64_t max_block, uint32_t frames_in_flight,
                               uint32_t ring_mask, rv_excision_rings* out) {
    if (c == nullptr || out == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_size_excision_rings: NULL");
    const uint64_t frames = std::max<uint32_t>(frames_in_flight, 1u);
    const uint64_t segment = 1ull << c->seg_log2;
    const uint64_t lag = std::max<uint64_t>((uint64_t)c->max_width + c->lead, segment);
    const uint64_t in_flight = max_block * frames;
    const uint64_t flags = bit_ceil64(in_flight + lag + 2u * (uint64_t)c->max_width + c->hang + c->lead + 1u);
    const uint64_t segs = bit_ceil64(in_flight / segment + c->segments + 4u);
    const uint64_t removed = bit_ceil64((max_block + lag) * frames);
    const uint64_t ring = ring_size(ring_mask);
    if (flags > ring || removed > ring || (segs << c->seg_log2) > ring)
        return set_error_fmt(RV_ERR_INVALID,
                             "impulse excision: a %llu sample ring is too small for %llu samples in flight and their scan",
                             (unsigned long long)ring, (unsigned long long)in_flight);
    out->seg_mask = (uint32_t)(segs - 1u);
    out->flag_mask = (uint32_t)(flags - 1u);
    out->removed_mask = (uint32_t)(removed - 1u);
    return rv::clear_error();
}

int32_t rv_excision_cursor_init(rv_excision_cursor* k, const rv_excision_config* c, uint32_t ring_mask,
                                const rv_excision_rings* rings, float threshold) {
    if (k == nullptr || c == nullptr || rings == nullptr)
        return set_error_fmt(RV_ERR_INVALID, "rv_excision_cursor_init: NULL");
    memset(k, 0, sizeof *k);
    k->config = *c;
    k->ring_mask = ring_mask;
    k->rings = *rings;
    k->threshold = threshold;
    return rv::clear_error();
}

// ExcisionCursor::plan: which samples each pass covers for the block
// [start, start + count) just written; a block that does not follow on from
// the last restarts the stage.
int32_t rv_excision_plan_block(rv_excision_cursor* k, uint64_t start, uint32_t count, rv_excision_plan* out) {
    if (k == nullptr || out == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_excision_plan_block: NULL");
    memset(out, 0, sizeof *out);
    out->segment = out->reference = out->flag = out->apply = idle_params();
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
        out->segment = cursor_params(*k, k->seg_next * segment, (uint32_t)(seg_end - k->seg_next));
        k->seg_next = seg_end;
    }
    if (end > k->flag_next) {
        const uint64_t lo = k->flag_next / segment, hi = (end - 1u) / segment;
        out->reference = cursor_params(*k, lo * segment, (uint32_t)(hi - lo + 1u));
        out->flag = cursor_params(*k, k->flag_next, (uint32_t)(end - k->flag_next));
        k->flag_next = end;
    }
    // the apply pass looks max_width + lead ahead and waits for whole segments
    const uint64_t reach = (uint64_t)k->config.max_width + k->config.lead;
    const uint64_t by_scan = end > reach ? end - reach : 0;
    const uint64_t apply_end = std::min(by_scan, (end / segment) * segment);
    if (apply_end > k->apply_next) {
        out->apply = cursor_params(*k, k->apply_next, (uint32_t)(apply_end - k->apply_next));
        k->apply_next = apply_end;
    }
    out->cleaned_end = k->apply_next;
    return rv::clear_error();
}

int32_t rv_excise_segment(void* stream, const rv_excision_config* config, const rv_excision_params* params,
                          const rv_cf32* raw, uint64_t raw_len, float* seg_power, uint64_t seg_len) {
    if (config == nullptr || params == nullptr || raw == nullptr || seg_power == nullptr)
        return set_error_fmt(RV_ERR_INVALID, "rv_excise_segment: NULL argument");
    const rv_excision_config c = with_pass(config, RV_EXCISE_SEGMENT);
    if (int32_t st = validate(c, *params, "rv_excise_segment")) return st;
    if (raw_len < ring_size(params->ring_mask) || seg_len < ring_size(params->seg_mask))
        return set_error_fmt(RV_ERR_INVALID, "rv_excise_segment: a ring is shorter than its mask");
    if ((reinterpret_cast<uintptr_t>(raw) & 15u) != 0u)
        return set_error_fmt(RV_ERR_INVALID, "rv_excise_segment: the sample ring must be 16-byte aligned");
    if (int32_t st = launch_segment((cudaStream_t)stream, c, *params, raw, seg_power)) return st;
    return rv::clear_error();
}

int32_t rv_excise_reference(void* stream, const rv_excision_config* config, const rv_excision_params* params,
                            const float* seg_power, float* seg_level, uint64_t seg_len) {
    if (config == nullptr || params == nullptr || seg_power == nullptr || seg_level == nullptr)
        return set_error_fmt(RV_ERR_INVALID, "rv_excise_reference: NULL argument");
    const rv_excision_config c = with_pass(config, RV_EXCISE_REFERENCE);
    if (int32_t st = validate(c, *params, "rv_excise_reference")) return st;
    if (seg_len < ring_size(params->seg_mask))
        return set_error_fmt(RV_ERR_INVALID, "rv_excise_reference: a segment ring is shorter than its mask");
    if (int32_t st = launch_reference((cudaStream_t)stream, c, *params, seg_power, seg_level)) return st;
    return rv::clear_error();
}

int32_t rv_excise_flag(void* stream, const rv_excision_config* config, const rv_excision_params* params,
                       const rv_cf32* raw, uint64_t raw_len, const float* seg_level, uint64_t seg_len, uint32_t* flags,
                       uint64_t flags_len) {
    if (config == nullptr || params == nullptr || raw == nullptr || seg_level == nullptr || flags == nullptr)
        return set_error_fmt(RV_ERR_INVALID, "rv_excise_flag: NULL argument");
    const rv_excision_config c = with_pass(config, RV_EXCISE_FLAG);
    if (int32_t st = validate(c, *params, "rv_excise_flag")) return st;
    if (raw_len < ring_size(params->ring_mask) || seg_len < ring_size(params->seg_mask) ||
        flags_len < ring_size(params->flag_mask))
        return set_error_fmt(RV_ERR_INVALID, "rv_excise_flag: a ring is shorter than its mask");
    if (int32_t st = launch_flag((cudaStream_t)stream, c, *params, raw, seg_level, flags)) return st;
    return rv::clear_error();
}

int32_t rv_excise_apply(void* stream, const rv_excision_config* config, const rv_excision_params* params,
                        const rv_cf32* raw, uint64_t raw_len, const uint32_t* flags, uint64_t flags_len,
                        rv_cf32* cleaned, rv_cf32* removed, uint64_t removed_len, uint32_t* counters) {
    if (config == nullptr || params == nullptr || raw == nullptr || flags == nullptr || cleaned == nullptr ||
        removed == nullptr || counters == nullptr)
        return set_error_fmt(RV_ERR_INVALID, "rv_excise_apply: NULL argument");
    const rv_excision_config c = with_pass(config, RV_EXCISE_APPLY);
    if (int32_t st = validate(c, *params, "rv_excise_apply")) return st;
    if (raw_len < ring_size(params->ring_mask) || flags_len < ring_size(params->flag_mask) ||
        removed_len < ring_size(params->removed_mask))
        return set_error_fmt(RV_ERR_INVALID, "rv_excise_apply: a ring is shorter than its mask");
    if (int32_t st = launch_apply((cudaStream_t)stream, c, *params, raw, flags, cleaned, removed, counters)) return st;
    return rv::clear_error();
}

int32_t rv_excise_block(void* stream, const rv_excision_config* config, const rv_excision_plan* plan, rv_cf32* ring,
                        uint64_t ring_len, float* seg_power, float* seg_level, uint64_t seg_len, uint32_t* flags,
                        uint64_t flags_len, rv_cf32* removed, uint64_t removed_len, uint32_t* counters) {
    if (config == nullptr || plan == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_excise_block: NULL argument");
    // every pass with work is validated before any is launched
    const rv_excision_params* passes[4] = {&plan->segment, &plan->reference, &plan->flag, &plan->apply};
    for (uint32_t k = 0; k < 4; ++k) {
        if (passes[k]->count == 0) continue;
        if (int32_t st = validate(with_pass(config, k), *passes[k], "rv_excise_block")) return st;
    }
    cudaStream_t s = (cudaStream_t)stream;
    if (plan->segment.count)
        if (int32_t st = rv_excise_segment(s, config, &plan->segment, ring, ring_len, seg_power, seg_len)) return st;
    if (plan->reference.count)
        if (int32_t st = rv_excise_reference(s, config, &plan->reference, seg_power, seg_level, seg_len)) return st;
    if (plan->flag.count)
        if (int32_t st = rv_excise_flag(s, config, &plan->flag, ring, ring_len, seg_level, seg_len, flags, flags_len))
            return st;
    if (plan->apply.count)
        if (int32_t st = rv_excise_apply(s, config, &plan->apply, ring, ring_len, flags, flags_len, ring, removed,
                                         removed_len, counters))
            return st;
    return rv::clear_error();
}

}  // extern "C"
