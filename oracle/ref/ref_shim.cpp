// Test-infrastructure only: a thin extern "C" wrapper over the reference's own
// CPU twins and host planner, compiled from the reference sources in place
// (see oracle/ref/Makefile) into oracle/_ref/libreftwins.so. The tests use it to
// pin the restated oracle (oracle/oracle.c) and the library's host planner
// against the reference itself. Nothing in the product links or loads it.
//
// Every wrapper converts this project's C structs (include/revenant_gb300.h,
// which mirror the reference's structs field for field) into the reference's
// types, calls the reference function named in its comment, and returns 0 or
// -1 with the reference's error message available from ref_last_error().

#include <complex>
#include <cstdint>
#include <cstring>
#include <span>
#include <string>
#include <vector>

#include "core/dsp/convert.h"
#include "core/dsp/front_end_correction.h"
#include "core/dsp/comb_cancel.h"
#include "core/dsp/impulse_excision.h"
#include "core/dsp/noise_reference.h"
#include "core/dsp/pfb.h"
#include "core/dsp/pfb_branch_reference.h"
#include "core/dsp/pfb_fft_reference.h"
#include "core/dsp/spectrum_levels_reference.h"
#include "core/dsp/spectrum_reference.h"
#include "core/dsp/vrx_reference.h"
#include "core/engine/vrx.h"
#include "include/revenant_gb300.h"
#include "lwdsp/primitives.h"
#include "lwdsp/spectrum.h"

namespace dsp = revenant::dsp;
namespace engine = revenant::engine;

namespace {

thread_local std::string g_error;

template <class T>
int32_t report(const T& result) {
    if (result) {
        g_error.clear();
        return 0;
    }
    g_error = result.error().message;
    return -1;
}

dsp::ComplexSpan cspan(rv_cf32* p, uint64_t n) {
    return dsp::ComplexSpan(reinterpret_cast<dsp::Complex32*>(p), n);
}
dsp::ConstComplexSpan ccspan(const rv_cf32* p, uint64_t n) {
    return dsp::ConstComplexSpan(reinterpret_cast<const dsp::Complex32*>(p), n);
}

dsp::GridParams grid_of(const rv_grid_params* g) {
    dsp::GridParams grid;
    grid.channels = g->channels;
    grid.taps_per_branch = g->taps_per_branch;
    grid.decimation = g->decimation;
    return grid;
}

engine::VrxParams request_of(const rv_vrx_request* r) {
    engine::VrxParams p;
    p.center = r->center;
    p.bandwidth = r->bandwidth;
    p.passband_low = r->passband_low;
    p.passband_high = r->passband_high;
    p.demod = static_cast<engine::Demod>(r->demod);
    p.deemphasis = static_cast<engine::Deemphasis>(r->deemphasis);
    p.stereo = r->stereo != 0;
    p.audio_rate = r->audio_rate;
    p.cw_pitch = r->cw_pitch;
    return p;
}

engine::VrxPlacement placement_of(const rv_vrx_placement* c) {
    engine::VrxPlacement p;
    p.channel = c->channel;
    p.channel_centre.numerator = c->centre_numerator;
    p.channel_centre.denominator = c->centre_denominator;
    p.residual_numerator = c->residual_numerator;
    p.residual_denominator = c->residual_denominator;
    p.channel_rate = c->channel_rate;
    p.granted_low = c->granted_low;
    p.granted_high = c->granted_high;
    p.bandwidth_clamped = c->bandwidth_clamped != 0;
    return p;
}

void placement_out(const engine::VrxPlacement& p, rv_vrx_placement* c) {
    c->channel = p.channel;
    c->bandwidth_clamped = p.bandwidth_clamped ? 1u : 0u;
    c->centre_numerator = p.channel_centre.numerator;
    c->centre_denominator = p.channel_centre.denominator;
    c->residual_numerator = p.residual_numerator;
    c->residual_denominator = p.residual_denominator;
    c->channel_rate = p.channel_rate;
    c->granted_low = p.granted_low;
    c->granted_high = p.granted_high;
}

}  // namespace

extern "C" {

const char* ref_last_error(void) { return g_error.c_str(); }

// core/dsp/convert.cpp reference_convert_{cu8,cs8,cs16,cs24}_cf32
int32_t ref_convert(int32_t format, const rv_convert_params* p, const void* packed,
                    uint64_t packed_bytes, rv_cf32* ring, uint64_t ring_len) {
    dsp::ConvertParams params{p->ring_mask, p->dst_offset, p->src_offset, p->count};
    std::span<const std::byte> bytes(static_cast<const std::byte*>(packed), packed_bytes);
    switch (format) {
        case RV_FORMAT_CU8: return report(dsp::reference_convert_cu8_cf32(bytes, params, cspan(ring, ring_len)));
        case RV_FORMAT_CS8: return report(dsp::reference_convert_cs8_cf32(bytes, params, cspan(ring, ring_len)));
        case RV_FORMAT_CS16: return report(dsp::reference_convert_cs16_cf32(bytes, params, cspan(ring, ring_len)));
        case RV_FORMAT_CS24: return report(dsp::reference_convert_cs24_cf32(bytes, params, cspan(ring, ring_len)));
        default: g_error = "unknown format"; return -1;
    }
}

// core/dsp/pfb_branch_reference.cpp:22
int32_t ref_pfb_branch(const rv_grid_params* g, const rv_pfb_branch_params* p, const float* taps,
                       uint64_t taps_len, const rv_cf32* ring, uint64_t ring_len, rv_cf32* out,
                       uint64_t out_len) {
    dsp::PfbBranchParams params{p->ring_mask, p->base_offset, p->block_count};
    return report(dsp::reference_pfb_branches(grid_of(g), dsp::ConstRealSpan(taps, taps_len),
                                              ccspan(ring, ring_len), params, cspan(out, out_len)));
}

// core/dsp/pfb_fft_reference.cpp:152
int32_t ref_pfb_fft(const rv_pfb_fft_params* p, const rv_cf32* branch, uint64_t branch_len,
                    const rv_cf32* twiddles, uint64_t tw_len, rv_cf32* ring, uint64_t ring_len) {
    dsp::PfbFftParams params;
    params.channels = p->channels;
    params.decimation = p->decimation;
    params.stages = p->stages;
    params.block_base = p->block_base;
    params.block_count = p->block_count;
    params.out_ring_blocks = p->out_ring_blocks;
    params.out_ring_mask = p->out_ring_mask;
    return report(dsp::reference_pfb_fft(params, ccspan(branch, branch_len), ccspan(twiddles, tw_len),
                                         cspan(ring, ring_len)));
}

// core/dsp/pfb_fft_reference.cpp reference_fft_radix2
int32_t ref_fft_radix2(const rv_cf32* twiddles, const rv_cf32* in, rv_cf32* out, uint32_t size,
                       uint32_t batch) {
    const uint64_t total = static_cast<uint64_t>(size) * batch;
    return report(dsp::reference_fft_radix2(ccspan(twiddles, size), ccspan(in, total),
                                            cspan(out, total), size, batch));
}

// core/dsp/spectrum_reference.cpp:286
int32_t ref_spectrum(const rv_spectrum_params* p, const rv_cf32* ring, uint64_t ring_len,
                     const rv_cf32* twiddles, uint64_t tw_len, const float* window,
                     uint64_t window_len, float* frame, uint64_t frame_len) {
    dsp::SpectrumParams params;
    params.channels = p->channels;
    params.transform = p->transform;
    params.stages = p->stages;
    params.chan_blocks = p->chan_blocks;
    params.chan_mask = p->chan_mask;
    params.in_offset = p->in_offset;
    return report(dsp::reference_spectrum(params, ccspan(ring, ring_len), ccspan(twiddles, tw_len),
                                          dsp::ConstRealSpan(window, window_len),
                                          dsp::RealSpan(frame, frame_len)));
}

// core/dsp/spectrum_levels_reference.cpp:75
int32_t ref_spectrum_levels(const rv_spectrum_levels_params* p, const float* frame,
                            uint64_t frame_len, float* levels) {
    dsp::SpectrumLevelsParams params{p->bins, p->low_permille, p->high_permille};
    return report(dsp::reference_spectrum_levels(params, dsp::ConstRealSpan(frame, frame_len),
                                                 dsp::RealSpan(levels, 2)));
}

// core/dsp/vrx_reference.cpp:489
int32_t ref_vrx_fine(const rv_vrx_fine_config* c, const rv_vrx_fine_params* p, const rv_cf32* chan,
                     uint64_t chan_len, const rv_cf32* taps, uint64_t taps_len, const rv_cf32* nco,
                     uint64_t nco_len, rv_cf32* fine, uint64_t fine_len) {
    dsp::VrxFineConfig config{c->taps, c->phases, c->nco_log2};
    dsp::VrxFineParams params;
    static_assert(sizeof(params) == sizeof(*p));
    std::memcpy(&params, p, sizeof(params));
    return report(dsp::reference_vrx_fine(config, params, ccspan(chan, chan_len),
                                          ccspan(taps, taps_len), ccspan(nco, nco_len),
                                          cspan(fine, fine_len)));
}

// core/dsp/vrx_reference.cpp:714
int32_t ref_vrx_demod(const rv_vrx_demod_config* c, const rv_vrx_demod_params* p,
                      const rv_cf32* fine, uint64_t fine_len, const float* weights,
                      uint64_t weights_len, float* audio, uint64_t audio_len) {
    dsp::VrxDemodConfig config;
    config.mode = c->mode;
    config.decimation = c->decimation;
    config.audio_taps = c->audio_taps;
    config.dc_taps = c->dc_taps;
    config.channels = c->channels;
    config.pilot_taps = c->pilot_taps;
    dsp::VrxDemodParams params;
    static_assert(sizeof(params) == sizeof(*p));
    std::memcpy(&params, p, sizeof(params));
    return report(dsp::reference_vrx_demod(config, params, ccspan(fine, fine_len),
                                           dsp::ConstRealSpan(weights, weights_len),
                                           dsp::RealSpan(audio, audio_len)));
}

// core/dsp/vrx_reference.cpp:1083
int32_t ref_vrx_carrier(const rv_vrx_carrier_config* c, const rv_vrx_carrier_params* p,
                        const rv_cf32* nco, uint64_t nco_len, rv_cf32* fine, uint64_t fine_len,
                        uint32_t* state) {
    dsp::VrxCarrierConfig config{c->power, c->nco_log2};
    dsp::VrxCarrierParams params;
    static_assert(sizeof(params) == sizeof(*p));
    std::memcpy(&params, p, sizeof(params));
    return report(dsp::reference_vrx_carrier(config, params, ccspan(nco, nco_len),
                                             cspan(fine, fine_len),
                                             std::span<std::uint32_t>(state, 8)));
}

// Deterministic transcendentals (core/dsp/vrx_reference.cpp:227-306,
// core/dsp/spectrum_reference.cpp det_log2).
float ref_det_rsqrt(float v) { return dsp::det_rsqrt(v); }
float ref_det_sqrt(float v) { return dsp::det_sqrt(v); }
float ref_det_recip(float v) { return dsp::det_recip(v); }
float ref_det_atan2(float y, float x) { return dsp::det_atan2(y, x); }
float ref_det_log2(float v) { return dsp::det_log2(v); }

// core/dsp/pfb_design.cpp:381
int32_t ref_design_prototype(const rv_grid_params* g, double atten, float* taps, uint64_t taps_len,
                             double* stopband, uint64_t* group_delay) {
    auto designed = dsp::design_prototype(grid_of(g), atten);
    if (!designed) return report(designed);
    if (designed->taps.size() != taps_len) {
        g_error = "ref_design_prototype: length mismatch";
        return -1;
    }
    std::memcpy(taps, designed->taps.data(), taps_len * sizeof(float));
    if (stopband) *stopband = designed->stopband_db;
    if (group_delay) *group_delay = designed->group_delay_samples;
    return 0;
}

// core/dsp/pfb_design.cpp:515
int32_t ref_build_twiddles(uint32_t channels, rv_cf32* out, uint64_t len) {
    auto table = dsp::build_twiddles(channels);
    if (!table) return report(table);
    if (table->size() != len) { g_error = "length mismatch"; return -1; }
    std::memcpy(out, table->data(), len * sizeof(rv_cf32));
    return 0;
}

// core/dsp/vrx_reference.cpp:364
int32_t ref_build_nco_table(uint32_t log2_size, rv_cf32* out, uint64_t len) {
    auto table = dsp::build_nco_table(log2_size);
    if (!table) return report(table);
    if (table->size() != len) { g_error = "length mismatch"; return -1; }
    std::memcpy(out, table->data(), len * sizeof(rv_cf32));
    return 0;
}

// core/dsp/spectrum_reference.cpp:195
int32_t ref_build_spectrum_window(uint32_t size, uint32_t taps_per_branch, double atten,
                                  float* out, uint64_t len) {
    auto table = dsp::build_spectrum_window(size, taps_per_branch, atten);
    if (!table) return report(table);
    if (table->size() != len) { g_error = "length mismatch"; return -1; }
    std::memcpy(out, table->data(), len * sizeof(float));
    return 0;
}

// core/engine/vrx_place.cpp:199
int32_t ref_place(const rv_grid_params* g, int64_t rate, const rv_vrx_request* r,
                  rv_vrx_placement* out) {
    auto placed = engine::place(grid_of(g), rate, request_of(r));
    if (!placed) return report(placed);
    placement_out(*placed, out);
    return 0;
}

uint32_t ref_channel_count_for(int64_t rate, int64_t widest) {
    return engine::channel_count_for(rate, widest);
}

// core/dsp/vrx_reference.cpp:2568
int32_t ref_plan_vrx(const rv_grid_params* g, int64_t rate, const rv_vrx_request* r,
                     const rv_vrx_placement* pl, rv_vrx_plan_info* info, rv_cf32* taps,
                     uint64_t taps_len, float* weights, uint64_t weights_len) {
    auto planned = dsp::plan_vrx(grid_of(g), rate, request_of(r), placement_of(pl));
    if (!planned) return report(planned);
    const dsp::VrxPlan& plan = *planned;
    std::memset(info, 0, sizeof(*info));
    placement_out(plan.placement, &info->placement);
    info->mode = plan.mode;
    info->bandwidth_clamped = plan.bandwidth_clamped ? 1u : 0u;
    info->channel_rate = plan.channel_rate;
    info->audio_rate = plan.audio_rate;
    info->demod_rate = plan.demod_rate;
    info->output_rate = plan.output_rate;
    info->passband_low = plan.passband.low;
    info->passband_high = plan.passband.high;
    info->bandwidth = plan.bandwidth;
    info->filter_numerator = plan.filter_numerator;
    info->filter_denominator = plan.filter_denominator;
    info->mix_numerator = plan.mix_numerator;
    info->mix_denominator = plan.mix_denominator;
    info->fine = rv_vrx_fine_config{plan.fine.taps, plan.fine.phases, plan.fine.nco_log2};
    info->stereo = plan.stereo ? 1u : 0u;
    info->fine_nco_delta = plan.fine_nco_delta;
    info->demod = rv_vrx_demod_config{plan.demod.mode,       plan.demod.decimation,
                                      plan.demod.audio_taps, plan.demod.dc_taps,
                                      plan.demod.channels,   plan.demod.pilot_taps};
    info->demod_gain = plan.demod_gain;
    info->carrier = rv_vrx_carrier_config{plan.carrier.power, plan.carrier.nco_log2};
    std::memcpy(&info->carrier_loop, &plan.carrier_loop, sizeof(info->carrier_loop));
    info->deviation = plan.deviation;
    info->deemphasis = static_cast<uint32_t>(plan.deemphasis);
    info->deemphasis_taps = plan.deemphasis_taps;
    info->audio_decimation_taps = plan.audio_decimation_taps;
    info->fine_tap_count = plan.fine_taps.size();
    info->demod_weight_count = plan.demod_weights.size();
    if (taps != nullptr) {
        if (taps_len != plan.fine_taps.size()) { g_error = "taps length mismatch"; return -1; }
        std::memcpy(taps, plan.fine_taps.data(), taps_len * sizeof(rv_cf32));
    }
    if (weights != nullptr) {
        if (weights_len != plan.demod_weights.size()) { g_error = "weights length mismatch"; return -1; }
        std::memcpy(weights, plan.demod_weights.data(), weights_len * sizeof(float));
    }
    g_error.clear();
    return 0;
}

// core/dsp/vrx_reference.cpp fine_block / demod_block / carrier_block: these
// take a VrxPlan, so the shim re-plans from the request (cheap) and calls them.
int32_t ref_fine_block(const rv_grid_params* g, int64_t rate, const rv_vrx_request* r,
                       uint32_t channel_base, uint32_t channel_mask, uint32_t fine_mask,
                       uint64_t first_output, uint32_t count, rv_vrx_fine_block* out) {
    auto placed = engine::place(grid_of(g), rate, request_of(r));
    if (!placed) return report(placed);
    auto planned = dsp::plan_vrx(grid_of(g), rate, request_of(r), *placed);
    if (!planned) return report(planned);
    auto block = dsp::fine_block(*planned, channel_base, channel_mask, fine_mask, first_output, count);
    if (!block) return report(block);
    std::memset(out, 0, sizeof(*out));
    std::memcpy(&out->params, &block->params, sizeof(out->params));
    out->first_input = block->first_input;
    out->oldest_input = block->oldest_input;
    out->newest_input = block->newest_input;
    return 0;
}

int32_t ref_demod_block(const rv_grid_params* g, int64_t rate, const rv_vrx_request* r,
                        uint32_t fine_mask, uint64_t first_audio, uint32_t count,
                        rv_vrx_demod_block* out) {
    auto placed = engine::place(grid_of(g), rate, request_of(r));
    if (!placed) return report(placed);
    auto planned = dsp::plan_vrx(grid_of(g), rate, request_of(r), *placed);
    if (!planned) return report(planned);
    auto block = dsp::demod_block(*planned, fine_mask, first_audio, count);
    if (!block) return report(block);
    std::memset(out, 0, sizeof(*out));
    std::memcpy(&out->params, &block->params, sizeof(out->params));
    out->first_fine = block->first_fine;
    out->oldest_fine = block->oldest_fine;
    return 0;
}

// lw-radio-dsp make_window (src/primitives.cpp:124); kind is lwdsp::Window's
// value (0 rectangular, 1 Hann, 2 Blackman-Harris).
int32_t ref_lwdsp_window(uint32_t kind, uint32_t n, float* out) {
    const auto w = lwdsp::make_window(static_cast<lwdsp::Window>(kind), static_cast<int>(n));
    std::memcpy(out, w.data(), w.size() * sizeof(float));
    return 0;
}

// lw-radio-dsp Spectrum::compute (src/spectrum.cpp:32-44) called once per
// frame of `size` samples on one Spectrum object, so the exponential average
// carries across frames as it does across the reference's calls; every call's
// dB row is written to db_out[frame * size ...].
int32_t ref_lwdsp_spectrum(uint32_t size, uint32_t kind, float averaging, const rv_cf32* iq,
                           uint64_t frames, float* db_out) {
    lwdsp::Spectrum spec({.size = static_cast<int>(size), .window = static_cast<lwdsp::Window>(kind),
                          .averaging = averaging});
    const auto* z = reinterpret_cast<const std::complex<float>*>(iq);
    for (uint64_t f = 0; f < frames; ++f)
        spec.compute(std::span<const std::complex<float>>(z + f * size, size),
                     std::span<float>(db_out + f * size, size));
    return 0;
}

// core/dsp/front_end_correction_reference.cpp reference_iq_moments
int32_t ref_iq_moments(const rv_iq_moments_params* p, const rv_cf32* ring, uint64_t ring_len, float* sums,
                       uint64_t sums_len) {
    dsp::IqMomentsParams params{p->ring_mask, p->src_offset, p->count};
    auto st = dsp::reference_iq_moments(
        std::span<const std::complex<float>>(reinterpret_cast<const std::complex<float>*>(ring), ring_len), params,
        std::span<float>(sums, sums_len));
    return st ? 0 : report(st);
}

// reference_iq_correct
int32_t ref_iq_correct(const rv_iq_correct_params* p, const rv_cf32* in, uint64_t in_len, rv_cf32* out,
                       uint64_t out_len) {
    dsp::IqCorrectParams params;
    params.ring_mask = p->ring_mask;
    params.offset = p->offset;
    params.count = p->count;
    params.dc_i = p->dc_i;
    params.dc_q = p->dc_q;
    params.cross = p->cross;
    params.scale = p->scale;
    auto st = dsp::reference_iq_correct(
        std::span<const std::complex<float>>(reinterpret_cast<const std::complex<float>*>(in), in_len), params,
        std::span<std::complex<float>>(reinterpret_cast<std::complex<float>*>(out), out_len));
    return st ? 0 : report(st);
}

// A FrontEndCorrector (core/dsp/front_end_correction.cpp) with its default
// configuration over `blocks` blocks: block b's chunk sums at
// sums + b * stride, `counts[b]` samples; after each update the estimate's
// fields go to estimates[b] and correction(dc, iq) to corrections[b].
int32_t ref_front_end_sequence(const float* sums, uint64_t stride, const uint32_t* counts, uint32_t blocks,
                               int64_t rate, int32_t dc, int32_t iq, rv_front_end* estimates,
                               rv_iq_correct_params* corrections) {
    dsp::FrontEndCorrector corrector;
    for (uint32_t b = 0; b < blocks; ++b) {
        const uint32_t count = counts[b];
        const std::size_t floats = (std::size_t)dsp::iq_moments_chunks(count) * dsp::kIqMomentsPerChunk;
        corrector.update(dsp::total_moments(std::span<const float>(sums + b * stride, floats), count), rate);
        const dsp::FrontEndEstimate& e = corrector.estimate();
        rv_front_end& o = estimates[b];
        std::memset(&o, 0, sizeof o);
        o.measured = e.measured ? 1u : 0u;
        o.iq_plausible = e.iq_plausible ? 1u : 0u;
        o.samples_seen = e.samples_seen;
        o.dc_i = e.dc_i;
        o.dc_q = e.dc_q;
        o.gain = e.gain;
        o.sin_phase = e.sin_phase;
        const dsp::IqCorrectParams c = corrector.correction(dc != 0, iq != 0);
        corrections[b] = rv_iq_correct_params{0u, 0u, 0u, c.dc_i, c.dc_q, c.cross, c.scale};
    }
    return 0;
}

// core/dsp/impulse_excision_reference.cpp
namespace {
dsp::ExcisionConfig xcfg(const rv_excision_config* c) {
    dsp::ExcisionConfig o;
    o.pass = c->pass;
    o.seg_log2 = c->seg_log2;
    o.segments = c->segments;
    o.max_width = c->max_width;
    o.hang = c->hang;
    o.lead = c->lead;
    return o;
}
dsp::ExcisionParams xpar(const rv_excision_params* p) {
    dsp::ExcisionParams o;
    std::memcpy(&o, p, sizeof o);
    return o;
}
void xout(const dsp::ExcisionParams& p, rv_excision_params* o) { std::memcpy(o, &p, sizeof *o); }
std::span<const std::complex<float>> xcs(const rv_cf32* p, uint64_t n) {
    return {reinterpret_cast<const std::complex<float>*>(p), n};
}
std::span<std::complex<float>> xms(rv_cf32* p, uint64_t n) { return {reinterpret_cast<std::complex<float>*>(p), n}; }
}  // namespace

int32_t ref_design_excision(int64_t rate, double max_width_seconds, rv_excision_config* out) {
    const dsp::ExcisionConfig c = dsp::design_excision(rate, max_width_seconds);
    out->pass = c.pass;
    out->seg_log2 = c.seg_log2;
    out->segments = c.segments;
    out->max_width = c.max_width;
    out->hang = c.hang;
    out->lead = c.lead;
    return 0;
}

float ref_excision_threshold(double db) { return dsp::excision_threshold(db); }

int32_t ref_size_excision_rings(const rv_excision_config* c, uint64_t max_block, uint32_t frames, uint32_t ring_mask,
                                rv_excision_rings* out) {
    auto r = dsp::size_excision_rings(xcfg(c), max_block, frames, ring_mask);
    if (!r) return report(r);
    out->seg_mask = r->seg_mask;
    out->flag_mask = r->flag_mask;
    out->removed_mask = r->removed_mask;
    return 0;
}

// An ExcisionCursor over `blocks` blocks [starts[b], starts[b] + counts[b]):
// each block's plan.
int32_t ref_excision_plans(const rv_excision_config* c, uint32_t ring_mask, const rv_excision_rings* rings,
                           float threshold, const uint64_t* starts, const uint32_t* counts, uint32_t blocks,
                           rv_excision_plan* plans) {
    dsp::ExcisionRings rr;
    rr.seg_mask = rings->seg_mask;
    rr.flag_mask = rings->flag_mask;
    rr.removed_mask = rings->removed_mask;
    dsp::ExcisionCursor cursor(xcfg(c), ring_mask, rr, threshold);
    for (uint32_t b = 0; b < blocks; ++b) {
        const dsp::ExcisionPlan p = cursor.plan(starts[b], counts[b]);
        rv_excision_plan& o = plans[b];
        std::memset(&o, 0, sizeof o);
        xout(p.segment, &o.segment);
        xout(p.reference, &o.reference);
        xout(p.flag, &o.flag);
        xout(p.apply, &o.apply);
        o.cleaned_end = p.cleaned_end;
        o.restarted = p.restarted ? 1u : 0u;
    }
    return 0;
}

int32_t ref_excise_segment(const rv_excision_config* c, const rv_excision_params* p, const rv_cf32* raw,
                           uint64_t raw_len, float* seg, uint64_t seg_len) {
    dsp::ExcisionConfig cc = xcfg(c);
    cc.pass = dsp::kExciseSegment;
    auto st = dsp::reference_excise_segment(cc, xpar(p), xcs(raw, raw_len), std::span<float>(seg, seg_len));
    return st ? 0 : report(st);
}

int32_t ref_excise_reference(const rv_excision_config* c, const rv_excision_params* p, const float* seg_power,
                             float* seg_level, uint64_t seg_len) {
    dsp::ExcisionConfig cc = xcfg(c);
    cc.pass = dsp::kExciseReference;
    auto st = dsp::reference_excise_reference(cc, xpar(p), std::span<const float>(seg_power, seg_len),
                                              std::span<float>(seg_level, seg_len));
    return st ? 0 : report(st);
}

int32_t ref_excise_flag(const rv_excision_config* c, const rv_excision_params* p, const rv_cf32* raw,
                        uint64_t raw_len, const float* seg_level, uint64_t seg_len, uint32_t* flags,
                        uint64_t flags_len) {
    dsp::ExcisionConfig cc = xcfg(c);
    cc.pass = dsp::kExciseFlag;
    auto st = dsp::reference_excise_flag(cc, xpar(p), xcs(raw, raw_len), std::span<const float>(seg_level, seg_len),
                                         std::span<std::uint32_t>(flags, flags_len));
    return st ? 0 : report(st);
}

int32_t ref_excise_apply(const rv_excision_config* c, const rv_excision_params* p, const rv_cf32* raw,
                         uint64_t raw_len, const uint32_t* flags, uint64_t flags_len, rv_cf32* cleaned,
                         rv_cf32* removed, uint64_t removed_len, uint32_t* counters) {
    dsp::ExcisionConfig cc = xcfg(c);
    cc.pass = dsp::kExciseApply;
    auto st = dsp::reference_excise_apply(cc, xpar(p), xcs(raw, raw_len),
                                          std::span<const std::uint32_t>(flags, flags_len),
                                          xms(cleaned, (uint64_t)p->ring_mask + 1u), xms(removed, removed_len),
                                          std::span<std::uint32_t>(counters, 4));
    return st ? 0 : report(st);
}

// core/dsp/noise_reference.cpp: the blanker, the line kernel and the
// spectral noise reduction, with their designers. The parameter blocks are
// the reference's own layouts, copied word for word.
static_assert(sizeof(dsp::BlankerParams) == sizeof(rv_blanker_params));
static_assert(sizeof(dsp::LineParams) == sizeof(rv_line_params));
static_assert(sizeof(dsp::SpectralParams) == sizeof(rv_spectral_params));

int32_t ref_design_blanker(int64_t rate, rv_blanker_config* out) {
    const dsp::BlankerConfig c = dsp::design_blanker(rate);
    out->pass = c.pass;
    out->window = c.window;
    out->guard = c.guard;
    out->hang = c.hang;
    out->lead = c.lead;
    return 0;
}

float ref_blanker_threshold(double db) { return dsp::blanker_threshold(db); }

namespace {
dsp::BlankerConfig xbc(const rv_blanker_config* c, uint32_t pass) {
    dsp::BlankerConfig o;
    o.pass = pass;
    o.window = c->window;
    o.guard = c->guard;
    o.hang = c->hang;
    o.lead = c->lead;
    return o;
}
dsp::BlankerParams xbp(const rv_blanker_params* p) {
    dsp::BlankerParams o;
    std::memcpy(&o, p, sizeof o);
    return o;
}
}  // namespace

int32_t ref_blank_detect(const rv_blanker_config* c, const rv_blanker_params* p, const rv_cf32* chan, uint64_t chan_len,
                         float* flags, uint64_t flags_len) {
    auto st = dsp::reference_blank_detect(xbc(c, dsp::kBlankDetect), xbp(p), xcs(chan, chan_len),
                                          std::span<float>(flags, flags_len));
    return st ? 0 : report(st);
}

int32_t ref_blank_apply(const rv_blanker_config* c, const rv_blanker_params* p, const rv_cf32* chan, uint64_t chan_len,
                        const float* flags, uint64_t flags_len, rv_cf32* blanked, uint64_t blanked_len) {
    auto st = dsp::reference_blank_apply(xbc(c, dsp::kBlankApply), xbp(p), xcs(chan, chan_len),
                                         std::span<const float>(flags, flags_len), xms(blanked, blanked_len));
    return st ? 0 : report(st);
}

int32_t ref_noise_line(const rv_line_config* c, const rv_line_params* p, float* audio, uint64_t audio_len,
                       float* state, uint64_t state_len) {
    dsp::LineConfig cc;
    cc.lanes = c->lanes;
    cc.taps = c->taps;
    cc.history = c->history;
    dsp::LineParams pp;
    std::memcpy(&pp, p, sizeof pp);
    auto st = dsp::reference_line(cc, pp, std::span<float>(audio, audio_len), std::span<float>(state, state_len));
    return st ? 0 : report(st);
}

int32_t ref_design_notch(double audio_hz, double depth_db, double width_hz, int64_t rate, rv_notch_design* out) {
    auto d = dsp::design_notch(audio_hz, depth_db, width_hz, rate);
    if (!d) return report(d);
    out->b0 = d->b0;
    out->b1 = d->b1;
    out->b2 = d->b2;
    out->a1 = d->a1;
    out->a2 = d->a2;
    return 0;
}

int32_t ref_spectral_config_for(int64_t rate, rv_spectral_config* out) {
    out->frame = dsp::spectral_config_for(rate).frame;
    return 0;
}

int32_t ref_design_spectral_tables(const rv_spectral_config* c, float* t, uint64_t len) {
    dsp::SpectralConfig cc;
    cc.frame = c->frame;
    const std::vector<float> v = dsp::design_spectral_tables(cc);
    if (len < v.size()) return -1;
    std::memcpy(t, v.data(), v.size() * sizeof(float));
    return 0;
}

int32_t ref_design_spectral_params(double strength, rv_spectral_params* out) {
    const dsp::SpectralParams p = dsp::spectral_params(strength);
    std::memcpy(out, &p, sizeof *out);
    return 0;
}

int32_t ref_noise_spectral(const rv_spectral_config* c, const rv_spectral_params* p, const float* tables,
                           uint64_t tables_len, float* audio, uint64_t audio_len, float* state, uint64_t state_len) {
    dsp::SpectralConfig cc;
    cc.frame = c->frame;
    dsp::SpectralParams pp;
    std::memcpy(&pp, p, sizeof pp);
    auto st = dsp::reference_spectral(cc, pp, std::span<const float>(tables, tables_len),
                                      std::span<float>(audio, audio_len), std::span<float>(state, state_len));
    return st ? 0 : report(st);
}

// core/dsp/vrx_reference.cpp: the display tap
uint32_t ref_display_max_decimation(void) { return dsp::display_max_decimation(); }

int32_t ref_display_ladder(int64_t rate, uint32_t* rungs, uint32_t capacity, uint32_t* count) {
    const std::vector<std::uint32_t> v = dsp::display_ladder(rate);
    *count = (uint32_t)v.size();
    for (uint32_t i = 0; i < *count && i < capacity; ++i) rungs[i] = v[i];
    return 0;
}

uint32_t ref_display_decimation(int64_t rate, int64_t reach) { return dsp::display_decimation(rate, reach); }

// place + plan_vrx + plan_vrx_display for a request, and optionally one
// display_block
int32_t ref_plan_vrx_display(const rv_grid_params* g, int64_t rate, const rv_vrx_request* r, rv_vrx_display_plan* out,
                             rv_cf32* taps, uint64_t taps_len, uint32_t channel_base, uint32_t channel_mask,
                             uint32_t display_mask, uint64_t first_output, uint32_t count, rv_vrx_fine_block* block) {
    auto placed = engine::place(grid_of(g), rate, request_of(r));
    if (!placed) return report(placed);
    auto planned = dsp::plan_vrx(grid_of(g), rate, request_of(r), *placed);
    if (!planned) return report(planned);
    auto disp = dsp::plan_vrx_display(*planned);
    if (!disp) return report(disp);
    const dsp::VrxDisplayPlan& d = *disp;
    std::memset(out, 0, sizeof *out);
    out->channel_rate = d.channel_rate;
    out->display_rate = d.display_rate;
    out->decimation = d.decimation;
    out->reach_hz = d.reach_hz;
    out->fine = rv_vrx_fine_config{d.fine.taps, d.fine.phases, d.fine.nco_log2};
    out->nco_delta = d.nco_delta;
    out->pass_hz = d.pass_hz;
    out->stop_hz = d.stop_hz;
    out->attenuation_db = d.attenuation_db;
    out->group_delay_channel_samples = d.group_delay_channel_samples;
    out->tap_count = d.taps.size();
    if (taps) {
        if (taps_len != d.taps.size()) return -1;
        std::memcpy(taps, d.taps.data(), d.taps.size() * sizeof(rv_cf32));
    }
    if (block && count) {
        auto b = dsp::display_block(d, channel_base, channel_mask, display_mask, first_output, count);
        if (!b) return report(b);
        std::memset(block, 0, sizeof *block);
        std::memcpy(&block->params, &b->params, sizeof(block->params));
        block->first_input = b->first_input;
        block->oldest_input = b->oldest_input;
        block->newest_input = b->newest_input;
    }
    return 0;
}

// core/dsp/comb_kernels_reference.cpp
static_assert(sizeof(dsp::CombLine) == sizeof(rv_comb_line));
static_assert(sizeof(dsp::CombParams) == sizeof(rv_comb_params));

uint32_t ref_comb_step(double hz, int64_t rate) { return dsp::comb_step(hz, rate); }

int32_t ref_comb_table(rv_cf32* t, uint64_t len) {
    const std::vector<dsp::Complex32> v = dsp::comb_table();
    if (len < v.size()) return -1;
    std::memcpy(t, v.data(), v.size() * sizeof(rv_cf32));
    return 0;
}

int32_t ref_comb_project(const rv_comb_params* p, const rv_cf32* raw, uint64_t raw_len, const rv_comb_line* lines,
                         uint64_t lines_len, const rv_cf32* table, uint64_t table_len, rv_cf32* proj, uint64_t proj_len) {
    dsp::CombParams pp;
    std::memcpy(&pp, p, sizeof pp);
    auto st = dsp::reference_comb_project(
        pp, xcs(raw, raw_len), std::span<const dsp::CombLine>(reinterpret_cast<const dsp::CombLine*>(lines), lines_len),
        xcs(table, table_len), xms(proj, proj_len));
    return st ? 0 : report(st);
}

int32_t ref_comb_subtract(const rv_comb_params* p, const rv_cf32* raw, uint64_t raw_len, const rv_comb_line* lines,
                          uint64_t lines_len, const rv_cf32* table, uint64_t table_len, rv_cf32* cleaned,
                          uint64_t cleaned_len, rv_cf32* removed, uint64_t removed_len) {
    dsp::CombParams pp;
    std::memcpy(&pp, p, sizeof pp);
    auto st = dsp::reference_comb_subtract(
        pp, xcs(raw, raw_len), std::span<const dsp::CombLine>(reinterpret_cast<const dsp::CombLine*>(lines), lines_len),
        xcs(table, table_len), xms(cleaned, cleaned_len), xms(removed, removed_len));
    return st ? 0 : report(st);
}

}  // extern "C"
