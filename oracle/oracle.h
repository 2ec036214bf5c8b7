/*
 * oracle.h — CPU restatement of the reference's receive-chain twins.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT. Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline / reference leg may load this library, and only as
 * the checker (or the timed CPU arm). The GPU library never links it and has
 * no CPU fallback.
 *
 * Each function restates, in plain C, the reference CPU twin cited beside it,
 * in the same operation order: fp32 with no contraction and denormals flushed
 * to zero, so that results are bit-identical to the twin (and to the CUDA
 * kernels). Parity of this restatement with the reference itself is pinned in
 * tests/test_oracle_pin.py against the reference's own twins compiled from
 * source (oracle/ref), and by the committed fixtures in tests/golden/.
 *
 * The *_f64 functions are double-precision restatements of the same maths
 * (not of the fp32 operation order), used as the error yardstick for the
 * reordered / split-precision paths.
 *
 * Return value: 0 on success, -1 on rejected parameters (message from
 * or_last_error()), mirroring the twins' Status.
 */
#ifndef REVENANT_ORACLE_H
#define REVENANT_ORACLE_H

#include <stdint.h>

#include "../include/revenant_gb300.h"

#ifdef __cplusplus
extern "C" {

/* scene noise field: siggen::Scene::fill_noise (core/dsp/synth/wideband.cpp:535-580) */
double or_scene_noise_sigma(double dbfs);
int32_t or_scene_noise(uint64_t seed, double sigma, uint64_t start, uint64_t count, rv_cf32* out);
int32_t or_scene_noise_draws(uint64_t seed, uint64_t start, uint64_t count, uint64_t* draws);
/* tone emitters: Modulator::accumulate_am / _nfm / _ssb (core/dsp/synth/modulators.cpp:1244-1366) */
int32_t or_emitter_accumulate(const rv_tone_emitter* e, uint64_t first, uint64_t count, double gain, rv_cf32* io);
int32_t or_emitter_accumulate_audio(const rv_tone_emitter* e, const float* audio, uint64_t len, uint32_t taps,
                                    uint64_t first, uint64_t count, double gain, rv_cf32* io);
#endif

const char* or_last_error(void);

/* The planner (planner.c): pfb_design.cpp:381-590 design_prototype and
 * build_twiddles, vrx_reference.cpp:364 build_nco_table, vrx_place.cpp place,
 * vrx_reference.cpp plan_vrx with its tables and the block parameters. */
int32_t or_design_prototype(const rv_grid_params* g, double attenuation_db, float* taps, uint64_t taps_len);
int32_t or_build_twiddles(uint32_t M, rv_cf32* out, uint64_t len);
int32_t or_build_nco_table(uint32_t log2, rv_cf32* out, uint64_t len);
int32_t or_place(const rv_grid_params* g, int64_t rate, const rv_vrx_request* r, rv_vrx_placement* out);
int32_t or_plan_vrx(const rv_grid_params* g, int64_t rate, const rv_vrx_request* r, const rv_vrx_placement* pl,
                    rv_vrx_plan_info* p, rv_cf32* taps, uint64_t taps_len, float* weights, uint64_t weights_len);
int32_t or_fine_block(const rv_vrx_plan_info* plan, uint32_t channel_base, uint32_t channel_mask, uint32_t fine_mask,
                      uint64_t first_output, uint32_t count, rv_vrx_fine_block* block);
uint32_t or_demod_fine_history(const rv_vrx_demod_config* c);
int32_t or_demod_block(const rv_vrx_plan_info* plan, uint32_t fine_mask, uint64_t first_audio, uint32_t count,
                       rv_vrx_demod_block* block);
int32_t or_carrier_block(const rv_vrx_plan_info* plan, uint32_t fine_mask, uint64_t first_fine, uint32_t count,
                         int32_t reset, float shift, rv_vrx_carrier_params* out);

float or_det_rsqrt(float v);
float or_det_sqrt(float v);
float or_det_recip(float v);
float or_det_atan2(float y, float x);
float or_det_log2(float v);

int32_t or_convert(int32_t format, const rv_convert_params* p, const void* packed,
                   uint64_t packed_bytes, rv_cf32* ring, uint64_t ring_len);
int32_t or_pfb_branch(const rv_grid_params* g, const rv_pfb_branch_params* p, const float* taps,
                      uint64_t taps_len, const rv_cf32* ring, uint64_t ring_len, rv_cf32* out,
                      uint64_t out_len);
int32_t or_pfb_fft(const rv_pfb_fft_params* p, const rv_cf32* branch, uint64_t branch_len,
                   const rv_cf32* twiddles, uint64_t tw_len, rv_cf32* ring, uint64_t ring_len);
int32_t or_fft_radix2(const rv_cf32* twiddles, const rv_cf32* in, rv_cf32* out, uint32_t size,
                      uint32_t batch);
int32_t or_spectrum(const rv_spectrum_params* p, const rv_cf32* ring, uint64_t ring_len,
                    const rv_cf32* twiddles, uint64_t tw_len, const float* window,
                    uint64_t window_len, float* frame, uint64_t frame_len);
int32_t or_spectrum_levels(const rv_spectrum_levels_params* p, const float* frame,
                           uint64_t frame_len, float* levels);
int32_t or_vrx_fine(const rv_vrx_fine_config* c, const rv_vrx_fine_params* p, const rv_cf32* chan,
                    uint64_t chan_len, const rv_cf32* taps, uint64_t taps_len, const rv_cf32* nco,
                    uint64_t nco_len, rv_cf32* fine, uint64_t fine_len);
int32_t or_vrx_demod(const rv_vrx_demod_config* c, const rv_vrx_demod_params* p,
                     const rv_cf32* fine, uint64_t fine_len, const float* weights,
                     uint64_t weights_len, float* audio, uint64_t audio_len);
int32_t or_vrx_carrier(const rv_vrx_carrier_config* c, const rv_vrx_carrier_params* p,
                       const rv_cf32* nco, uint64_t nco_len, rv_cf32* fine, uint64_t fine_len,
                       uint32_t* state);

/* Whole coarse chain for a contiguous cs16 capture: convert -> branch -> FFT,
 * block by block, over `threads` host threads (0 = all). Output is the
 * channel-major ring [M][out_ring_blocks]. Used as the timed CPU arm and as
 * the checker of the fused GPU coarse kernel. */
int32_t or_coarse_cs16(const rv_grid_params* g, const float* taps, const rv_cf32* twiddles,
                       const void* packed, uint64_t samples, uint64_t first_block,
                       uint32_t block_count, uint32_t out_ring_blocks, rv_cf32* channel_ring,
                       int32_t threads);

/* FP64 yardstick: PFB channelizer (branch FIR + exact M-point DFT + phase
 * correction) of cf32 input x (as double), for blocks [0, block_count):
 * y[k][m] = sum_r branch_r(m) * exp(-2 pi i k (M - r mod M)/M) * exp(-2 pi i k m D / M).
 * Output channel-major [M][block_count] complex double. */
int32_t or_pfb_branch_wide(const rv_grid_params* g, const rv_pfb_branch_params* p, const float* taps,
                           uint64_t taps_len, const rv_cf32* ring, uint64_t ring_len, rv_cf32* out,
                           uint64_t out_len);
int32_t or_pfb_f64(const rv_grid_params* g, const float* taps, const rv_cf32* ring,
                   uint32_t ring_mask, uint32_t base_offset, uint32_t block_count,
                   uint32_t block_base, double* out_re, double* out_im);

#ifdef __cplusplus
}

/* scene noise field: siggen::Scene::fill_noise (core/dsp/synth/wideband.cpp:535-580) */
double or_scene_noise_sigma(double dbfs);
int32_t or_scene_noise(uint64_t seed, double sigma, uint64_t start, uint64_t count, rv_cf32* out);
int32_t or_scene_noise_draws(uint64_t seed, uint64_t start, uint64_t count, uint64_t* draws);
/* tone emitters: Modulator::accumulate_am / _nfm / _ssb (core/dsp/synth/modulators.cpp:1244-1366) */
int32_t or_emitter_accumulate(const rv_tone_emitter* e, uint64_t first, uint64_t count, double gain, rv_cf32* io);
int32_t or_emitter_accumulate_audio(const rv_tone_emitter* e, const float* audio, uint64_t len, uint32_t taps,
                                    uint64_t first, uint64_t count, double gain, rv_cf32* io);
#endif


/* front-end correction: twins of core/dsp/front_end_correction_reference.cpp
 * and the host FrontEndCorrector (core/dsp/front_end_correction.cpp) */
int32_t or_iq_moments(const rv_iq_moments_params* p, const rv_cf32* ring, uint64_t ring_len, float* sums,
                      uint64_t sums_len);
int32_t or_iq_correct(const rv_iq_correct_params* p, const rv_cf32* in, uint64_t in_len, rv_cf32* out,
                      uint64_t out_len);
int32_t or_front_end_update(rv_front_end* st, const float* sums, uint64_t sums_len, uint32_t count, int64_t rate);
int32_t or_front_end_correction(const rv_front_end* st, int32_t dc, int32_t iq, rv_iq_correct_params* out);

/* impulse excision: twins of core/dsp/impulse_excision_reference.cpp */
int32_t or_design_excision(int64_t source_rate, double max_width_seconds, rv_excision_config* out);
float or_excision_threshold(double threshold_db);
int32_t or_size_excision_rings(const rv_excision_config* c, uint64_t max_block, uint32_t frames_in_flight,
                               uint32_t ring_mask, rv_excision_rings* out);
int32_t or_excision_cursor_init(rv_excision_cursor* k, const rv_excision_config* c, uint32_t ring_mask,
                                const rv_excision_rings* rings, float threshold);
int32_t or_excision_plan_block(rv_excision_cursor* k, uint64_t start, uint32_t count, rv_excision_plan* out);
int32_t or_excise_segment(const rv_excision_config* c, const rv_excision_params* p, const rv_cf32* raw,
                          uint64_t raw_len, float* seg_power, uint64_t seg_len);
int32_t or_excise_reference(const rv_excision_config* c, const rv_excision_params* p, const float* seg_power,
                            float* seg_level, uint64_t seg_len);
int32_t or_excise_flag(const rv_excision_config* c, const rv_excision_params* p, const rv_cf32* raw,
                       uint64_t raw_len, const float* seg_level, uint64_t seg_len, uint32_t* flags,
                       uint64_t flags_len);
int32_t or_excise_apply(const rv_excision_config* c, const rv_excision_params* p, const rv_cf32* raw,
                        uint64_t raw_len, const uint32_t* flags, uint64_t flags_len, rv_cf32* cleaned,
                        rv_cf32* removed, uint64_t removed_len, uint32_t* counters);

/* per-receiver noise stages: twins of core/dsp/noise_reference.cpp */
int32_t or_design_blanker(int64_t channel_rate, rv_blanker_config* out);
float or_blanker_threshold(double threshold_db);
int32_t or_blank_detect(const rv_blanker_config* c, const rv_blanker_params* p, const rv_cf32* chan,
                        uint64_t chan_len, float* flags, uint64_t flags_len);
int32_t or_blank_apply(const rv_blanker_config* c, const rv_blanker_params* p, const rv_cf32* chan,
                       uint64_t chan_len, const float* flags, uint64_t flags_len, rv_cf32* blanked,
                       uint64_t blanked_len);
int32_t or_noise_line(const rv_line_config* c, const rv_line_params* p, float* audio, uint64_t audio_len,
                      float* state, uint64_t state_len);
int32_t or_design_notch(double audio_hz, double depth_db, double width_hz, int64_t audio_rate, rv_notch_design* d);
int32_t or_spectral_config_for(int64_t audio_rate, rv_spectral_config* out);
int32_t or_design_spectral_tables(const rv_spectral_config* c, float* t, uint64_t len);
int32_t or_design_spectral_params(double strength, rv_spectral_params* o);
int32_t or_noise_spectral(const rv_spectral_config* c, const rv_spectral_params* p, const float* tables,
                          uint64_t tables_len, float* audio, uint64_t audio_len, float* state, uint64_t state_len);

/* comb cancellation: twins of core/dsp/comb_kernels_reference.cpp */
uint32_t or_comb_step(double frequency_hz, int64_t rate);
int32_t or_comb_table(rv_cf32* t, uint64_t len);
int32_t or_comb_project(const rv_comb_params* p, const rv_cf32* raw, uint64_t raw_len, const rv_comb_line* lines,
                        uint64_t lines_len, const rv_cf32* table, uint64_t table_len, rv_cf32* proj,
                        uint64_t proj_len);
int32_t or_comb_subtract(const rv_comb_params* p, const rv_cf32* raw, uint64_t raw_len, const rv_comb_line* lines,
                         uint64_t lines_len, const rv_cf32* table, uint64_t table_len, rv_cf32* cleaned,
                         uint64_t cleaned_len, rv_cf32* removed, uint64_t removed_len);

/* scene noise field: siggen::Scene::fill_noise (core/dsp/synth/wideband.cpp:535-580) */
double or_scene_noise_sigma(double dbfs);
int32_t or_scene_noise(uint64_t seed, double sigma, uint64_t start, uint64_t count, rv_cf32* out);
int32_t or_scene_noise_draws(uint64_t seed, uint64_t start, uint64_t count, uint64_t* draws);
/* tone emitters: Modulator::accumulate_am / _nfm / _ssb (core/dsp/synth/modulators.cpp:1244-1366) */
int32_t or_emitter_accumulate(const rv_tone_emitter* e, uint64_t first, uint64_t count, double gain, rv_cf32* io);
int32_t or_emitter_accumulate_audio(const rv_tone_emitter* e, const float* audio, uint64_t len, uint32_t taps,
                                    uint64_t first, uint64_t count, double gain, rv_cf32* io);
#endif
