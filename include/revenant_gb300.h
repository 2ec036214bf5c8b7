/*
 * revenant_gb300.h — the C ABI of the GB300 receive chain.
 *
 * This library stands in for the reference's Vulkan operator surface on the
 * receive path: core/gpu (Context, Buffer, ComputePipeline + record_dispatch)
 * together with the hot-path shaders in core/shaders. Every launch takes the
 * same parameter structs the reference's shaders take as push and
 * specialisation constants, byte for byte, so a caller that builds a
 * PfbBranchParams / VrxFineParams / ... for the reference can hand the same
 * bytes here. Host-side planning (prototype and table design, receiver
 * placement, plan_vrx, per-block parameter derivation) is exported too, so a
 * caller without the reference's core/dsp can drive the chain.
 *
 * Conventions (mirroring core/error.h and core/plugin/engine_plugin_abi.h):
 *   - every entry point returns int32: RV_OK (0) or a negative RV_ERR_*;
 *   - the message for the most recent failure on the calling thread is
 *     returned by rv_last_error();
 *   - no C++ exception crosses this boundary;
 *   - pointers named *_dev are CUDA device pointers, all other pointers are
 *     host pointers; lengths are ELEMENT counts of the pointed-to type;
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default);
 *   - launches are asynchronous on `stream` and never allocate; parameters
 *     are validated on the host before the launch, with the same rules as the
 *     reference's validate() twins, and a rejected launch enqueues nothing.
 */
#ifndef REVENANT_GB300_H
#define REVENANT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (core/error.h Status / Error{message, code}) ---------- */
#define RV_OK 0
#define RV_ERR_INVALID (-1)     /* parameters rejected by host validation   */
#define RV_ERR_CUDA (-2)        /* a CUDA runtime call failed               */
#define RV_ERR_NO_DEVICE (-3)   /* no usable sm_103 device                  */
#define RV_ERR_NO_MEMORY (-4)   /* allocation failed                        */
#define RV_ERR_UNSUPPORTED (-5) /* shape outside what this build implements */
#define RV_ERR_TIMEOUT (-6)     /* a bounded device wait gave up            */

/* Message for the most recent failure on this thread ("" if none). The
 * pointer stays valid until the next failing call on the same thread. */
const char* rv_last_error(void);

/* Library version; bumps on any ABI change. */
#define RV_ABI_VERSION 1
int32_t rv_abi_version(void);

/* ---- value types ------------------------------------------------------- */

/* std::complex<float> / std430 vec2 (core/dsp/types.h:40-45). */
typedef struct rv_cf32 {
    float re;
    float im;
} rv_cf32;

/* core/dsp/convert.h:116-143 ConvertParams: four packed uint32. */
typedef struct rv_convert_params {
    uint32_t ring_mask;
    uint32_t dst_offset;
    uint32_t src_offset; /* in SAMPLES, not bytes */
    uint32_t count;
} rv_convert_params;

/* core/dsp/pfb.h:32-71 GridParams (M, L+1, D). */
typedef struct rv_grid_params {
    uint32_t channels;
    uint32_t taps_per_branch;
    uint32_t decimation;
} rv_grid_params;

/* core/dsp/pfb_branch_reference.h:28-53 PfbBranchParams. */
typedef struct rv_pfb_branch_params {
    uint32_t ring_mask;
    uint32_t base_offset;
    uint32_t block_count;
} rv_pfb_branch_params;

/* core/dsp/pfb_fft_reference.h:36-69 PfbFftParams: the FFT kernel's three
 * specialisation constants (M, D, log2 M) then its four push constants. */
typedef struct rv_pfb_fft_params {
    uint32_t channels;
    uint32_t decimation;
    uint32_t stages;
    uint32_t block_base;
    uint32_t block_count;
    uint32_t out_ring_blocks;
    uint32_t out_ring_mask;
} rv_pfb_fft_params;

/* core/dsp/spectrum_reference.h SpectrumParams (spec M, N, log2 N; push
 * chan_blocks, chan_mask, in_offset). */
typedef struct rv_spectrum_params {
    uint32_t channels;
    uint32_t transform;
    uint32_t stages;
    uint32_t chan_blocks;
    uint32_t chan_mask;
    uint32_t in_offset;
} rv_spectrum_params;

/* core/dsp/spectrum_levels_reference.h SpectrumLevelsParams. */
typedef struct rv_spectrum_levels_params {
    uint32_t bins;
    uint32_t low_permille;
    uint32_t high_permille;
} rv_spectrum_levels_params;

/* core/dsp/vrx_reference.h VrxFineConfig (spec T, P, nco_log2). */
typedef struct rv_vrx_fine_config {
    uint32_t taps;
    uint32_t phases;
    uint32_t nco_log2;
} rv_vrx_fine_config;

/* core/dsp/vrx_reference.h:232-271 VrxFineParams: fifteen 32-bit words. */
typedef struct rv_vrx_fine_params {
    uint32_t chan_base;
    uint32_t chan_mask;
    uint32_t in_offset;
    uint32_t out_offset;
    uint32_t out_mask;
    uint32_t count;
    uint32_t step_whole;
    uint32_t step_rem;
    uint32_t out_rate;
    uint32_t frac0;
    uint32_t nco_phase_high;
    uint32_t nco_phase_low;
    uint32_t nco_delta_high;
    uint32_t nco_delta_low;
    float inv_out_rate;
} rv_vrx_fine_params;

/* Demodulator modes: engine::Demod (core/engine/vrx.h) numbering. */
#define RV_DEMOD_RAW 0
#define RV_DEMOD_AM 1
#define RV_DEMOD_NFM 2
#define RV_DEMOD_WFM 3
#define RV_DEMOD_USB 4
#define RV_DEMOD_LSB 5
#define RV_DEMOD_DSB 6
#define RV_DEMOD_CW 7
#define RV_DEMOD_P25P1 8
#define RV_DEMOD_DSTAR 9
#define RV_DEMOD_TETRA 10
#define RV_DEMOD_DMR 11
#define RV_DEMOD_SAM 12

/* core/dsp/vrx_reference.h VrxDemodConfig (the demod kernel's seven
 * specialisation constants minus channel_power). */
typedef struct rv_vrx_demod_config {
    uint32_t mode;
    uint32_t decimation;
    uint32_t audio_taps;
    uint32_t dc_taps;
    uint32_t channels;
    uint32_t pilot_taps;
} rv_vrx_demod_config;

/* core/dsp/vrx_reference.h:584 VrxDemodParams: four 32-bit words. */
typedef struct rv_vrx_demod_params {
    uint32_t in_mask;
    uint32_t in_offset;
    uint32_t count;
    float gain;
} rv_vrx_demod_params;

/* core/dsp/vrx_reference.h VrxCarrierConfig; power 1 = PLL, 2 = Costas. */
typedef struct rv_vrx_carrier_config {
    uint32_t power;
    uint32_t nco_log2;
} rv_vrx_carrier_config;

/* core/dsp/vrx_reference.h:716 VrxCarrierParams: fourteen 32-bit words. */
typedef struct rv_vrx_carrier_params {
    uint32_t in_mask;
    uint32_t in_offset;
    uint32_t count;
    uint32_t flags;
    float shift;
    float k1_acquire;
    float k2_acquire;
    float k1_track;
    float k2_track;
    float level_alpha;
    float lock_alpha;
    float clamp_radians;
    uint32_t hold_in;
    uint32_t hold_out;
} rv_vrx_carrier_params;

#define RV_CARRIER_STATE_WORDS 8

/* ---- receiver requests and plans (core/engine/vrx.h, vrx_reference.h) -- */

/* The planning-relevant subset of engine::VrxParams. */
typedef struct rv_vrx_request {
    int64_t center;        /* Hz relative to the source centre */
    int64_t bandwidth;     /* Hz; 0 = the mode's default passband */
    int64_t passband_low;  /* explicit edges win when either is non-zero */
    int64_t passband_high;
    uint32_t demod;        /* RV_DEMOD_* */
    uint32_t deemphasis;   /* 0 default, 1 none, 2 75us, 3 50us */
    uint32_t stereo;       /* 0/1 */
    uint32_t reserved;
    int64_t audio_rate;    /* 0 = 48000 */
    int64_t cw_pitch;      /* Hz, CW only */
} rv_vrx_request;

/* engine::VrxPlacement (core/engine/vrx.h). */
typedef struct rv_vrx_placement {
    uint32_t channel;
    uint32_t bandwidth_clamped;
    int64_t centre_numerator;
    int64_t centre_denominator;
    int64_t residual_numerator;
    int64_t residual_denominator;
    int64_t channel_rate;
    int64_t granted_low;
    int64_t granted_high;
} rv_vrx_placement;

/* The scalar part of dsp::VrxPlan (core/dsp/vrx_reference.h). The two
 * tables (fine taps, demod weights) are returned separately. */
typedef struct rv_vrx_plan_info {
    rv_vrx_placement placement;
    uint32_t mode;
    uint32_t bandwidth_clamped;
    int64_t channel_rate;
    int64_t audio_rate;
    int64_t demod_rate;
    int64_t output_rate;
    int64_t passband_low;
    int64_t passband_high;
    int64_t bandwidth;
    int64_t filter_numerator;
    int64_t filter_denominator;
    int64_t mix_numerator;
    int64_t mix_denominator;
    rv_vrx_fine_config fine;
    uint32_t stereo;
    uint64_t fine_nco_delta;
    rv_vrx_demod_config demod;
    float demod_gain;
    rv_vrx_carrier_config carrier;
    rv_vrx_carrier_params carrier_loop;
    int64_t deviation;
    uint32_t deemphasis;
    uint32_t deemphasis_taps;
    uint32_t audio_decimation_taps;
    uint32_t reserved;
    uint64_t fine_tap_count;     /* phases * taps + 1 */
    uint64_t demod_weight_count; /* audio + dc + 2*pilot (+ 2*audio rotation) */
} rv_vrx_plan_info;

/* dsp::VrxFineBlock / VrxDemodBlock bookkeeping. */
typedef struct rv_vrx_fine_block {
    rv_vrx_fine_params params;
    uint32_t reserved;
    uint64_t first_input;
    uint64_t oldest_input;
    uint64_t newest_input;
} rv_vrx_fine_block;

typedef struct rv_vrx_demod_block {
    rv_vrx_demod_params params;
    uint64_t first_fine;
    uint64_t oldest_fine;
} rv_vrx_demod_block;

/* ===================================================================== *
 * Runtime: context, buffers, streams  (core/gpu/context.h, buffer.h)     *
 * ===================================================================== */

typedef struct rv_context rv_context;
typedef struct rv_buffer rv_buffer;

/* core/gpu/context.h:26-58 DeviceInfo. */
typedef struct rv_device_info {
    char name[256];
    int32_t device_index;
    int32_t sm_count;
    int32_t cc_major;
    int32_t cc_minor;
    uint64_t total_memory;
    uint64_t max_shared_per_block; /* opt-in bytes */
    uint64_t l2_bytes;
} rv_device_info;

/* Context::create (core/gpu/context.cpp:274). device_index < 0 reads
 * REVENANT_GPU_INDEX, else 0 (core/gpu/context.cpp:174). */
int32_t rv_context_create(int32_t device_index, rv_context** out);
int32_t rv_context_destroy(rv_context* context);
int32_t rv_context_device_info(const rv_context* context, rv_device_info* out);
/* The context's own stream (core/gpu Context::submit's queue). */
void* rv_context_stream(const rv_context* context);
int32_t rv_context_synchronize(rv_context* context);
/* A further (non-blocking) stream on the context's device, for work that
 * overlaps the context stream's. */
int32_t rv_stream_create(rv_context* context, void** out);
int32_t rv_stream_destroy(void* stream);
int32_t rv_stream_synchronize(void* stream);

/* core/gpu/buffer.h:33-39 MemoryKind. */
#define RV_MEMORY_DEVICE_LOCAL 0
#define RV_MEMORY_UPLOAD 1   /* pinned, host-written */
#define RV_MEMORY_READBACK 2 /* pinned, host-read */

int32_t rv_buffer_create(rv_context* context, uint64_t bytes, int32_t kind, rv_buffer** out);
int32_t rv_buffer_destroy(rv_buffer* buffer);
/* Device address (device-local) or host address (pinned kinds). */
void* rv_buffer_address(const rv_buffer* buffer);
uint64_t rv_buffer_size(const rv_buffer* buffer);
/* Synchronous copies on the context stream (core/gpu CommandRunner::copy). */
int32_t rv_buffer_upload(rv_buffer* buffer, uint64_t offset, const void* src, uint64_t bytes);
int32_t rv_buffer_download(const rv_buffer* buffer, uint64_t offset, void* dst, uint64_t bytes);
int32_t rv_buffer_clear(rv_buffer* buffer);
/* Synchronous copy between any two addresses (host or device) on the
 * context stream (core/gpu/kernel.h CommandRunner::copy). */
int32_t rv_copy(rv_context* context, void* dst, const void* src, uint64_t bytes);

/* ===================================================================== *
 * Plain kernels: one launch per reference dispatch, bit-identical to the  *
 * reference's CPU twins (fp32, no contraction, denormals flushed).        *
 * ===================================================================== */

/* core/shaders/convert_{cu8,cs8,cs16,cs24}_cf32.comp; twins
 * core/dsp/convert.cpp reference_convert_*. `packed_dev` is the staging
 * buffer as raw bytes (packed_bytes long, whole 32-bit words are read). */
#define RV_FORMAT_CU8 0
#define RV_FORMAT_CS8 1
#define RV_FORMAT_CS16 2
#define RV_FORMAT_CS24 3
int32_t rv_convert(void* stream, int32_t format, const rv_convert_params* params,
                   const void* packed_dev, uint64_t packed_bytes, rv_cf32* ring_dev,
                   uint64_t ring_len);

/* core/shaders/pfb_branch.comp; twin core/dsp/pfb_branch_reference.cpp:22. */
int32_t rv_pfb_branch(void* stream, const rv_grid_params* grid, const rv_pfb_branch_params* params,
                      const float* taps_dev, uint64_t taps_len, const rv_cf32* ring_dev,
                      uint64_t ring_len, rv_cf32* branch_dev, uint64_t branch_len);

/* core/shaders/pfb_fft.comp; twin core/dsp/pfb_fft_reference.cpp:152. */
int32_t rv_pfb_fft(void* stream, const rv_pfb_fft_params* params, const rv_cf32* branch_dev,
                   uint64_t branch_len, const rv_cf32* twiddles_dev, uint64_t twiddles_len,
                   rv_cf32* channel_ring_dev, uint64_t channel_ring_len);

/* core/shaders/spectrum.comp; twin core/dsp/spectrum_reference.cpp:286.
 * window holds N window taps then N/2 correction gains. */
int32_t rv_spectrum(void* stream, const rv_spectrum_params* params,
                    const rv_cf32* channel_ring_dev, uint64_t channel_ring_len,
                    const rv_cf32* twiddles_dev, uint64_t twiddles_len, const float* window_dev,
                    uint64_t window_len, float* frame_dev, uint64_t frame_len);

/* Front-end DC and IQ-imbalance correction (core/dsp/front_end_correction.h,
 * front_end_correction_reference.cpp; shaders iq_moments.comp, iq_correct.comp):
 * per 64-sample chunk the five sums (I, Q, I^2, Q^2, IQ) in float, in order;
 * the host totals them in double and updates the running estimate; the
 * correction i' = I - dc_i, q' = cross * i' + scale * (Q - dc_q) in place. */
#define RV_IQ_MOMENTS_CHUNK 64u
#define RV_IQ_MOMENTS_PER_CHUNK 5u
typedef struct rv_iq_moments_params { /* IqMomentsParams, 12 B */
    uint32_t ring_mask;
    uint32_t src_offset;
    uint32_t count;
} rv_iq_moments_params;
typedef struct rv_iq_correct_params { /* IqCorrectParams, 28 B */
    uint32_t ring_mask;
    uint32_t offset;
    uint32_t count;
    float dc_i;
    float dc_q;
    float cross;
    float scale;
} rv_iq_correct_params;
int32_t rv_iq_moments(void* stream, const rv_iq_moments_params* params, const rv_cf32* ring_dev,
                      uint64_t ring_len, float* sums_dev, uint64_t sums_len);
int32_t rv_iq_correct(void* stream, const rv_iq_correct_params* params, const rv_cf32* in_dev,
                      uint64_t in_len, rv_cf32* out_dev, uint64_t out_len);
/* FrontEndCorrector (core/dsp/front_end_correction.cpp) as a plain struct:
 * the configuration, the estimate and the running second moments. */
typedef struct rv_front_end {
    double dc_time_constant_s;    /* 0.1 */
    double iq_time_constant_s;    /* 1.0 */
    double max_gain_error_db;     /* 6 */
    double max_phase_error_deg;   /* 30 */
    uint32_t measured;
    uint32_t iq_plausible;
    uint64_t samples_seen;
    double dc_i, dc_q, gain, sin_phase;
    double m_ii, m_qq, m_iq;
} rv_front_end;
/* FrontEndCorrector() with the reference's defaults, then reset(). */
int32_t rv_front_end_init(rv_front_end* state);
int32_t rv_front_end_reset(rv_front_end* state);
/* total_moments over chunk sums of a `count`-sample block, then update(). */
int32_t rv_front_end_update(rv_front_end* state, const float* chunk_sums, uint64_t sums_len, uint32_t count,
                            int64_t rate);
/* correction(dc, iq): the parameters' dc/cross/scale fields (ring fields untouched). */
int32_t rv_front_end_correction(const rv_front_end* state, int32_t dc, int32_t iq, rv_iq_correct_params* out);

/* Averaged power spectrum, lw-radio-dsp's Spectrum::compute
 * (third_party/lw-radio-dsp/src/spectrum.cpp:32-44, src/fft.cpp:31-50): frames
 * of `size` samples, window, FFT, |X|^2 * norm (norm = 1/(sum w)^2), fftshift,
 * averaged, 10 log10(max(p, 1e-30)) dB. MEAN: one output spectrum per
 * `average` consecutive frames; EXPONENTIAL: avg = alpha*avg + (1-alpha)*p
 * over all frames, one output. avg_dev (optional, N floats per output)
 * receives the linear average; with `resume` it also seeds the exponential
 * average, as lwdsp keeps it between calls. Tolerance-level agreement with an
 * FP64 restatement (the reference transforms with pocketfft). */
#define RV_AVERAGE_MEAN 0
#define RV_AVERAGE_EXPONENTIAL 1
#define RV_WINDOW_RECTANGULAR 0
#define RV_WINDOW_HANN 1
#define RV_WINDOW_BLACKMAN_HARRIS 2
typedef struct rv_spectrum_average_params {
    uint32_t size;    /* N, a power of two in [16, 8192] */
    uint32_t frames;  /* consecutive N-sample frames in the input */
    uint32_t average; /* frames per output spectrum (MEAN) */
    uint32_t mode;    /* RV_AVERAGE_* */
    float alpha;      /* exponential weight (EXPONENTIAL), lwdsp's `averaging` */
    float norm;       /* 1 / (sum of the window)^2 */
    uint32_t resume;  /* EXPONENTIAL: 1 = continue from the average in avg_dev */
    uint32_t reserved;
} rv_spectrum_average_params;
int32_t rv_spectrum_average(void* stream, const rv_spectrum_average_params* params,
                            const rv_cf32* iq_dev, uint64_t iq_len, const float* window_dev,
                            uint64_t window_len, const rv_cf32* twiddles_dev, uint64_t twiddles_len,
                            float* out_dev, uint64_t out_len, float* avg_dev, uint64_t avg_len);
/* make_window (third_party/lw-radio-dsp/src/primitives.cpp:124): n floats of
 * the symmetric window; *norm = 1 / (sum of the floats, in double)^2. */
int32_t rv_build_lwdsp_window(uint32_t kind, uint32_t n, float* window, double* norm);

/* core/shaders/spectrum_levels.comp; twin
 * core/dsp/spectrum_levels_reference.cpp:75. levels_dev receives 2 floats. */
int32_t rv_spectrum_levels(void* stream, const rv_spectrum_levels_params* params,
                           const float* frame_dev, uint64_t frame_len, float* levels_dev);

/* core/shaders/vrx_fine.comp; twin core/dsp/vrx_reference.cpp:489. */
int32_t rv_vrx_fine(void* stream, const rv_vrx_fine_config* config,
                    const rv_vrx_fine_params* params, const rv_cf32* channel_ring_dev,
                    uint64_t channel_ring_len, const rv_cf32* taps_dev, uint64_t taps_len,
                    const rv_cf32* nco_dev, uint64_t nco_len, rv_cf32* fine_ring_dev,
                    uint64_t fine_ring_len);

/* core/shaders/vrx_demod.comp; twin core/dsp/vrx_reference.cpp:714. */
int32_t rv_vrx_demod(void* stream, const rv_vrx_demod_config* config,
                     const rv_vrx_demod_params* params, const rv_cf32* fine_ring_dev,
                     uint64_t fine_ring_len, const float* weights_dev, uint64_t weights_len,
                     float* audio_dev, uint64_t audio_len);

/* core/shaders/vrx_carrier.comp; twin core/dsp/vrx_reference.cpp:1083.
 * Rotates the fine ring in place and carries 8 state words. */
int32_t rv_vrx_carrier(void* stream, const rv_vrx_carrier_config* config,
                       const rv_vrx_carrier_params* params, const rv_cf32* nco_dev,
                       uint64_t nco_len, rv_cf32* fine_ring_dev, uint64_t fine_ring_len,
                       uint32_t* state_dev);

/* Branch filter then FFT (rv_pfb_branch + rv_pfb_fft, same outputs bit for
 * bit) with the branch values between them kept in a fixed array inside the
 * library, for callers that may not allocate device memory on their path:
 * per-block processing callbacks, where cudaMalloc can stall the device while
 * samples keep arriving, and plugins or hosts that work inside a device-memory
 * budget they do not own. No counterpart in the reference. The array holds
 * RV_NOALLOC_BRANCH_VALUES complex values (block_count * M at most), stays
 * allocated on every GPU that loads the library, and is shared by all calls on
 * a device: calls whose work overlaps on the GPU race on it. The first call on
 * a device looks the array's address up (cudaGetSymbolAddress) and should come
 * before any stream capture. Calls no cudaMalloc / cudaFree. */
#define RV_NOALLOC_BRANCH_VALUES (1u << 20)
int32_t rv_pfb_channelize_noalloc(void* stream, const rv_grid_params* grid,
                                  const rv_pfb_branch_params* branch_params,
                                  const rv_pfb_fft_params* fft_params, const float* taps_dev,
                                  uint64_t taps_len, const rv_cf32* ring_dev, uint64_t ring_len,
                                  const rv_cf32* twiddles_dev, uint64_t twiddles_len,
                                  rv_cf32* channel_ring_dev, uint64_t channel_ring_len);

/* ===================================================================== *
 * Fused kernels (same outputs as the plain chain, bit for bit)           *
 * ===================================================================== */

/* Parameters of the fused coarse chain: PfbBranchParams' ring view of the
 * raw input plus PfbFftParams' output view. */
typedef struct rv_coarse_params {
    uint32_t ring_mask;       /* raw ring capacity in samples, minus one */
    uint32_t base_offset;     /* ring position of x[mD] for block 0 */
    uint32_t block_count;
    uint32_t block_base;      /* absolute output block index of block 0 */
    uint32_t out_ring_blocks; /* channel ring blocks per channel, power of two */
    uint32_t out_ring_mask;
    /* Samples at the start of block 0's filter support (the M*T samples
     * ending at x[base_offset]) that precede the stream and read as 0.0, as
     * a freshly zeroed cf32 ring does in the plain path; at most M*T - 1,
     * zero once the stream has M*T - 1 samples of history. A native ring
     * cannot hold that zero itself: no cu8 code converts to 0.0. */
    uint32_t lead_zero;
} rv_coarse_params;

/* convert -> pfb_branch -> pfb_fft in one launch, reading the staging ring
 * in its native format (RV_FORMAT_CS16: one 32-bit word per sample;
 * RV_FORMAT_CU8: two samples per word) and writing the channel-major ring
 * [M][out_ring_blocks]. Output is bit-identical to rv_convert (whole ring,
 * dst_offset 0) followed by rv_pfb_branch and rv_pfb_fft with the same
 * offsets (core/engine/graph.cpp:5118-5199). Grids without a fused
 * instantiation return RV_ERR_UNSUPPORTED. */
int32_t rv_coarse_fused(void* stream, const rv_grid_params* grid, int32_t format,
                        const rv_coarse_params* params, const void* raw_ring_dev,
                        uint64_t raw_ring_bytes, const float* taps_dev, uint64_t taps_len,
                        const rv_cf32* twiddles_dev, uint64_t twiddles_len,
                        rv_cf32* channel_ring_dev, uint64_t channel_ring_len);

/* ===================================================================== *
 * The chain: raw IQ -> channel ring -> N receivers -> audio               *
 * (core/engine/graph.h Graph::on_block + core/engine/vrx_stage.cpp       *
 * DemodStage::record, with the same cursor arithmetic)                   *
 * ===================================================================== */

#define RV_CHAIN_BATCHED 0 /* fused coarse kernel + one launch per receiver stage */
#define RV_CHAIN_PLAIN 1   /* one launch per stage per receiver, as the reference records */
#define RV_CHAIN_FAST 2    /* batched, the fine stage on the tensor cores (split BF16 GEMMs, FP32
                            * accumulation), the DC-removal and mono audio FIRs with fused
                            * multiply-adds: to a stated tolerance, not bit for bit */
#define RV_CHAIN_HOISTED 3 /* the plain recording with the detector hoisted: one launch per stage per
                            * receiver (fine, carrier, detector, audio), the detector once per fine
                            * sample as the batched chain does; the same audio bit for bit (a
                            * comparison mode: it isolates what batching adds) */

typedef struct rv_chain rv_chain;

/* rv_chain_autotune's findings: receivers of the same rates, taps and
 * pattern period form a class; each class's fine-tile shapes that fit shared
 * memory were timed on one run of its own tiles and the fastest kept (the
 * rule's shape unless another was more than 3 % faster), within the shared
 * memory of the rule's largest shape (a launch's CTAs all reserve the
 * largest); the choices are kept only when every tiled receiver's run is
 * faster with them together; then the tile count per SM (2, 4 or 8). Times: the fine tiles of one run of every tiled
 * receiver, rule's shapes at 4 tiles per SM against the tuned ones. */
typedef struct rv_chain_tune_report {
    uint32_t receivers;        /* tiled receivers */
    uint32_t classes;          /* receiver classes tuned */
    uint32_t classes_changed;  /* classes whose shape differs from the rule's */
    uint32_t shapes_timed;
    uint32_t tiles_per_sm;     /* the chosen tile count per SM */
    uint32_t shapes_reverted;  /* 1: the classes' choices together were not faster; the rule's kept */
    double default_ms;
    double tuned_ms;
} rv_chain_tune_report;

typedef struct rv_chain_config {
    rv_grid_params grid;
    uint32_t reserved;
    int64_t rate;             /* input samples per second; a multiple of D */
    int32_t format;           /* RV_FORMAT_CS16 or RV_FORMAT_CU8 */
    int32_t mode;             /* RV_CHAIN_BATCHED or RV_CHAIN_PLAIN */
    uint32_t max_run_samples; /* largest count one rv_chain_run may carry */
    uint32_t keep_audio;      /* 1: accumulate audio for rv_chain_read_audio */
    double attenuation_db;    /* prototype stopband target, 0 = 120 dB */
    uint32_t profile;         /* 1: time each stage with CUDA events into rv_chain_stats
                               * (not with pipelined runs) */
    uint32_t pipelined;       /* batched only. 1: rv_chain_run returns once the run is queued;
                               * the next run is prepared, and its input copied on a second
                               * stream, while this one executes. A run's audio reaches
                               * rv_chain_read_audio when the run after next begins or at
                               * rv_chain_drain (read_audio, receiver_info and get_stats
                               * drain first). Host input must stay valid and unchanged
                               * until the next rv_chain_run or rv_chain_drain returns. */
} rv_chain_config;

typedef struct rv_chain_stats {
    uint64_t runs;
    uint64_t blocks;      /* channel blocks produced */
    uint64_t launches;    /* kernel launches issued */
    uint64_t work_items;  /* batched work items */
    uint64_t audio_bytes; /* bytes read back to the host */
    /* device time per stage, summed over runs, when profiling is on
     * (CUDA events on the chain's stream; core/engine/graph.h GraphStats) */
    double input_ms;      /* host/device copy of the run's samples */
    double coarse_ms;     /* convert + branch + FFT */
    double fine_ms;       /* fine stage (+ carrier) */
    double demod_ms;      /* detector + audio */
    double readback_ms;   /* audio to the host */
    uint64_t graph_launches; /* runs replayed from the captured graph */
    uint64_t graph_captures; /* times the graph was (re)captured */
    double graph_ms;      /* captured runs: work-list upload + the whole graph */
    double host_ms;       /* host time from a run's start until its launches are queued
                           * (cursor and work-list building, uploads and launch calls) */
} rv_chain_stats;

/* Allocates the chain's rings (the only allocating calls of the chain API
 * are create and add_receiver). */
int32_t rv_chain_create(rv_context* context, const rv_chain_config* config, rv_chain** out);
int32_t rv_chain_destroy(rv_chain* chain);
/* engine::place + dsp::plan_vrx, tables uploaded; the receiver starts at the
 * first channel block of the next run (DemodStage::anchor_to). */
int32_t rv_chain_add_receiver(rv_chain* chain, const rv_vrx_request* request, uint32_t* id);
/* Consumes `count` input samples in the chain's format. where = 0: host
 * memory, 1: device memory. Produces every channel block, fine sample and
 * audio frame whose inputs now exist; audio is read back before it returns. */
int32_t rv_chain_run(rv_chain* chain, const void* samples, uint64_t count, int32_t where);
int32_t rv_chain_receiver_info(const rv_chain* chain, uint32_t id, rv_vrx_plan_info* info,
                               uint64_t* audio_frames, uint64_t* first_audio);
/* Drains up to `capacity` floats of accumulated audio (frames x channels). */
int32_t rv_chain_read_audio(rv_chain* chain, uint32_t id, float* dst, uint64_t capacity,
                            uint64_t* written);
int32_t rv_chain_get_stats(const rv_chain* chain, rv_chain_stats* stats);
/* Batched chains only (RV_ERR_UNSUPPORTED for a plain one). From the next run
 * on, the coarse kernel and every batched receiver kernel run from one
 * captured CUDA graph: each run uploads its work lists and a small count
 * header (the kernels read their item counts and the coarse parameters from
 * it) and replays the graph with a single cudaGraphLaunch. The graph is
 * captured again only when a run's work lists outgrow its capacities or a
 * buffer it names moved (a receiver was added). Outputs are bit-identical to
 * the direct batched run. */
int32_t rv_chain_capture_graph(rv_chain* chain);
/* Times the batched chain's fine-tile shapes per receiver class on
 * `run_samples`-sample runs and keeps the fastest (outputs do not depend on
 * the shape). Call after the receivers are added and before the first run
 * (it writes their fine rings, then clears them); RV_ERR_UNSUPPORTED for a
 * plain, hoisted or fast chain. */
int32_t rv_chain_autotune(rv_chain* chain, uint32_t run_samples, rv_chain_tune_report* report);
/* The spectrum stage (Graph::on_block's spectrum dispatch, a6): with
 * `transform` N > 0, every run that completes N or more channel blocks
 * computes one frame of the last N blocks (M * N / 2 dB bins, the central half
 * of each channel's transform), covering source samples [first block * D -
 * the prototype's group delay, + N * D) (SpectrumFrame). An attached detector
 * (same context) consumes every frame on the device as it is made.
 * transform 0 turns the stage off. */
struct rv_detector;
int32_t rv_chain_set_spectrum(rv_chain* chain, uint32_t transform, struct rv_detector* detector);
/* The latest frame (drains first): its bins, start, count and sequence number. */
int32_t rv_chain_read_spectrum(rv_chain* chain, float* out, uint64_t capacity, uint64_t* bins, uint64_t* start,
                               uint64_t* count, uint64_t* sequence);
/* Graph::set_front_end_correction: from the next run on, each run's samples
 * get their moments measured and are corrected with the estimate built from
 * the runs `lag` or more before it (the engine's estimate lags by its frames
 * in flight; a pipelined chain needs lag >= 2). Switching on resets the
 * estimate. Off by default. */
int32_t rv_chain_set_front_end(rv_chain* chain, int32_t dc_removal, int32_t iq_correction, uint32_t lag);
/* The current estimate (Graph::front_end_correction); drains first. */
int32_t rv_chain_front_end_estimate(rv_chain* chain, rv_front_end* out);
/* Graph's span-wide impulse excision (EngineConfig::impulse_excision,
 * core/engine/graph.cpp:1461-1525): from the next run on, every run's samples
 * are excised in place after the front-end correction (rv_excise_block over
 * the run's ExcisionCursor plan, the stage designed by design_excision for
 * the chain's rate and max_width_seconds, threshold in dB: 15 is the
 * reference's default), and the channelizer reads only the samples the stage
 * has finished. In the batched mode the samples then pass through a cf32 ring
 * the fused channelizer reads. Off by default; switching on restarts the
 * stage. Drains first. */
int32_t rv_chain_set_impulse_excision(rv_chain* chain, int32_t on, double threshold_db, double max_width_seconds);
/* Samples excised, runs excised, runs spared and samples examined since the
 * chain was created (drains first). */
int32_t rv_chain_excision_counters(rv_chain* chain, uint64_t* out4);
/* Waits for all of the chain's device work (a run returns with its audio
 * read back already; this is the engine's drain at stop). */
int32_t rv_chain_drain(rv_chain* chain);
/* A receiver's device rings: fine samples (cf32) and detector values (f32),
 * both indexed by fine sample index modulo (mask + 1). Detector values exist
 * only in the batched mode. */
int32_t rv_chain_receiver_rings(const rv_chain* chain, uint32_t id, const rv_cf32** fine,
                                const float** detector, uint32_t* mask);
/* The device channel ring [M][ring_blocks] (block m at slot m mod ring_blocks). */
int32_t rv_chain_channel_ring(const rv_chain* chain, const rv_cf32** ring, uint32_t* ring_blocks);

/* ===================================================================== *
 * Span-wide impulse excision (core/dsp/impulse_excision.h,
 * impulse_excision_reference.cpp; core/shaders/impulse_excise.comp): on the
 * cf32 sample ring, after the front-end correction and before the
 * channelizer. Segment powers, their running median, per-sample flags, and
 * the apply pass that zeroes (to -0) every run of marked samples no longer
 * than max_width and writes what it removed beside it, so cleaned + removed
 * == raw bit for bit.
 * ===================================================================== */
enum {
    RV_EXCISE_SEGMENT = 0,
    RV_EXCISE_REFERENCE = 1,
    RV_EXCISE_FLAG = 2,
    RV_EXCISE_APPLY = 3,
    RV_EXCISE_MAX_SEGMENTS = 64,
    RV_EXCISE_MAX_WIDTH = 4096,
    RV_EXCISE_MAX_SEG_LOG2 = 12,
    RV_EXCISE_MAX_GUARD = 16,
    RV_EXCISE_COUNTER_SAMPLES = 0, /* counters[4]: samples excised, */
    RV_EXCISE_COUNTER_EVENTS = 1,  /* runs excised, */
    RV_EXCISE_COUNTER_SPARED = 2,  /* runs left alone as too long */
    RV_EXCISE_COUNTERS = 4
};

/* ExcisionConfig (impulse_excision.h:150-160): the kernel's specialisation
 * constants. `pass` is set by each entry point. */
typedef struct rv_excision_config {
    uint32_t pass;
    uint32_t seg_log2;  /* segment of 2^seg_log2 samples */
    uint32_t segments;  /* K, the median's window */
    uint32_t max_width; /* longest run excised */
    uint32_t hang;
    uint32_t lead;
} rv_excision_config;

/* ExcisionParams (impulse_excision.h:176-187): eight packed words. */
typedef struct rv_excision_params {
    uint32_t ring_mask;
    uint32_t first;     /* ring slot of the first sample (segment passes: of the first segment) */
    uint32_t count;     /* samples (segment passes: segments) */
    uint32_t seg_mask;
    uint32_t flag_mask;
    uint32_t removed_mask;
    int32_t history;    /* samples of the current run before `first` */
    float threshold;    /* power ratio */
} rv_excision_params;

typedef struct rv_excision_rings {
    uint32_t seg_mask;
    uint32_t flag_mask;
    uint32_t removed_mask;
} rv_excision_rings;

/* ExcisionPlan: one block's four passes (count 0: nothing to do). */
typedef struct rv_excision_plan {
    rv_excision_params segment;
    rv_excision_params reference;
    rv_excision_params flag;
    rv_excision_params apply;
    uint64_t cleaned_end; /* one past the last sample finished: the channelizer reads below it */
    uint32_t restarted;
    uint32_t reserved;
} rv_excision_plan;

/* ExcisionCursor (impulse_excision.h:232-270), as plain state. */
typedef struct rv_excision_cursor {
    rv_excision_config config;
    uint32_t ring_mask;
    rv_excision_rings rings;
    float threshold;
    uint32_t running;
    uint32_t reserved;
    uint64_t valid_from;
    uint64_t next_in;
    uint64_t seg_next;
    uint64_t flag_next;
    uint64_t apply_next;
} rv_excision_cursor;

/* design_excision / excision_threshold / size_excision_rings (host). */
int32_t rv_design_excision(int64_t source_rate, double max_width_seconds, rv_excision_config* out);
float rv_excision_threshold(double threshold_db);
int32_t rv_size_excision_rings(const rv_excision_config* config, uint64_t max_block, uint32_t frames_in_flight,
                               uint32_t ring_mask, rv_excision_rings* out);
/* ExcisionCursor: construct (running = 0), reset (set running = 0), plan. */
int32_t rv_excision_cursor_init(rv_excision_cursor* cursor, const rv_excision_config* config, uint32_t ring_mask,
                                const rv_excision_rings* rings, float threshold);
int32_t rv_excision_plan_block(rv_excision_cursor* cursor, uint64_t start, uint32_t count, rv_excision_plan* out);

/* The four passes on the device (one launch each, validated as the twins
 * validate; the lengths are the buffers' element counts). `raw` and
 * `cleaned` may be the same ring. */
int32_t rv_excise_segment(void* stream, const rv_excision_config* config, const rv_excision_params* params,
                          const rv_cf32* raw_dev, uint64_t raw_len, float* seg_power_dev, uint64_t seg_len);
int32_t rv_excise_reference(void* stream, const rv_excision_config* config, const rv_excision_params* params,
                            const float* seg_power_dev, float* seg_level_dev, uint64_t seg_len);
int32_t rv_excise_flag(void* stream, const rv_excision_config* config, const rv_excision_params* params,
                       const rv_cf32* raw_dev, uint64_t raw_len, const float* seg_level_dev, uint64_t seg_len,
                       uint32_t* flags_dev, uint64_t flags_len);
int32_t rv_excise_apply(void* stream, const rv_excision_config* config, const rv_excision_params* params,
                        const rv_cf32* raw_dev, uint64_t raw_len, const uint32_t* flags_dev, uint64_t flags_len,
                        rv_cf32* cleaned_dev, rv_cf32* removed_dev, uint64_t removed_len, uint32_t* counters_dev);
/* Graph::record_impulse_excision: a plan's passes in order on one ring, in place. */
int32_t rv_excise_block(void* stream, const rv_excision_config* config, const rv_excision_plan* plan,
                        rv_cf32* ring_dev, uint64_t ring_len, float* seg_power_dev, float* seg_level_dev,
                        uint64_t seg_len, uint32_t* flags_dev, uint64_t flags_len, rv_cf32* removed_dev,
                        uint64_t removed_len, uint32_t* counters_dev);

/* ===================================================================== *
 * Comb / spur cancellation on the sample ring (core/dsp/comb_cancel.h,
 * comb_kernels_reference.cpp; core/shaders/comb_project.comp,
 * comb_subtract.comp): the projection of each tracked line onto the block in
 * sub-blocks, and the subtraction of the lines' sum with the removed part
 * written beside it. The tracker that turns projections into amplitudes is
 * host bookkeeping of the reference's (CombTracker) and not part of this.
 * ===================================================================== */
enum { RV_COMB_TABLE_LOG2 = 12, RV_COMB_TABLE_SIZE = 4096, RV_COMB_MAX_LINES = 1024, RV_COMB_MAX_SUB_BLOCKS = 16 };

/* CombLine (comb_cancel.h:248-256): tone_l(n) = table[(phase0 + n step) >> 20]. */
typedef struct rv_comb_line {
    uint32_t phase0;
    uint32_t step;
    uint32_t pad0;
    uint32_t pad1;
    rv_cf32 amplitude;  /* what subtract removes; project ignores it */
} rv_comb_line;

/* CombParams (comb_cancel.h:276-288): eight packed words. */
typedef struct rv_comb_params {
    uint32_t ring_mask;
    uint32_t first;
    uint32_t count;
    uint32_t lines;
    uint32_t sub_blocks;
    uint32_t removed_mask;
    uint32_t pad0;
    uint32_t pad1;
} rv_comb_params;

/* comb_step / comb_table (comb_kernels_reference.cpp). */
uint32_t rv_comb_step(double frequency_hz, int64_t rate);
int32_t rv_comb_table(rv_cf32* table, uint64_t len);
/* projections[l * sub_blocks + s] = sum over sub-block s of x(n) conj(tone_l(n)),
 * in 64-sample chunks added in order. */
int32_t rv_comb_project(void* stream, const rv_comb_params* params, const rv_cf32* raw_dev, uint64_t raw_len,
                        const rv_comb_line* lines_dev, uint64_t lines_len, const rv_cf32* table_dev, uint64_t table_len,
                        rv_cf32* projections_dev, uint64_t projections_len);
/* cleaned = x - sum_l a_l tone_l(n); removed = the sum (raw and cleaned may be one ring). */
int32_t rv_comb_subtract(void* stream, const rv_comb_params* params, const rv_cf32* raw_dev, uint64_t raw_len,
                         const rv_comb_line* lines_dev, uint64_t lines_len, const rv_cf32* table_dev, uint64_t table_len,
                         rv_cf32* cleaned_dev, uint64_t cleaned_len, rv_cf32* removed_dev, uint64_t removed_len);

/* ===================================================================== *
 * Per-receiver noise stages (core/dsp/noise_reference.h,
 * noise_reference.cpp; core/shaders/noise_blank.comp, noise_line.comp,
 * noise_spectral.comp): the impulse blanker on a receiver's coarse channel,
 * the line kernel (manual notch cascade and adaptive line enhancer) and the
 * spectral noise reduction on its mono audio. Same parameter blocks, same
 * state layouts, same bits as the twins.
 * ===================================================================== */
enum {
    RV_BLANK_DETECT = 0,
    RV_BLANK_APPLY = 1,
    RV_BLANK_MIN_WINDOW = 16,
    RV_BLANK_MAX_WINDOW = 256,
    RV_LINE_NOTCH = 1,
    RV_LINE_ALE = 2,
    RV_LINE_GUARD = 4,
    RV_LINE_MAX_NOTCHES = 4,
    RV_LINE_MAX_STRIDE = 8,
    RV_LINE_NOTCH_COUNT_SHIFT = 8,    /* bits [8, 10): sections after the first */
    RV_LINE_STATE_POSITION = 4,
    RV_LINE_STATE_GUARD = 8,
    RV_LINE_STATE_MORE = 12,
    RV_LINE_STATE_WEIGHTS = 24,
    RV_SPECTRAL_MIN_FRAME = 64,
    RV_SPECTRAL_MAX_FRAME = 512
};

/* BlankerConfig / BlankerParams (noise_reference.h:117-168). */
typedef struct rv_blanker_config {
    uint32_t pass;  /* set by each entry point */
    uint32_t window;
    uint32_t guard;
    uint32_t hang;
    uint32_t lead;
} rv_blanker_config;

typedef struct rv_blanker_params {
    uint32_t chan_base;  /* the channel's first slot in the channel-major ring */
    uint32_t chan_mask;
    uint32_t chan_first;
    uint32_t out_mask;   /* flag and blanked rings */
    uint32_t out_first;
    uint32_t count;
    float threshold;
} rv_blanker_params;

/* LineConfig / LineSection / LineParams (noise_reference.h:277-385). */
typedef struct rv_line_config {
    uint32_t lanes;
    uint32_t taps;
    uint32_t history;  /* power of two */
} rv_line_config;

typedef struct rv_line_section {
    float b0, b1, b2, a1, a2;
} rv_line_section;

typedef struct rv_line_params {
    uint32_t count;
    uint32_t flags;   /* RV_LINE_* and the section count */
    uint32_t stride;
    uint32_t delay;
    float b0, b1, b2, a1, a2;
    float mu, leak, eps;
    float gb0, gb1, gb2, ga1, ga2;
    rv_line_section more[3];
} rv_line_params;

/* NotchDesign (noise_reference.h:395-401), before rounding to float. */
typedef struct rv_notch_design {
    double b0, b1, b2, a1, a2;
} rv_notch_design;

/* SpectralConfig / SpectralParams (noise_reference.h:483-524). */
typedef struct rv_spectral_config {
    uint32_t frame;  /* N, a power of two in [64, 512]; hop N/2 */
} rv_spectral_config;

typedef struct rv_spectral_params {
    uint32_t count;
    float smoothing, smoothing_complement;
    float gamma, beta, rise;
    float bias, alpha, floor_gain, eps;
} rv_spectral_params;

/* design_blanker / blanker_threshold (noise_reference.cpp:112-125). */
int32_t rv_design_blanker(int64_t channel_rate, rv_blanker_config* out);
float rv_blanker_threshold(double threshold_db);
/* The blanker's two passes (noise_blank.comp): flags (floats 0/1) into
 * out_mask + 1 slots, then the blanked samples. chan_len counts the whole
 * channel-major ring (chan_base + chan_mask + 1 at least). */
int32_t rv_blank_detect(void* stream, const rv_blanker_config* config, const rv_blanker_params* params,
                        const rv_cf32* channel_ring_dev, uint64_t channel_len, float* flags_dev, uint64_t flags_len);
int32_t rv_blank_apply(void* stream, const rv_blanker_config* config, const rv_blanker_params* params,
                       const rv_cf32* channel_ring_dev, uint64_t channel_len, const float* flags_dev,
                       uint64_t flags_len, rv_cf32* blanked_dev, uint64_t blanked_len);

/* design_notch (noise_reference.cpp:424-459). */
int32_t rv_design_notch(double audio_hz, double depth_db, double width_hz, int64_t audio_rate, rv_notch_design* out);
/* line_state_size: floats of the line kernel's state. */
uint64_t rv_line_state_size(const rv_line_config* config);
/* The line kernel (noise_line.comp): `count` audio samples in place, the
 * state (line_state_size floats) read and written. */
int32_t rv_noise_line(void* stream, const rv_line_config* config, const rv_line_params* params, float* audio_dev,
                      uint64_t audio_len, float* state_dev, uint64_t state_len);

/* spectral_config_for / design_spectral_tables (4 N floats) / spectral_params
 * (noise_reference.cpp:493-554; spectral_params as rv_design_spectral_params)
 * and the state size. */
int32_t rv_spectral_config_for(int64_t audio_rate, rv_spectral_config* out);
int32_t rv_design_spectral_tables(const rv_spectral_config* config, float* tables, uint64_t len);
int32_t rv_design_spectral_params(double strength, rv_spectral_params* out);
uint64_t rv_spectral_state_size(const rv_spectral_config* config);
/* The spectral noise reduction (noise_spectral.comp): in place, one frame
 * of latency, the state read and written. */
int32_t rv_noise_spectral(void* stream, const rv_spectral_config* config, const rv_spectral_params* params,
                          const float* tables_dev, uint64_t tables_len, float* audio_dev, uint64_t audio_len,
                          float* state_dev, uint64_t state_len);

/* ===================================================================== *
 * Wideband detector (core/detect/detector.h:1316-1460, detector.cpp:186-1586):
 * the exponential average of the spectrum frames, and at every decision the
 * noise floor, the summed-bin width ladder and the candidate bands, then the
 * residual rejection. The per-bin average, the noise-floor percentiles and
 * interpolation, the prefix sums and the ladder's deflections and peaks run
 * on the GPU; the greedy band growth, candidate emission and track
 * association run on the host. Each live track's band power is measured on
 * the GPU for every frame (Detector::measure_levels) and folded into the
 * track at the next decision or tracks() call.
 * ===================================================================== */
typedef struct rv_detector_config {
    int64_t source_rate;          /* source samples per second */
    int64_t source_center;        /* Hz */
    uint32_t bins;                /* SpectrumGeometry::bins */
    uint32_t noise_knots;         /* DetectorConfig defaults in brackets: 32 */
    int64_t bin_width_numerator;  /* SpectrumGeometry's exact bin width and bin-0 frequency */
    int64_t bin_width_denominator;
    int64_t bin_zero_numerator;
    int64_t bin_zero_denominator;
    double detection_threshold_db;    /* 6 */
    double average_seconds;           /* 1 */
    double decision_interval_seconds; /* 0.1 */
    uint32_t noise_window_knots;      /* 8 */
    uint32_t max_sum_bins;            /* 0: bit_floor(bins / 8) */
    double noise_percentile;          /* 0.10 */
    double noise_percentile_high;     /* 0.40 */
    double noise_excision_sigma;      /* 4 */
    uint32_t max_peaks;               /* 0: bins */
    uint32_t split_gap_bins;          /* 8 */
    double edge_floor_fraction;       /* 0 */
    double edge_floor_sigma;          /* 3 */
    double occupied_power_fraction;   /* 0.99 */
    double split_gap_db;              /* 1 */
    double residual_rate_tolerance;   /* 0.25 */
    uint32_t residual_decisions;      /* 4 */
    /* tracking (Detector::update_tracks, core/detect/detector.h:900-1206) */
    uint32_t birth_hits;              /* 3: consecutive decisions before a track is born */
    uint32_t max_tracks;              /* 512 */
    uint32_t grid_channels;           /* 0: tracks carry no coarse channel */
    double association_overlap;       /* 0.3 */
    double confidence_rise;           /* 0.35 */
    double confidence_half_life_seconds; /* 1 */
    double drop_confidence;           /* 0.05 */
    double centre_smoothing;          /* 0.4 */
    double channel_hysteresis;        /* 0.15 */
    double bootstrap_hold_seconds;    /* 3 */
} rv_detector_config;

/* TrackState (core/detect/detector.h:271). */
enum { RV_TRACK_PENDING = 0, RV_TRACK_LIVE = 1, RV_TRACK_HELD = 2, RV_TRACK_MERGED = 3 };

/* Track (core/detect/detector.h:361-577): the fields the tracker maintains
 * from candidates and frames. Classification, probes, refinement, emitter
 * memory, spur and HD-hybrid marks come from probing and are not carried. */
typedef struct rv_detector_track {
    uint64_t id;                  /* issued from 1, never reused */
    uint32_t state;               /* RV_TRACK_* */
    uint32_t held_spells;
    int64_t center;               /* Hz, smoothed */
    int64_t bandwidth;            /* Hz, smoothed, >= 1 */
    double snr_2500_db;           /* smoothed */
    double margin_confidence;     /* of the smoothed snr */
    double confidence;
    uint64_t first_seen;          /* decision instants (source sample indices) */
    uint64_t last_seen;
    uint64_t last_detected;
    uint32_t hits;
    uint32_t misses;
    int64_t channel_index;        /* nearest coarse channel, with hysteresis */
    uint32_t channel;             /* channel_index reduced into [0, grid_channels) */
    uint32_t channel_valid;
    uint64_t merged_into;         /* parent id while merged */
    uint32_t level_first_bin;     /* the bins of its latest candidate */
    uint32_t level_last_bin;
    uint32_t level_bins_known;
    uint32_t level_frames;        /* frames measured over those bins while live */
    double level_mean_db;         /* running mean and sum of squared deviations */
    double level_m2;              /* of the band power, dB (Welford) */
    double peak_to_mean;          /* BandShape of its latest candidate */
    double concentration;
    double lower_fraction;
    double skirt_fraction;
    uint64_t skirt_bins_available;
    uint32_t shape_measured;
    uint32_t reserved;
} rv_detector_track;

/* Candidate + BandShape (core/detect/detector.h:299-359, shape.h:53-75). */
typedef struct rv_detector_candidate {
    int64_t center;               /* Hz */
    int64_t bandwidth;            /* Hz */
    double snr_2500_db;
    double margin_confidence;
    double noise_floor_dbfs;
    double peak_dbfs;
    uint32_t first_bin;
    uint32_t last_bin;
    double peak_to_mean;
    double concentration;
    double lower_fraction;
    double skirt_fraction;
    uint64_t skirt_bins_available;
    uint32_t measured;
    uint32_t reserved;
} rv_detector_candidate;

typedef struct rv_detector_stats {
    uint64_t frames;
    uint64_t decisions;
    uint64_t frames_rejected;
    uint64_t candidates;             /* summed over decisions, after residual rejection */
    uint64_t peaks_overflowed;
    uint64_t candidates_residual;
    uint64_t residual_parts_degenerate;
    double device_ms;                /* stream time of the decisions (CUDA events around each
                                      * decision's kernels, read-back and host part) */
    double host_ms;                  /* host part of the decisions */
    uint64_t tracks_born;
    uint64_t tracks_dropped;
    uint64_t births_refused;
    uint64_t merges;
    uint64_t splits;
} rv_detector_stats;

typedef struct rv_detector rv_detector;
/* Detector::create: the same validation and derived constants. */
int32_t rv_detector_create(rv_context* context, const rv_detector_config* config, rv_detector** out);
int32_t rv_detector_destroy(rv_detector* detector);
/* Detector::consume of one frame of `bins` dB values (where = 0: host memory,
 * 1: device memory) covering source samples [start, start + count); *decided
 * is 1 when the frame completed a decision. */
int32_t rv_detector_consume(rv_detector* detector, const float* power_db, uint64_t start, uint64_t count,
                            int32_t where, int32_t* decided);
/* `frames` consecutive frames at power_db + f * bins, frame f covering
 * [start + f * hop, start + f * hop + count): consume() for each, with the
 * averaging of all the frames up to each decision in one launch. Returns the
 * number of decisions in *decisions; candidates() then holds the last one's. */
int32_t rv_detector_consume_frames(rv_detector* detector, const float* power_db, uint32_t frames, uint64_t start,
                                   uint64_t hop, uint64_t count, int32_t where, uint32_t* decisions);
/* Detector::candidates after the latest decision. */
int32_t rv_detector_candidates(const rv_detector* detector, rv_detector_candidate* out, uint32_t capacity,
                               uint32_t* count);
/* Detector::averaged_power / noise_floor (bins doubles each; either may be NULL). */
int32_t rv_detector_state(rv_detector* detector, double* average, double* floor, uint64_t bins);
int32_t rv_detector_get_stats(const rv_detector* detector, rv_detector_stats* stats);
/* Detector::tracks (all = 0: every track but the pending ones, ascending in
 * centre then id) or every track including pending ones (all = 1). Waits for
 * the frames in flight, whose band powers the tracks' levels include. */
int32_t rv_detector_tracks(rv_detector* detector, int32_t all, rv_detector_track* out, uint32_t capacity,
                           uint32_t* count);

/* The tracker alone, on the host (Detector::update_tracks over candidates
 * the caller supplies, and measure_levels over band powers it supplies):
 * the same state machine rv_detector runs after each decision. */
typedef struct rv_tracker rv_tracker;
int32_t rv_tracker_create(const rv_detector_config* config, rv_tracker** out);
int32_t rv_tracker_destroy(rv_tracker* tracker);
/* One decision at source sample `now`, `elapsed_seconds` after the previous
 * one, with that decision's candidates (ascending, as rv_detector hands them). */
int32_t rv_tracker_update(rv_tracker* tracker, uint64_t now, double elapsed_seconds,
                          const rv_detector_candidate* candidates, uint32_t count);
/* The bins whose power each frame contributes to a track's level: pairs
 * (first, last) of the live tracks with known bins below `bins`, in track
 * order; *count pairs. */
int32_t rv_tracker_level_bins(const rv_tracker* tracker, uint32_t bins, uint32_t* first_last, uint32_t capacity,
                              uint32_t* count);
/* Folds `frames` frames of band powers: sums[f * tracks + k] is the linear
 * power summed over pair k's bins in frame f, for the pairs level_bins gave
 * for the same `bins` (tracks = its count). */
int32_t rv_tracker_fold_levels(rv_tracker* tracker, uint32_t bins, const double* sums, uint32_t frames,
                               uint32_t tracks);
int32_t rv_tracker_tracks(const rv_tracker* tracker, int32_t all, rv_detector_track* out, uint32_t capacity,
                          uint32_t* count);
int32_t rv_tracker_get_stats(const rv_tracker* tracker, rv_detector_stats* stats);

/* ===================================================================== *
 * Host planning (core/dsp/pfb_design.cpp, vrx_reference.cpp,             *
 * core/engine/vrx_place.cpp), restated; results equal the reference's.   *
 * ===================================================================== */

int32_t rv_validate_grid(const rv_grid_params* grid);
/* design_prototype (core/dsp/pfb_design.cpp:381). taps_len = M*(L+1). */
int32_t rv_design_prototype(const rv_grid_params* grid, double attenuation_db, float* taps,
                            uint64_t taps_len, double* stopband_db, uint64_t* group_delay);
/* Grids past the reference's channel cap (kMaxChannels = 2048,
 * core/dsp/pfb_design.cpp:67), up to 16384 channels: C4's M = 4096 PFB.
 * design_prototype and the branch dispatch with the same arithmetic; the
 * FFT dispatch is rv_pfb_fft (up to 16384 channels) with rv_build_fft_twiddles. */
int32_t rv_design_prototype_wide(const rv_grid_params* grid, double attenuation_db, float* taps,
                                 uint64_t taps_len, double* stopband_db, uint64_t* group_delay);
/* C4's split-precision DFT on the tensor cores (tcgen05): rv_pfb_fft's
 * outputs for M = 4096 (the channel ring, phase correction included),
 * computed as two 64-point DFT GEMM stages with hi + lo split operands in
 * FP16 or BF16 and FP32 accumulators. Accurate to a stated tolerance against
 * FP64, not bit-identical to rv_pfb_fft. Asynchronous on `stream` (it can be
 * captured in a graph): a CTA whose bounded wait on the tensor cores or a
 * bulk copy runs out stops, waits (bounded) for what it has in flight and
 * counts itself on the device; rv_pfb_dft_tc_status reads and clears that
 * count (synchronising `stream`) and returns RV_ERR_TIMEOUT when it is not
 * zero. rv_pfb_dft_tc_stop_for_test makes every later call stop each CTA
 * before it issues a copy or an MMA (a test of the stop path); 0 clears it. */
#define RV_DFT_FP16 0
#define RV_DFT_BF16 1
int32_t rv_pfb_dft_tc(void* stream, const rv_pfb_fft_params* params, const rv_cf32* branch_dev, uint64_t branch_len,
                      const rv_cf32* twiddles_dev, uint64_t twiddles_len, rv_cf32* ring_dev, uint64_t ring_len,
                      int32_t precision);
int32_t rv_pfb_dft_tc_status(void* stream, uint32_t* timeouts);
int32_t rv_pfb_dft_tc_stop_for_test(void* stream, int32_t stop);
int32_t rv_pfb_branch_wide(void* stream, const rv_grid_params* grid, const rv_pfb_branch_params* params,
                           const float* taps_dev, uint64_t taps_len, const rv_cf32* ring_dev,
                           uint64_t ring_len, rv_cf32* out_dev, uint64_t out_len);
/* build_twiddles (core/dsp/pfb_design.cpp:515); M entries. */
int32_t rv_build_twiddles(uint32_t channels, rv_cf32* table, uint64_t table_len);
/* build_twiddles' first-octant construction for any power of two up to 65536
 * (the reference caps its channel grid at 2048; the averaged spectrum and
 * wider transforms use this). Equal to rv_build_twiddles where both apply. */
int32_t rv_build_fft_twiddles(uint32_t n, rv_cf32* table, uint64_t len);
/* build_nco_table (core/dsp/vrx_reference.cpp:364); 2^log2 entries. */
int32_t rv_build_nco_table(uint32_t log2_size, rv_cf32* table, uint64_t table_len);
/* build_spectrum_window (core/dsp/spectrum_reference.cpp:195); 3N/2 floats. */
int32_t rv_build_spectrum_window(uint32_t transform, uint32_t taps_per_branch,
                                 double attenuation_db, float* window, uint64_t window_len);
/* engine::place (core/engine/vrx_place.cpp:199). */
int32_t rv_place(const rv_grid_params* grid, int64_t rate, const rv_vrx_request* request,
                 rv_vrx_placement* placement);
/* engine::channel_count_for (core/engine/vrx_place.cpp:187). */
uint32_t rv_channel_count_for(int64_t rate, int64_t widest_receiver_hz);
/* dsp::plan_vrx (core/dsp/vrx_reference.cpp:2568). Fills `info`; when the
 * table pointers are non-NULL also writes the fine tap table
 * (info->fine_tap_count entries) and demod weights (info->demod_weight_count).
 * Call once with NULL tables to learn the sizes. */
int32_t rv_plan_vrx(const rv_grid_params* grid, int64_t rate, const rv_vrx_request* request,
                    const rv_vrx_placement* placement, rv_vrx_plan_info* info,
                    rv_cf32* fine_taps, uint64_t fine_taps_len, float* demod_weights,
                    uint64_t demod_weights_len);
/* dsp::fine_block / demod_block / carrier_block (vrx_reference.cpp:2830+). */
int32_t rv_fine_block(const rv_vrx_plan_info* plan, uint32_t channel_base, uint32_t channel_mask,
                      uint32_t fine_mask, uint64_t first_output, uint32_t count,
                      rv_vrx_fine_block* block);
int32_t rv_demod_block(const rv_vrx_plan_info* plan, uint32_t fine_mask, uint64_t first_audio,
                       uint32_t count, rv_vrx_demod_block* block);
int32_t rv_carrier_block(const rv_vrx_plan_info* plan, uint32_t fine_mask, uint64_t first_fine,
                         uint32_t count, int32_t reset, float shift,
                         rv_vrx_carrier_params* params);
/* The display tap (core/dsp/vrx_reference.h:1639-1766): the fine stage
 * again, one polyphase branch of RV_DISPLAY_TAPS taps and an integer
 * decimation R from the channel rate's ladder, reading the same channel with
 * the receiver's own mix, so a passband pane shows the channel before any
 * receiver filter. Its launches are rv_vrx_fine with `fine` below. */
enum { RV_DISPLAY_TAPS = 256 };
typedef struct rv_vrx_display_plan {
    int64_t channel_rate;
    int64_t display_rate;
    uint32_t decimation;
    uint32_t reserved;
    int64_t reach_hz;
    rv_vrx_fine_config fine;  /* taps 256, phases 1, the receiver's nco_log2 */
    uint32_t reserved2;
    uint64_t nco_delta;       /* the fine stage's mix at the display rate */
    double pass_hz;
    double stop_hz;
    double attenuation_db;
    double group_delay_channel_samples;
    uint64_t tap_count;       /* taps + 1 */
} rv_vrx_display_plan;

uint32_t rv_display_max_decimation(void);
/* display_ladder: the rungs R may take, ascending from 1 (*count of them). */
int32_t rv_display_ladder(int64_t channel_rate, uint32_t* rungs, uint32_t capacity, uint32_t* count);
uint32_t rv_display_decimation(int64_t channel_rate, int64_t reach_hz);
/* plan_vrx_display for a receiver's plan; writes the tap table when `taps`
 * is not NULL (tap_count entries). */
int32_t rv_plan_vrx_display(const rv_vrx_plan_info* plan, rv_vrx_display_plan* out, rv_cf32* taps, uint64_t taps_len);
/* display_block: rv_vrx_fine parameters for display outputs
 * [first_output, first_output + count). */
int32_t rv_display_block(const rv_vrx_display_plan* plan, uint32_t channel_base, uint32_t channel_mask,
                         uint32_t display_mask, uint64_t first_output, uint32_t count, rv_vrx_fine_block* block);

/* dsp::demod_fine_history (core/dsp/vrx_reference.h). */
uint32_t rv_demod_fine_history(const rv_vrx_demod_config* config);

/* ===================================================================== *
 * Scene noise (core/dsp/synth/wideband.cpp siggen::Scene::fill_noise):   *
 * the synthesiser's Gaussian noise field, 4096-sample blocks each drawn  *
 * from its own MT19937-64 seeded from (seed ^ block), two draws per      *
 * sample, Box-Muller in FP64. The draws equal the reference's bit for    *
 * bit; a sample can differ from the reference's in its last FP32 bit     *
 * (CUDA's FP64 log/sin/cos against the C library's).                   *
 * ===================================================================== */

/* The per-component sigma of a noise floor of `dbfs` over the full band
 * (wideband.cpp:108-111, :200-203). */
double rv_scene_noise_sigma(double noise_power_full_band_dbfs);
/* Samples [start, start + count) of the noise field into out_dev (cf32). */
int32_t rv_scene_noise(void* stream, uint64_t seed, double sigma, uint64_t start, uint64_t count, rv_cf32* out_dev,
                       uint64_t out_len);
/* The raw draws of the same samples, two per sample (draws_len >= 2 count),
 * for pinning the generator. */
int32_t rv_scene_noise_draws(void* stream, uint64_t seed, uint64_t start, uint64_t count, uint64_t* draws_dev,
                             uint64_t draws_len);

/* A tone-modulated emitter of the scene synthesiser (siggen::ModulatorSpec
 * with no supplied audio; core/dsp/synth/modulators.h). */
#define RV_EMITTER_CW 0  /* siggen::Modulation::Cw: the text keyed in Morse */
#define RV_EMITTER_AM 1  /* siggen::Modulation::Am */
#define RV_EMITTER_NFM 2 /* siggen::Modulation::Nfm */
#define RV_EMITTER_USB 3 /* siggen::Modulation::Usb: tone(s) as one exact rotation each */
#define RV_EMITTER_LSB 4 /* siggen::Modulation::Lsb */
#define RV_EMITTER_FSK2 5 /* siggen::Modulation::Fsk2: continuous-phase binary FSK of random bits */
#define RV_EMITTER_BPSK 6 /* siggen::Modulation::Bpsk: root-raised-cosine pulses of random bits */
#define RV_EMITTER_QPSK 7 /* siggen::Modulation::Qpsk: two bits a symbol, Gray mapped */
typedef struct rv_tone_emitter {
    int32_t modulation;      /* RV_EMITTER_CW, _AM, _NFM, _USB, _LSB, _FSK2, _BPSK or _QPSK */
    int32_t reserved;
    int64_t rate;            /* samples per second */
    int64_t carrier_offset;  /* Hz from DC */
    int64_t tone_hz;         /* the modulating tone */
    int64_t deviation;       /* NFM peak deviation, Hz */
    double amplitude;        /* peak carrier amplitude */
    double initial_phase;    /* radians */
    double modulation_index; /* AM */
    int64_t tone2_hz;        /* SSB second tone, 0 = one tone */
    int64_t audio_low_hz;    /* SSB audio passband the tones must sit in */
    int64_t audio_high_hz;
    double words_per_minute; /* CW (PARIS timing: a dot is 1.2 / WPM seconds) */
    double rise_fall_ms;     /* CW raised-cosine edges */
    double message_gap_dots; /* CW silence after the message */
    char text[64];           /* CW message, NUL-terminated */
    uint64_t seed;           /* FSK and PSK payload seed (the random bits) */
    double symbol_rate;      /* FSK and PSK baud */
    uint64_t symbol_count;   /* FSK and PSK payload length in symbols */
    double rolloff;          /* PSK root-raised-cosine rolloff, 0..1 */
    uint64_t span_symbols;   /* PSK pulse span either side, in symbols (the reference's default is 8) */
} rv_tone_emitter;
/* Modulator::accumulate (modulators.cpp:1204-1323): adds `gain` times the
 * emitter's samples at emitter indices [first, first + count) to
 * out_dev[0 .. count), as Scene::render_range does for a burst (first = the
 * range's start less the burst's). Synchronous on `stream` (its host anchor
 * table is copied first). */
int32_t rv_emitter_accumulate(void* stream, const rv_tone_emitter* emitter, uint64_t first, uint64_t count,
                              double gain, rv_cf32* out_dev, uint64_t out_len);
/* The same for an AM, NFM, USB or LSB emitter modulated by supplied audio
 * (ModulatorSpec::audio: one value per sample at the emitter's rate, zero
 * past its end; modulators.cpp:1048-1053, :756-781 the FM phase integral,
 * :807-836 and :1169-1193 the Hilbert phasing network of `hilbert_taps`
 * (odd, >= 3) taps for SSB). */
int32_t rv_emitter_accumulate_audio(void* stream, const rv_tone_emitter* emitter, const float* audio,
                                    uint64_t audio_len, uint32_t hilbert_taps, uint64_t first, uint64_t count,
                                    double gain, rv_cf32* out_dev, uint64_t out_len);

/* Scene::create's random population (core/dsp/synth/wideband.cpp:375-482;
 * RandomPopulation, wideband.h:211-236) for palettes of the built modes
 * (all eight: CW, AM, NFM, USB, LSB, FSK2, BPSK, QPSK): the emitters and their bursts, laid out from
 * std::mt19937_64 draws exactly as the reference lays them out, sorted by
 * start. A scene is then rv_scene_noise plus, in this order, each burst's
 * rv_emitter_accumulate over its window at its gain. */
typedef struct rv_scene_population {
    uint64_t seed;
    int64_t rate;
    int64_t duration_samples;       /* 0 = unbounded (one always-on burst each) */
    double noise_dbfs;              /* full-band noise floor */
    uint32_t emitter_count;
    uint32_t bursts_per_emitter;
    int64_t span_low_hz;
    int64_t span_high_hz;
    double snr_min_db;              /* in the occupied bandwidth */
    double snr_max_db;
    double min_burst_seconds;
    double max_burst_seconds;
    uint32_t palette_count;         /* 0 = every modulation */
    int32_t palette[8];             /* RV_EMITTER_* (siggen::Modulation values) */
} rv_scene_population;

typedef struct rv_scene_burst {
    rv_tone_emitter emitter;
    uint64_t start;                 /* stream indices; end = UINT64_MAX for always on */
    uint64_t end;
    double gain;
    double mean_power;              /* EmitterTruth (wideband.h:82-150) */
    double snr_in_occupied_bandwidth_db;
    int64_t extent_low_hz;
    int64_t extent_high_hz;
    uint64_t payload_seed;
} rv_scene_burst;

/* *count = every burst; the first `capacity` written to out (may be NULL). */
int32_t rv_scene_plan(const rv_scene_population* population, rv_scene_burst* out, uint32_t capacity,
                      uint32_t* count);

/* ===================================================================== *
 * Capture segments (core/capture/format.h, core/capture/writer.cpp): the  *
 * rolling capture's on-disk SigMF recordings, so a capture replays       *
 * through the chain. Host only.                                          *
 *   <root>/<YYYY-MM-DD>/<stem>.sigmf-data   raw samples, source format   *
 *   <root>/<YYYY-MM-DD>/<stem>.sigmf-meta   JSON, written on close       *
 *   stem = rev-<yyyymmddThhmmss.fffZ>-<centre Hz>-<epoch %016x>-<first>  *
 * An open segment is <stem>.open.sigmf-data plus <stem>.open.revenant.   *
 * ===================================================================== */

/* core:recorder is "Revenant " RV_CAPTURE_RECORDER_VERSION. */
#define RV_CAPTURE_RECORDER_VERSION "gb300"

/* WriterConfig (core/capture/writer.h). Zero disables each limit. */
typedef struct rv_capture_config {
    uint64_t max_segment_bytes;    /* a block that would pass it closes "size" first */
    double max_segment_seconds;    /* a segment holding this much closes "size" */
    uint64_t retention_bytes;      /* closed + open bytes kept; oldest closed go first */
    int64_t retention_max_age_ns;  /* age from a segment's first sample */
    uint64_t stream_epoch;         /* 0 = drawn at open */
    int32_t recover_on_start;      /* close what a dead writer left open first */
    int32_t reserved;
} rv_capture_config;

/* A source block (core/source/source.h SourceBlock with its
 * BlockTimestamp): sample_count samples from stream index first_index. */
typedef struct rv_capture_block {
    uint64_t first_index;
    int64_t epoch_anchor_ns; /* wall clock of stream index 0 */
    int64_t rate;            /* samples per second */
    int64_t center;          /* Hz */
    uint64_t sample_count;
    uint64_t dropped_before; /* samples the device lost just before this block */
    int32_t format;          /* RV_FORMAT_CU8, _CS8, _CS16 or _CS24 */
    int32_t reserved;
} rv_capture_block;

/* Annotation (core/capture/format.h) as the detector files it: a track's
 * extent in samples and Hz. core:label is the family, else "signal". */
typedef struct rv_capture_annotation {
    uint64_t sample_count;
    int64_t freq_lower;
    int64_t freq_upper;
    double confidence;
    double peak_db;
    double snr_db;
    uint64_t track_id;
    int32_t has_track_id;
    int32_t reserved;
    char family[32];
} rv_capture_annotation;

typedef struct rv_capture_writer_stats {
    uint64_t segments_written;
    uint64_t bytes_written;
    uint64_t segments_deleted;
    uint64_t delete_failures;
    uint64_t annotations_discarded;
    uint64_t annotations_merged_late;
    uint64_t retained_bytes;
    uint64_t recovered;      /* segments closed as "recovered" at open */
    uint64_t stream_epoch;
} rv_capture_writer_stats;

typedef struct rv_capture_segment {
    char day[16];            /* YYYY-MM-DD directory */
    char stem[96];
    char close_reason[16];   /* retune, rate, format, loss, size, stop, recovered */
    int64_t rate;
    int64_t center;
    int32_t format;
    int32_t has_gain;
    double gain_db;
    uint64_t stream_epoch;
    uint64_t first_index;
    int64_t epoch_anchor_ns;
    uint64_t dropped_before;
    uint64_t samples;
} rv_capture_segment;

typedef struct rv_capture_writer rv_capture_writer;

/* SegmentWriter::start (core/capture/writer.cpp). hw = core:hw (may be NULL). */
int32_t rv_capture_writer_open(const char* root, const rv_capture_config* config, const char* hw,
                               rv_capture_writer** out);
/* SegmentWriter::consume + process: closes the open segment when the block
 * does not continue it, opens one when none is open, appends the block.
 * byte_count = sample_count * bytes per sample of the format. */
int32_t rv_capture_writer_write(rv_capture_writer* w, const rv_capture_block* block, const void* bytes,
                                uint64_t byte_count);
/* SegmentWriter::set_gain_db: in force for segments opened from now. */
int32_t rv_capture_writer_set_gain(rv_capture_writer* w, int32_t has_gain, double gain_db);
/* SegmentWriter::add_annotation: [absolute_start, + sample_count) in
 * stream indices, filed into every segment it overlaps. */
int32_t rv_capture_writer_annotate(rv_capture_writer* w, uint64_t absolute_start, const rv_capture_annotation* a);
/* The clock retention ages against; 0 = the system clock. */
int32_t rv_capture_writer_set_clock(rv_capture_writer* w, int64_t now_ns);
int32_t rv_capture_writer_get_stats(const rv_capture_writer* w, rv_capture_writer_stats* out);
/* SegmentWriter::stop: closes the open segment ("stop"), frees the writer. */
int32_t rv_capture_writer_close(rv_capture_writer* w);
/* The catalog: closed segments under root, by day then stem; *count = all
 * of them, the first `capacity` written to out (out may be NULL). */
int32_t rv_capture_list(const char* root, rv_capture_segment* out, uint32_t capacity, uint32_t* count);
/* Samples [offset, offset + count) of a listed segment, in its format. */
int32_t rv_capture_read(const char* root, const rv_capture_segment* segment, uint64_t offset, uint64_t count,
                        void* out);
/* recover_open_segments: closes segments a dead writer left open
 * ("recovered"). counts = {recovered, removed empty, failed}. */
int32_t rv_capture_recover(const char* root, uint32_t counts[3]);

/* ===================================================================== *
 * Learned detection proposal. No counterpart in the reference: its       *
 * detector (core/detect/detector.cpp:526-1942) scans every bin at every  *
 * decision. Here a small spectrogram CNN proposes the bins worth a look  *
 * and the detector's own decision rules confirm them there              *
 * (rv_detector_set_regions), the full-band decision serving as fallback. *
 * ===================================================================== */

/* Spectrogram tiles: RV_TILE_FRAMES frames x RV_TILE_BINS bins x 2 channels
 * (the dB of exponential averages of the linear power, frame by frame, with
 * a tenth of average_seconds and with average_seconds as time constant, both
 * less the tile row's noise floor and divided by 10), BF16, channels
 * innermost. A row of tiles covers every bin of RV_TILE_FRAMES consecutive
 * frames. */
#define RV_TILE_FRAMES 64u
#define RV_TILE_BINS 256u
#define RV_TILE_CHANNELS 2u
#define RV_CNN_CELLS 32u      /* logits per tile: one per 8-bin cell */
#define RV_CNN_CELL_BINS 8u

/* The network (fixed): conv 4x4/4 2->64, conv 2x2/2 64->128, conv 2x3/(2,1)
 * pad (0,1) 128->128, conv 4x3/(4,1) pad (0,1) 128->64 (ReLU after each),
 * 1x1 64->1; 231,873 FP32 parameters, weights [cout][kh][kw][cin] then the
 * biases, layer after layer. Forward and backward run as BF16 implicit GEMMs
 * on the tcgen05 tensor cores with FP32 accumulation, on the context's
 * stream. */
typedef struct rv_cnn rv_cnn;
typedef struct rv_cnn_train_config {
    float learning_rate;   /* Adam */
    float beta1;
    float beta2;
    float epsilon;
    float weight_decay;    /* added to the gradient (L2) */
    float pos_weight;      /* weight of the positive term of the cross-entropy */
} rv_cnn_train_config;

uint64_t rv_cnn_param_count(void);
/* He-normal weights from `seed`, zero biases; activations for max_batch tiles. */
int32_t rv_cnn_create(rv_context* context, uint32_t max_batch, uint64_t seed, rv_cnn** out);
int32_t rv_cnn_destroy(rv_cnn* cnn);
int32_t rv_cnn_set_params(rv_cnn* cnn, const float* host, uint64_t count);
int32_t rv_cnn_get_params(rv_cnn* cnn, float* host, uint64_t count);
/* The gradient of the last backward or training step. */
int32_t rv_cnn_get_grads(rv_cnn* cnn, float* host, uint64_t count);
void* rv_cnn_stream(const rv_cnn* cnn);
/* Later calls enqueue on `stream` (NULL: the context's); waits for the old one. */
int32_t rv_cnn_set_stream(rv_cnn* cnn, void* stream);
/* Logits [batch][RV_CNN_CELLS] of `batch` tiles (BF16, layout above); the
 * activations stay for rv_cnn_backward. logits_dev may be NULL. */
int32_t rv_cnn_forward(rv_cnn* cnn, const void* tiles_dev, uint32_t batch, float* logits_dev, uint64_t logits_len);
/* Parameter gradient of sum(dlogits * logits) for the last forward batch. */
int32_t rv_cnn_backward(rv_cnn* cnn, const float* dlogits_dev, uint64_t dlogits_len);
/* Forward, weighted binary cross-entropy against labels [batch][RV_CNN_CELLS]
 * (0 or 1, mean over the batch), backward and one Adam step. *loss_host (may
 * be NULL; then nothing waits) receives the batch's loss. */
int32_t rv_cnn_train_step(rv_cnn* cnn, const void* tiles_dev, const float* labels_dev, uint32_t batch,
                          const rv_cnn_train_config* config, float* loss_host);
/* Waits for the stream; RV_ERR_TIMEOUT (count in *timeouts) when a bounded
 * tensor-core wait ran out since the network was created. */
int32_t rv_cnn_status(rv_cnn* cnn, uint32_t* timeouts);
/* The network's GEMM kernel on its own: D[m][n] = sum_k A[m][k] B[n][k],
 * FP32 row-major operands rounded to BF16, FP32 accumulation. Bounded waits
 * that run out are counted in *status_dev. */
int32_t rv_gemm_bf16(void* stream, const float* a_dev, const float* b_dev, uint32_t m, uint32_t n, uint32_t k,
                     float* d_dev, uint32_t* status_dev);

/* The tile builder and the proposals. */
typedef struct rv_proposal_config {
    uint32_t bins;             /* frame bins, a multiple of RV_TILE_BINS */
    uint32_t hold_rows;        /* a proposed cell stays in force this many further tile rows */
    double frame_seconds;      /* source seconds between frames */
    double average_seconds;    /* time constant of the averaged channel (the detector's average_seconds) */
    float threshold;           /* logit above which a cell is proposed */
    uint32_t pad_bins;         /* bins added either side of each run of proposed cells */
} rv_proposal_config;

typedef struct rv_proposer rv_proposer;
int32_t rv_proposer_create(rv_context* context, const rv_proposal_config* config, rv_proposer** out);
int32_t rv_proposer_destroy(rv_proposer* proposer);
/* One row of tiles (bins / RV_TILE_BINS tiles) from RV_TILE_FRAMES frames of
 * `bins` dB values on the device, advancing the averaged channel. */
int32_t rv_proposer_tiles(rv_proposer* proposer, const float* frames_dev, uint64_t frames_len, void* tiles_dev,
                          uint64_t tiles_len);
/* The cells of one tile row whose logit is above the threshold, held for
 * hold_rows rows, merged into ascending disjoint bin ranges [lo, hi)
 * (ranges[2 i], ranges[2 i + 1]) padded by pad_bins; *count = ranges. */
int32_t rv_proposer_regions(rv_proposer* proposer, const float* logits_dev, uint64_t logits_len, uint32_t* ranges,
                            uint32_t capacity, uint32_t* count);
/* Later calls enqueue on `stream` (NULL: the context's); waits for the old one. */
int32_t rv_proposer_set_stream(rv_proposer* proposer, void* stream);
/* The averaged channel and the floors start again (a new capture). */
int32_t rv_proposer_reset(rv_proposer* proposer);

/* Confirmation: the detector's next decisions evaluate the noise floor, the
 * ladder, the peaks and the candidate growth only inside `count` ascending
 * disjoint bin ranges [lo, hi); the average keeps accumulating over every
 * bin. ranges = NULL returns to the full band (the plain detector). */
int32_t rv_detector_set_regions(rv_detector* detector, const uint32_t* ranges, uint32_t count);
/* Keeps every decision's candidates, each with its decision instant (the
 * source sample index), until read; enabling or disabling clears the log. */
int32_t rv_detector_log_candidates(rv_detector* detector, int32_t enable);
/* Moves up to `capacity` logged candidates (oldest first) out of the log;
 * *count = the candidates logged before the call (out = NULL: count only). */
int32_t rv_detector_read_log(rv_detector* detector, uint64_t* instants, rv_detector_candidate* out, uint32_t capacity,
                             uint32_t* count);

#ifdef __cplusplus
}
#endif

#endif /* REVENANT_GB300_H */
