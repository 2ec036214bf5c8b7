"""ctypes mirror of include/revenant_gb300.h (structs and constants).

Field order and widths match the C header exactly; tests/test_abi.py checks
sizes and that the shared library exports every declared entry point.
"""
import ctypes as C

U32, U64, I32, I64, F32, F64 = C.c_uint32, C.c_uint64, C.c_int32, C.c_int64, C.c_float, C.c_double

RV_OK = 0
RV_ERR_INVALID = -1
RV_ERR_CUDA = -2
RV_ERR_NO_DEVICE = -3
RV_ERR_NO_MEMORY = -4
RV_ERR_UNSUPPORTED = -5
RV_ERR_TIMEOUT = -6

FORMAT_CU8, FORMAT_CS8, FORMAT_CS16, FORMAT_CS24 = 0, 1, 2, 3
BYTES_PER_SAMPLE = {FORMAT_CU8: 2, FORMAT_CS8: 2, FORMAT_CS16: 4, FORMAT_CS24: 6}

DEMOD = dict(raw=0, am=1, nfm=2, wfm=3, usb=4, lsb=5, dsb=6, cw=7, p25p1=8, dstar=9, tetra=10,
             dmr=11, sam=12)

MEMORY_DEVICE_LOCAL, MEMORY_UPLOAD, MEMORY_READBACK = 0, 1, 2


class _S(C.Structure):
    def __repr__(self):
        return "%s(%s)" % (type(self).__name__,
                           ", ".join("%s=%r" % (n, getattr(self, n)) for n, _ in self._fields_))

    def as_dict(self):
        out = {}
        for n, _ in self._fields_:
            v = getattr(self, n)
            out[n] = v.as_dict() if isinstance(v, _S) else v
        return out


class CF32(_S):
    _fields_ = [("re", F32), ("im", F32)]


class ConvertParams(_S):
    _fields_ = [("ring_mask", U32), ("dst_offset", U32), ("src_offset", U32), ("count", U32)]


class GridParams(_S):
    _fields_ = [("channels", U32), ("taps_per_branch", U32), ("decimation", U32)]


class PfbBranchParams(_S):
    _fields_ = [("ring_mask", U32), ("base_offset", U32), ("block_count", U32)]


class PfbFftParams(_S):
    _fields_ = [("channels", U32), ("decimation", U32), ("stages", U32), ("block_base", U32),
                ("block_count", U32), ("out_ring_blocks", U32), ("out_ring_mask", U32)]


class SpectrumParams(_S):
    _fields_ = [("channels", U32), ("transform", U32), ("stages", U32), ("chan_blocks", U32),
                ("chan_mask", U32), ("in_offset", U32)]


class SpectrumLevelsParams(_S):
    _fields_ = [("bins", U32), ("low_permille", U32), ("high_permille", U32)]


class VrxFineConfig(_S):
    _fields_ = [("taps", U32), ("phases", U32), ("nco_log2", U32)]


class VrxFineParams(_S):
    _fields_ = [("chan_base", U32), ("chan_mask", U32), ("in_offset", U32), ("out_offset", U32),
                ("out_mask", U32), ("count", U32), ("step_whole", U32), ("step_rem", U32),
                ("out_rate", U32), ("frac0", U32), ("nco_phase_high", U32), ("nco_phase_low", U32),
                ("nco_delta_high", U32), ("nco_delta_low", U32), ("inv_out_rate", F32)]


class VrxDemodConfig(_S):
    _fields_ = [("mode", U32), ("decimation", U32), ("audio_taps", U32), ("dc_taps", U32),
                ("channels", U32), ("pilot_taps", U32)]


class VrxDemodParams(_S):
    _fields_ = [("in_mask", U32), ("in_offset", U32), ("count", U32), ("gain", F32)]


class VrxCarrierConfig(_S):
    _fields_ = [("power", U32), ("nco_log2", U32)]


class VrxCarrierParams(_S):
    _fields_ = [("in_mask", U32), ("in_offset", U32), ("count", U32), ("flags", U32),
                ("shift", F32), ("k1_acquire", F32), ("k2_acquire", F32), ("k1_track", F32),
                ("k2_track", F32), ("level_alpha", F32), ("lock_alpha", F32),
                ("clamp_radians", F32), ("hold_in", U32), ("hold_out", U32)]


class CoarseParams(_S):
    _fields_ = [("ring_mask", U32), ("base_offset", U32), ("block_count", U32), ("block_base", U32),
                ("out_ring_blocks", U32), ("out_ring_mask", U32), ("lead_zero", U32)]


class SpectrumAverageParams(_S):
    _fields_ = [("size", U32), ("frames", U32), ("average", U32), ("mode", U32), ("alpha", F32), ("norm", F32),
                ("resume", U32), ("reserved", U32)]


AVERAGE_MEAN, AVERAGE_EXPONENTIAL = 0, 1
WINDOW_RECTANGULAR, WINDOW_HANN, WINDOW_BLACKMAN_HARRIS = 0, 1, 2


class IqMomentsParams(_S):
    _fields_ = [("ring_mask", U32), ("src_offset", U32), ("count", U32)]


class IqCorrectParams(_S):
    _fields_ = [("ring_mask", U32), ("offset", U32), ("count", U32), ("dc_i", F32), ("dc_q", F32), ("cross", F32),
                ("scale", F32)]


class FrontEnd(_S):
    _fields_ = [("dc_time_constant_s", F64), ("iq_time_constant_s", F64), ("max_gain_error_db", F64),
                ("max_phase_error_deg", F64), ("measured", U32), ("iq_plausible", U32), ("samples_seen", U64),
                ("dc_i", F64), ("dc_q", F64), ("gain", F64), ("sin_phase", F64), ("m_ii", F64), ("m_qq", F64),
                ("m_iq", F64)]


class DetectorConfig(_S):
    _fields_ = [("source_rate", I64), ("source_center", I64), ("bins", U32), ("noise_knots", U32),
                ("bin_width_numerator", I64), ("bin_width_denominator", I64), ("bin_zero_numerator", I64),
                ("bin_zero_denominator", I64), ("detection_threshold_db", F64), ("average_seconds", F64),
                ("decision_interval_seconds", F64), ("noise_window_knots", U32), ("max_sum_bins", U32),
                ("noise_percentile", F64), ("noise_percentile_high", F64), ("noise_excision_sigma", F64),
                ("max_peaks", U32), ("split_gap_bins", U32), ("edge_floor_fraction", F64),
                ("edge_floor_sigma", F64), ("occupied_power_fraction", F64), ("split_gap_db", F64),
                ("residual_rate_tolerance", F64), ("residual_decisions", U32), ("birth_hits", U32),
                ("max_tracks", U32), ("grid_channels", U32), ("association_overlap", F64),
                ("confidence_rise", F64), ("confidence_half_life_seconds", F64), ("drop_confidence", F64),
                ("centre_smoothing", F64), ("channel_hysteresis", F64), ("bootstrap_hold_seconds", F64)]


def tracking_defaults(c):
    """DetectorConfig's tracking defaults (core/detect/detector.h:900-1206)."""
    c.birth_hits, c.max_tracks, c.grid_channels = 3, 512, 0
    c.association_overlap, c.confidence_rise, c.confidence_half_life_seconds = 0.3, 0.35, 1.0
    c.drop_confidence, c.centre_smoothing, c.channel_hysteresis, c.bootstrap_hold_seconds = 0.05, 0.4, 0.15, 3.0
    return c


EXCISE_SEGMENT, EXCISE_REFERENCE, EXCISE_FLAG, EXCISE_APPLY = 0, 1, 2, 3
EXCISE_COUNTER_SAMPLES, EXCISE_COUNTER_EVENTS, EXCISE_COUNTER_SPARED = 0, 1, 2


class ExcisionConfig(_S):
    _fields_ = [("pass_", U32), ("seg_log2", U32), ("segments", U32), ("max_width", U32), ("hang", U32),
                ("lead", U32)]


class ExcisionParams(_S):
    _fields_ = [("ring_mask", U32), ("first", U32), ("count", U32), ("seg_mask", U32), ("flag_mask", U32),
                ("removed_mask", U32), ("history", I32), ("threshold", F32)]


class ExcisionRings(_S):
    _fields_ = [("seg_mask", U32), ("flag_mask", U32), ("removed_mask", U32)]


class ExcisionPlan(_S):
    _fields_ = [("segment", ExcisionParams), ("reference", ExcisionParams), ("flag", ExcisionParams),
                ("apply", ExcisionParams), ("cleaned_end", U64), ("restarted", U32), ("reserved", U32)]


class ExcisionCursor(_S):
    _fields_ = [("config", ExcisionConfig), ("ring_mask", U32), ("rings", ExcisionRings), ("threshold", F32),
                ("running", U32), ("reserved", U32), ("valid_from", U64), ("next_in", U64), ("seg_next", U64),
                ("flag_next", U64), ("apply_next", U64)]


class VrxDisplayPlan(_S):
    _fields_ = [("channel_rate", I64), ("display_rate", I64), ("decimation", U32), ("reserved", U32),
                ("reach_hz", I64), ("fine", VrxFineConfig), ("reserved2", U32), ("nco_delta", U64), ("pass_hz", F64),
                ("stop_hz", F64), ("attenuation_db", F64), ("group_delay_channel_samples", F64), ("tap_count", U64)]


COMB_TABLE_SIZE = 4096


class CombLine(_S):
    _fields_ = [("phase0", U32), ("step", U32), ("pad0", U32), ("pad1", U32), ("amp_re", F32), ("amp_im", F32)]


class CombParams(_S):
    _fields_ = [("ring_mask", U32), ("first", U32), ("count", U32), ("lines", U32), ("sub_blocks", U32),
                ("removed_mask", U32), ("pad0", U32), ("pad1", U32)]


DFT_FP16, DFT_BF16 = 0, 1
EMITTER_CW, EMITTER_AM, EMITTER_NFM, EMITTER_USB, EMITTER_LSB, EMITTER_FSK2, EMITTER_BPSK, EMITTER_QPSK = range(8)


class ToneEmitter(_S):
    _fields_ = [("modulation", I32), ("reserved", I32), ("rate", I64), ("carrier_offset", I64), ("tone_hz", I64),
                ("deviation", I64), ("amplitude", F64), ("initial_phase", F64), ("modulation_index", F64),
                ("tone2_hz", I64), ("audio_low_hz", I64), ("audio_high_hz", I64), ("words_per_minute", F64),
                ("rise_fall_ms", F64), ("message_gap_dots", F64), ("text", C.c_char * 64), ("seed", U64),
                ("symbol_rate", F64), ("symbol_count", U64), ("rolloff", F64), ("span_symbols", U64)]


class ScenePopulation(_S):
    _fields_ = [("seed", U64), ("rate", I64), ("duration_samples", I64), ("noise_dbfs", F64), ("emitter_count", U32),
                ("bursts_per_emitter", U32), ("span_low_hz", I64), ("span_high_hz", I64), ("snr_min_db", F64),
                ("snr_max_db", F64), ("min_burst_seconds", F64), ("max_burst_seconds", F64), ("palette_count", U32),
                ("palette", I32 * 8)]


class SceneBurst(_S):
    _fields_ = [("emitter", ToneEmitter), ("start", U64), ("end", U64), ("gain", F64), ("mean_power", F64),
                ("snr_in_occupied_bandwidth_db", F64), ("extent_low_hz", I64), ("extent_high_hz", I64),
                ("payload_seed", U64)]


class CaptureConfig(_S):
    _fields_ = [("max_segment_bytes", U64), ("max_segment_seconds", F64), ("retention_bytes", U64),
                ("retention_max_age_ns", I64), ("stream_epoch", U64), ("recover_on_start", I32), ("reserved", I32)]


class CaptureBlock(_S):
    _fields_ = [("first_index", U64), ("epoch_anchor_ns", I64), ("rate", I64), ("center", I64),
                ("sample_count", U64), ("dropped_before", U64), ("format", I32), ("reserved", I32)]


class CaptureAnnotation(_S):
    _fields_ = [("sample_count", U64), ("freq_lower", I64), ("freq_upper", I64), ("confidence", F64),
                ("peak_db", F64), ("snr_db", F64), ("track_id", U64), ("has_track_id", I32), ("reserved", I32),
                ("family", C.c_char * 32)]


class CaptureWriterStats(_S):
    _fields_ = [(n, U64) for n in ("segments_written", "bytes_written", "segments_deleted", "delete_failures",
                                   "annotations_discarded", "annotations_merged_late", "retained_bytes",
                                   "recovered", "stream_epoch")]


class CaptureSegment(_S):
    _fields_ = [("day", C.c_char * 16), ("stem", C.c_char * 96), ("close_reason", C.c_char * 16), ("rate", I64),
                ("center", I64), ("format", I32), ("has_gain", I32), ("gain_db", F64), ("stream_epoch", U64),
                ("first_index", U64), ("epoch_anchor_ns", I64), ("dropped_before", U64), ("samples", U64)]


LINE_NOTCH, LINE_ALE, LINE_GUARD, LINE_NOTCH_COUNT_SHIFT = 1, 2, 4, 8
LINE_STATE_WEIGHTS = 24


class BlankerConfig(_S):
    _fields_ = [("pass_", U32), ("window", U32), ("guard", U32), ("hang", U32), ("lead", U32)]


class BlankerParams(_S):
    _fields_ = [("chan_base", U32), ("chan_mask", U32), ("chan_first", U32), ("out_mask", U32), ("out_first", U32),
                ("count", U32), ("threshold", F32)]


class LineConfig(_S):
    _fields_ = [("lanes", U32), ("taps", U32), ("history", U32)]


class LineSection(_S):
    _fields_ = [("b0", F32), ("b1", F32), ("b2", F32), ("a1", F32), ("a2", F32)]


class LineParams(_S):
    _fields_ = [("count", U32), ("flags", U32), ("stride", U32), ("delay", U32), ("b0", F32), ("b1", F32),
                ("b2", F32), ("a1", F32), ("a2", F32), ("mu", F32), ("leak", F32), ("eps", F32), ("gb0", F32),
                ("gb1", F32), ("gb2", F32), ("ga1", F32), ("ga2", F32), ("more", LineSection * 3)]


class NotchDesign(_S):
    _fields_ = [("b0", F64), ("b1", F64), ("b2", F64), ("a1", F64), ("a2", F64)]


class SpectralConfig(_S):
    _fields_ = [("frame", U32)]


class SpectralParams(_S):
    _fields_ = [("count", U32), ("smoothing", F32), ("smoothing_complement", F32), ("gamma", F32), ("beta", F32),
                ("rise", F32), ("bias", F32), ("alpha", F32), ("floor_gain", F32), ("eps", F32)]


TRACK_PENDING, TRACK_LIVE, TRACK_HELD, TRACK_MERGED = 0, 1, 2, 3


class DetectorTrack(_S):
    _fields_ = [("id", U64), ("state", U32), ("held_spells", U32), ("center", I64), ("bandwidth", I64),
                ("snr_2500_db", F64), ("margin_confidence", F64), ("confidence", F64), ("first_seen", U64),
                ("last_seen", U64), ("last_detected", U64), ("hits", U32), ("misses", U32), ("channel_index", I64),
                ("channel", U32), ("channel_valid", U32), ("merged_into", U64), ("level_first_bin", U32),
                ("level_last_bin", U32), ("level_bins_known", U32), ("level_frames", U32), ("level_mean_db", F64),
                ("level_m2", F64), ("peak_to_mean", F64), ("concentration", F64), ("lower_fraction", F64),
                ("skirt_fraction", F64), ("skirt_bins_available", U64), ("shape_measured", U32), ("reserved", U32)]


class DetectorCandidate(_S):
    _fields_ = [("center", I64), ("bandwidth", I64), ("snr_2500_db", F64), ("margin_confidence", F64),
                ("noise_floor_dbfs", F64), ("peak_dbfs", F64), ("first_bin", U32), ("last_bin", U32),
                ("peak_to_mean", F64), ("concentration", F64), ("lower_fraction", F64), ("skirt_fraction", F64),
                ("skirt_bins_available", U64), ("measured", U32), ("reserved", U32)]


class DetectorStats(_S):
    _fields_ = [("frames", U64), ("decisions", U64), ("frames_rejected", U64), ("candidates", U64),
                ("peaks_overflowed", U64), ("candidates_residual", U64), ("residual_parts_degenerate", U64),
                ("device_ms", F64), ("host_ms", F64), ("tracks_born", U64), ("tracks_dropped", U64),
                ("births_refused", U64), ("merges", U64), ("splits", U64)]


class VrxRequest(_S):
    _fields_ = [("center", I64), ("bandwidth", I64), ("passband_low", I64), ("passband_high", I64),
                ("demod", U32), ("deemphasis", U32), ("stereo", U32), ("reserved", U32),
                ("audio_rate", I64), ("cw_pitch", I64)]


class VrxPlacement(_S):
    _fields_ = [("channel", U32), ("bandwidth_clamped", U32), ("centre_numerator", I64),
                ("centre_denominator", I64), ("residual_numerator", I64),
                ("residual_denominator", I64), ("channel_rate", I64), ("granted_low", I64),
                ("granted_high", I64)]


class VrxPlanInfo(_S):
    _fields_ = [("placement", VrxPlacement), ("mode", U32), ("bandwidth_clamped", U32),
                ("channel_rate", I64), ("audio_rate", I64), ("demod_rate", I64),
                ("output_rate", I64), ("passband_low", I64), ("passband_high", I64),
                ("bandwidth", I64), ("filter_numerator", I64), ("filter_denominator", I64),
                ("mix_numerator", I64), ("mix_denominator", I64), ("fine", VrxFineConfig),
                ("stereo", U32), ("fine_nco_delta", U64), ("demod", VrxDemodConfig),
                ("demod_gain", F32), ("carrier", VrxCarrierConfig),
                ("carrier_loop", VrxCarrierParams), ("deviation", I64), ("deemphasis", U32),
                ("deemphasis_taps", U32), ("audio_decimation_taps", U32), ("reserved", U32),
                ("fine_tap_count", U64), ("demod_weight_count", U64)]


class VrxFineBlock(_S):
    _fields_ = [("params", VrxFineParams), ("reserved", U32), ("first_input", U64),
                ("oldest_input", U64), ("newest_input", U64)]


class VrxDemodBlock(_S):
    _fields_ = [("params", VrxDemodParams), ("first_fine", U64), ("oldest_fine", U64)]


class DeviceInfo(_S):
    _fields_ = [("name", C.c_char * 256), ("device_index", I32), ("sm_count", I32),
                ("cc_major", I32), ("cc_minor", I32), ("total_memory", U64),
                ("max_shared_per_block", U64), ("l2_bytes", U64)]


CHAIN_BATCHED, CHAIN_PLAIN, CHAIN_FAST, CHAIN_HOISTED = 0, 1, 2, 3


class ChainConfig(_S):
    _fields_ = [("grid", GridParams), ("reserved", U32), ("rate", I64), ("format", I32), ("mode", I32),
                ("max_run_samples", U32), ("keep_audio", U32), ("attenuation_db", C.c_double),
                ("profile", U32), ("pipelined", U32)]


class ChainStats(_S):
    _fields_ = [("runs", U64), ("blocks", U64), ("launches", U64), ("work_items", U64), ("audio_bytes", U64),
                ("input_ms", C.c_double), ("coarse_ms", C.c_double), ("fine_ms", C.c_double),
                ("demod_ms", C.c_double), ("readback_ms", C.c_double), ("graph_launches", U64),
                ("graph_captures", U64), ("graph_ms", C.c_double), ("host_ms", C.c_double)]


class ChainTuneReport(_S):
    _fields_ = [("receivers", U32), ("classes", U32), ("classes_changed", U32), ("shapes_timed", U32),
                ("tiles_per_sm", U32), ("shapes_reverted", U32), ("default_ms", C.c_double), ("tuned_ms", C.c_double)]


class CnnTrainConfig(_S):
    _fields_ = [("learning_rate", F32), ("beta1", F32), ("beta2", F32), ("epsilon", F32), ("weight_decay", F32),
                ("pos_weight", F32)]


class ProposalConfig(_S):
    _fields_ = [("bins", U32), ("hold_rows", U32), ("frame_seconds", F64), ("average_seconds", F64),
                ("threshold", F32), ("pad_bins", U32)]


TILE_FRAMES, TILE_BINS, TILE_CHANNELS, CNN_CELLS, CNN_CELL_BINS = 64, 256, 2, 32, 8

EXTRA_STRUCTS = {"rv_cnn_train_config": CnnTrainConfig, "rv_proposal_config": ProposalConfig, "rv_iq_moments_params": IqMomentsParams, "rv_iq_correct_params": IqCorrectParams,
                 "rv_front_end": FrontEnd, "rv_detector_config": DetectorConfig, "rv_detector_candidate": DetectorCandidate,
                 "rv_detector_track": DetectorTrack, "rv_excision_config": ExcisionConfig,
                 "rv_excision_params": ExcisionParams, "rv_excision_rings": ExcisionRings,
                 "rv_excision_plan": ExcisionPlan, "rv_excision_cursor": ExcisionCursor,
                 "rv_vrx_display_plan": VrxDisplayPlan, "rv_comb_line": CombLine, "rv_capture_config": CaptureConfig, "rv_tone_emitter": ToneEmitter, "rv_scene_population": ScenePopulation,
                 "rv_scene_burst": SceneBurst,
                 "rv_capture_block": CaptureBlock, "rv_capture_annotation": CaptureAnnotation,
                 "rv_capture_writer_stats": CaptureWriterStats, "rv_capture_segment": CaptureSegment, "rv_comb_params": CombParams, "rv_blanker_config": BlankerConfig, "rv_blanker_params": BlankerParams,
                 "rv_line_config": LineConfig, "rv_line_section": LineSection, "rv_line_params": LineParams,
                 "rv_notch_design": NotchDesign, "rv_spectral_config": SpectralConfig,
                 "rv_spectral_params": SpectralParams,
                 "rv_detector_stats": DetectorStats, "rv_spectrum_average_params": SpectrumAverageParams, "rv_coarse_params": CoarseParams, "rv_chain_config": ChainConfig, "rv_chain_stats": ChainStats}


def request(center=0, bandwidth=0, demod="nfm", deemphasis=0, stereo=True, audio_rate=0,
            passband_low=0, passband_high=0, cw_pitch=700):
    r = VrxRequest()
    r.center = center
    r.bandwidth = bandwidth
    r.passband_low = passband_low
    r.passband_high = passband_high
    r.demod = DEMOD[demod] if isinstance(demod, str) else demod
    r.deemphasis = deemphasis
    r.stereo = 1 if stereo else 0
    r.audio_rate = audio_rate
    r.cw_pitch = cw_pitch
    return r
