// extern "C" access to the reference's own wideband detector
// (core/detect/detector.cpp), compiled from the reference sources by
// oracle/ref/Makefile into oracle/_ref/libdetref.so. TEST INFRASTRUCTURE: the
// tests and the golden-fixture script use it to pin rv_detector_* against the
// reference; nothing in the product links it.
#include <cstdint>
#include <cstring>
#include <optional>
#include <span>
#include <string>

#include "core/detect/detector.h"
#include "include/revenant_gb300.h"

using namespace revenant;

namespace {
std::string g_error;

struct RefDetector {
    engine::SpectrumGeometry geometry;
    std::optional<detect::Detector> detector;
};
}  // namespace

extern "C" {

const char* refdet_last_error(void) { return g_error.c_str(); }

int32_t refdet_create(const rv_detector_config* c, void** out) {
    detect::DetectorConfig cfg;
    cfg.source_rate = c->source_rate;
    cfg.source_center = c->source_center;
    cfg.detection_threshold_db = c->detection_threshold_db;
    cfg.average_seconds = c->average_seconds;
    cfg.decision_interval_seconds = c->decision_interval_seconds;
    cfg.noise_knots = c->noise_knots;
    cfg.noise_window_knots = c->noise_window_knots;
    cfg.noise_percentile = c->noise_percentile;
    cfg.noise_percentile_high = c->noise_percentile_high;
    cfg.noise_excision_sigma = c->noise_excision_sigma;
    cfg.max_sum_bins = c->max_sum_bins;
    cfg.max_peaks = c->max_peaks;
    cfg.edge_floor_fraction = c->edge_floor_fraction;
    cfg.edge_floor_sigma = c->edge_floor_sigma;
    cfg.occupied_power_fraction = c->occupied_power_fraction;
    cfg.split_gap_bins = c->split_gap_bins;
    cfg.split_gap_db = c->split_gap_db;
    cfg.residual_rate_tolerance = c->residual_rate_tolerance;
    cfg.residual_decisions = c->residual_decisions;
    cfg.birth_hits = c->birth_hits;
    cfg.max_tracks = c->max_tracks;
    cfg.grid_channels = c->grid_channels;
    cfg.association_overlap = c->association_overlap;
    cfg.confidence_rise = c->confidence_rise;
    cfg.confidence_half_life_seconds = c->confidence_half_life_seconds;
    cfg.drop_confidence = c->drop_confidence;
    cfg.centre_smoothing = c->centre_smoothing;
    cfg.channel_hysteresis = c->channel_hysteresis;
    cfg.bootstrap_hold_seconds = c->bootstrap_hold_seconds;
    auto* r = new RefDetector;
    r->geometry.transform = c->bins;
    r->geometry.bins_per_channel = c->bins;
    r->geometry.channels = 1;
    r->geometry.bins = c->bins;
    r->geometry.bin_width_numerator = c->bin_width_numerator;
    r->geometry.bin_width_denominator = c->bin_width_denominator;
    r->geometry.bin_zero_numerator = c->bin_zero_numerator;
    r->geometry.bin_zero_denominator = c->bin_zero_denominator;
    auto made = detect::Detector::create(cfg, r->geometry);
    if (!made) {
        g_error = made.error().message;
        delete r;
        return -2;
    }
    r->detector.emplace(std::move(*made));
    *out = r;
    return 0;
}

void refdet_destroy(void* d) { delete static_cast<RefDetector*>(d); }

int32_t refdet_consume(void* d, const float* power_db, uint64_t start, uint64_t count, int32_t* decided) {
    auto* r = static_cast<RefDetector*>(d);
    const uint64_t before = r->detector->stats().decisions;
    engine::SpectrumFrame frame;
    frame.power_db = std::span<const float>(power_db, r->geometry.bins);
    frame.geometry = r->geometry;
    frame.start = start;
    frame.count = count;
    auto st = r->detector->consume(frame);
    if (!st) {
        g_error = st.error().message;
        return -2;
    }
    if (decided) *decided = r->detector->stats().decisions != before ? 1 : 0;
    return 0;
}

int32_t refdet_candidates(void* d, rv_detector_candidate* out, uint32_t capacity, uint32_t* count) {
    auto* r = static_cast<RefDetector*>(d);
    const auto cands = r->detector->candidates();
    *count = (uint32_t)cands.size();
    for (size_t i = 0; i < cands.size() && i < capacity; ++i) {
        const detect::Candidate& c = cands[i];
        rv_detector_candidate& o = out[i];
        std::memset(&o, 0, sizeof o);
        o.center = c.center;
        o.bandwidth = c.bandwidth;
        o.snr_2500_db = c.snr_2500_db;
        o.margin_confidence = c.margin_confidence;
        o.noise_floor_dbfs = c.noise_floor_dbfs;
        o.peak_dbfs = c.peak_dbfs;
        o.first_bin = c.first_bin;
        o.last_bin = c.last_bin;
        o.peak_to_mean = c.shape.peak_to_mean;
        o.concentration = c.shape.concentration;
        o.lower_fraction = c.shape.lower_fraction;
        o.skirt_fraction = c.shape.skirt_fraction;
        o.skirt_bins_available = c.shape.skirt_bins_available;
        o.measured = c.shape.measured ? 1u : 0u;
    }
    return 0;
}

// Detector::tracks(): every track but the pending ones.
int32_t refdet_tracks(void* d, rv_detector_track* out, uint32_t capacity, uint32_t* count) {
    auto* r = static_cast<RefDetector*>(d);
    const auto tracks = r->detector->tracks();
    *count = (uint32_t)tracks.size();
    for (size_t i = 0; i < tracks.size() && i < capacity; ++i) {
        const detect::Track& t = tracks[i];
        rv_detector_track& o = out[i];
        std::memset(&o, 0, sizeof o);
        o.id = t.id;
        o.state = (uint32_t)t.state;
        o.held_spells = t.held_spells;
        o.center = t.center;
        o.bandwidth = t.bandwidth;
        o.snr_2500_db = t.snr_2500_db;
        o.margin_confidence = t.margin_confidence;
        o.confidence = t.confidence;
        o.first_seen = t.first_seen;
        o.last_seen = t.last_seen;
        o.last_detected = t.last_detected;
        o.hits = t.hits;
        o.misses = t.misses;
        o.channel_index = t.channel_index;
        o.channel = t.channel;
        o.channel_valid = t.channel_valid ? 1u : 0u;
        o.merged_into = t.merged_into;
        o.level_first_bin = t.level_first_bin;
        o.level_last_bin = t.level_last_bin;
        o.level_bins_known = t.level_bins_known ? 1u : 0u;
        o.level_frames = t.level_frames;
        o.level_mean_db = t.level_mean_db;
        o.level_m2 = t.level_m2;
        o.peak_to_mean = t.shape.peak_to_mean;
        o.concentration = t.shape.concentration;
        o.lower_fraction = t.shape.lower_fraction;
        o.skirt_fraction = t.shape.skirt_fraction;
        o.skirt_bins_available = t.shape.skirt_bins_available;
        o.shape_measured = t.shape.measured ? 1u : 0u;
    }
    return 0;
}

int32_t refdet_state(void* d, double* average, double* floor, uint64_t bins) {
    auto* r = static_cast<RefDetector*>(d);
    const auto a = r->detector->averaged_power();
    const auto f = r->detector->noise_floor();
    if (bins != a.size()) return -1;
    if (average) std::memcpy(average, a.data(), bins * sizeof(double));
    if (floor) std::memcpy(floor, f.data(), bins * sizeof(double));
    return 0;
}

int32_t refdet_stats(void* d, rv_detector_stats* s) {
    auto* r = static_cast<RefDetector*>(d);
    const auto& st = r->detector->stats();
    std::memset(s, 0, sizeof *s);
    s->frames = st.frames;
    s->decisions = st.decisions;
    s->frames_rejected = st.frames_rejected;
    s->candidates = st.candidates;
    s->peaks_overflowed = st.peaks_overflowed;
    s->candidates_residual = st.candidates_residual;
    s->residual_parts_degenerate = st.residual_parts_degenerate;
    s->tracks_born = st.tracks_born;
    s->tracks_dropped = st.tracks_dropped;
    s->births_refused = st.births_refused;
    s->merges = st.merges;
    s->splits = st.splits;
    return 0;
}

}  // extern "C"
