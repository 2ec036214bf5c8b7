// Track association for the wideband detector.
//
// Detector::update_tracks (core/detect/detector.cpp:1585-1941) turns each
// decision's candidates into tracks with identities that persist across
// decisions: candidates and tracks are paired where their bands overlap
// enough, the pairs are taken best first one to one, several older tracks
// claiming one candidate merge into the eldest, assigned tracks are smoothed
// towards their candidate, unassigned ones are held with a decaying
// confidence and dropped, and unclaimed candidates start pending tracks that
// are born after birth_hits consecutive decisions. measure_levels
// (:629-646) keeps a running mean and variance of each live track's band
// power over the frames. The parts of the reference's tracker that consume
// probe results (classification, emitter memory, keyups, spur and HD-hybrid
// marks) are not carried: without probes they leave every field here as it is.
#include "tracker.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <tuple>

namespace rv {
int32_t set_error_fmt(int32_t code, const char* fmt, ...);
int32_t clear_error();

namespace {

constexpr uint32_t kUnassigned = 0xFFFFFFFFu;

// (numerator / denominator) rounded half away from zero, in integers
// (divide_nearest, core/detect/detector.cpp:82-88).
int64_t divide_nearest(int64_t numerator, int64_t denominator) {
    if (denominator == 0) return 0;
    const int64_t half = denominator / 2;
    return numerator >= 0 ? (numerator + half) / denominator : (numerator - half) / denominator;
}

struct Band {
    double low, high;
};
Band band_of(int64_t center, int64_t bandwidth) {
    const double half = 0.5 * (double)std::max<int64_t>(1, bandwidth);
    return {(double)center - half, (double)center + half};
}

struct Pair {
    uint32_t track, candidate;
    double score;
    uint64_t first_seen, id;
};

bool by_centre(const rv_detector_track& a, const rv_detector_track& b) {
    return a.center != b.center ? a.center < b.center : a.id < b.id;
}

void take_shape(rv_detector_track& t, const rv_detector_candidate& c) {
    t.peak_to_mean = c.peak_to_mean;
    t.concentration = c.concentration;
    t.lower_fraction = c.lower_fraction;
    t.skirt_fraction = c.skirt_fraction;
    t.skirt_bins_available = c.skirt_bins_available;
    t.shape_measured = c.measured;
}

int32_t out_of_range(double v, double lo, double hi, const char* what) {
    if (!std::isfinite(v)) return set_error_fmt(RV_ERR_INVALID, "rv_detector: %s is not a finite number", what);
    if (v < lo || v > hi) return set_error_fmt(RV_ERR_INVALID, "rv_detector: %s is %g, outside %g to %g", what, v, lo, hi);
    return RV_OK;
}

}  // namespace

int32_t validate_tracking(const rv_detector_config& c) {
    if (int32_t st = out_of_range(c.association_overlap, 0.001, 1.0, "association_overlap")) return st;
    if (int32_t st = out_of_range(c.confidence_rise, 0.001, 1.0, "confidence_rise")) return st;
    if (int32_t st = out_of_range(c.confidence_half_life_seconds, 1.0e-6, 3600.0, "confidence_half_life_seconds"))
        return st;
    if (int32_t st = out_of_range(c.drop_confidence, 0.0, 0.999, "drop_confidence")) return st;
    if (int32_t st = out_of_range(c.centre_smoothing, 0.001, 1.0, "centre_smoothing")) return st;
    if (int32_t st = out_of_range(c.bootstrap_hold_seconds, 1.0e-6, 3600.0, "bootstrap_hold_seconds")) return st;
    if (int32_t st = out_of_range(c.channel_hysteresis, 0.0, 10.0, "channel_hysteresis")) return st;
    if (c.birth_hits == 0)
        return set_error_fmt(RV_ERR_INVALID, "rv_detector: birth_hits of zero would make every noise excursion a track");
    if (c.max_tracks == 0) return set_error_fmt(RV_ERR_INVALID, "rv_detector: max_tracks must be at least one");
    if (c.source_rate <= 0) return set_error_fmt(RV_ERR_INVALID, "rv_detector: source_rate must be positive");
    return RV_OK;
}

// Detector::update_channel (core/detect/detector.cpp:1978-2007): the nearest
// coarse channel, moved only when the centre is more than half a channel plus
// the hysteresis away from the current one.
void Tracker::set_channel(rv_detector_track& t) const {
    if (cfg_.grid_channels == 0) {
        t.channel_valid = 0;
        t.channel = 0;
        t.channel_index = 0;
        return;
    }
    const int64_t channels = (int64_t)cfg_.grid_channels;
    const int64_t baseband = t.center - cfg_.source_center;
    const double exact = (double)baseband * (double)channels / (double)cfg_.source_rate;
    if (!t.channel_valid || std::abs(exact - (double)t.channel_index) > 0.5 + cfg_.channel_hysteresis) {
        t.channel_index = divide_nearest(baseband * channels, cfg_.source_rate);
        t.channel_valid = 1;
    }
    int64_t wrapped = t.channel_index % channels;
    if (wrapped < 0) wrapped += channels;
    t.channel = (uint32_t)wrapped;
}

void Tracker::update(uint64_t now, double elapsed, const rv_detector_candidate* cand, uint32_t ncand) {
    std::sort(all_.begin(), all_.end(), by_centre);
    const uint32_t ntracks = (uint32_t)all_.size();

    // Candidate bands, once.
    std::vector<Band> cb(ncand);
    for (uint32_t c = 0; c < ncand; ++c) cb[c] = band_of(cand[c].center, cand[c].bandwidth);

    // Gate on overlap over the narrower band, score on overlap over the wider.
    // Candidates ascend in frequency, so a track's sweep stops at the first
    // candidate wholly above it.
    std::vector<Pair> pairs;
    for (uint32_t t = 0; t < ntracks; ++t) {
        const Band tb = band_of(all_[t].center, all_[t].bandwidth);
        const double tw = tb.high - tb.low;
        for (uint32_t c = 0; c < ncand; ++c) {
            if (cb[c].high < tb.low) continue;
            if (cb[c].low > tb.high) break;
            const double w = cb[c].high - cb[c].low;
            const double overlap = std::min(tb.high, cb[c].high) - std::max(tb.low, cb[c].low);
            if (overlap <= 0.0) continue;
            if (overlap / std::min(tw, w) < cfg_.association_overlap) continue;
            pairs.push_back(Pair{t, c, overlap / std::max(tw, w), all_[t].first_seen, all_[t].id});
        }
    }
    std::sort(pairs.begin(), pairs.end(), [](const Pair& a, const Pair& b) {
        if (a.score != b.score) return a.score > b.score;
        return std::tie(a.first_seen, a.id, a.candidate) < std::tie(b.first_seen, b.id, b.candidate);
    });

    // One to one, best first.
    std::vector<uint32_t> cand_of(ntracks, kUnassigned), track_of(ncand, kUnassigned);
    for (const Pair& p : pairs) {
        if (cand_of[p.track] != kUnassigned || track_of[p.candidate] != kUnassigned) continue;
        cand_of[p.track] = p.candidate;
        track_of[p.candidate] = p.track;
    }

    // Merges: every born track gated to a candidate and left without one
    // joins the candidate's claimants; the eldest (first_seen, then id) keeps
    // the candidate and the others become its children. A pending owner
    // loses its candidate to any born claimant.
    std::vector<uint32_t> gated;
    for (uint32_t c = 0; c < ncand; ++c) {
        const uint32_t owner = track_of[c];
        if (owner == kUnassigned) continue;
        gated.clear();
        if (all_[owner].state != RV_TRACK_PENDING) gated.push_back(owner);
        for (const Pair& p : pairs) {
            if (p.candidate != c || p.track == owner) continue;
            if (cand_of[p.track] != kUnassigned || all_[p.track].state == RV_TRACK_PENDING) continue;
            gated.push_back(p.track);
        }
        if (gated.empty() || (gated.size() == 1 && gated[0] == owner)) continue;
        uint32_t eldest = gated[0];
        for (uint32_t t : gated)
            if (std::tie(all_[t].first_seen, all_[t].id) < std::tie(all_[eldest].first_seen, all_[eldest].id)) eldest = t;
        if (eldest != owner) {
            cand_of[owner] = kUnassigned;
            cand_of[eldest] = c;
            track_of[c] = eldest;
        }
        const uint64_t parent = all_[eldest].id;
        for (uint32_t t : gated) {
            if (t == eldest) continue;
            rv_detector_track& child = all_[t];
            if (child.state != RV_TRACK_MERGED || child.merged_into != parent) ++merges_;
            child.state = RV_TRACK_MERGED;
            child.merged_into = parent;
            child.last_seen = now;  // last_detected stays: the hold still bounds a child
        }
    }

    const double decay = std::exp2(-elapsed / cfg_.confidence_half_life_seconds);
    const double hold_samples = cfg_.bootstrap_hold_seconds * (double)cfg_.source_rate;
    std::vector<rv_detector_track> next;
    next.reserve(all_.size() + ncand);
    for (uint32_t t = 0; t < ntracks; ++t) {
        rv_detector_track k = all_[t];
        const uint32_t a = cand_of[t];
        if (a != kUnassigned) {
            const rv_detector_candidate& c = cand[a];
            if (k.state == RV_TRACK_MERGED) ++splits_;
            k.merged_into = 0;
            const double s = k.state == RV_TRACK_PENDING ? 1.0 : cfg_.centre_smoothing;
            const double centre = (double)k.center + s * (double)(c.center - k.center);
            const double width = (double)k.bandwidth + s * (double)(c.bandwidth - k.bandwidth);
            k.center = (int64_t)std::llround(centre);
            k.bandwidth = std::max<int64_t>(1, (int64_t)std::llround(width));
            k.snr_2500_db += s * (c.snr_2500_db - k.snr_2500_db);
            k.margin_confidence = margin_confidence(k.snr_2500_db, cfg_.detection_threshold_db);
            take_shape(k, c);
            if (k.level_bins_known && (k.level_first_bin != c.first_bin || k.level_last_bin != c.last_bin)) {
                k.level_frames = 0;  // a level over other bins is another quantity
                k.level_mean_db = 0.0;
                k.level_m2 = 0.0;
            }
            k.level_first_bin = c.first_bin;
            k.level_last_bin = c.last_bin;
            k.level_bins_known = 1;
            ++k.hits;
            k.misses = 0;
            k.last_detected = now;
            k.last_seen = now;
            k.confidence += (1.0 - k.confidence) * cfg_.confidence_rise;
            if (k.state == RV_TRACK_PENDING) {
                if (k.hits >= cfg_.birth_hits) {
                    k.state = RV_TRACK_LIVE;
                    ++born_;
                }
            } else {
                k.state = RV_TRACK_LIVE;
            }
            set_channel(k);
            next.push_back(k);
            continue;
        }
        if (k.state == RV_TRACK_PENDING) continue;  // birth is consecutive or nothing
        if (k.state != RV_TRACK_MERGED) {
            if (k.state == RV_TRACK_LIVE) ++k.held_spells;
            ++k.misses;
            k.state = RV_TRACK_HELD;
            k.confidence *= decay;
        }
        k.last_seen = now;
        if (k.confidence < cfg_.drop_confidence || (double)(now - k.last_detected) > hold_samples) {
            ++dropped_;
            continue;
        }
        next.push_back(k);
    }

    for (uint32_t c = 0; c < ncand; ++c) {
        if (track_of[c] != kUnassigned) continue;
        if (next.size() >= cfg_.max_tracks) {
            ++refused_;
            continue;
        }
        const rv_detector_candidate& d = cand[c];
        rv_detector_track k;
        std::memset(&k, 0, sizeof k);
        k.id = next_id_++;
        k.state = RV_TRACK_PENDING;
        k.center = d.center;
        k.bandwidth = std::max<int64_t>(1, d.bandwidth);
        k.snr_2500_db = d.snr_2500_db;
        k.margin_confidence = d.margin_confidence;
        take_shape(k, d);
        k.level_first_bin = d.first_bin;
        k.level_last_bin = d.last_bin;
        k.level_bins_known = 1;
        k.confidence = cfg_.confidence_rise;
        k.first_seen = k.last_seen = k.last_detected = now;
        k.hits = 1;
        if (k.hits >= cfg_.birth_hits) {
            k.state = RV_TRACK_LIVE;
            ++born_;
        }
        set_channel(k);
        next.push_back(k);
    }
    all_ = std::move(next);
    std::sort(all_.begin(), all_.end(), by_centre);
}

void Tracker::level_bins(uint32_t bins, std::vector<uint32_t>& first_last) const {
    first_last.clear();
    for (const rv_detector_track& t : all_) {
        if (t.state != RV_TRACK_LIVE || !t.level_bins_known || t.level_last_bin >= bins) continue;
        first_last.push_back(t.level_first_bin);
        first_last.push_back(t.level_last_bin);
    }
}

void Tracker::fold_levels(const double* sums, uint32_t frames, uint32_t tracks, uint32_t bins) {
    std::vector<rv_detector_track*> measured;
    for (rv_detector_track& t : all_)
        if (t.state == RV_TRACK_LIVE && t.level_bins_known && t.level_last_bin < bins) measured.push_back(&t);
    const uint32_t n = std::min<uint32_t>(tracks, (uint32_t)measured.size());
    for (uint32_t f = 0; f < frames; ++f)
        for (uint32_t k = 0; k < n; ++k) {
            rv_detector_track& t = *measured[k];
            const double level = 10.0 * std::log10(std::max(sums[(uint64_t)f * tracks + k], 1e-30));
            ++t.level_frames;
            const double delta = level - t.level_mean_db;
            t.level_mean_db += delta / (double)t.level_frames;
            t.level_m2 += delta * (level - t.level_mean_db);
        }
}

void Tracker::tracks(bool all, std::vector<rv_detector_track>& out) const {
    out.clear();
    for (const rv_detector_track& t : all_)
        if (all || t.state != RV_TRACK_PENDING) out.push_back(t);
}

}  // namespace rv

struct rv_tracker {
    rv::Tracker tracker;
    explicit rv_tracker(const rv_detector_config& c) : tracker(c) {}
};

extern "C" {

int32_t rv_tracker_create(const rv_detector_config* config, rv_tracker** out) {
    if (config == nullptr || out == nullptr) return rv::set_error_fmt(RV_ERR_INVALID, "rv_tracker_create: NULL argument");
    *out = nullptr;
    if (int32_t st = rv::validate_tracking(*config)) return st;
    *out = new rv_tracker(*config);
    return rv::clear_error();
}

int32_t rv_tracker_destroy(rv_tracker* t) {
    delete t;
    return rv::clear_error();
}

int32_t rv_tracker_update(rv_tracker* t, uint64_t now, double elapsed_seconds, const rv_detector_candidate* candidates,
                          uint32_t count) {
    if (t == nullptr || (candidates == nullptr && count > 0))
        return rv::set_error_fmt(RV_ERR_INVALID, "rv_tracker_update: NULL argument");
    if (!std::isfinite(elapsed_seconds) || elapsed_seconds < 0.0)
        return rv::set_error_fmt(RV_ERR_INVALID, "rv_tracker_update: elapsed_seconds is %g", elapsed_seconds);
    t->tracker.update(now, elapsed_seconds, candidates, count);
    return rv::clear_error();
}

int32_t rv_tracker_level_bins(const rv_tracker* t, uint32_t bins, uint32_t* first_last, uint32_t capacity,
                              uint32_t* count) {
    if (t == nullptr || count == nullptr) return rv::set_error_fmt(RV_ERR_INVALID, "rv_tracker_level_bins: NULL argument");
    std::vector<uint32_t> fl;
    t->tracker.level_bins(bins, fl);
    *count = (uint32_t)(fl.size() / 2);
    if (first_last)
        for (uint32_t i = 0; i < *count && i < capacity; ++i) {
            first_last[2 * i] = fl[2 * i];
            first_last[2 * i + 1] = fl[2 * i + 1];
        }
    return rv::clear_error();
}

int32_t rv_tracker_fold_levels(rv_tracker* t, uint32_t bins, const double* sums, uint32_t frames, uint32_t tracks) {
    if (t == nullptr || (sums == nullptr && frames > 0 && tracks > 0))
        return rv::set_error_fmt(RV_ERR_INVALID, "rv_tracker_fold_levels: NULL argument");
    t->tracker.fold_levels(sums, frames, tracks, bins);
    return rv::clear_error();
}

int32_t rv_tracker_tracks(const rv_tracker* t, int32_t all, rv_detector_track* out, uint32_t capacity,
                          uint32_t* count) {
    if (t == nullptr || count == nullptr) return rv::set_error_fmt(RV_ERR_INVALID, "rv_tracker_tracks: NULL argument");
    std::vector<rv_detector_track> v;
    t->tracker.tracks(all != 0, v);
    *count = (uint32_t)v.size();
    if (out)
        for (uint32_t i = 0; i < *count && i < capacity; ++i) out[i] = v[i];
    return rv::clear_error();
}

int32_t rv_tracker_get_stats(const rv_tracker* t, rv_detector_stats* stats) {
    if (t == nullptr || stats == nullptr) return rv::set_error_fmt(RV_ERR_INVALID, "rv_tracker_get_stats: NULL argument");
    std::memset(stats, 0, sizeof *stats);
    t->tracker.add_stats(*stats);
    return rv::clear_error();
}

}  // extern "C"
