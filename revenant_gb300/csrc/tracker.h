// Track association over detector candidates (host side of rv_detector and
// the standalone rv_tracker_*).
#pragma once

#include <stdint.h>

#include <cmath>
#include <vector>

#include "revenant_gb300.h"

namespace rv {

// characterise::margin_confidence (core/characterise/transform.cpp:272-279):
// zero below the threshold, then 1 - exp(-excess / 6 dB) / 2.
inline double margin_confidence(double margin_db, double threshold_db) {
    if (margin_db < threshold_db) return 0.0;
    return 1.0 - 0.5 * std::exp(-(margin_db - threshold_db) / 6.0);
}

// Checks the tracking fields of a detector configuration (the ranges
// Detector::create enforces, core/detect/detector.cpp:260-300).
int32_t validate_tracking(const rv_detector_config& c);

class Tracker {
public:
    explicit Tracker(const rv_detector_config& c) : cfg_(c) {}

    // Detector::update_tracks (core/detect/detector.cpp:1585-1941) for the
    // decision at `now`, `elapsed` seconds after the previous one.
    void update(uint64_t now, double elapsed, const rv_detector_candidate* cand, uint32_t count);
    // Tracks whose band power measure_levels takes from each frame: live,
    // bins known and inside the frame; (first, last) pairs in track order.
    void level_bins(uint32_t bins, std::vector<uint32_t>& first_last) const;
    // Folds frames of band powers for the tracks level_bins named (in the
    // same order), one frame at a time, as measure_levels does per frame.
    void fold_levels(const double* sums, uint32_t frames, uint32_t tracks, uint32_t bins);
    void tracks(bool all, std::vector<rv_detector_track>& out) const;
    void add_stats(rv_detector_stats& s) const {
        s.tracks_born = born_;
        s.tracks_dropped = dropped_;
        s.births_refused = refused_;
        s.merges = merges_;
        s.splits = splits_;
    }

private:
    void set_channel(rv_detector_track& t) const;

    rv_detector_config cfg_;
    std::vector<rv_detector_track> all_;  // ascending (center, id)
    uint64_t next_id_ = 1;
    uint64_t born_ = 0, dropped_ = 0, refused_ = 0, merges_ = 0, splits_ = 0;
};

}  // namespace rv
