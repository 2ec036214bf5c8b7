"""Seeded spectrum-frame scenes for the wideband detector tests.

A frame is `bins` dB values: noise with an exponential (two-degree-of-freedom
chi-square) power distribution around a floor with a gentle tilt, plus bands
that switch on and off at given frames (flat or raised-cosine shaped). Frames
are quantised to 1/256 dB and kept as int16 so that a committed fixture
reproduces them exactly on any machine.
"""
import numpy as np

QUANTUM = 256.0


def scene(bins, frames, seed, bands, floor_db=-100.0, tilt_db=3.0):
    """bands: (first_bin, width, snr_db, on_frame, off_frame, shape) tuples;
    shape "flat", "cos" (raised cosine) or "keyN" (flat, keyed off every
    other N frames)."""
    rng = np.random.default_rng(seed)
    k = np.arange(bins, dtype=np.float64)
    floor = 10.0 ** ((floor_db + tilt_db * np.sin(2.0 * np.pi * k / bins)) / 10.0)
    out = np.zeros((frames, bins), np.int16)
    for f in range(frames):
        p = floor * rng.exponential(1.0, bins)
        for first, width, snr_db, on, off, shape in bands:
            if not (on <= f < off):
                continue
            if shape.startswith("key") and (f // int(shape[3:])) % 2 == 1:
                continue
            idx = np.arange(first, first + width)
            x = (idx - first + 0.5) / width
            level = 10.0 ** (snr_db / 10.0) * floor[idx]
            if shape == "cos":
                level = level * np.sin(np.pi * x) ** 2
            p[idx] += level * rng.exponential(1.0, width) ** 0.25
        db = 10.0 * np.log10(np.maximum(p, 1e-30))
        out[f] = np.clip(np.round(db * QUANTUM), -32768, 32767).astype(np.int16)
    return out


def to_db(quantised):
    return (quantised.astype(np.float32) / np.float32(QUANTUM)).astype(np.float32)


# The scene of the committed fixture: 2048 bins of 1 kHz at 2.048 MS/s, one
# frame per 2048 source samples; bands that appear, vanish (their residual
# decays through the average) and split.
FIXTURE = dict(bins=2048, frames=120, seed=21, bands=[
    (300, 40, 12.0, 0, 120, "flat"),
    (700, 9, 20.0, 10, 70, "flat"),
    (1000, 200, 6.0, 0, 120, "cos"),
    (1500, 3, 25.0, 30, 120, "flat"),
    (1520, 60, 8.0, 0, 40, "cos"),
    (1800, 120, 15.0, 50, 120, "flat"),
    (1940, 1, 30.0, 0, 120, "flat"),
])
FIXTURE_RATE = 2_048_000
FIXTURE_HOP = 2048


# The tracker's scene: 1024 bins of 1 kHz at 1.024 MS/s, one frame per
# millisecond. Two bands a bridge joins for 40 frames (a merge, then a split),
# a band that stops (held, then dropped), a keyed carrier (held spells), and a
# strong narrow band that appears on a wide one (births beside a live track).
TRACKER = dict(bins=1024, frames=240, seed=7, bands=[
    (150, 20, 15.0, 0, 240, "flat"),
    (230, 20, 15.0, 0, 240, "flat"),
    (170, 60, 15.0, 60, 100, "flat"),
    (500, 40, 12.0, 0, 100, "cos"),
    (700, 8, 20.0, 0, 240, "key64"),
    (860, 60, 10.0, 30, 240, "flat"),
    (880, 6, 25.0, 120, 200, "flat"),
])


def tracker_config(abi):
    """The detector configuration of the tracker's scene."""
    c = fixture_config(abi)
    bins = TRACKER["bins"]
    c.bins = bins
    c.source_rate = bins * 1000
    c.bin_width_numerator, c.bin_width_denominator = bins * 1000, bins
    c.bin_zero_numerator = -bins * 1000 // 2
    c.confidence_half_life_seconds = 0.02
    c.bootstrap_hold_seconds = 0.12
    c.grid_channels = 16
    return c


def fixture_config(abi):
    """The detector configuration the fixture was made with."""
    c = abi.DetectorConfig()
    c.source_rate = FIXTURE_RATE
    c.source_center = 100_000_000
    c.bins = FIXTURE["bins"]
    c.noise_knots = 32
    c.bin_width_numerator = FIXTURE_RATE
    c.bin_width_denominator = FIXTURE["bins"]
    c.bin_zero_numerator = -FIXTURE_RATE // 2
    c.bin_zero_denominator = 1
    c.detection_threshold_db = 6.0
    c.average_seconds = 0.04
    c.decision_interval_seconds = 0.008
    c.noise_window_knots = 8
    c.max_sum_bins = 0
    c.noise_percentile = 0.10
    c.noise_percentile_high = 0.40
    c.noise_excision_sigma = 4.0
    c.max_peaks = 0
    c.split_gap_bins = 8
    c.edge_floor_fraction = 0.0
    c.edge_floor_sigma = 3.0
    c.occupied_power_fraction = 0.99
    c.split_gap_db = 1.0
    c.residual_rate_tolerance = 0.25
    c.residual_decisions = 4
    return abi.tracking_defaults(c)


def fast_tracking(c):
    """Tracking fast enough for the fixture's 0.12 s to hold, drop, merge and
    split tracks: a half-life of 4 ms, a 20 ms hold, a channel grid."""
    c.confidence_half_life_seconds = 0.004
    c.bootstrap_hold_seconds = 0.02
    c.birth_hits = 2
    c.grid_channels = 64
    c.max_tracks = 12
    return c
