"""CPU restatement of the learned proposal's tile builder and region merger
(revenant_gb300/csrc/proposal.cu), in FP64.

TEST INFRASTRUCTURE ONLY: tests/test_gpu_proposal.py compares the GPU's
tiles and ranges with these. The reference has no counterpart (its detector
reads frames directly); the rules restated here are this project's own.
"""
import math

import numpy as np

TILE_FRAMES, TILE_BINS, CELLS, CELL_BINS = 64, 256, 32, 8


def alphas(frame_seconds, average_seconds):
    a = min(1.0, max(1e-6, 1.0 - math.exp(-frame_seconds / average_seconds)))
    q = min(1.0, max(1e-6, 1.0 - math.exp(-10.0 * frame_seconds / average_seconds)))
    return a, q


def tile_row(frames_db, state, alpha, alpha_short):
    """One row of tiles from TILE_FRAMES frames [64][bins] (dB). `state` is a
    dict carrying 'long' and 'short' averages (absent: start fresh from the
    first frame). Returns float64 [tiles][64][256][2]."""
    frames = np.asarray(frames_db, np.float64)
    bins = frames.shape[1]
    lin = np.exp2(frames * (math.log2(10.0) / 10.0))
    a = state.get("long")
    q = state.get("short")
    long_db = np.empty_like(frames)
    short_db = np.empty_like(frames)
    for f in range(TILE_FRAMES):
        if a is None:
            a, q = lin[f].copy(), lin[f].copy()
        else:
            a = a + alpha * (lin[f] - a)
            q = q + alpha_short * (lin[f] - q)
        long_db[f] = 10.0 * np.log10(np.maximum(a, 1e-30))
        short_db[f] = 10.0 * np.log10(np.maximum(q, 1e-30))
    state["long"], state["short"] = a, q
    tiles = bins // TILE_BINS
    means = long_db.reshape(TILE_FRAMES, tiles, TILE_BINS).mean(axis=(0, 2))
    floor = np.sort(means)[(tiles - 1) // 2]
    out = np.stack([(short_db - floor) / 10.0, (long_db - floor) / 10.0], axis=-1)  # [64][bins][2]
    return out.reshape(TILE_FRAMES, tiles, TILE_BINS, 2).transpose(1, 0, 2, 3)


def regions(flag_rows, bins, pad_bins):
    """Ranges [lo, hi) from the held rows' cell flags (a list of [cells]
    arrays): cells on in any row, padded by pad_bins, merged."""
    on = np.zeros(len(flag_rows[0]), bool)
    for row in flag_rows:
        on |= np.asarray(row, bool)
    out = []
    for c in np.flatnonzero(on):
        lo, hi = max(0, c * CELL_BINS - pad_bins), min(bins, (c + 1) * CELL_BINS + pad_bins)
        if out and lo <= out[-1][1]:
            out[-1][1] = max(out[-1][1], hi)
        else:
            out.append([lo, hi])
    return np.asarray(out, np.uint32).reshape(-1, 2)
