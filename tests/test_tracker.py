"""Track association (rv_tracker_*, rv_detector_tracks) against the reference's
own Detector::update_tracks and measure_levels (core/detect/detector.cpp).

tests/golden/detector.npz holds, for every decision of two seeded scenes, the
reference detector's candidates and its tracks (tests/golden/make_detector.py;
the reference compiled from its sources into oracle/_ref/libdetref.so). The
tracker scene merges two tracks and splits them again, holds and drops a band
that stops, counts a keyed carrier's held spells and maps tracks to a 16-channel
grid; the fixture scene is run with the default tracking and with fast
tracking (drops within the scene).

The bar:
  * host tracker fed the reference's own candidates: every field bit for bit,
    except the level statistics, whose per-frame band powers this test forms
    with the C library's exp2f, as the reference does, but sums in numpy
    (pairwise, the reference sequentially): LEVEL_REL relative on the mean
    and on m2 (absolute below 1);
  * rv_detector on the GPU, which associates its own candidates: integers
    exactly, the dB figures and shape ratios within REL_CAND (the candidates'
    own tolerance), confidence exactly, levels within GPU_LEVEL_REL (the device
    rounds a double exp2 to float where the C library's exp2f is not
    correctly rounded: one float ulp on some bins, measured ~2e-10 relative on
    the mean and ~3e-8 on m2 by the host sums above with numpy's exp2).
"""
import ctypes as C
import ctypes.util as ctypes_util
import os

import numpy as np
import pytest

import detector_scenes as ds
from bindings import candidates_from_array, detector_reference, tracks_array
from revenant_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "detector.npz")
LEVEL_REL = 1e-12
GPU_LEVEL_REL = 1e-6
REL_CAND = 1e-6
KDB = np.float32(0.332192809488736234787)
LEVELS = ("level_mean_db", "level_m2")
SOFT = ("snr_2500_db", "margin_confidence", "peak_to_mean", "concentration", "lower_fraction", "skirt_fraction")


def golden():
    return np.load(GOLDEN)


def scenes(g):
    """(name, frames in dB, config, hop, decision frames, candidates key, tracks key)."""
    fx = ds.FIXTURE
    return {
        "fixture": (ds.to_db(g["frames_q"]), ds.fixture_config(abi), ds.FIXTURE_HOP, g["decision_frames"],
                    "candidates_%d", "tracks_%d"),
        "fixture_fast": (ds.to_db(g["frames_q"]), ds.fast_tracking(ds.fixture_config(abi)), ds.FIXTURE_HOP,
                         g["decision_frames"], "candidates_%d", "fast_tracks_%d"),
        "tracker": (ds.to_db(g["trk_frames_q"]), ds.tracker_config(abi), ds.TRACKER["bins"], g["trk_decision_frames"],
                    "trk_candidates_%d", "trk_tracks_%d"),
    }, fx


def same_tracks(got, want, where, soft=0.0, level_rel=LEVEL_REL):
    assert len(got) == len(want), "%s: %d tracks, want %d\n got %s\nwant %s" % (
        where, len(got), len(want), got[["id", "state", "center"]], want[["id", "state", "center"]])
    for name in got.dtype.names:
        g, w = got[name], want[name]
        if name in LEVELS:
            rel = np.abs(g - w) / np.maximum(1.0, np.abs(w))
            assert np.all(rel <= level_rel), "%s: %s %s vs %s" % (where, name, g, w)
        elif name in SOFT and soft > 0.0:
            rel = np.abs(g - w) / np.maximum(1.0, np.abs(w))
            assert np.all(rel <= soft), "%s: %s %s vs %s" % (where, name, g, w)
        else:
            assert np.array_equal(g, w), "%s: %s %s vs %s" % (where, name, g, w)


_LIBM = C.CDLL(ctypes_util.find_library("m") or "libm.so.6")
_LIBM.exp2f.restype = C.c_float
_LIBM.exp2f.argtypes = [C.c_float]


def band_powers(frame, pairs):
    """measure_levels' band power of each (first, last) pair: the C library's
    exp2f of each bin's float argument, as the reference calls it, summed in
    float64."""
    x = (frame * KDB).astype(np.float32)
    out = []
    for a, b in pairs:
        out.append(np.array([_LIBM.exp2f(float(v)) for v in x[a:b + 1]], np.float64).sum())
    return np.array(out, np.float64)


def first_elapsed(cfg):
    return max(cfg.decision_interval_seconds, cfg.bin_width_denominator / cfg.bin_width_numerator)


# -- CPU: the host tracker over the reference's candidates ---------------------

@pytest.mark.parametrize("scene", ["fixture", "fixture_fast", "tracker"])
def test_host_tracker_matches_reference(rv, scene):
    from revenant_gb300.detector import Tracker
    g = golden()
    frames, cfg, hop, decisions, ckey, tkey = scenes(g)[0][scene]
    trk = Tracker(cfg)
    bins = frames.shape[1]
    prev, k = None, 0
    for f in range(frames.shape[0]):
        pairs = trk.level_bins(bins)
        if len(pairs):
            trk.fold_levels(bins, band_powers(frames[f], pairs)[None, :])
        if k < len(decisions) and f == decisions[k]:
            now = (f + 1) * hop
            elapsed = first_elapsed(cfg) if prev is None else (now - prev) / cfg.source_rate
            trk.update(now, elapsed, candidates_from_array(g[ckey % k]))
            same_tracks(trk.tracks(), g[tkey % k], "%s decision %d" % (scene, k))
            prev, k = now, k + 1
    assert k == len(decisions)
    st = trk.stats()
    want = {"fixture": "track_stats", "fixture_fast": "fast_track_stats", "tracker": "trk_track_stats"}[scene]
    assert (st.tracks_born, st.tracks_dropped, st.births_refused, st.merges, st.splits) == tuple(
        int(x) for x in g[want])
    trk.close()


def test_tracker_scene_exercises_every_transition():
    """The scene does what its comment says: a merge, a split, a drop, held
    tracks and live tracks on several channels."""
    g = golden()
    born, dropped, _, merges, splits = (int(x) for x in g["trk_track_stats"])
    assert merges >= 1 and splits >= 1 and dropped >= 1 and born >= 6
    states = np.concatenate([g["trk_tracks_%d" % k]["state"] for k in range(len(g["trk_decision_frames"]))])
    assert {abi.TRACK_LIVE, abi.TRACK_HELD, abi.TRACK_MERGED} <= set(int(s) for s in states)
    last = g["trk_tracks_%d" % (len(g["trk_decision_frames"]) - 1)]
    assert len(set(int(c) for c in last["channel"])) >= 3 and np.all(last["channel_valid"] == 1)
    assert np.any(last["held_spells"] > 0) and np.any(last["level_frames"] > 10)


def test_reference_tracks_reproduce_golden():
    lib = detector_reference()
    if lib is None:
        pytest.skip("reference detector not built (reference sources absent on this machine)")
    g = golden()
    frames, cfg, hop, decisions, _, tkey = scenes(g)[0]["tracker"]
    det = C.c_void_p()
    assert lib.refdet_create(C.byref(cfg), C.byref(det)) == 0
    k = 0
    for f in range(frames.shape[0]):
        row = np.ascontiguousarray(frames[f])
        decided = C.c_int32()
        assert lib.refdet_consume(det, row.ctypes.data, f * hop, hop, C.byref(decided)) == 0
        if decided.value:
            n = C.c_uint32()
            buf = (abi.DetectorTrack * 512)()
            lib.refdet_tracks(det, buf, 512, C.byref(n))
            assert tracks_array(list(buf)[:n.value]).tobytes() == g[tkey % k].tobytes()
            k += 1
    assert k == len(decisions)
    lib.refdet_destroy(det)


@pytest.mark.parametrize("field,value", [("association_overlap", 0.0), ("confidence_rise", 1.5),
                                         ("confidence_half_life_seconds", 0.0), ("drop_confidence", 1.0),
                                         ("centre_smoothing", 0.0), ("bootstrap_hold_seconds", float("nan")),
                                         ("channel_hysteresis", 11.0), ("birth_hits", 0), ("max_tracks", 0)])
def test_tracker_rejects_bad_configs(rv, field, value):
    cfg = ds.fixture_config(abi)
    setattr(cfg, field, value)
    h = C.c_void_p()
    assert rv.rv_tracker_create(C.byref(cfg), C.byref(h)) == abi.RV_ERR_INVALID, field
    assert field in rv.rv_last_error().decode()


def test_max_tracks_refuses_births(rv):
    """More unclaimed candidates than max_tracks: the rest are refused."""
    from revenant_gb300.detector import Tracker
    g = golden()
    cfg = ds.fixture_config(abi)
    cfg.max_tracks = 3
    trk = Tracker(cfg)
    cands = candidates_from_array(g["candidates_0"])
    trk.update(2048, 0.008, cands)
    assert len(trk.tracks(all_tracks=True)) == 3
    assert trk.stats().births_refused == len(cands) - 3
    trk.close()


# -- GPU: rv_detector's tracks against the reference's --------------------------

@pytest.mark.gpu
@pytest.mark.parametrize("scene,batched", [("tracker", False), ("tracker", True), ("fixture_fast", True)])
def test_gpu_detector_tracks_match_reference(gpu, scene, batched):
    from revenant_gb300.detector import Detector
    g = golden()
    frames, cfg, hop, decisions, _, tkey = scenes(g)[0][scene]
    det = Detector(gpu, cfg)
    decisions = [int(f) for f in decisions]
    if batched:
        first = 0
        for k, f in enumerate(decisions):
            assert det.consume_frames(frames[first:f + 1], first * hop, hop, hop) == 1
            same_tracks(det.tracks(), g[tkey % k], "%s decision %d" % (scene, k), soft=REL_CAND,
                            level_rel=GPU_LEVEL_REL)
            first = f + 1
    else:
        k = 0
        for f in range(frames.shape[0]):
            if det.consume(frames[f], f * hop, hop):
                same_tracks(det.tracks(), g[tkey % k], "%s decision %d" % (scene, k), soft=REL_CAND,
                            level_rel=GPU_LEVEL_REL)
                k += 1
        assert k == len(decisions)
    det.close()
