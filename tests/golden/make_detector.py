"""Writes tests/golden/detector.npz from the reference's own wideband detector.

Runs core/detect/detector.cpp (compiled from the reference sources into
oracle/_ref/libdetref.so by oracle/ref/Makefile) over the seeded fixture scene
of tests/detector_scenes.py and stores the scene's quantised frames, every
decision's candidates and the averaged power and noise floor after the last
frame, so that machines without the reference sources can check
rv_detector_* against it.

    python tests/golden/make_detector.py
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
import detector_scenes as ds  # noqa: E402
from bindings import candidates_array, detector_reference, tracks_array  # noqa: E402
from revenant_gb300 import abi  # noqa: E402


def reference_tracks(lib, det):
    n = C.c_uint32()
    buf = (abi.DetectorTrack * 4096)()
    lib.refdet_tracks(det, buf, 4096, C.byref(n))
    return tracks_array(list(buf)[:n.value])


def run_reference(frames_q, cfg, hop):
    lib = detector_reference()
    if lib is None:
        raise SystemExit("oracle/_ref/libdetref.so is missing; run oracle/ref/Makefile first")
    det = C.c_void_p()
    if lib.refdet_create(C.byref(cfg), C.byref(det)) != 0:
        raise SystemExit(lib.refdet_last_error().decode())
    frames = ds.to_db(frames_q)
    decisions = []
    for f in range(frames.shape[0]):
        row = np.ascontiguousarray(frames[f])
        decided = C.c_int32()
        if lib.refdet_consume(det, row.ctypes.data, f * hop, hop, C.byref(decided)) != 0:
            raise SystemExit(lib.refdet_last_error().decode())
        if decided.value:
            n = C.c_uint32()
            buf = (abi.DetectorCandidate * 4096)()
            lib.refdet_candidates(det, buf, 4096, C.byref(n))
            decisions.append((f, candidates_array(list(buf)[:n.value]), reference_tracks(lib, det)))
    bins = frames.shape[1]
    avg, flo = np.zeros(bins), np.zeros(bins)
    lib.refdet_state(det, avg.ctypes.data, flo.ctypes.data, bins)
    st = abi.DetectorStats()
    lib.refdet_stats(det, C.byref(st))
    lib.refdet_destroy(det)
    return decisions, avg, flo, st


def main():
    fx = ds.FIXTURE
    frames_q = ds.scene(fx["bins"], fx["frames"], fx["seed"], fx["bands"])
    decisions, avg, flo, st = run_reference(frames_q, ds.fixture_config(abi), ds.FIXTURE_HOP)
    out = {"frames_q": frames_q, "average": avg, "floor": flo,
           "decision_frames": np.array([f for f, _, _ in decisions], np.int64),
           "stats": np.array([st.frames, st.decisions, st.candidates, st.peaks_overflowed,
                              st.candidates_residual], np.uint64),
           "track_stats": np.array([st.tracks_born, st.tracks_dropped, st.births_refused, st.merges, st.splits],
                                   np.uint64)}
    for k, (_, cands, tracks) in enumerate(decisions):
        out["candidates_%d" % k] = cands
        out["tracks_%d" % k] = tracks
    # the same scene with fast tracking: the tracker holds, drops, merges and
    # splits within the fixture (the candidates do not depend on tracking)
    fast, _, _, fst = run_reference(frames_q, ds.fast_tracking(ds.fixture_config(abi)), ds.FIXTURE_HOP)
    for k, ((f, cands, tracks), (f2, cands2, _)) in enumerate(zip(fast, decisions)):
        assert f == f2 and cands.tobytes() == cands2.tobytes()
        out["fast_tracks_%d" % k] = tracks
    out["fast_track_stats"] = np.array([fst.tracks_born, fst.tracks_dropped, fst.births_refused, fst.merges,
                                        fst.splits], np.uint64)
    # the tracker's scene: merges, splits, holds, drops, channels
    tr = ds.TRACKER
    trk_q = ds.scene(tr["bins"], tr["frames"], tr["seed"], tr["bands"])
    trk, _, _, tst = run_reference(trk_q, ds.tracker_config(abi), tr["bins"])
    out["trk_frames_q"] = trk_q
    out["trk_decision_frames"] = np.array([f for f, _, _ in trk], np.int64)
    for k, (_, cands, tracks) in enumerate(trk):
        out["trk_candidates_%d" % k] = cands
        out["trk_tracks_%d" % k] = tracks
    out["trk_track_stats"] = np.array([tst.tracks_born, tst.tracks_dropped, tst.births_refused, tst.merges,
                                       tst.splits], np.uint64)
    print("tracker scene: %d decisions, stats (born, dropped, refused, merges, splits) %s"
          % (len(trk), out["trk_track_stats"]))
    np.savez_compressed(os.path.join(HERE, "detector.npz"), **out)
    print("wrote detector.npz: %d decisions, %d candidates in total" % (len(decisions), sum(len(c) for _, c, _ in decisions)))
    for (f, c, t), (_, _, ft) in zip(decisions, fast):
        print(f, [(int(x["first_bin"]), int(x["last_bin"]), round(float(x["snr_2500_db"]), 2)) for x in c])
        print("   tracks", [(int(x["id"]), int(x["state"])) for x in t], "fast", [(int(x["id"]), int(x["state"]),
                                                                             int(x["merged_into"])) for x in ft])
    print("track stats", out["track_stats"], "fast", out["fast_track_stats"])


if __name__ == "__main__":
    main()
