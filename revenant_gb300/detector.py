"""Host mirror of the wideband detector API (rv_detector_*).

``Detector(device, config)`` wraps one rv_detector: feed spectrum frames with
``consume(frame_db, start, count)`` or many at once with ``consume_frames``,
read the latest decision's ``candidates()`` and the ``state()`` arrays. All the
work happens in librevenant_gb300.so.
"""
import ctypes as C

import numpy as np

from . import abi
from .library import check, lib


def _dtype(struct):
    return np.dtype([(name, np.int64 if t is C.c_int64 else np.uint64 if t is C.c_uint64 else
                      np.uint32 if t is C.c_uint32 else np.float64) for name, t in struct._fields_])


CANDIDATE_DTYPE = _dtype(abi.DetectorCandidate)
TRACK_DTYPE = _dtype(abi.DetectorTrack)


def _to_array(buf, n, struct, dtype):
    out = np.zeros(n, dtype)
    for i in range(n):
        for name, _ in struct._fields_:
            out[i][name] = getattr(buf[i], name)
    return out


def _read_tracks(fn, handle, all_tracks):
    n = C.c_uint32()
    check(fn(handle, int(all_tracks), None, 0, C.byref(n)))
    buf = (abi.DetectorTrack * max(n.value, 1))()
    check(fn(handle, int(all_tracks), buf, n.value, C.byref(n)))
    return _to_array(buf, n.value, abi.DetectorTrack, TRACK_DTYPE)


class Detector:
    def __init__(self, device, config):
        self.device = device
        self.config = config
        self.bins = config.bins
        handle = C.c_void_p()
        check(lib().rv_detector_create(device.handle, C.byref(config), C.byref(handle)))
        self.handle = handle

    def consume(self, frame_db, start, count):
        """One frame (numpy float32 of `bins` values on the host); True when it decided."""
        frame = np.ascontiguousarray(frame_db, np.float32)
        decided = C.c_int32()
        check(lib().rv_detector_consume(self.handle, frame.ctypes.data, start, count, 0, C.byref(decided)))
        return bool(decided.value)

    def consume_frames(self, frames, start, hop, count, device=False):
        """frames: numpy [n][bins] float32 on the host, or a device address (device=True, n = frames)."""
        made = C.c_uint32()
        if device:
            address, n = frames
            check(lib().rv_detector_consume_frames(self.handle, address, n, start, hop, count, 1, C.byref(made)))
        else:
            f = np.ascontiguousarray(frames, np.float32)
            check(lib().rv_detector_consume_frames(self.handle, f.ctypes.data, f.shape[0], start, hop, count, 0,
                                                   C.byref(made)))
        return made.value

    def candidates(self):
        n = C.c_uint32()
        check(lib().rv_detector_candidates(self.handle, None, 0, C.byref(n)))
        buf = (abi.DetectorCandidate * max(n.value, 1))()
        check(lib().rv_detector_candidates(self.handle, buf, n.value, C.byref(n)))
        return _to_array(buf, n.value, abi.DetectorCandidate, CANDIDATE_DTYPE)

    def tracks(self, all_tracks=False):
        """Detector::tracks (pending ones too with all_tracks)."""
        return _read_tracks(lib().rv_detector_tracks, self.handle, all_tracks)

    def state(self):
        avg = np.zeros(self.bins, np.float64)
        flo = np.zeros(self.bins, np.float64)
        check(lib().rv_detector_state(self.handle, avg.ctypes.data, flo.ctypes.data, self.bins))
        return avg, flo

    def stats(self):
        s = abi.DetectorStats()
        check(lib().rv_detector_get_stats(self.handle, C.byref(s)))
        return s

    def set_regions(self, ranges):
        """Confirm only inside bin ranges ([n][2] lo, hi), or the full band (None)."""
        if ranges is None:
            check(lib().rv_detector_set_regions(self.handle, None, 0))
            return
        r = np.ascontiguousarray(ranges, np.uint32).reshape(-1, 2)
        check(lib().rv_detector_set_regions(self.handle, r.ctypes.data, r.shape[0]))

    def log_candidates(self, enable=True):
        check(lib().rv_detector_log_candidates(self.handle, int(enable)))

    def read_log(self):
        """(instants, candidates) of every decision since the last read."""
        n = C.c_uint32()
        check(lib().rv_detector_read_log(self.handle, None, None, 0, C.byref(n)))
        buf = (abi.DetectorCandidate * max(n.value, 1))()
        inst = np.zeros(max(n.value, 1), np.uint64)
        check(lib().rv_detector_read_log(self.handle, inst.ctypes.data, buf, n.value, C.byref(n)))
        return inst[:n.value], _to_array(buf, n.value, abi.DetectorCandidate, CANDIDATE_DTYPE)

    def close(self):
        if self.handle:
            lib().rv_detector_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Tracker:
    """The tracker alone on the host (rv_tracker_*): candidates in, tracks out."""

    def __init__(self, config):
        handle = C.c_void_p()
        check(lib().rv_tracker_create(C.byref(config), C.byref(handle)))
        self.handle = handle

    def update(self, now, elapsed_seconds, candidates):
        """candidates: a sequence of abi.DetectorCandidate."""
        arr = (abi.DetectorCandidate * max(len(candidates), 1))(*candidates)
        check(lib().rv_tracker_update(self.handle, now, elapsed_seconds, arr, len(candidates)))

    def level_bins(self, bins):
        n = C.c_uint32()
        check(lib().rv_tracker_level_bins(self.handle, bins, None, 0, C.byref(n)))
        out = np.zeros((max(n.value, 1), 2), np.uint32)
        check(lib().rv_tracker_level_bins(self.handle, bins, out.ctypes.data, n.value, C.byref(n)))
        return out[:n.value]

    def fold_levels(self, bins, sums):
        """sums: [frames][tracks] float64 band powers for level_bins(bins)."""
        s = np.ascontiguousarray(sums, np.float64)
        check(lib().rv_tracker_fold_levels(self.handle, bins, s.ctypes.data, s.shape[0], s.shape[1]))

    def tracks(self, all_tracks=False):
        return _read_tracks(lib().rv_tracker_tracks, self.handle, all_tracks)

    def stats(self):
        s = abi.DetectorStats()
        check(lib().rv_tracker_get_stats(self.handle, C.byref(s)))
        return s

    def close(self):
        if self.handle:
            lib().rv_tracker_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
