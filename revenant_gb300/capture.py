"""Host mirror of the rolling capture's segments (rv_capture_*; the reference's
core/capture/writer.h SegmentWriter and recover_open_segments).

``SegmentWriter(root, epoch=..., max_segment_bytes=...)`` takes source blocks
(``write(samples, first_index, rate=, center=, anchor_ns=, fmt=,
dropped_before=)``) and rolls SigMF segments under ``root`` on loss, restart,
format, rate, retune and size; ``annotate`` files a detector track into every
segment it overlaps. ``segments(root)`` lists the closed segments, ``read``
returns one's samples, ``replay`` yields a stream's samples back in index
order, and ``recover(root)`` closes what a writer that died left open. All the
work happens in librevenant_gb300.so.
"""
import ctypes as C

import numpy as np

from . import abi
from .library import check, lib

FORMATS = {"cu8": 0, "cs8": 1, "cs16": 2, "cs24": 3}
BYTES_PER_SAMPLE = {0: 2, 1: 2, 2: 4, 3: 6}


def _bytes(path):
    return str(path).encode()


def _format(fmt):
    return FORMATS[fmt] if isinstance(fmt, str) else int(fmt)


def annotation(sample_count, freq_lower, freq_upper, confidence=0.0, peak_db=0.0, snr_db=0.0, family="",
               track_id=None):
    a = abi.CaptureAnnotation()
    a.sample_count, a.freq_lower, a.freq_upper = sample_count, freq_lower, freq_upper
    a.confidence, a.peak_db, a.snr_db = confidence, peak_db, snr_db
    a.family = family.encode()
    if track_id is not None:
        a.has_track_id, a.track_id = 1, track_id
    return a


class SegmentWriter:
    def __init__(self, root, epoch=0, max_segment_bytes=0, max_segment_seconds=0.0, retention_bytes=0,
                 retention_max_age_ns=0, recover_on_start=True, hw=""):
        cfg = abi.CaptureConfig()
        cfg.max_segment_bytes, cfg.max_segment_seconds = max_segment_bytes, max_segment_seconds
        cfg.retention_bytes, cfg.retention_max_age_ns = retention_bytes, retention_max_age_ns
        cfg.stream_epoch, cfg.recover_on_start = epoch, int(recover_on_start)
        handle = C.c_void_p()
        check(lib().rv_capture_writer_open(_bytes(root), C.byref(cfg), hw.encode(), C.byref(handle)))
        self.handle = handle

    def write(self, data, first_index, rate, center, anchor_ns=0, fmt="cs16", dropped_before=0):
        """One source block: `data` is the block's raw bytes (any numpy array
        or bytes object in the format's layout)."""
        f = _format(fmt)
        raw = np.ascontiguousarray(np.frombuffer(data, np.uint8) if isinstance(data, (bytes, bytearray))
                                   else data).view(np.uint8).reshape(-1)
        b = abi.CaptureBlock()
        b.first_index, b.epoch_anchor_ns, b.rate, b.center = first_index, anchor_ns, rate, center
        b.sample_count, b.dropped_before, b.format = raw.size // BYTES_PER_SAMPLE.get(f, 2), dropped_before, f
        check(lib().rv_capture_writer_write(self.handle, C.byref(b), raw.ctypes.data, raw.size))

    def set_gain(self, gain_db):
        check(lib().rv_capture_writer_set_gain(self.handle, int(gain_db is not None), gain_db or 0.0))

    def annotate(self, absolute_start, ann):
        check(lib().rv_capture_writer_annotate(self.handle, absolute_start, C.byref(ann)))

    def set_clock(self, now_ns):
        check(lib().rv_capture_writer_set_clock(self.handle, now_ns))

    def stats(self):
        s = abi.CaptureWriterStats()
        check(lib().rv_capture_writer_get_stats(self.handle, C.byref(s)))
        return s.as_dict()

    def close(self):
        if self.handle:
            h, self.handle = self.handle, None
            check(lib().rv_capture_writer_close(h))

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def segments(root):
    """The closed segments under root by day then stem (rv_capture_segment list)."""
    n = C.c_uint32()
    check(lib().rv_capture_list(_bytes(root), None, 0, C.byref(n)))
    buf = (abi.CaptureSegment * max(n.value, 1))()
    check(lib().rv_capture_list(_bytes(root), buf, n.value, C.byref(n)))
    return list(buf[:n.value])


def read(root, segment, offset=0, count=None):
    """The segment's raw bytes for samples [offset, offset + count)."""
    count = segment.samples - offset if count is None else count
    out = np.empty(count * BYTES_PER_SAMPLE[segment.format], np.uint8)
    check(lib().rv_capture_read(_bytes(root), C.byref(segment), offset, count, out.ctypes.data))
    return out


def replay(root, stream_epoch=None):
    """(segment, raw bytes) of one stream epoch's segments in index order."""
    segs = [s for s in segments(root) if stream_epoch is None or s.stream_epoch == stream_epoch]
    for s in sorted(segs, key=lambda s: (s.stream_epoch, s.first_index)):
        yield s, read(root, s)


def recover(root):
    """{recovered, removed_empty, failed} after closing dead writers' segments."""
    counts = (C.c_uint32 * 3)()
    check(lib().rv_capture_recover(_bytes(root), counts))
    return dict(recovered=counts[0], removed_empty=counts[1], failed=counts[2])
