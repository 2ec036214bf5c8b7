"""The rolling capture's segments (core/capture/writer.cpp, format.h) against
the reference's own SegmentWriter compiled into oracle/_ref/libcapref.so: the
same blocks, gains and annotations through both writers leave the same files,
byte for byte (data, meta and names), across the roll reasons (size, retune,
loss, rate, format, restart), retention by bytes and by age, annotations that
span segments, and recovery of segments a dead writer left open. Then the
catalog and reader give back exactly what was written, the stems parse, and
the reference's own writer-test cases hold (tests/capture/test_writer.cpp).
"""
import ctypes as C
import json
import os

import numpy as np
import pytest

from revenant_gb300 import capture
from revenant_gb300.library import LibraryError

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CAPREF = os.path.join(ROOT, "oracle", "_ref", "libcapref.so")

RATE = 1_000_000
ANCHOR = 1_791_806_400_000_000_000  # 2026-10-12T12:00:00Z
BLOCK = 1000
HW = 'test "dongle"\nline two'
HALF_DAY = 43_200


class RefWriter:
    """The reference's SegmentWriter through the shim, with capture.SegmentWriter's calls."""

    def __init__(self, lib, root, epoch=0, max_segment_bytes=0, max_segment_seconds=0.0, retention_bytes=0,
                 retention_max_age_ns=0, recover_on_start=True, hw="", now_ns=0):
        self.lib = lib
        self.h = lib.refcap_open(str(root).encode(), max_segment_bytes, max_segment_seconds, retention_bytes,
                                 retention_max_age_ns, epoch, int(recover_on_start), hw.encode(), now_ns)
        assert self.h

    def write(self, data, first_index, rate, center, anchor_ns=0, fmt="cs16", dropped_before=0):
        f = capture.FORMATS[fmt]
        raw = np.ascontiguousarray(data).view(np.uint8).reshape(-1)
        n = raw.size // capture.BYTES_PER_SAMPLE[f]
        assert self.lib.refcap_write(self.h, first_index, anchor_ns, rate, center, n, dropped_before, f,
                                     raw.ctypes.data, raw.size) == 0

    def set_gain(self, gain_db):
        self.lib.refcap_set_gain(self.h, int(gain_db is not None), gain_db or 0.0)

    def set_clock(self, now_ns):
        self.lib.refcap_set_clock(self.h, now_ns)

    def annotate(self, start, a):
        self.lib.refcap_annotate(self.h, start, a.sample_count, a.freq_lower, a.freq_upper, a.confidence,
                                 a.peak_db, a.snr_db, a.has_track_id, a.track_id, a.family)

    def stats(self):
        out = (C.c_uint64 * 7)()
        self.lib.refcap_stats(self.h, out)
        keys = ("segments_written", "bytes_written", "segments_deleted", "annotations_discarded",
                "annotations_merged_late", "retained_bytes", "stream_epoch")
        return dict(zip(keys, out))

    def close(self):
        self.lib.refcap_close(self.h)


@pytest.fixture(scope="module")
def capref():
    if not os.path.exists(CAPREF):
        pytest.skip("reference capture writer not built (reference sources absent on this machine)")
    lib = C.CDLL(CAPREF)
    lib.refcap_open.restype = C.c_void_p
    lib.refcap_open.argtypes = [C.c_char_p, C.c_uint64, C.c_double, C.c_uint64, C.c_int64, C.c_uint64, C.c_int,
                                C.c_char_p, C.c_int64]
    lib.refcap_write.argtypes = [C.c_void_p, C.c_uint64, C.c_int64, C.c_int64, C.c_int64, C.c_uint64, C.c_uint64,
                                 C.c_int, C.c_void_p, C.c_uint64]
    lib.refcap_set_gain.argtypes = [C.c_void_p, C.c_int, C.c_double]
    lib.refcap_set_clock.argtypes = [C.c_void_p, C.c_int64]
    lib.refcap_annotate.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64, C.c_int64, C.c_int64, C.c_double,
                                    C.c_double, C.c_double, C.c_int, C.c_uint64, C.c_char_p]
    lib.refcap_stats.argtypes = [C.c_void_p, C.c_void_p]
    lib.refcap_close.argtypes = [C.c_void_p]
    lib.refcap_recover.argtypes = [C.c_char_p, C.c_void_p]
    return lib


def block_bytes(start, count, fmt="cu8"):
    """Each sample's bytes depend on its index, so a sample out of place shows."""
    idx = np.arange(start, start + count, dtype=np.uint64)
    bps = capture.BYTES_PER_SAMPLE[capture.FORMATS[fmt]]
    out = np.empty((count, bps), np.uint8)
    for k in range(bps):
        out[:, k] = ((idx * np.uint64(7) + np.uint64(k)) >> np.uint64(8 * (k % 4))) & np.uint64(0xFF)
    return out.reshape(-1)


def tree(root):
    """{relative path: bytes} of every file under root."""
    out = {}
    for d, _, files in os.walk(root):
        for f in files:
            p = os.path.join(d, f)
            with open(p, "rb") as fh:
                out[os.path.relpath(p, root)] = fh.read()
    return out


def assert_same_tree(a, b):
    ta, tb = tree(a), tree(b)
    assert sorted(ta) == sorted(tb)
    for k in ta:
        assert ta[k] == tb[k], k


def both(capref, tmp_path, script, **cfg):
    """Run one script of writer calls through both writers; their roots."""
    roots = []
    for kind in ("rv", "ref"):
        root = tmp_path / kind
        w = capture.SegmentWriter(root, **cfg) if kind == "rv" else RefWriter(capref, root, **cfg)
        script(w)
        w.close()
        roots.append(root)
    return roots


def metas(root):
    out = []
    for d, _, files in os.walk(root):
        for f in sorted(files):
            if f.endswith(".sigmf-meta"):
                with open(os.path.join(d, f)) as fh:
                    out.append((f, json.load(fh)))
    return sorted(out, key=lambda m: m[1]["global"]["revenant:first_index"])


def test_roll_reasons_match_reference(capref, tmp_path):
    """tests/capture/test_writer.cpp "Segments roll on retune, rate, size and loss"."""
    def script(w):
        at = 0
        for _ in range(5):
            w.write(block_bytes(at, BLOCK), at, RATE, 100_000_000, ANCHOR, "cu8")
            at += BLOCK
        w.write(block_bytes(at, BLOCK), at, RATE, 101_000_000, ANCHOR, "cu8")
        at += BLOCK
        w.write(block_bytes(at + 500, BLOCK), at + 500, RATE, 101_000_000, ANCHOR, "cu8", dropped_before=500)
        at += 500 + BLOCK
        w.write(block_bytes(at, BLOCK), at, 2 * RATE, 101_000_000, ANCHOR, "cu8")

    a, b = both(capref, tmp_path, script, epoch=0x1234, max_segment_bytes=4 * BLOCK * 2, hw=HW)
    assert_same_tree(a, b)
    m = metas(a)
    assert [x[1]["global"]["revenant:close_reason"] for x in m] == ["size", "retune", "loss", "rate", "stop"]
    assert m[3][1]["global"]["revenant:dropped_before"] == 500 and m[1][1]["global"]["revenant:dropped_before"] == 0
    assert not any(".open" in k for k in tree(a))


@pytest.mark.parametrize("fmt", ["cu8", "cs8", "cs16", "cs24"])
def test_formats_gain_and_seconds_limit_match_reference(capref, tmp_path, fmt):
    def script(w):
        at = 0
        w.set_gain(29.7)
        for k in range(7):
            if k == 3:
                w.set_gain(None)
            if k == 5:
                w.set_gain(-3.25)
            w.write(block_bytes(at, BLOCK, fmt), at, 4 * BLOCK, -145_500_000, ANCHOR + 123_456_789, fmt)
            at += BLOCK
        # a format change closes with "format"
        other = "cs16" if fmt != "cs16" else "cu8"
        w.write(block_bytes(at, BLOCK, other), at, 4 * BLOCK, -145_500_000, ANCHOR + 123_456_789, other)

    a, b = both(capref, tmp_path, script, epoch=0xABCDEF0123, max_segment_seconds=0.5, hw="rtl\tsdr")
    assert_same_tree(a, b)
    reasons = [x[1]["global"]["revenant:close_reason"] for x in metas(a)]
    assert reasons[-2:] == ["format", "stop"] and "size" in reasons


def test_meta_keys_stem_and_annotations(tmp_path):
    """tests/capture/test_writer.cpp "A meta carries every key format.h names"."""
    root = tmp_path / "c"
    with capture.SegmentWriter(root, epoch=0x1234, hw=HW) as w:
        w.set_gain(29.7)
        for at in range(0, 4 * BLOCK, BLOCK):
            w.write(block_bytes(at, BLOCK), at, RATE, 145_500_000, ANCHOR, "cu8")
        w.annotate(2500, capture.annotation(1500, 145_490_000, 145_510_000, 0.75, -20.5, 18.0, "nbfm", 42))
    (day, files), = [(os.path.basename(d), f) for d, _, f in os.walk(root) if f]
    assert day == "2026-10-12"
    assert sorted(files) == ["rev-20261012T120000.000Z-145500000-0000000000001234-0.sigmf-data",
                             "rev-20261012T120000.000Z-145500000-0000000000001234-0.sigmf-meta"]
    text = open(os.path.join(root, day, sorted(files)[1])).read()
    for key in ['"core:datatype":"cu8"', '"core:sample_rate":1000000', '"core:version":"1.',
                '"core:recorder":"Revenant ', '"core:hw":"test \\"dongle\\"\\nline two"', '"name":"revenant"',
                '"version":"1.1.0"', '"optional":true', '"revenant:stream_epoch":4660', '"revenant:first_index":0',
                '"revenant:epoch_anchor_ns":1791806400000000000', '"revenant:dropped_before":0',
                '"revenant:close_reason":"stop"', '"revenant:gain_db":29.7', '"core:frequency":145500000',
                '"core:datetime":"2026-10-12T12:00:00.000000000Z"', '"core:sample_start":2500',
                '"core:sample_count":1500', '"core:freq_lower_edge":145490000', '"core:label":"nbfm"',
                '"core:generator":"revenant-detect"', '"revenant:confidence":0.75', '"revenant:family":"nbfm"',
                '"revenant:track_id":42']:
        assert key in text, key
    seg, = capture.segments(root)
    assert seg.samples == 4 * BLOCK and seg.has_gain and seg.gain_db == 29.7 and seg.center == 145_500_000


def test_annotations_across_segments_match_reference(capref, tmp_path):
    """tests/capture/test_writer.cpp "A track spanning closed segments is filed in
    every one with its id": parts inside closed segments merge late, parts
    past the open segment wait for the next."""
    def script(w):
        at = 0
        for k in range(9):
            w.write(block_bytes(at, BLOCK), at, RATE, 100_000_000, ANCHOR, "cu8")
            at += BLOCK
            if k == 4:  # spans segments 0 and 1 (both closed by now) and the open one
                w.annotate(1500, capture.annotation(3000, 99_990_000, 100_010_000, 0.5, -30.0, 12.0, "", 7))
            if k == 5:  # a point inside a closed segment, and one past the stream's end so far
                w.annotate(2100, capture.annotation(0, 1, 2, 0.25, -40.0, 6.0, "am"))
                w.annotate(8200, capture.annotation(600, 5, 9, 1.0, float("inf"), -1.5, "usb", 8))
        w.annotate(8900, capture.annotation(2000, 3, 4, 0.125, -1.0, 2.0, "ft8", 9))

    a, b = both(capref, tmp_path, script, epoch=77, max_segment_bytes=2 * BLOCK * 2)
    ma, mb = metas(a), metas(b)
    assert [x[0] for x in ma] == [x[0] for x in mb]
    for (_, x), (_, y) in zip(ma, mb):
        key = lambda e: (e["core:sample_start"], e["core:sample_count"], e["core:freq_lower_edge"])
        assert sorted(x.pop("annotations"), key=key) == sorted(y.pop("annotations"), key=key)
        assert x == y
    filed = [(m[1]["global"]["revenant:first_index"], e["core:sample_start"], e["core:sample_count"],
              e.get("revenant:track_id")) for m in metas(a) for e in m[1]["annotations"]]
    assert (0, 1500, 500, 7) in filed and (2000, 0, 2000, 7) in filed and (4000, 0, 500, 7) in filed
    assert (2000, 100, 0, None) in filed and (8000, 200, 600, 8) in filed and (8000, 900, 100, 9) in filed


def test_restart_opens_a_new_epoch(capref, tmp_path):
    for kind in ("rv", "ref"):
        root = tmp_path / kind
        w = capture.SegmentWriter(root, epoch=5) if kind == "rv" else RefWriter(capref, root, epoch=5)
        w.write(block_bytes(0, BLOCK), 0, RATE, 1, ANCHOR, "cu8")
        w.write(block_bytes(BLOCK, BLOCK), BLOCK, RATE, 1, ANCHOR, "cu8")
        w.write(block_bytes(0, BLOCK), 0, RATE, 1, ANCHOR, "cu8")  # index went back: a new run
        epoch = w.stats()["stream_epoch"]
        w.close()
        m = metas(root)
        assert [x[1]["global"]["revenant:close_reason"] for x in m] == ["stop", "stop"]
        epochs = {x[1]["global"]["revenant:stream_epoch"] for x in m}
        assert 5 in epochs and epoch in epochs and epoch != 5 and 0 < epoch < 1 << 63


@pytest.mark.parametrize("mode", ["bytes", "age"])
def test_retention_matches_reference(capref, tmp_path, mode):
    """tests/capture/test_writer.cpp retention cases: oldest closed segments go
    first, and an emptied day directory goes with them."""
    day = 86_400 * 10**9
    cfg = dict(epoch=3, max_segment_bytes=3 * HALF_DAY * 2)
    if mode == "bytes":
        cfg["retention_bytes"] = 8 * HALF_DAY * 2 + 3000
    else:
        cfg["retention_max_age_ns"] = 2 * day

    def script(w):
        # at 1 S/s a block of 43,200 samples is half a day, so segments fall
        # in several day directories; the clock reads the end of each block
        at = 0
        for k in range(12):
            w.set_clock(ANCHOR + (k + 1) * day // 2)
            w.write(block_bytes(at, HALF_DAY), at, 1, 7, ANCHOR, "cu8")
            at += HALF_DAY

    a, b = both(capref, tmp_path, script, **cfg)
    assert_same_tree(a, b)
    assert 0 < len(tree(a)) < 2 * 4  # some segments were deleted
    days = sorted(os.listdir(a))
    assert days == sorted(os.listdir(b)) and all(os.listdir(os.path.join(a, d)) for d in days)


def test_recovery_matches_reference(capref, tmp_path):
    """tests/capture/test_writer.cpp "Recovery finalises a segment a dead writer
    left open": a partial trailing sample is cut, an empty leftover removed, a
    meta already present kept, a leftover without its side file reported."""
    def plant(root):
        d = root / "2026-10-12"
        d.mkdir(parents=True)
        stems = ["rev-20261012T120000.000Z-100000000-0000000000000001-0",
                 "rev-20261012T120001.000Z--2500-0000000000000001-1000000",
                 "rev-20261012T120002.000Z-7-0000000000000001-2000000",
                 "rev-20261012T120003.000Z-7-0000000000000001-3000000"]
        (d / (stems[0] + ".open.sigmf-data")).write_bytes(block_bytes(0, 777, "cs16").tobytes() + b"\x01\x02")
        (d / (stems[0] + ".open.revenant")).write_text(
            "rate=1000000\nformat=cs16\nanchor_ns=%d\ndropped_before=12\ngain_db=7.5\nhw=dongle x\n" % ANCHOR)
        (d / (stems[1] + ".open.sigmf-data")).write_bytes(b"")
        (d / (stems[1] + ".open.revenant")).write_text("rate=1000000\nformat=cu8\nanchor_ns=%d\n" % ANCHOR)
        (d / (stems[2] + ".open.sigmf-data")).write_bytes(block_bytes(5, 100, "cu8").tobytes())
        (d / (stems[2] + ".open.revenant")).write_text(
            "rate=1000000\nformat=cu8\nanchor_ns=%d\ndropped_before=0\nhw=\n" % ANCHOR)
        (d / (stems[2] + ".sigmf-meta")).write_text('{"kept": true}\n')
        (d / (stems[3] + ".open.sigmf-data")).write_bytes(b"abcd")

    for kind in ("rv", "ref"):
        plant(tmp_path / kind)
    got = capture.recover(tmp_path / "rv")
    out = (C.c_uint64 * 3)()
    assert capref.refcap_recover(str(tmp_path / "ref").encode(), out) == 0
    assert (got["recovered"], got["removed_empty"], got["failed"]) == tuple(out) == (2, 1, 1)
    assert_same_tree(tmp_path / "rv", tmp_path / "ref")


def test_recover_on_start_then_write(capref, tmp_path):
    """A writer opened over a dead writer's leftovers closes them first and
    its retention counts them."""
    def plant(root):
        d = root / "2026-10-12"
        d.mkdir(parents=True)
        stem = "rev-20261012T115959.000Z-5-0000000000000009-0"
        (d / (stem + ".open.sigmf-data")).write_bytes(block_bytes(0, 3000, "cu8").tobytes())
        (d / (stem + ".open.revenant")).write_text("rate=1000000\nformat=cu8\nanchor_ns=%d\n" % (ANCHOR - 10**9))

    for kind in ("rv", "ref"):
        plant(tmp_path / kind)

    def script(w):
        for at in range(0, 6 * BLOCK, BLOCK):
            w.write(block_bytes(at, BLOCK), at, RATE, 5, ANCHOR, "cu8")

    a, b = both(capref, tmp_path, script, epoch=10, max_segment_bytes=2 * BLOCK * 2,
                retention_bytes=3 * 2 * BLOCK * 2 + 2000)
    assert_same_tree(a, b)
    assert not any(k.startswith("2026-10-12/rev-20261012T115959") for k in tree(a))  # recovered, then aged out


def test_catalog_read_and_replay_round_trip(tmp_path):
    root = tmp_path / "c"
    rng = np.random.default_rng(1)
    stream = rng.integers(-32768, 32767, size=(50_000, 2), dtype=np.int16)
    runs = [4096, 10_000, 1, 7_000, 8192, 20_711]
    with capture.SegmentWriter(root, epoch=99, max_segment_bytes=30_000 * 4) as w:
        at = 0
        for n in runs:
            w.write(stream[at:at + n], at, 2_400_000, 433_920_000, ANCHOR, "cs16")
            at += n
    segs = capture.segments(root)
    assert [s.close_reason for s in segs] == [b"size", b"stop"]
    assert sum(s.samples for s in segs) == stream.shape[0]
    got = np.concatenate([raw for _, raw in capture.replay(root, 99)]).view(np.int16).reshape(-1, 2)
    assert np.array_equal(got, stream)
    s = segs[1]
    part = capture.read(root, s, 1000, 333).view(np.int16).reshape(-1, 2)
    assert np.array_equal(part, stream[s.first_index + 1000:s.first_index + 1333])
    with pytest.raises(LibraryError):
        capture.read(root, s, s.samples - 10, 11)


def test_bad_blocks_are_rejected(tmp_path):
    with capture.SegmentWriter(tmp_path / "c", epoch=1) as w:
        with pytest.raises(LibraryError):
            w.write(np.zeros(10, np.uint8), 0, 0, 1, fmt="cu8")  # rate must be positive
        with pytest.raises(LibraryError):
            w.write(np.zeros(10, np.uint8), 0, RATE, 1, fmt=9)  # unknown format
        w.write(np.zeros(0, np.uint8), 0, RATE, 1, fmt="cu8")  # an empty block opens nothing on disk
    assert capture.segments(tmp_path / "c") == []
