"""A capture replays through the chain: a cu8 stream written by the segment
writer (rolling on size, blocks of uneven sizes), read back segment by
segment and fed to the batched chain, gives the audio the chain gives when fed
the stream directly, bit for bit; and a cs16 capture at 20 MS/s (the
detection workload's format) through the plain and batched chains alike.
"""
import numpy as np
import pytest

import signals
from revenant_gb300 import abi, capture
from revenant_gb300.chain import Chain

pytestmark = pytest.mark.gpu

ANCHOR = 1_791_806_400_000_000_000
C1_REQUESTS = [dict(center=200_000, bandwidth=200_000, demod="wfm"), dict(center=-300_000, bandwidth=12_500, demod="nfm"),
               dict(center=500_000, bandwidth=10_000, demod="am"), dict(center=100_000, bandwidth=3_000, demod="usb")]


def run_chain(gpu, grid, rate, fmt, reqs, parts, mode):
    ch = Chain(gpu, grid=grid, rate=rate, fmt=fmt, mode=mode, max_run_samples=1 << 18)
    ids = [ch.add_receiver(abi.request(**r)) for r in reqs]
    for p in parts:
        ch.run(p)
    ch.drain()
    out = [ch.audio(i) for i in ids]
    ch.close()
    return out


def write_capture(root, codes, runs, rate, center, fmt, bps_values, max_bytes):
    with capture.SegmentWriter(root, epoch=0x5EED, max_segment_bytes=max_bytes) as w:
        at = 0
        for n in runs:
            w.write(codes[at * bps_values:(at + n) * bps_values], at, rate, center, ANCHOR, fmt)
            at += n


def replayed(root, dtype):
    return [raw.view(dtype) for _, raw in capture.replay(root, 0x5EED)]


def assert_same(a, b):
    for x, y in zip(a, b):
        assert x.size == y.size and x.size > 0
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))


def test_cu8_capture_replays_bit_for_bit(gpu, tmp_path):
    runs = [4096, 30000, 65536, 1000, 20000, 10000]
    z = signals.scene(sum(runs), 2_400_000, [("wfm", 200_000, 1.0), ("nfm", -300_000, 0.3), ("am", 500_000, 0.3)],
                      snr_db=25.0, seed=11)
    codes = signals.quantise(z, "cu8")
    write_capture(tmp_path, codes, runs, 2_400_000, 98_000_000, "cu8", 2, max_bytes=50_000 * 2)
    parts = replayed(tmp_path, np.uint8)
    assert len(parts) > 2 and np.array_equal(np.concatenate(parts), codes)
    direct = run_chain(gpu, (8, 17, 4), 2_400_000, abi.FORMAT_CU8, C1_REQUESTS, [codes[:2 * 70_000], codes[2 * 70_000:]],
                       abi.CHAIN_BATCHED)
    again = run_chain(gpu, (8, 17, 4), 2_400_000, abi.FORMAT_CU8, C1_REQUESTS, parts, abi.CHAIN_BATCHED)
    assert_same(direct, again)


@pytest.mark.parametrize("mode", ["plain", "batched"])
def test_cs16_capture_at_20msps_replays_bit_for_bit(gpu, tmp_path, mode):
    runs = [1 << 16, 50_000, 1 << 17, 77_777, 1 << 16]
    rate = 20_000_000
    z = signals.scene(sum(runs), rate, [("nfm", 1_000_000, 0.3), ("am", -3_000_000, 0.3), ("usb", 7_500_000, 0.2)],
                      snr_db=30.0, seed=12)
    codes = signals.quantise(z, "cs16")
    write_capture(tmp_path, codes, runs, rate, 433_000_000, "cs16", 2, max_bytes=150_000 * 4)
    parts = replayed(tmp_path, np.int16)
    assert len(parts) >= 2 and np.array_equal(np.concatenate(parts), codes)
    reqs = [dict(center=1_000_000, bandwidth=12_500, demod="nfm"), dict(center=-3_000_000, bandwidth=10_000, demod="am"),
            dict(center=7_500_000, bandwidth=3_000, demod="usb")]
    m = abi.CHAIN_PLAIN if mode == "plain" else abi.CHAIN_BATCHED
    direct = run_chain(gpu, (64, 17, 32), rate, abi.FORMAT_CS16, reqs,
                       [codes[k:k + 2 * (1 << 17)] for k in range(0, codes.size, 2 * (1 << 17))], m)
    again = run_chain(gpu, (64, 17, 32), rate, abi.FORMAT_CS16, reqs, parts, m)
    assert_same(direct, again)
