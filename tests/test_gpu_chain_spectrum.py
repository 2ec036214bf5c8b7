"""The chain's spectrum stage (Graph::on_block's spectrum dispatch) and an
attached detector.

Per run the frame must equal the oracle's spectrum (core/dsp/
spectrum_reference.cpp, restated) of the oracle chain's channel ring over the
same blocks, bit for bit, with the engine's SpectrumFrame start and count; the
batched chain's frames must equal the plain chain's; a detector attached to a
chain must decide exactly as one fed the same frames from the host.
"""
import ctypes as C

import numpy as np
import pytest

import signals
from bindings import same_bits
from oracle_chain import OracleChain
from revenant_gb300 import abi
from revenant_gb300.chain import Chain
from revenant_gb300.library import lib

pytestmark = pytest.mark.gpu

RATE, GRID, N = 2_400_000, (8, 17, 4), 512
RUNS = [8192, 30000, 16384, 4096, 20000, 40000, 12000, 30000]


@pytest.fixture(scope="module")
def codes():
    z = signals.scene(sum(RUNS), RATE, [("wfm", 200_000, 1.0), ("am", 500_000, 0.3), ("nfm", -300_000, 0.3)],
                      snr_db=30.0, seed=12)
    return signals.quantise(z, "cu8")


def oracle_frame(oc, first_block, blocks):
    one_past = first_block + blocks
    if blocks == 0 or one_past < N:
        return None
    M = GRID[0]
    tw = np.zeros((N, 2), np.float32)
    assert lib().rv_build_twiddles(N, tw.ctypes.data, N) == 0
    win = np.zeros(N + N // 2, np.float32)
    assert lib().rv_build_spectrum_window(N, GRID[1], 120.0, win.ctypes.data, win.size) == 0
    p = abi.SpectrumParams()
    p.channels, p.transform, p.stages = M, N, int(np.log2(N))
    p.chan_blocks, p.chan_mask = oc.chan_blocks, oc.chan_blocks - 1
    p.in_offset = (one_past - N) & (oc.chan_blocks - 1)
    out = np.zeros(M * N // 2, np.float32)
    assert oc.ora.spectrum(p, oc.chan, tw, win, out) == 0
    return out


def test_chain_spectrum_frames_match_oracle(gpu, codes):
    oc = OracleChain(GRID, RATE, abi.FORMAT_CU8, [])
    chains = {}
    for mode in (abi.CHAIN_PLAIN, abi.CHAIN_BATCHED):
        ch = Chain(gpu, grid=GRID, rate=RATE, fmt=abi.FORMAT_CU8, mode=mode, max_run_samples=max(RUNS))
        ch.add_receiver(abi.request(center=500_000, bandwidth=10_000, demod="am"))
        ch.set_spectrum(N)
        chains[mode] = ch
    at, seq = 0, 0
    D = GRID[2]
    group_delay = GRID[0] * (GRID[1] - 1) // 2
    for n in RUNS:
        first_block = oc.next_block
        oc.run(codes[2 * at:2 * (at + n)], n)
        blocks = oc.next_block - first_block
        want = oracle_frame(oc, first_block, blocks)
        frames = []
        for mode, ch in chains.items():
            ch.run(codes[2 * at:2 * (at + n)])
            frame, start, count, sequence = ch.spectrum()
            frames.append(frame)
            if want is not None:
                assert same_bits(frame, want), "mode %d run at %d" % (mode, at)
                assert start == (first_block + blocks - N) * D - group_delay and count == N * D
        if want is not None:
            seq += 1
        assert chains[abi.CHAIN_BATCHED].spectrum()[3] == seq
        at += n
    for ch in chains.values():
        ch.close()


def test_attached_detector_decides_as_a_standalone_one(gpu, codes):
    from revenant_gb300.detector import Detector
    import detector_scenes as ds
    bins = GRID[0] * N // 2
    cfg = ds.fixture_config(abi)
    cfg.bins, cfg.source_rate, cfg.source_center = bins, RATE, 100_000_000
    cfg.bin_width_numerator, cfg.bin_width_denominator = RATE, GRID[0] * N
    cfg.bin_zero_numerator, cfg.bin_zero_denominator = -RATE // 2, 1
    cfg.average_seconds, cfg.decision_interval_seconds = 0.01, 0.005
    attached, standalone = Detector(gpu, cfg), Detector(gpu, cfg)
    ch = Chain(gpu, grid=GRID, rate=RATE, fmt=abi.FORMAT_CU8, mode=abi.CHAIN_BATCHED, max_run_samples=max(RUNS))
    ch.add_receiver(abi.request(center=500_000, bandwidth=10_000, demod="am"))
    ch.set_spectrum(N, attached)
    at, last_seq = 0, 0
    for n in RUNS * 2:
        n = min(n, len(codes) // 2 - at)
        if n <= 0:
            break
        ch.run(codes[2 * at:2 * (at + n)])
        frame, start, count, seq = ch.spectrum()
        if seq != last_seq:
            standalone.consume(frame, start, count)
            last_seq = seq
        at += n
    assert attached.stats().frames == standalone.stats().frames > 0
    assert attached.stats().decisions == standalone.stats().decisions > 0
    assert attached.candidates().tobytes() == standalone.candidates().tobytes()
    a, b = attached.state(), standalone.state()
    assert same_bits(a[0], b[0]) and same_bits(a[1], b[1])
    ch.close()
    attached.close()
    standalone.close()
