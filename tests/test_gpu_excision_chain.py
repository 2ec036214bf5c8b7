"""Impulse excision inside the chain (Graph::plan_impulse_excision and
record_impulse_excision, core/engine/graph.cpp:1461-1525, 5025-5052).

The capture carries impulses of one to sixty samples (the stage's max_width
at 2.4 MS/s is 48) and a burst. With the stage switched on after the first
run, the plain chain (convert, front end, excision in place, then the
reference's recording with the channelizer held back to the stage's cleaned
end) must equal the oracle chain bit for bit, audio and counters; the batched
chain (converted and corrected into a cf32 ring, excised there, read by the
fused channelizer) must equal the plain chain; a pipelined captured chain
must equal a synchronous one; and the stage must have changed the audio.
"""
import numpy as np
import pytest

import signals
from oracle_chain import OracleChain
from revenant_gb300 import abi
from revenant_gb300.chain import Chain

pytestmark = pytest.mark.gpu

RATE = 2_400_000
GRID = (8, 17, 4)
RUNS = [8192, 30000, 16384, 4096, 20000, 40000, 12000, 30000, 25000]


def impulsive_capture(n, seed=5):
    z = signals.scene(n, RATE, [("wfm", 200_000, 1.0), ("am", 500_000, 0.3), ("nfm", -300_000, 0.3)], snr_db=30.0,
                      seed=seed)
    rng = np.random.default_rng(seed)
    pos = 12_000
    while pos < n - 100:
        w = int(rng.integers(1, 61))
        z[pos:pos + w] += rng.uniform(8, 20) * np.exp(2j * np.pi * rng.uniform(0, 1, w))
        pos += int(rng.integers(1_500, 6_000))
    z[100_000:103_000] += 6.0 * np.exp(2j * np.pi * 0.11 * np.arange(3000))  # a burst the stage spares
    return signals.quantise(z, "cs16")


def requests():
    return [abi.request(center=200_000, bandwidth=200_000, demod="wfm", stereo=True),
            abi.request(center=500_000, bandwidth=10_000, demod="am"),
            abi.request(center=-300_000, bandwidth=12_500, demod="nfm")]


def feed(chain, codes, switch_at=1, front_end=None, off_at=None, oracle=False):
    at = 0
    for k, n in enumerate(RUNS):
        if k == switch_at:
            chain.set_impulse_excision(True, 15.0, 20e-6)
            if front_end:
                chain.set_front_end(True, True, front_end)
        if off_at is not None and k == off_at:
            chain.set_impulse_excision(False)
        part = codes[2 * at:2 * (at + n)]
        if oracle:
            chain.run(part, n)
        else:
            chain.run(part)
        at += n


def make(mode, pipelined=False, captured=False):
    ch = Chain(GPU[0], grid=GRID, rate=RATE, fmt=abi.FORMAT_CS16, mode=mode, max_run_samples=max(RUNS),
               pipelined=pipelined)
    if captured:
        ch.capture_graph()
    ids = [ch.add_receiver(r) for r in requests()]
    return ch, ids


GPU = []


@pytest.fixture(autouse=True)
def _gpu(gpu):
    GPU[:] = [gpu]


@pytest.fixture(scope="module")
def codes():
    return impulsive_capture(sum(RUNS))


def audio_of(ch, ids):
    ch.drain()
    return [ch.audio(i) for i in ids]


def assert_same(a, b, what):
    for i, (x, y) in enumerate(zip(a, b)):
        assert x.size == y.size and x.size > 0, "%s: receiver %d sizes %d %d" % (what, i, x.size, y.size)
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), "%s: receiver %d differs" % (what, i)


def test_plain_chain_excision_matches_oracle(codes):
    oc = OracleChain(GRID, RATE, abi.FORMAT_CS16, requests())
    orig = oc.set_impulse_excision

    def set_ex(on, threshold_db=15.0, max_width_seconds=20e-6):
        orig(on, threshold_db, max_width_seconds, max_block=max(RUNS))
    oc.set_impulse_excision = set_ex
    feed(oc, codes, oracle=True)
    ch, ids = make(abi.CHAIN_PLAIN)
    feed(ch, codes)
    assert_same(audio_of(ch, ids), [oc.audio(i) for i in range(len(ids))], "plain vs oracle")
    got = ch.excision_counters()
    want = (int(oc.ex_counters[0]), int(oc.ex_counters[1]), int(oc.ex_counters[2]), oc.ex_examined)
    assert got == want, (got, want)
    assert got[1] > 10 and got[2] >= 1  # impulses excised, the burst spared
    ch.close()


@pytest.mark.parametrize("front_end", [None, 1])
def test_batched_chain_excision_matches_plain(codes, front_end):
    outs, counts = [], []
    for mode in (abi.CHAIN_PLAIN, abi.CHAIN_BATCHED):
        ch, ids = make(mode)
        feed(ch, codes, front_end=front_end)
        outs.append(audio_of(ch, ids))
        counts.append(ch.excision_counters())
        ch.close()
    assert_same(outs[0], outs[1], "batched vs plain")
    assert counts[0] == counts[1]


def test_batched_chain_excision_switched_off_matches_plain(codes):
    outs = []
    for mode in (abi.CHAIN_PLAIN, abi.CHAIN_BATCHED):
        ch, ids = make(mode)
        feed(ch, codes, off_at=6)
        outs.append(audio_of(ch, ids))
        ch.close()
    assert_same(outs[0], outs[1], "batched vs plain, excision off at run 6")


def test_pipelined_captured_chain_excision_matches_synchronous(codes):
    outs = []
    for pipelined, captured in ((False, False), (True, True)):
        ch, ids = make(abi.CHAIN_BATCHED, pipelined=pipelined, captured=captured)
        feed(ch, codes, front_end=2)
        outs.append(audio_of(ch, ids))
        ch.close()
    assert_same(outs[0], outs[1], "pipelined captured vs synchronous")


def test_excision_changes_the_audio(codes):
    outs = []
    for on in (False, True):
        ch, ids = make(abi.CHAIN_BATCHED)
        feed(ch, codes, switch_at=1 if on else -1)
        outs.append(audio_of(ch, ids))
        ch.close()
    # the held-back channelizer hands out fewer samples by the end, and what
    # it hands out differs where impulses were cut
    for x, y in zip(outs[0], outs[1]):
        n = min(x.size, y.size)
        assert n > 0 and not np.array_equal(x[:n].view(np.uint32), y[:n].view(np.uint32))
