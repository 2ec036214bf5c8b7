"""C2's grid in the chain: M = 1024 channels, D = 512, T = 16 (a 16,384-tap
prototype) at 61.44 MS/s cs16, which the generic fused channelizer kernel
covers (grids sized at run time). The batched chain's audio must equal the
plain chain's bit for bit, and the plain chain's the oracle chain's, across
runs of uneven sizes; with impulse excision on as well (the fused kernel then
reads the cleaned cf32 ring); and the chain replayed from a captured graph
must equal it directly launched.
"""
import numpy as np
import pytest

import signals
from oracle_chain import OracleChain
from revenant_gb300 import abi
from revenant_gb300.chain import Chain

pytestmark = pytest.mark.gpu

GRID, RATE = (1024, 16, 512), 61_440_000
RUNS = [1 << 17, 70_000, 1 << 16, 200_000, 12_345, 1 << 17]


def requests():
    return signals.random_receivers(12, RATE, seed=2, modes=("nfm", "am", "usb", "lsb"), bw=(3_000, 40_000),
                                    grid=GRID)


@pytest.fixture(scope="module")
def capture():
    n = sum(RUNS)
    z = signals.scene(n, RATE, [("nfm", 1_000_000, 0.3), ("am", -3_000_000, 0.3), ("usb", 7_500_000, 0.2)],
                      snr_db=30.0, seed=2)
    return signals.quantise(z, "cs16")


def feed(chain, codes, oracle=False, excise_at=None):
    at = 0
    for k, n in enumerate(RUNS):
        if excise_at is not None and k == excise_at:
            chain.set_impulse_excision(True, 15.0, 20e-6)
        part = codes[2 * at:2 * (at + n)]
        if oracle:
            chain.run(part, n)
        else:
            chain.run(part)
        at += n


def make(gpu, mode):
    ch = Chain(gpu, grid=GRID, rate=RATE, fmt=abi.FORMAT_CS16, mode=mode, max_run_samples=max(RUNS))
    ids = [ch.add_receiver(r) for r in requests()]
    return ch, ids


def audio_of(ch, ids):
    ch.drain()
    return [ch.audio(i) for i in ids]


def assert_same(a, b, what):
    for i, (x, y) in enumerate(zip(a, b)):
        assert x.size == y.size and x.size > 0, "%s: receiver %d sizes %d %d" % (what, i, x.size, y.size)
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), "%s: receiver %d differs" % (what, i)


def test_c2_plain_chain_matches_oracle(gpu, capture):
    oc = OracleChain(GRID, RATE, abi.FORMAT_CS16, requests(), ring_log2=21, chan_log2=12)
    feed(oc, capture, oracle=True)
    ch, ids = make(gpu, abi.CHAIN_PLAIN)
    feed(ch, capture)
    assert_same(audio_of(ch, ids), [oc.audio(i) for i in range(len(ids))], "plain vs oracle")
    ch.close()


@pytest.mark.parametrize("excise_at", [None, 2])
def test_c2_batched_chain_matches_plain(gpu, capture, excise_at):
    outs = []
    for mode in (abi.CHAIN_PLAIN, abi.CHAIN_BATCHED):
        ch, ids = make(gpu, mode)
        feed(ch, capture, excise_at=excise_at)
        outs.append(audio_of(ch, ids))
        ch.close()
    assert_same(outs[0], outs[1], "batched vs plain")


def test_c2_captured_chain_matches_direct(gpu, capture):
    outs = []
    for graph in (False, True):
        ch, ids = make(gpu, abi.CHAIN_BATCHED)
        if graph:
            ch.capture_graph()
        feed(ch, capture)
        outs.append(audio_of(ch, ids))
        ch.close()
    assert_same(outs[0], outs[1], "captured vs direct")
