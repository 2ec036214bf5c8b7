"""Front-end correction inside the chain (Graph::record_front_end_correction).

The input carries a DC offset and an IQ imbalance. The plain chain (moments,
estimate, in-place correction, then the reference's recording) must equal the
oracle chain bit for bit; the batched chain, whose fused kernel corrects each
sample with the parameters of the run it arrived in, must equal the plain
chain; a pipelined captured chain (estimate two runs behind) must equal a
synchronous chain with the same lag. The estimate read back must be the
oracle's.
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
RUNS = [8192, 30000, 16384, 4096, 20000, 40000, 12000, 30000]  # the correction switches on after run 1


def impaired_capture(n, seed=11):
    z = signals.scene(n, RATE, [("wfm", 200_000, 1.0), ("am", 500_000, 0.3), ("nfm", -300_000, 0.3)], snr_db=30.0,
                      seed=seed)
    i = z.real + 0.04
    q = 1.15 * (z.imag * np.cos(np.deg2rad(5.0)) + z.real * np.sin(np.deg2rad(5.0))) - 0.03
    return signals.quantise(i + 1j * q, "cu8")


def requests():
    return [abi.request(center=200_000, bandwidth=200_000, demod="wfm", stereo=True),
            abi.request(center=500_000, bandwidth=10_000, demod="am"),
            abi.request(center=-300_000, bandwidth=12_500, demod="nfm")]


def feed(chain, codes, switch_at=1, lag=1, oracle=False):
    at = 0
    for k, n in enumerate(RUNS):
        if k == switch_at:
            chain.set_front_end(True, True, lag)
        part = codes[2 * at:2 * (at + n)]
        if oracle:
            chain.run(part, n)
        else:
            chain.run(part)
        at += n


def make(mode, pipelined=False, captured=False):
    ch = Chain(GPU[0], grid=GRID, rate=RATE, fmt=abi.FORMAT_CU8, mode=mode,
               max_run_samples=max(RUNS), pipelined=pipelined)
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
    return impaired_capture(sum(RUNS))


def audio_of(ch, ids):
    ch.drain()
    return [ch.audio(i) for i in ids]


def assert_same(a, b, what):
    for i, (x, y) in enumerate(zip(a, b)):
        assert x.size == y.size and x.size > 0, "%s: receiver %d sizes %d %d" % (what, i, x.size, y.size)
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), "%s: receiver %d differs" % (what, i)


def test_plain_chain_front_end_matches_oracle(codes):
    oc = OracleChain(GRID, RATE, abi.FORMAT_CU8, requests())
    feed(oc, codes, oracle=True)
    ch, ids = make(abi.CHAIN_PLAIN)
    feed(ch, codes)
    assert_same(audio_of(ch, ids), [oc.audio(i) for i in range(len(ids))], "plain vs oracle")
    est = ch.front_end_estimate()
    for name in ("measured", "iq_plausible", "samples_seen", "dc_i", "dc_q", "gain", "sin_phase", "m_ii", "m_qq", "m_iq"):
        assert getattr(est, name) == getattr(oc.fe, name), name
    # and it measured the impairment: the DC of the quantised input's last runs
    tail = codes[-2 * 60000:].astype(np.float64)
    i_mean = np.mean((tail[0::2] - 127.5) / 127.5)
    q_mean = np.mean((tail[1::2] - 127.5) / 127.5)
    assert est.measured and est.iq_plausible
    assert abs(est.dc_i - i_mean) < 2e-3 and abs(est.dc_q - q_mean) < 2e-3, (est.dc_i, i_mean, est.dc_q, q_mean)
    assert 1.05 < est.gain < 1.25 and 0.04 < est.sin_phase < 0.14
    ch.close()


@pytest.mark.parametrize("lag", [1, 2])
def test_batched_chain_front_end_matches_plain(codes, lag):
    outs = []
    for mode in (abi.CHAIN_PLAIN, abi.CHAIN_BATCHED):
        ch, ids = make(mode)
        feed(ch, codes, lag=lag)
        outs.append(audio_of(ch, ids))
        ch.close()
    assert_same(outs[0], outs[1], "batched vs plain, lag %d" % lag)


def test_pipelined_captured_chain_front_end_matches_synchronous(codes):
    outs = []
    for pipelined, captured in ((False, False), (True, True)):
        ch, ids = make(abi.CHAIN_BATCHED, pipelined=pipelined, captured=captured)
        feed(ch, codes, lag=2)
        outs.append(audio_of(ch, ids))
        ch.close()
    assert_same(outs[0], outs[1], "pipelined captured vs synchronous")


def test_pipelined_chain_refuses_lag_one():
    ch, _ = make(abi.CHAIN_BATCHED, pipelined=True)
    with pytest.raises(Exception):
        ch.set_front_end(True, True, 1)
    ch.close()
